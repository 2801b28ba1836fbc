"""Python mirror of the reference's lattice construction API over the C ABI.

    lat = DeviceLattice3D(nx, ny, nz, omega)             # MultiBlockLattice3D(nx,ny,nz,new BGKdynamics(omega))
    lat.periodicity(True, False, False)                  # lattice.periodicity().toggle(...)
    lat.define_dynamics(box, BOUNCEBACK)                 # defineDynamics(lattice, box, new BounceBack)
    lat.add_velocity_boundary(box, 0, -1)                # bc->addVelocityBoundary0N(box, lattice)
    lat.set_boundary_velocity(box, (u, 0, 0))            # setBoundaryVelocity(lattice, box, u)
    lat.initialize_at_equilibrium(box, 1.0, (0, 0, 0))   # initializeAtEquilibrium(...)
    lat.initialize()                                     # lattice.initialize()
    lat.collide_and_stream()                             # lattice.collideAndStream()
    e = lat.compute_average_energy()                     # computeAverageEnergy(lattice)

Boxes are inclusive (x0, x1, y0, y1, z0, z1), like Box3D.  Populations are
exchanged as FP64 f-bar in [x][y][z][19] order.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import native as N


class Context:
    """One GPU, one stream (plbgpu_create)."""

    def __init__(self, device: int = 0):
        self.lib = N.load()
        h = ctypes.c_void_p()
        rc = self.lib.plbgpu_create(device, ctypes.byref(h))
        if rc != N.OK:
            raise N.PlbGpuError(rc, f"cannot create a context on CUDA device {device}")
        self.h = h

    def launch_count(self) -> int:
        v = ctypes.c_ulonglong()
        N.check(self.h, self.lib.plbgpu_launch_count(self.h, ctypes.byref(v)))
        return int(v.value)

    def stream(self) -> int:
        v = ctypes.c_void_p()
        N.check(self.h, self.lib.plbgpu_get_stream(self.h, ctypes.byref(v)))
        return int(v.value or 0)

    def synchronize(self):
        N.check(self.h, self.lib.plbgpu_synchronize(self.h))

    def fp64_rate(self) -> float:
        """Measured FP64 pipe rate, adds + multiplies per second."""
        v = ctypes.c_double()
        N.check(self.h, self.lib.plbgpu_measure_fp64_rate(self.h, ctypes.byref(v)))
        return float(v.value)

    def close(self):
        if self.h:
            self.lib.plbgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class DeviceLattice3D:
    def __init__(self, nx, ny, nz, omega=1.0, precision="fp64", ctx: Context | None = None,
                 rho0=1.0, bb_rho=0.0):
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        self.shape = (int(nx), int(ny), int(nz))
        self.precision = N.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        h = ctypes.c_int()
        self._check(self.lib.plbgpu_add_domain(self.ctx.h, *self.shape, self.precision, ctypes.byref(h)))
        self.handle = h.value
        self.set_params(omega, rho0, bb_rho)

    # ----------------------------------------------------------------- helpers
    def _check(self, rc):
        return N.check(self.ctx.h, rc)

    @property
    def bounding_box(self):
        nx, ny, nz = self.shape
        return (0, nx - 1, 0, ny - 1, 0, nz - 1)

    def _box(self, box):
        return tuple(int(v) for v in (self.bounding_box if box is None else box))

    @staticmethod
    def _cells(box):
        return (box[1] - box[0] + 1) * (box[3] - box[2] + 1) * (box[5] - box[4] + 1)

    # ----------------------------------------------------------------- setup
    def set_params(self, omega, rho0=1.0, bb_rho=0.0):
        self.omega, self.rho0, self.bb_rho = float(omega), float(rho0), float(bb_rho)
        self._check(self.lib.plbgpu_set_params(self.ctx.h, self.handle, self.omega, self.rho0, self.bb_rho))

    def periodicity(self, px, py, pz):
        self._check(self.lib.plbgpu_set_periodicity(self.ctx.h, self.handle, int(bool(px)), int(bool(py)),
                                                    int(bool(pz))))

    def define_dynamics(self, box, kind):
        self._check(self.lib.plbgpu_define_dynamics(self.ctx.h, self.handle, *self._box(box), int(kind)))

    def set_kinds(self, kinds, box=None):
        box = self._box(box)
        k = np.ascontiguousarray(kinds, np.uint8).reshape(-1)
        self._check(self.lib.plbgpu_set_kinds(self.ctx.h, self.handle, *box,
                                              k.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), k.size))

    def get_kinds(self, box=None):
        box = self._box(box)
        out = np.zeros(self._cells(box), np.uint8)
        self._check(self.lib.plbgpu_get_kinds(self.ctx.h, self.handle, *box,
                                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), out.size))
        return out.reshape(box[1] - box[0] + 1, box[3] - box[2] + 1, box[5] - box[4] + 1)

    def add_boundary(self, box, kind):
        """A face, edge or corner kind over the box plus the data-processor
        record the reference's boundary instantiator integrates with it."""
        self._check(self.lib.plbgpu_add_boundary(self.ctx.h, self.handle, *self._box(box), int(kind)))

    def add_velocity_boundary(self, box, direction, orientation, zou_he=False):
        fam = N.ZOUHE_VELOCITY if zou_he else N.REG_VELOCITY
        self.add_boundary(box, N.face_kind(fam, direction, orientation))

    def add_external_velocity_edge(self, box, plane, normal1, normal2):
        """addExternalVelocityEdge{plane}{N|P}{N|P}(box, lattice) of the local
        regularized condition: finished after every step (and by
        initialize()) by the finite-difference edge processor."""
        self.add_boundary(box, N.edge_kind(plane, normal1, normal2))

    def add_external_velocity_corner(self, x, y, z, x_normal, y_normal, z_normal):
        """addExternalVelocityCorner{N|P}{N|P}{N|P}(x, y, z, lattice)."""
        self.add_boundary((x, x, y, y, z, z), N.corner_kind(x_normal, y_normal, z_normal))

    def set_velocity_condition_on_block_boundaries(self, box=None):
        """setVelocityConditionOnBlockBoundaries(lattice, box): regularized
        velocity faces, edges and corners on the box's surface."""
        self._check(self.lib.plbgpu_set_velocity_condition_on_block_boundaries(self.ctx.h, self.handle,
                                                                              *self._box(box)))

    def add_pressure_boundary(self, box, direction, orientation, zou_he=False):
        fam = N.ZOUHE_PRESSURE if zou_he else N.REG_PRESSURE
        self.add_boundary(box, N.face_kind(fam, direction, orientation))

    def processors(self):
        """The data-processor list saved lattice states describe: dicts of
        name ("%TD" for double_<Descriptor>), domain, data, level, blocks."""
        n = ctypes.c_int(0)
        self._check(self.lib.plbgpu_processor_count(self.ctx.h, self.handle, ctypes.byref(n)))
        out = []
        for i in range(n.value):
            name, data = ctypes.create_string_buffer(1024), ctypes.create_string_buffer(4096)
            dom, level, nb = (ctypes.c_longlong * 6)(), ctypes.c_longlong(0), ctypes.c_int(0)
            blocks = (ctypes.c_longlong * 64)()
            self._check(self.lib.plbgpu_get_processor(self.ctx.h, self.handle, i, name, 1024, dom, data, 4096,
                                                      ctypes.byref(level), blocks, 64, ctypes.byref(nb)))
            out.append({"name": name.value.decode(), "domain": tuple(dom), "data": data.value.decode(),
                        "level": level.value, "blocks": tuple(blocks[:nb.value])})
        return out

    def add_processor(self, name, domain, data="0 0 ", level=0, blocks=(0,)):
        dom = (ctypes.c_longlong * 6)(*[int(v) for v in domain])
        bl = (ctypes.c_longlong * max(1, len(blocks)))(*[int(v) for v in blocks])
        self._check(self.lib.plbgpu_add_processor(self.ctx.h, self.handle, name.encode(), dom, data.encode(),
                                                  int(level), bl, len(blocks)))

    def clear_processors(self):
        self._check(self.lib.plbgpu_clear_processors(self.ctx.h, self.handle))

    def load_processors(self, plb_path):
        """readXmlProcessors: append the processors a saved description lists."""
        self._check(self.lib.plbgpu_load_processors(self.ctx.h, self.handle, str(plb_path).encode()))

    def set_boundary_velocity(self, box, u):
        box = self._box(box)
        u = np.asarray(u, np.float64)
        if u.size == 3:
            self._check(self.lib.plbgpu_set_boundary_velocity(self.ctx.h, self.handle, *box, *map(float, u.ravel())))
        else:
            u = np.ascontiguousarray(u).reshape(-1)
            self._check(self.lib.plbgpu_set_boundary_velocity_field(self.ctx.h, self.handle, *box, _dp(u), u.size))

    def set_boundary_density(self, box, rho):
        box = self._box(box)
        r = np.asarray(rho, np.float64)
        if r.size == 1:
            self._check(self.lib.plbgpu_set_boundary_density(self.ctx.h, self.handle, *box, float(r)))
        else:
            r = np.ascontiguousarray(r).reshape(-1)
            self._check(self.lib.plbgpu_set_boundary_density_field(self.ctx.h, self.handle, *box, _dp(r), r.size))

    def set_external_vector(self, box, force):
        box = self._box(box)
        f = np.asarray(force, np.float64)
        if f.size == 3:
            self._check(self.lib.plbgpu_set_force(self.ctx.h, self.handle, *box, *map(float, f.ravel())))
        else:
            f = np.ascontiguousarray(f).reshape(-1)
            self._check(self.lib.plbgpu_set_force_field(self.ctx.h, self.handle, *box, _dp(f), f.size))

    def initialize_momentum_exchange(self):
        self._check(self.lib.plbgpu_initialize_momentum_exchange(self.ctx.h, self.handle))

    def initialize_at_equilibrium(self, box, rho, u):
        box = self._box(box)
        r = np.asarray(rho, np.float64)
        if r.size == 1:
            self._check(self.lib.plbgpu_initialize_at_equilibrium(self.ctx.h, self.handle, *box, float(r),
                                                                  *map(float, np.asarray(u, np.float64).ravel())))
        else:
            ru = np.concatenate([r.reshape(-1, 1), np.asarray(u, np.float64).reshape(-1, 3)], axis=1)
            ru = np.ascontiguousarray(ru).reshape(-1)
            self._check(self.lib.plbgpu_initialize_at_equilibrium_field(self.ctx.h, self.handle, *box, _dp(ru),
                                                                        ru.size))

    def initialize(self):
        self._check(self.lib.plbgpu_initialize(self.ctx.h, self.handle))

    # ----------------------------------------------------------------- transfer
    def send(self, f, box=None):
        box = self._box(box)
        a = np.ascontiguousarray(f, np.float64).reshape(-1)
        self._check(self.lib.plbgpu_send(self.ctx.h, self.handle, *box, _dp(a), a.size))

    def receive(self, box=None, out=None):
        """Populations of a box as [x][y][z][19] FP64 f-bar; `out` (a
        C-contiguous float64 array of that many values) is filled and
        returned instead of a new array."""
        box = self._box(box)
        shape = (box[1] - box[0] + 1, box[3] - box[2] + 1, box[5] - box[4] + 1, 19)
        if out is None:
            out = np.empty(shape, np.float64)
        elif (out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or out.size != self._cells(box) * 19):
            raise ValueError(f"receive: out must be a C-contiguous float64 array of {self._cells(box) * 19} values")
        flat = out.reshape(-1)
        self._check(self.lib.plbgpu_receive(self.ctx.h, self.handle, *box, _dp(flat), flat.size))
        return out.reshape(shape)

    # ----------------------------------------------------------------- stepping
    def run_host(self, f, nsteps, stats_every=0, out=None):
        """Send f, run nsteps steps and receive the state into `out` (which may
        be f) in one call (plbgpu_run_host): bit for bit send +
        collide_and_stream + receive, with the transfers overlapped with ramps
        of x-slab steps at both ends when the GPU addresses both buffers
        directly.  Returns (state, statistics records (k, 7) of every
        stats_every-th and of the last step, in the internal_statistics()
        "raw" layout)."""
        a = np.ascontiguousarray(f, np.float64).reshape(-1)
        if out is None:
            out = np.empty(self.shape + (19,))
        if not (out.flags["C_CONTIGUOUS"] and out.dtype == np.float64 and out.size == a.size):
            raise ValueError("out must be a C-contiguous float64 array of the domain's size x 19")
        nrec = (nsteps + stats_every - 1) // stats_every if stats_every > 0 else 0
        st = np.zeros((max(nrec, 1), 7))
        self._check(self.lib.plbgpu_run_host(self.ctx.h, self.handle, _dp(a), _dp(out.reshape(-1)), a.size,
                                             int(nsteps), int(stats_every), _dp(st), st.size))
        return out, st[:nrec]

    def collide_and_stream(self, nsteps=1, stats=False):
        self._check(self.lib.plbgpu_collide_and_stream(self.ctx.h, self.handle, int(nsteps), int(bool(stats))))

    def compute_rhobar_j(self):
        """BoxRhoBarJfunctional3D over the domain into the external fields."""
        self._check(self.lib.plbgpu_compute_rhobar_j(self.ctx.h, self.handle))

    def set_rhobar_j(self, rho_bar, j, box=None):
        """External fields over a box: rho_bar (cells), j (cells x 3)."""
        box = self._box(box)
        n = self._cells(box)
        v = np.empty((n, 4))
        v[:, 0] = np.asarray(rho_bar, np.float64).reshape(n)
        v[:, 1:] = np.asarray(j, np.float64).reshape(n, 3)
        self._check(self.lib.plbgpu_set_rhobar_j(self.ctx.h, self.handle, *box, _dp(v), v.size))

    def get_rhobar_j(self, box=None):
        """(rho_bar [x][y][z], j [x][y][z][3]) of the external fields."""
        box = self._box(box)
        n = self._cells(box)
        v = np.empty((n, 4))
        self._check(self.lib.plbgpu_get_rhobar_j(self.ctx.h, self.handle, *box, _dp(v), v.size))
        shape = (box[1] - box[0] + 1, box[3] - box[2] + 1, box[5] - box[4] + 1)
        return v[:, 0].reshape(shape), v[:, 1:].reshape(shape + (3,))

    def collide_and_stream_external(self, nsteps=1, recompute=True, stats=False):
        """ExternalRhoJcollideAndStream3D steps (with BoxRhoBarJfunctional3D
        after each when recompute)."""
        self._check(self.lib.plbgpu_collide_and_stream_external(self.ctx.h, self.handle, int(nsteps),
                                                                int(bool(recompute)), int(bool(stats))))

    def select_sparse_blocks(self, field, blocks):
        """computeSparseManagement over the regular distribution `blocks` =
        (bx, by, bz): blocks without a non-zero `field` value leave the
        lattice.  Returns the keep flags, shape blocks."""
        f = np.ascontiguousarray(field, np.int32).reshape(-1)
        keep = np.zeros(int(np.prod(blocks)), np.uint8)
        self._check(self.lib.plbgpu_select_sparse_blocks(
            self.ctx.h, self.handle, f.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), f.size, *map(int, blocks),
            keep.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), keep.size))
        return keep.reshape(tuple(blocks))

    def save_binary_block(self, path, what="lattice", enforce_uint=False):
        """saveBinaryBlock of the lattice (or "forced_lattice", "density",
        "velocity", "rho_bar", "j") to `path`."""
        self._check(self.lib.plbgpu_save_binary_block(self.ctx.h, self.handle, N.BLOCKS[what],
                                                      os.fsencode(path), int(bool(enforce_uint))))

    def load_binary_block(self, path, what="lattice", enforce_uint=False):
        """loadBinaryBlock into the lattice ("lattice", "forced_lattice") or
        the external fields ("rho_bar", "j")."""
        self._check(self.lib.plbgpu_load_binary_block(self.ctx.h, self.handle, N.BLOCKS[what],
                                                      os.fsencode(path), int(bool(enforce_uint))))

    def save_state(self, base, what="lattice"):
        """parallelIO::save: <base>.plb and <base>.dat (static content)."""
        self._check(self.lib.plbgpu_save_state(self.ctx.h, self.handle, N.BLOCKS[what], os.fsencode(base)))

    def load_state(self, plb_path, what="lattice"):
        """parallelIO::load(plb, block, false): the populations (and force) of a
        state, with or without dynamic content."""
        self._check(self.lib.plbgpu_load_state(self.ctx.h, self.handle, N.BLOCKS[what], os.fsencode(plb_path)))

    def save_state_dynamic(self, base, what="lattice"):
        """parallelIO::save(lattice, base, true): each cell's dynamics chain
        before its populations."""
        self._check(self.lib.plbgpu_save_state_dynamic(self.ctx.h, self.handle, N.BLOCKS[what],
                                                       os.fsencode(base)))

    def load_state_dynamic(self, plb_path, what="lattice"):
        """parallelIO::load(plb, lattice, true): cell kinds, boundary values,
        momentum-exchange directions, parameters and populations from the
        state."""
        self._check(self.lib.plbgpu_load_state_dynamic(self.ctx.h, self.handle, N.BLOCKS[what],
                                                       os.fsencode(plb_path)))

    def time_steps(self, nsteps, stats=False) -> float:
        ms = ctypes.c_float()
        self._check(self.lib.plbgpu_time_steps(self.ctx.h, self.handle, int(nsteps), int(bool(stats)),
                                               ctypes.byref(ms)))
        return float(ms.value)

    def internal_statistics(self):
        out = np.zeros(7)
        self._check(self.lib.plbgpu_get_stats(self.ctx.h, self.handle, _dp(out)))
        return dict(avRhoBar=out[0], avUSqr=out[1], maxUSqr=out[2], drag=out[3:6].copy(), count=int(out[6]),
                    raw=out)

    def reduce(self, box=None):
        box = self._box(box)
        e = ctypes.c_double()
        r = ctypes.c_double()
        self._check(self.lib.plbgpu_reduce(self.ctx.h, self.handle, *box, ctypes.byref(e), ctypes.byref(r)))
        return e.value, r.value

    def compute_velocity(self, box=None):
        """computeVelocity(lattice, box): (nx, ny, nz, 3) FP64."""
        box = self._box(box)
        out = np.empty(self._cells(box) * 3, np.float64)
        self._check(self.lib.plbgpu_compute_velocity(self.ctx.h, self.handle, *box, _dp(out), out.size))
        return out.reshape(box[1] - box[0] + 1, box[3] - box[2] + 1, box[5] - box[4] + 1, 3)

    def compute_density(self, box=None):
        """computeDensity(lattice, box): (nx, ny, nz) FP64."""
        box = self._box(box)
        out = np.empty(self._cells(box), np.float64)
        self._check(self.lib.plbgpu_compute_density(self.ctx.h, self.handle, *box, _dp(out), out.size))
        return out.reshape(box[1] - box[0] + 1, box[3] - box[2] + 1, box[5] - box[4] + 1)

    # ----------------------------------------------------------------- adjoint
    def adjoint_forward(self, T, K=0):
        """Run T steps keeping a checkpoint every K steps (discrete adjoint);
        K = 0 picks the smallest interval that fits in device memory.
        Returns the interval used."""
        self._check(self.lib.plbgpu_adjoint_forward(self.ctx.h, self.handle, int(T), int(K)))
        k = ctypes.c_int()
        self._check(self.lib.plbgpu_adjoint_interval(self.ctx.h, self.handle, ctypes.byref(k)))
        return k.value

    def _objective(self, u_target, weights, drag):
        """(kind, values) of the one objective given: "mismatch" (u_target),
        "weighted" (weights) or "drag" (a direction)."""
        given = [(k, v) for k, v in (("mismatch", u_target), ("weighted", weights), ("drag", drag)) if v is not None]
        if len(given) != 1:
            raise ValueError("give exactly one objective: u_target (mismatch), weights (weighted velocity) "
                             "or drag (a direction)")
        kind, v = given[0]
        v = np.ascontiguousarray(v, np.float64).reshape(-1)
        if kind == "drag" and v.size != 3:
            raise ValueError("drag needs a direction of 3 components")
        return kind, v

    def adjoint_backward(self, u_target=None, want_force=True, weights=None, drag=None):
        """Gradients of the last adjoint_forward run.  Objective J = 1/2 sum
        |u(T) - u*|^2 (u_target = u*), J = sum w . u(T) (weights = w, e.g.
        the mean flux), or J = drag . D(T) with D the momentum-exchange drag
        (drag = direction).  Returns J, dJ/dF (nx,ny,nz,3), dJ/domega and
        the device time of the sweep in ms."""
        kind, v = self._objective(u_target, weights, drag)
        J = ctypes.c_double()
        go = ctypes.c_double()
        ms = ctypes.c_float()
        g = np.empty(3 * self._cells(self.bounding_box) if want_force else 0, np.float64)
        gp = _dp(g) if want_force else None
        if kind == "drag":
            rc = self.lib.plbgpu_adjoint_backward_drag(self.ctx.h, self.handle, _dp(v), ctypes.byref(J), gp, g.size,
                                                       ctypes.byref(go), ctypes.byref(ms))
        else:
            fn = self.lib.plbgpu_adjoint_backward_weighted if kind == "weighted" else self.lib.plbgpu_adjoint_backward
            rc = fn(self.ctx.h, self.handle, _dp(v), v.size, ctypes.byref(J), gp, g.size, ctypes.byref(go),
                    ctypes.byref(ms))
        self._check(rc)
        grad = g.reshape(self.shape + (3,)) if want_force else None
        return J.value, grad, go.value, ms.value

    def adjoint_steady(self, weights=None, iterations=1000, want_force=True, drag=None):
        """Gradients of J = sum w . u (weights) or J = drag . D (drag) at the
        current (converged) state from `iterations` reverse steps around it.
        Returns J, dJ/dF, dJ/domega and the device time in ms."""
        kind, v = self._objective(None, weights, drag)
        J = ctypes.c_double()
        go = ctypes.c_double()
        ms = ctypes.c_float()
        g = np.empty(3 * self._cells(self.bounding_box) if want_force else 0, np.float64)
        gp = _dp(g) if want_force else None
        if kind == "drag":
            rc = self.lib.plbgpu_adjoint_steady_drag(self.ctx.h, self.handle, int(iterations), _dp(v),
                                                     ctypes.byref(J), gp, g.size, ctypes.byref(go), ctypes.byref(ms))
        else:
            rc = self.lib.plbgpu_adjoint_steady_weighted(self.ctx.h, self.handle, int(iterations), _dp(v), v.size,
                                                         ctypes.byref(J), gp, g.size, ctypes.byref(go),
                                                         ctypes.byref(ms))
        self._check(rc)
        grad = g.reshape(self.shape + (3,)) if want_force else None
        return J.value, grad, go.value, ms.value

    def tangent_linear(self, T, dforce, domega, u_target=None, weights=None, drag=None):
        """(J, grad J . (dforce, domega)) from a dual-number run of T steps;
        the objective as in adjoint_backward."""
        kind, v = self._objective(u_target, weights, drag)
        df = None if dforce is None else np.ascontiguousarray(dforce, np.float64).reshape(-1)
        dfp, dfn = (None, 0) if df is None else (_dp(df), df.size)
        J = ctypes.c_double()
        dj = ctypes.c_double()
        if kind == "drag":
            rc = self.lib.plbgpu_tangent_linear_drag(self.ctx.h, self.handle, int(T), dfp, dfn, float(domega), _dp(v),
                                                     ctypes.byref(J), ctypes.byref(dj))
        else:
            fn = self.lib.plbgpu_tangent_linear_weighted if kind == "weighted" else self.lib.plbgpu_tangent_linear
            rc = fn(self.ctx.h, self.handle, int(T), dfp, dfn, float(domega), _dp(v), v.size, ctypes.byref(J),
                    ctypes.byref(dj))
        self._check(rc)
        return J.value, dj.value

    def compute_average_energy(self, box=None):
        return self.reduce(box)[0]

    def compute_average_density(self, box=None):
        return self.reduce(box)[1]

    def device_bytes(self) -> int:
        b = ctypes.c_ulonglong()
        self._check(self.lib.plbgpu_domain_info(self.ctx.h, self.handle, None, None, None, None, ctypes.byref(b)))
        return int(b.value)

    def close(self):
        if self.handle is not None and self.ctx.h:
            self.lib.plbgpu_remove_domain(self.ctx.h, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lattice_from_description(nx, ny, nz, periodic, omega, flags, bcval=None, force=None, rho0=1.0,
                             bb_rho=0.0, precision="fp64", ctx=None, sparse=None):
    """Configure a device lattice from per-cell arrays (kinds, face values in
    3 components -- velocity, or density in component 0 -- and Guo force).
    sparse = (field, (bx, by, bz)) makes it a sparse lattice
    (select_sparse_blocks) before the momentum-exchange masks are built."""
    from .native import REG_VELOCITY, REG_PRESSURE, ZOUHE_VELOCITY, ZOUHE_PRESSURE
    lat = DeviceLattice3D(nx, ny, nz, omega, precision, ctx, rho0, bb_rho)
    lat.periodicity(*periodic)
    flags = np.ascontiguousarray(flags, np.uint8).reshape(nx, ny, nz)
    lat.set_kinds(flags)
    if sparse is not None:
        lat.select_sparse_blocks(sparse[0], sparse[1])
    kinds = set(np.unique(flags).tolist())
    if bcval is not None and any(REG_VELOCITY <= k < N.NKINDS for k in kinds):
        bc = np.asarray(bcval, np.float64).reshape(nx, ny, nz, 3)
        vel = np.zeros_like(bc)
        is_press = ((flags >= REG_PRESSURE) & (flags < REG_PRESSURE + 6)) | \
                   ((flags >= ZOUHE_PRESSURE) & (flags < ZOUHE_PRESSURE + 6))
        is_vel = ((flags >= REG_VELOCITY) & (flags < REG_PRESSURE)) | \
                 ((flags >= ZOUHE_VELOCITY) & (flags < ZOUHE_PRESSURE)) | \
                 ((flags >= N.VELOCITY_EDGE) & (flags < N.NKINDS))
        vel[is_vel] = bc[is_vel]
        vel[is_press, 0] = bc[is_press, 0]
        lat.set_boundary_velocity(None, vel)   # the three planes; density lives in component 0
    if force is not None and N.GUO in kinds:
        lat.set_external_vector(None, force)
    if N.MOMENTUM_EXCHANGE in kinds:
        lat.initialize_momentum_exchange()
    return lat
