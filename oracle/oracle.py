"""ctypes front end of the CPU oracle (oracle/plb_oracle.c).

TEST INFRASTRUCTURE.  Only the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use this module, as the checker or as the
timed CPU baseline.  The product library never calls it.
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libplboracle.so")


class _Params(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("periodic", ctypes.c_int * 3),
                ("omega", ctypes.c_double), ("rho0", ctypes.c_double), ("bbRho", ctypes.c_double)]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        u8 = ctypes.POINTER(ctypes.c_uint8)
        for name in ("orc_run",):
            fn = getattr(_lib, name)
            fn.argtypes = [ctypes.POINTER(_Params), u8, dp, dp, dp, ctypes.c_int, dp]
            fn.restype = ctypes.c_int
        _lib.orc_initialize.argtypes = [ctypes.POINTER(_Params), u8, dp, dp, dp]
        _lib.orc_reduce.argtypes = [ctypes.POINTER(_Params), u8, dp, dp, dp, dp, dp]
        _lib.orc_velocity.argtypes = [ctypes.POINTER(_Params), u8, dp, dp, dp, dp]
        _lib.orc_mebb_masks.argtypes = [ctypes.POINTER(_Params), u8, ctypes.POINTER(ctypes.c_uint32)]
        _lib.orc_rhobar_j.argtypes = [ctypes.POINTER(_Params), u8, dp, dp, dp, dp, dp]
        _lib.orc_run_external.argtypes = [ctypes.POINTER(_Params), u8, dp, dp, dp, dp, dp, ctypes.c_int,
                                          ctypes.c_int, dp]
        _lib.orc_run_external.restype = ctypes.c_int
        _lib.orc_sparse_blocks.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int32), ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.POINTER(ctypes.c_uint8)]
        _lib.orc_sparse_blocks.restype = ctypes.c_int
        _lib.orc_voxelize.argtypes = [dp, ctypes.c_long, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_int32)]
        _lib.orc_voxelize.restype = ctypes.c_int
        _lib.orc_set_threads.argtypes = [ctypes.c_int]
        _lib.orc_max_threads.restype = ctypes.c_int
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class OracleLattice:
    """A lattice description for the oracle (same fields as the golden cases)."""

    def __init__(self, nx, ny, nz, periodic, omega, flags, bcval=None, force=None,
                 rho0=1.0, bb_rho=0.0):
        self.shape = (nx, ny, nz)
        n = nx * ny * nz
        self.p = _Params(nx, ny, nz, (ctypes.c_int * 3)(*[int(v) for v in periodic]),
                         float(omega), float(rho0), float(bb_rho))
        self.flags = np.ascontiguousarray(flags, np.uint8).reshape(n)
        # the C code reads the face values of face / edge / corner cells and
        # the force of Guo cells only: a lattice without such cells gets a
        # three-value stand-in instead of n * 3 zeros (large lattices)
        kinds = np.unique(self.flags)
        needs_bc = bool(np.any((kinds >= 6) & (kinds < 50)))
        needs_force = bool(np.any(kinds == 1))
        self.bcval = np.ascontiguousarray(
            (np.zeros((n, 3)) if needs_bc else np.zeros(3)) if bcval is None else bcval, np.float64).reshape(-1)
        self.force = np.ascontiguousarray(
            (np.zeros((n, 3)) if needs_force else np.zeros(3)) if force is None else force, np.float64).reshape(-1)

    @classmethod
    def from_golden(cls, g, meta):
        return cls(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"],
                   g["flags"], g["bcval"], g["force"], meta.get("rho0", 1.0),
                   meta.get("bb_rho", 0.0))

    def _u8(self):
        return self.flags.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))

    def initialize(self, f):
        f = np.ascontiguousarray(f, np.float64).copy()
        lib().orc_initialize(ctypes.byref(self.p), self._u8(), _dp(self.bcval), _dp(self.force),
                             _dp(f))
        return f

    def run(self, f, nsteps, with_stats=True, inplace=False):
        """Advance f ([x][y][z][19] f-bar) by nsteps; returns (f, stats[nsteps, 7]).
        inplace: advance the caller's C-contiguous float64 array itself."""
        if inplace:
            if f.dtype != np.float64 or not f.flags["C_CONTIGUOUS"]:
                raise ValueError("run(inplace=True) needs a C-contiguous float64 array")
        else:
            f = np.ascontiguousarray(f, np.float64).copy()
        stats = np.zeros((max(nsteps, 1), 7)) if with_stats else None
        rc = lib().orc_run(ctypes.byref(self.p), self._u8(), _dp(self.bcval), _dp(self.force),
                           _dp(f), int(nsteps), _dp(stats) if with_stats else None)
        if rc != 0:
            raise MemoryError("oracle allocation failed")
        return f, stats

    def reduce(self, f):
        f = np.ascontiguousarray(f, np.float64)
        e = ctypes.c_double()
        d = ctypes.c_double()
        lib().orc_reduce(ctypes.byref(self.p), self._u8(), _dp(self.bcval), _dp(self.force),
                         _dp(f), ctypes.byref(e), ctypes.byref(d))
        return e.value, d.value

    def velocity(self, f):
        """computeVelocity of every cell, shape (nx, ny, nz, 3)."""
        f = np.ascontiguousarray(f, np.float64)
        out = np.zeros(self.flags.size * 3)
        lib().orc_velocity(ctypes.byref(self.p), self._u8(), _dp(self.bcval), _dp(self.force), _dp(f), _dp(out))
        return out.reshape(self.shape + (3,))

    def rhobar_j(self, f):
        """BoxRhoBarJfunctional3D: (rho-bar (nx, ny, nz), j (nx, ny, nz, 3))."""
        f = np.ascontiguousarray(f, np.float64)
        rb = np.zeros(self.flags.size)
        j = np.zeros(self.flags.size * 3)
        lib().orc_rhobar_j(ctypes.byref(self.p), self._u8(), _dp(self.bcval), _dp(self.force), _dp(f),
                           _dp(rb), _dp(j))
        return rb.reshape(self.shape), j.reshape(self.shape + (3,))

    def run_external(self, f, rho_bar, j, nsteps, recompute=True):
        """ExternalRhoJcollideAndStream3D for nsteps with the given fields (and,
        with recompute, BoxRhoBarJfunctional3D after each step); returns
        (f, rho_bar, j, stats[nsteps, 7])."""
        f = np.ascontiguousarray(f, np.float64).copy()
        rb = np.ascontiguousarray(rho_bar, np.float64).reshape(self.shape).copy()
        jj = np.ascontiguousarray(j, np.float64).reshape(self.shape + (3,)).copy()
        stats = np.zeros((max(nsteps, 1), 7))
        rc = lib().orc_run_external(ctypes.byref(self.p), self._u8(), _dp(self.bcval), _dp(self.force),
                                    _dp(f), _dp(rb), _dp(jj), int(bool(recompute)), int(nsteps), _dp(stats))
        if rc != 0:
            raise MemoryError("oracle allocation failed")
        return f, rb, jj, stats

    def mebb_masks(self):
        out = np.zeros(self.flags.size, np.uint32)
        lib().orc_mebb_masks(ctypes.byref(self.p), self._u8(),
                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
        return out


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return int(lib().orc_max_threads())


def binary_block(records, enforce_uint=False):
    """saveBinaryBlock's byte stream for a block whose cells serialize to
    `records` (float64, cells in x-major order, z fastest, the values of one
    cell contiguous): the byte count (uint64, or uint32 with enforce_uint) and
    the data, each base64-encoded on its own with '=' padding and no line
    breaks (io/serializerIO_3D.cpp:37-49, io/serializerIO.cpp:64-86,
    io/base64.hh:35-115, multiBlock/multiBlockSerializer3D.cpp:61-129)."""
    import base64
    import struct
    data = np.ascontiguousarray(records, dtype="<f8").tobytes()
    head = struct.pack("<I" if enforce_uint else "<Q", len(data))
    return base64.b64encode(head) + base64.b64encode(data)


def sparse_blocks(field, blocks):
    """computeSparseManagement's block selection over the regular distribution
    with blocks = (bx, by, bz): keep[bx, by, bz] (1 = kept)."""
    field = np.ascontiguousarray(field, np.int32)
    nx, ny, nz = field.shape
    bx, by, bz = blocks
    keep = np.zeros(bx * by * bz, np.uint8)
    lib().orc_sparse_blocks(nx, ny, nz, field.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), bx, by, bz,
                            keep.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    return keep.reshape(bx, by, bz)


def voxelize(triangles, shape, border_width=1):
    """voxelize(mesh, Box3D(0..nx-1, ...), borderWidth) restated: voxel flags
    (1 outside, 2 outerBorder, 3 inside, 4 innerBorder) of the closed mesh
    given as triangles (t, 3, 3) in lattice coordinates."""
    tri = np.ascontiguousarray(triangles, np.float64).reshape(-1, 9)
    nx, ny, nz = shape
    flags = np.zeros(nx * ny * nz, np.int32)
    rc = lib().orc_voxelize(_dp(tri), tri.shape[0], nx, ny, nz, int(border_width),
                            flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    return flags.reshape(nx, ny, nz)


def regular_ranges(n, b):
    """Block boundaries of createRegularDistribution3D along one axis."""
    starts = [0]
    for i in range(b):
        starts.append(starts[-1] + n // b + (1 if i < n % b else 0))
    return starts


def sparse_cell_mask(shape, blocks, keep):
    """Cells inside kept blocks (bool [nx, ny, nz])."""
    mask = np.zeros(shape, bool)
    r = [regular_ranges(n, b) for n, b in zip(shape, blocks)]
    for ix in range(blocks[0]):
        for iy in range(blocks[1]):
            for iz in range(blocks[2]):
                if keep[ix, iy, iz]:
                    mask[r[0][ix]:r[0][ix + 1], r[1][iy]:r[1][iy + 1], r[2][iz]:r[2][iz + 1]] = True
    return mask


def state_files(records, shape, cell_dim, family, descriptor, dat_name):
    """parallelIO::save(block, base, false) of a block as one component, the
    whole bounding box: the description (<base>.plb, in the layout of the
    reference's XML writer: io/multiBlockWriter3D.cpp:53-137,
    libraryInterfaces/TINYXML_xmlIO.hh:229-272) and the raw records
    (<base>.dat: cells x-major, z fastest, `cell_dim` float64 each, no header;
    io/mpiParallelIO.cpp:92-150).  Returns (plb text, dat bytes)."""
    data = np.ascontiguousarray(records, dtype="<f8").tobytes()
    nx, ny, nz = shape
    box = f"0 {nx - 1} 0 {ny - 1} 0 {nz - 1}"
    lines = ['<?xml version="1.0" ?>', "<Block3D>", "    <General>",
             f"        <Family> {family} </Family>", "        <Datatype> double </Datatype>"]
    if descriptor:
        lines.append(f"        <Descriptor> {descriptor} </Descriptor>")
    lines += [f"        <cellDim> {cell_dim} </cellDim>", "        <dynamicContent> False </dynamicContent>",
              "        <globalId> 0 </globalId>", "    </General>", "    <Structure>",
              f"        <BoundingBox> {box} </BoundingBox>", "        <EnvelopeWidth> 1 </EnvelopeWidth>",
              "        <GridLevel> 0 </GridLevel>", "        <NumComponents> 1 </NumComponents>", "    </Structure>",
              "    <Data>", f"        <File> {dat_name} </File>", f"        <Component> {box} </Component>",
              f"        <Offsets> {len(data)} </Offsets>", "    </Data>", "</Block3D>", ""]
    return "\n".join(lines), data



# ---------------------------------------------------------------- states with dynamic content

_BASIC_DYNAMICS = ["BGK", "BGK_ExternalForce_Guo", "BGK_Incompressible", "BounceBack", "MomentumExchangeBounceBack",
                   "NoDynamics"]
_FACE_FAMILIES = ["Boundary_RegularizedVelocity", "Boundary_RegularizedDensity", "Boundary_ZouHeVelocity",
                  "Boundary_ZouHePressure"]
_K_FACE, _K_EDGE, _K_END = 6, 30, 50
_K_INCBGK, _K_BB, _K_MEBB, _K_NODYN = 2, 3, 4, 5


def dynamics_name(kind):
    """Registry name of the dynamics class of a cell kind (the names of
    meta::dynamicsRegistration, e.g. regularizedBoundaryDynamics.hh:44-47)."""
    if kind < _K_FACE:
        return _BASIC_DYNAMICS[kind]
    if kind < _K_EDGE:
        r = kind - _K_FACE
        face = r % 6
        return f"{_FACE_FAMILIES[r // 6]}_{face // 2}_{1 if face % 2 else -1}"
    return "Boundary_StoreVelocity"


def _is_density_kind(kind):
    return 12 <= kind < 18 or 24 <= kind < 30


def _d(v):
    return (8, struct.pack("<d", v))


def _cell_values(kind, bc, mask, omega, rho0, bb_rho):
    """What each dynamics of the cell's chain serializes, outermost first
    (core/dynamics.hh:119-122, 445-450, 770-773, 955-958;
    boundaryCondition/bounceBackModels.hh:75-84; boundaryDynamics.hh:238-242,
    315-321): a list of (value size, bytes) per dynamics."""
    if kind in (0, 1):
        return [[_d(omega)]]
    if kind == _K_INCBGK:
        return [[_d(omega), _d(1.0 / rho0)]]
    if kind in (_K_BB, _K_NODYN):
        return [[_d(bb_rho)]]
    if kind == _K_MEBB:
        dirs = [i for i in range(19) if (int(mask) >> i) & 1]
        return [[_d(bb_rho), (4, struct.pack("<i", len(dirs)))] + [(8, struct.pack("<q", i)) for i in dirs]
                + [(8, struct.pack("<q", a)) for a in range(3)]]
    if _is_density_kind(kind):
        stored = [_d(float(bc[0]) - 1.0)]
    else:
        stored = [_d(float(bc[a])) for a in range(3)]
    return [stored + [(1, bytes([1 if kind >= _K_EDGE else 0]))], [_d(omega)]]


def _chain_bytes(ids, values):
    """HierarchicSerializer (core/hierarchicSerializer.h:152-230): numDynamics,
    then per dynamics its id, its number of values and runs of values of one
    size (size, count, values)."""
    out = bytearray(struct.pack("<i", len(ids)))
    for did, vals in zip(ids, values):
        out += struct.pack("<ii", did, len(vals))
        i = 0
        while i < len(vals):
            j = i
            while j < len(vals) and vals[j][0] == vals[i][0]:
                j += 1
            out += struct.pack("<ii", vals[i][0], j - i)
            for _, b in vals[i:j]:
                out += b
            i = j
    return bytes(out)


def _own_ids(kind):
    return 31 if kind >= _K_EDGE else kind + 1


def dynamic_state_files(kinds, bcval, masks, records, cell_dim, descriptor, dat_name, omega, rho0, bb_rho,
                        ids=None):
    """parallelIO::save(lattice, base, true) of a lattice as one component:
    every cell's dynamics chain, then its `cell_dim` static values
    (atomicBlock/blockLattice3D.hh:703-722), and a description whose
    DynamicsDict maps the ids to names (io/multiBlockWriter3D.cpp:92-110).
    ids: name -> id (default: the library's own ids, kind + 1 and 31 for
    stored-velocity cells).  Returns (plb text, dat bytes)."""
    shape = kinds.shape
    recs = np.ascontiguousarray(records, dtype="<f8").reshape(-1, cell_dim)
    kf = kinds.reshape(-1)
    bf = np.asarray(bcval, dtype=np.float64).reshape(-1, 3)
    mf = np.asarray(masks).reshape(-1) if masks is not None else np.zeros(kf.size, np.uint32)
    idof = (lambda name, k: ids[name]) if ids else (lambda name, k: 1 if name == "BGK" else _own_ids(k))
    out = bytearray()
    dict_ = {}
    for c in range(kf.size):
        k = int(kf[c])
        if k == 255:   # outside the lattice of a sparse domain: NoDynamics, zero populations
            k = _K_NODYN
        names = [dynamics_name(k)] + (["BGK"] if k >= _K_FACE else [])
        chain_ids = [idof(names[0], k)] + ([idof("BGK", 0)] if k >= _K_FACE else [])
        for nm, i in zip(names, chain_ids):
            dict_[nm] = i
        out += _chain_bytes(chain_ids, _cell_values(k, bf[c], mf[c], omega, rho0, bb_rho))
        out += recs[c].tobytes()
    plb, _ = state_files(np.zeros((0, cell_dim)), shape, cell_dim, "BlockLattice3D", descriptor, dat_name)
    plb = plb.replace("<dynamicContent> False </dynamicContent>", "<dynamicContent> True </dynamicContent>")
    plb = plb.replace("<Offsets> 0 </Offsets>", f"<Offsets> {len(out)} </Offsets>")
    block = ["        <DynamicsDict>"] + [f"            <{n}> {dict_[n]} </{n}>" for n in sorted(dict_)] + \
            ["        </DynamicsDict>"]
    plb = plb.replace("    </Data>", "\n".join(block) + "\n    </Data>")
    return plb, bytes(out)


def _surface_kind(x, y, z, shape):
    side = [(-1 if q == 0 else (1 if q == n - 1 else 0)) for q, n in zip((x, y, z), shape)]
    count = sum(s != 0 for s in side)
    if count == 3:
        return 42 + 4 * (side[0] > 0) + 2 * (side[1] > 0) + (side[2] > 0)
    if count == 2:
        plane = [i for i in range(3) if side[i] == 0][0]
        return _K_EDGE + 4 * plane + 2 * (side[(plane + 1) % 3] > 0) + (side[(plane + 2) % 3] > 0)
    raise ValueError("a stored-velocity cell that is not on an edge or corner of the lattice")


def read_dynamic_state(plb, dat, shape):
    """Decode a lattice state with dynamic content (any number of components):
    kinds, boundary values (velocity, or the density rho-bar + 1 in [..., 0]),
    momentum-exchange fluid-direction masks, static records, and the sets of
    omegas, 1/rho0s and wall densities the cells hold
    (blockLattice3D.hh:812-845, hierarchicSerializer.h)."""
    import re
    cell_dim = int(re.search(r"<cellDim>([^<]*)</cellDim>", plb).group(1))
    boxes = [tuple(map(int, m.split())) for m in re.findall(r"<Component[^>]*>([^<]*)</Component>", plb)]
    offsets = list(map(int, re.search(r"<Offsets>([^<]*)</Offsets>", plb).group(1).split()))
    dd = re.search(r"<DynamicsDict>(.*?)</DynamicsDict>", plb, re.S).group(1)
    names = {int(v): n for n, v in re.findall(r"<([^/>]+)>\s*(-?\d+)\s*</\1>", dd)}
    name_kind = {dynamics_name(k): k for k in range(_K_EDGE)}
    nx, ny, nz = shape
    kinds = np.full(shape, 255, np.uint8)
    bc = np.zeros(shape + (3,))
    masks = np.zeros(shape, np.uint32)
    recs = np.zeros(shape + (cell_dim,))
    omegas, inv_rho0s, rhos = set(), set(), set()
    pos, start = 0, 0
    for (x0, x1, y0, y1, z0, z1), end in zip(boxes, offsets):
        for x in range(x0, x1 + 1):
            for y in range(y0, y1 + 1):
                for z in range(z0, z1 + 1):
                    (nd,) = struct.unpack_from("<i", dat, pos)
                    pos += 4
                    chain = []
                    for _ in range(nd):
                        did, nv = struct.unpack_from("<ii", dat, pos)
                        pos += 8
                        vals = []
                        while len(vals) < nv:
                            size, count = struct.unpack_from("<ii", dat, pos)
                            pos += 8
                            vals += [dat[pos + r * size:pos + (r + 1) * size] for r in range(count)]
                            pos += size * count
                        chain.append((names[did], vals))
                    top, v = chain[0]
                    if top == "Boundary_StoreVelocity" or name_kind.get(top, -1) >= _K_FACE:
                        k = _surface_kind(x, y, z, shape) if top == "Boundary_StoreVelocity" else name_kind[top]
                        if _is_density_kind(k):
                            bc[x, y, z, 0] = struct.unpack("<d", v[0])[0] + 1.0
                        else:
                            bc[x, y, z] = [struct.unpack("<d", v[a])[0] for a in range(3)]
                        assert chain[1][0] == "BGK"
                        omegas.add(struct.unpack("<d", chain[1][1][0])[0])
                    else:
                        k = name_kind[top]
                        first = struct.unpack("<d", v[0])[0]
                        if k in (0, 1):
                            omegas.add(first)
                        elif k == _K_INCBGK:
                            omegas.add(first)
                            inv_rho0s.add(struct.unpack("<d", v[1])[0])
                        else:
                            rhos.add(first)
                        if k == _K_MEBB:
                            (n,) = struct.unpack("<i", v[1])
                            for b in v[2:2 + n]:
                                masks[x, y, z] |= np.uint32(1 << struct.unpack("<q", b)[0])
                    kinds[x, y, z] = k
                    recs[x, y, z] = np.frombuffer(dat, "<f8", cell_dim, pos)
                    pos += 8 * cell_dim
        assert pos == end, (pos, end)
        start = end
    return dict(kinds=kinds, bc=bc, masks=masks, records=recs, omegas=omegas, inv_rho0s=inv_rho0s, rhos=rhos,
                names=names)
