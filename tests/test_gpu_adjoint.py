"""Discrete adjoint of the collide-and-stream step.

The gradients of J = 1/2 sum |u(T) - u*|^2, of a weighted velocity (the mean
flux) and of the momentum-exchange drag with respect to the per-cell Guo
force and omega, from the checkpointed reverse sweep and from the steady
adjoint, are checked against
  - a forward-mode dual-number directional derivative of the same GPU FP64
    path (plbgpu_tangent_linear): agreement to 1e-9 relative;
  - central finite differences of the CPU oracle (the reference's FP64 step,
    bit for bit), or of converged FP64 runs for the steady adjoint:
    agreement to 1e-5 relative.
"""
import numpy as np
import pytest

import oracle as O
from palabos_gb300 import native as N
from palabos_gb300 import workloads

pytestmark = pytest.mark.gpu


def _case(shape=(12, 10, 8), T=24, seed=3):
    wl = workloads.forced_channel(shape, omega=1.6, seed=seed, sigma=1e-4, drive=1e-3)
    rng = np.random.default_rng(seed + 1)
    u_target = 1e-3 * rng.standard_normal(shape + (3,))
    return wl, u_target, T


def _oracle_objective(wl, f0, force, omega, T, u_target):
    ol = O.OracleLattice(*wl.shape, wl.periodic, omega, wl.kinds, None, force)
    f, _ = ol.run(f0, T, with_stats=False)
    u = ol.velocity(f)
    return 0.5 * float(np.sum((u - u_target) ** 2))


@pytest.mark.parametrize("K", [0, 1, 4, 24])
def test_adjoint_matches_tangent_linear(K):
    wl, u_target, T = _case()
    lat = wl.lattice("fp64")
    f0 = lat.receive()
    rng = np.random.default_rng(11)
    dF = rng.standard_normal(wl.shape + (3,))
    dF[wl.kinds != 1] = 0.0
    domega = 0.7
    J_t, dJ = lat.tangent_linear(T, dF, domega, u_target)
    used = lat.adjoint_forward(T, K)
    assert used == (K if K else 1)     # K = 0: a small domain keeps every state
    J, gF, gO, _ = lat.adjoint_backward(u_target)
    assert J == pytest.approx(J_t, rel=1e-13)
    adj = float(np.sum(gF * dF)) + gO * domega
    assert adj == pytest.approx(dJ, rel=1e-9), (adj, dJ)
    # the domain continued from step T: same state as a plain run
    lat2 = wl.lattice("fp64")
    lat2.send(f0)
    lat2.collide_and_stream(T)
    assert np.array_equal(lat.receive(), lat2.receive())


def test_adjoint_matches_reference_finite_differences():
    wl, u_target, T = _case()
    lat = wl.lattice("fp64")
    f0 = lat.receive()
    lat.adjoint_forward(T, 6)
    J, gF, gO, _ = lat.adjoint_backward(u_target)
    assert J == pytest.approx(_oracle_objective(wl, f0, wl.force, wl.omega, T, u_target), rel=1e-12)
    rng = np.random.default_rng(5)
    fluid = np.argwhere(wl.kinds == 1)
    h = 1e-6
    for k in range(6):
        x, y, z = fluid[rng.integers(len(fluid))]
        d = int(rng.integers(3))
        fp = wl.force.copy()
        fm = wl.force.copy()
        fp[x, y, z, d] += h
        fm[x, y, z, d] -= h
        fd = (_oracle_objective(wl, f0, fp, wl.omega, T, u_target) -
              _oracle_objective(wl, f0, fm, wl.omega, T, u_target)) / (2 * h)
        assert gF[x, y, z, d] == pytest.approx(fd, rel=1e-5, abs=1e-12 * max(1.0, abs(fd))), (k, gF[x, y, z, d], fd)
    fd = (_oracle_objective(wl, f0, wl.force, wl.omega + h, T, u_target) -
          _oracle_objective(wl, f0, wl.force, wl.omega - h, T, u_target)) / (2 * h)
    assert gO == pytest.approx(fd, rel=1e-5), (gO, fd)


def test_fp32_adjoint_tracks_fp64():
    wl, u_target, T = _case()
    g = {}
    for prec in ("fp64", "fp32"):
        lat = wl.lattice(prec)
        lat.adjoint_forward(T, 6)
        J, gF, gO, _ = lat.adjoint_backward(u_target)
        g[prec] = (J, gF, gO)
    J64, g64, o64 = g["fp64"]
    J32, g32, o32 = g["fp32"]
    assert J32 == pytest.approx(J64, rel=1e-4)
    assert np.abs(g32 - g64).max() <= 1e-3 * np.abs(g64).max()
    assert o32 == pytest.approx(o64, rel=1e-3)


def test_adjoint_rejects_unsupported_cells():
    from palabos_gb300 import DeviceLattice3D, PlbGpuError
    lat = DeviceLattice3D(6, 6, 6, 1.2)
    lat.define_dynamics((0, 5, 0, 5, 0, 5), N.GUO)
    lat.define_dynamics((2, 2, 2, 2, 2, 2), N.edge_kind(0, -1, -1))   # an edge reading Guo-forced cells
    with pytest.raises(PlbGpuError):
        lat.adjoint_forward(4, 2)
    lat2 = DeviceLattice3D(6, 6, 6, 1.2)
    with pytest.raises(PlbGpuError):
        lat2.adjoint_forward(5, 2)      # K must divide T
    with pytest.raises(PlbGpuError):
        lat2.adjoint_forward(4, -1)
    with pytest.raises(PlbGpuError):
        lat2.adjoint_backward(np.zeros((6, 6, 6, 3)))   # no forward run yet
    import ctypes
    k = ctypes.c_int()
    assert N.ERRORS[lat2.lib.plbgpu_adjoint_interval(lat2.ctx.h, lat2.handle, ctypes.byref(k))] == "PLBGPU_ERR_STATE"


@pytest.mark.slow
def test_forced_channel_gradient_full_size():
    """The Guo-forced channel at full size (128x64x64, Guo forcing, T = 2000, checkpoint
    every 100 steps): adjoint gradient against central finite differences of
    the CPU oracle for omega and three force components, to 1e-5 relative."""
    T, K = 2000, 100
    tgt = workloads.forced_channel(seed=5678).lattice("fp64")
    tgt.collide_and_stream(T)
    u_target = tgt.compute_velocity()
    wl = workloads.forced_channel(seed=1234)
    lat = wl.lattice("fp64")
    f0 = lat.receive()
    lat.adjoint_forward(T, K)
    J, gF, gO, _ = lat.adjoint_backward(u_target)
    O.set_threads(O.max_threads())
    assert J == pytest.approx(_oracle_objective(wl, f0, wl.force, wl.omega, T, u_target), rel=1e-10)
    h = 1e-5
    fd = (_oracle_objective(wl, f0, wl.force, wl.omega + h, T, u_target) -
          _oracle_objective(wl, f0, wl.force, wl.omega - h, T, u_target)) / (2 * h)
    assert gO == pytest.approx(fd, rel=1e-5), (gO, fd)
    rng = np.random.default_rng(2)
    fluid = np.argwhere(wl.kinds == 1)
    hF = 1e-8
    for _ in range(3):
        x, y, z = fluid[rng.integers(len(fluid))]
        fp = wl.force.copy()
        fm = wl.force.copy()
        fp[x, y, z, 0] += hF
        fm[x, y, z, 0] -= hF
        fd = (_oracle_objective(wl, f0, fp, wl.omega, T, u_target) -
              _oracle_objective(wl, f0, fm, wl.omega, T, u_target)) / (2 * hF)
        assert gF[x, y, z, 0] == pytest.approx(fd, rel=1e-5), (gF[x, y, z, 0], fd)


def _flux_weights(shape):
    """J = mean x-velocity over all cells (the superficial velocity)."""
    w = np.zeros(shape + (3,))
    w[..., 0] = 1.0 / np.prod(shape)
    return w


@pytest.mark.parametrize("K", [1, 6])
def test_weighted_adjoint_matches_tangent_linear(K):
    wl, _, T = _case()
    rng = np.random.default_rng(21)
    w = rng.standard_normal(wl.shape + (3,))
    lat = wl.lattice("fp64")
    dF = rng.standard_normal(wl.shape + (3,))
    dF[wl.kinds != 1] = 0.0
    J_t, dJ = lat.tangent_linear(T, dF, -0.4, weights=w)
    lat.adjoint_forward(T, K)
    J, gF, gO, _ = lat.adjoint_backward(weights=w)
    assert J == pytest.approx(J_t, rel=1e-13)
    adj = float(np.sum(gF * dF)) + gO * -0.4
    assert adj == pytest.approx(dJ, rel=1e-9), (adj, dJ)


def test_weighted_adjoint_matches_reference_finite_differences():
    """Mean-flux objective against central differences of the CPU oracle."""
    wl, _, T = _case()
    w = _flux_weights(wl.shape)
    lat = wl.lattice("fp64")
    f0 = lat.receive()
    lat.adjoint_forward(T, 4)
    J, gF, gO, _ = lat.adjoint_backward(weights=w)

    def objective(force, omega):
        ol = O.OracleLattice(*wl.shape, wl.periodic, omega, wl.kinds, None, force)
        f, _ = ol.run(f0, T, with_stats=False)
        return float(np.sum(ol.velocity(f) * w))

    assert J == pytest.approx(objective(wl.force, wl.omega), rel=1e-12)
    h = 1e-6
    fd = (objective(wl.force, wl.omega + h) - objective(wl.force, wl.omega - h)) / (2 * h)
    assert gO == pytest.approx(fd, rel=1e-5), (gO, fd)
    rng = np.random.default_rng(8)
    fluid = np.argwhere(wl.kinds == 1)
    for _ in range(3):
        x, y, z = fluid[rng.integers(len(fluid))]
        fp = wl.force.copy()
        fm = wl.force.copy()
        fp[x, y, z, 0] += h
        fm[x, y, z, 0] -= h
        fd = (objective(fp, wl.omega) - objective(fm, wl.omega)) / (2 * h)
        assert gF[x, y, z, 0] == pytest.approx(fd, rel=1e-5), (gF[x, y, z, 0], fd)


def _converged_packing(omega, force=None, steps=6000, prec="fp64"):
    wl = workloads.sphere_packing(n=20, porosity=0.6, rmin=2.5, rmax=4.5, seed=5, force=1e-5, omega=omega)
    if force is not None:
        wl.force = force
    lat = wl.lattice(prec)
    lat.collide_and_stream(steps)
    return wl, lat


def test_steady_adjoint_permeability_gradient():
    """dk/domega and dk/dF of a converged sphere packing from the steady
    adjoint, against central differences of converged forward runs."""
    omega = 1.2
    wl, lat = _converged_packing(omega)
    w = _flux_weights(wl.shape)
    u = lat.compute_velocity()
    J, gF, gO, _ = lat.adjoint_steady(w, 3000)
    assert J == pytest.approx(float(np.mean(u[..., 0])), rel=1e-12)
    J2, _, gO2, _ = lat.adjoint_steady(w, 6000, want_force=False)
    assert gO2 == pytest.approx(gO, rel=1e-9)       # the sum has converged

    def flux(om, force=None):
        _, l2 = _converged_packing(om, force)
        return float(np.mean(l2.compute_velocity()[..., 0]))

    h = 1e-5
    fd = (flux(omega + h) - flux(omega - h)) / (2 * h)
    assert gO == pytest.approx(fd, rel=1e-5), (gO, fd)
    k = workloads.permeability(J, 1e-5, omega)
    dk = workloads.permeability_derivative(J, gO, 1e-5, omega)
    k_p = workloads.permeability(flux(omega + h), 1e-5, omega + h)
    k_m = workloads.permeability(flux(omega - h), 1e-5, omega - h)
    assert dk == pytest.approx((k_p - k_m) / (2 * h), rel=1e-5)
    assert k > 0
    rng = np.random.default_rng(4)
    fluid = np.argwhere(wl.kinds == 1)
    hF = 1e-8
    for _ in range(2):
        x, y, z = fluid[rng.integers(len(fluid))]
        fp = wl.force.copy()
        fm = wl.force.copy()
        fp[x, y, z, 0] += hF
        fm[x, y, z, 0] -= hF
        fd = (flux(omega, fp) - flux(omega, fm)) / (2 * hF)
        assert gF[x, y, z, 0] == pytest.approx(fd, rel=1e-5), (gF[x, y, z, 0], fd)


def test_steady_adjoint_fp32_tracks_fp64():
    g = {}
    for prec in ("fp64", "fp32"):
        wl, lat = _converged_packing(1.2, prec=prec)
        J, gF, gO, _ = lat.adjoint_steady(_flux_weights(wl.shape), 3000)
        g[prec] = (J, gF, gO)
    assert g["fp32"][0] == pytest.approx(g["fp64"][0], rel=1e-4)
    assert g["fp32"][2] == pytest.approx(g["fp64"][2], rel=1e-3)
    assert np.abs(g["fp32"][1] - g["fp64"][1]).max() <= 1e-3 * np.abs(g["fp64"][1]).max()


def _obstacle_channel(shape=(12, 10, 8), T=24, seed=3):
    """The forced channel with a 2x2x2 momentum-exchange block in its middle."""
    wl, _, T = _case(shape, T, seed)
    kinds = wl.kinds.copy()
    cx, cy, cz = (s // 2 for s in shape)
    kinds[cx - 1:cx + 1, cy - 1:cy + 1, cz - 1:cz + 1] = N.MOMENTUM_EXCHANGE
    wl.kinds = kinds
    return wl, T


DRAG_DIR = np.array([1.0, 0.3, -0.2])


def _oracle_drag(wl, f0, force, omega, T):
    """direction . drag of the state after T steps (the drag step T + 1 records)."""
    ol = O.OracleLattice(*wl.shape, wl.periodic, omega, wl.kinds, None, force)
    f, _ = ol.run(f0, T, with_stats=False)
    _, st = ol.run(f, 1, with_stats=True)
    return float(np.dot(DRAG_DIR, st[0, 3:6]))


@pytest.mark.parametrize("K", [1, 4])
def test_drag_adjoint_matches_tangent_linear(K):
    wl, T = _obstacle_channel()
    lat = wl.lattice("fp64")
    rng = np.random.default_rng(31)
    dF = rng.standard_normal(wl.shape + (3,))
    dF[wl.kinds != N.GUO] = 0.0
    J_t, dJ = lat.tangent_linear(T, dF, 0.3, drag=DRAG_DIR)
    lat.adjoint_forward(T, K)
    J, gF, gO, _ = lat.adjoint_backward(drag=DRAG_DIR)
    assert J == pytest.approx(J_t, rel=1e-13)
    assert J != 0.0
    adj = float(np.sum(gF * dF)) + gO * 0.3
    assert adj == pytest.approx(dJ, rel=1e-9), (adj, dJ)


def test_drag_adjoint_matches_reference_finite_differences():
    wl, T = _obstacle_channel()
    lat = wl.lattice("fp64")
    f0 = lat.receive()
    lat.adjoint_forward(T, 6)
    J, gF, gO, _ = lat.adjoint_backward(drag=DRAG_DIR)
    assert J == pytest.approx(_oracle_drag(wl, f0, wl.force, wl.omega, T), rel=1e-12)
    h = 1e-6
    fd = (_oracle_drag(wl, f0, wl.force, wl.omega + h, T) - _oracle_drag(wl, f0, wl.force, wl.omega - h, T)) / (2 * h)
    assert gO == pytest.approx(fd, rel=1e-5), (gO, fd)
    rng = np.random.default_rng(9)
    fluid = np.argwhere(wl.kinds == N.GUO)
    for _ in range(3):
        x, y, z = fluid[rng.integers(len(fluid))]
        fp = wl.force.copy()
        fm = wl.force.copy()
        fp[x, y, z, 0] += h
        fm[x, y, z, 0] -= h
        fd = (_oracle_drag(wl, f0, fp, wl.omega, T) - _oracle_drag(wl, f0, fm, wl.omega, T)) / (2 * h)
        assert gF[x, y, z, 0] == pytest.approx(fd, rel=1e-5, abs=1e-9 * abs(gF).max()), (gF[x, y, z, 0], fd)


def _converged_sphere_drag(omega, force=None, steps=8000):
    """Channel 16^3, periodic x, bounce-back walls at the y and z ends, Guo
    force 1e-5 along x, momentum-exchange sphere of radius 3 in the middle:
    the sphere takes a share of the applied force that depends on the flow
    (in a fully periodic box it would take all of it, whatever omega)."""
    n = 16
    X, Y, Z = np.meshgrid(*(np.arange(n),) * 3, indexing="ij")
    kinds = np.full((n, n, n), N.GUO, np.uint8)
    kinds[:, 0, :] = kinds[:, -1, :] = kinds[:, :, 0] = kinds[:, :, -1] = N.BOUNCEBACK
    kinds[(X - 7.5) ** 2 + (Y - 7.5) ** 2 + (Z - 7.5) ** 2 <= 9.0] = N.MOMENTUM_EXCHANGE
    F = np.zeros((n, n, n, 3))
    F[..., 0] = 1e-5
    wl = workloads.Workload("sphere_in_channel", (n, n, n), omega, (1, 0, 0), kinds,
                            force=F if force is None else force)
    lat = wl.lattice("fp64")
    lat.collide_and_stream(steps)
    return wl, lat


def test_steady_drag_adjoint():
    omega = 1.0
    wl, lat = _converged_sphere_drag(omega)
    J, gF, gO, _ = lat.adjoint_steady(iterations=4000, drag=DRAG_DIR)
    _, _, gO2, _ = lat.adjoint_steady(iterations=8000, want_force=False, drag=DRAG_DIR)
    assert gO2 == pytest.approx(gO, rel=1e-9, abs=1e-15)

    def drag(om, force=None):
        _, l2 = _converged_sphere_drag(om, force)
        J2, _, _, _ = l2.adjoint_steady(iterations=0, want_force=False, drag=DRAG_DIR)
        return J2

    assert J == pytest.approx(drag(omega), rel=1e-13)
    assert 0 < J < 1e-5 * 14 * 14 * 16      # a share of the applied force
    h = 1e-5
    fd = (drag(omega + h) - drag(omega - h)) / (2 * h)
    assert gO == pytest.approx(fd, rel=1e-5, abs=1e-9 * J), (gO, fd)
    rng = np.random.default_rng(12)
    fluid = np.argwhere(wl.kinds == N.GUO)
    hF = 1e-8
    for _ in range(2):
        x, y, z = fluid[rng.integers(len(fluid))]
        fp = wl.force.copy()
        fm = wl.force.copy()
        fp[x, y, z, 0] += hF
        fm[x, y, z, 0] -= hF
        fd = (drag(omega, fp) - drag(omega, fm)) / (2 * hF)
        assert gF[x, y, z, 0] == pytest.approx(fd, rel=1e-5), (gF[x, y, z, 0], fd)


def test_adjoint_objective_arguments():
    from palabos_gb300 import DeviceLattice3D, PlbGpuError
    lat = DeviceLattice3D(6, 6, 6, 1.2)
    with pytest.raises(ValueError):
        lat.adjoint_backward()                       # neither objective
    with pytest.raises(ValueError):
        lat.tangent_linear(2, None, 0.1, np.zeros((6, 6, 6, 3)), np.zeros((6, 6, 6, 3)))
    with pytest.raises(PlbGpuError):
        lat.adjoint_steady(np.zeros((6, 6, 3)), 4)   # wrong size
    with pytest.raises(PlbGpuError):
        lat.adjoint_steady(np.zeros((6, 6, 6, 3)), -1)
    with pytest.raises(ValueError):
        lat.adjoint_backward(drag=(1.0, 0.0))            # a direction has 3 components
    with pytest.raises(PlbGpuError):
        lat.adjoint_steady(iterations=2, drag=(1.0, 0.0, 0.0))   # no momentum-exchange masks


def _face_channel(faces="regularized", omega=1.8, shape=(24, 12, 12)):
    """Channel past a momentum-exchange sphere with a velocity inlet and a
    pressure outlet, regularized or Zou/He."""
    wl = workloads.channel_sphere(shape, (8.2, 5.6, 6.3), 2.5, 0.05, omega)
    if faces == "zouhe":
        k = wl.kinds.copy()
        k[k == N.face_kind(N.REG_VELOCITY, 0, -1)] = N.face_kind(N.ZOUHE_VELOCITY, 0, -1)
        k[k == N.face_kind(N.REG_PRESSURE, 0, +1)] = N.face_kind(N.ZOUHE_PRESSURE, 0, +1)
        wl.kinds = k
    return wl


def _permuted(wl, perm):
    """The workload with its axes permuted (new axis a = old axis perm[a]):
    face kinds turned with it, velocity values rotated, densities kept."""
    import dataclasses
    kinds = np.ascontiguousarray(np.transpose(wl.kinds, perm))
    bc = np.ascontiguousarray(np.transpose(wl.bcval, perm + (3,)))
    out = kinds.copy()
    for fam in (N.REG_VELOCITY, N.REG_PRESSURE, N.ZOUHE_VELOCITY, N.ZOUHE_PRESSURE):
        for d in range(3):
            for o in (-1, 1):
                m = kinds == N.face_kind(fam, d, o)
                out[m] = N.face_kind(fam, perm.index(d), o)
                if fam in (N.REG_VELOCITY, N.ZOUHE_VELOCITY):
                    bc[m] = bc[m][:, list(perm)]
    return dataclasses.replace(wl, shape=tuple(wl.shape[a] for a in perm), kinds=out, bcval=bc,
                               periodic=tuple(wl.periodic[a] for a in perm))


@pytest.mark.parametrize("faces", ["regularized", "zouhe"])
@pytest.mark.parametrize("perm", [(1, 0, 2), (2, 1, 0)])
def test_face_adjoint_every_orientation_matches_tangent_linear(faces, perm):
    """The channel turned to run along y and along z: the closed-form reverse
    of the face completion for the other four face orientations."""
    wl = _permuted(_face_channel(faces), perm)
    lat = wl.lattice("fp64")
    lat.collide_and_stream(3)
    J_t, dJ = lat.tangent_linear(12, None, 0.41, drag=DRAG_DIR)
    lat.adjoint_forward(12, 4)
    J, _, gO, _ = lat.adjoint_backward(drag=DRAG_DIR, want_force=False)
    assert J == pytest.approx(J_t, rel=1e-13) and J != 0.0
    assert gO * 0.41 == pytest.approx(dJ, rel=1e-9), (gO * 0.41, dJ)


@pytest.mark.parametrize("warm", [0, 3])
@pytest.mark.parametrize("faces", ["regularized", "zouhe"])
@pytest.mark.parametrize("K", [1, 5])
def test_face_adjoint_drag_matches_tangent_linear(faces, K, warm):
    """Velocity inlet, pressure outlet: the face cells' reverse step (dual
    passes over their completion and collision) against the dual-number run,
    from a freshly initialized state and from one whose faces are pending."""
    wl = _face_channel(faces)
    T = 20
    lat = wl.lattice("fp64")
    lat.collide_and_stream(warm)
    J_t, dJ = lat.tangent_linear(T, None, 0.37, drag=DRAG_DIR)
    lat.adjoint_forward(T, K)
    J, _, gO, _ = lat.adjoint_backward(drag=DRAG_DIR, want_force=False)
    assert J == pytest.approx(J_t, rel=1e-13) and J != 0.0
    assert gO * 0.37 == pytest.approx(dJ, rel=1e-9), (gO * 0.37, dJ)


def test_face_adjoint_weighted_matches_tangent_linear():
    wl = _face_channel("regularized")
    lat = wl.lattice("fp64")
    lat.collide_and_stream(2)
    w = np.random.default_rng(17).standard_normal(wl.shape + (3,))
    J_t, dJ = lat.tangent_linear(16, None, -0.8, weights=w)
    lat.adjoint_forward(16, 4)
    J, _, gO, _ = lat.adjoint_backward(weights=w, want_force=False)
    assert J == pytest.approx(J_t, rel=1e-13)
    assert gO * -0.8 == pytest.approx(dJ, rel=1e-9)


def test_face_adjoint_drag_matches_reference_finite_differences():
    wl = _face_channel("regularized")
    T = 20
    lat = wl.lattice("fp64")
    lat.collide_and_stream(3)
    f0 = lat.receive()   # faces completed, as the reference holds them after a step
    lat.adjoint_forward(T, 5)
    J, _, gO, _ = lat.adjoint_backward(drag=DRAG_DIR, want_force=False)

    def drag(omega):
        ol = O.OracleLattice(*wl.shape, wl.periodic, omega, wl.kinds, wl.bcval, None)
        f, _ = ol.run(f0, T, with_stats=False)
        _, st = ol.run(f, 1, with_stats=True)
        return float(np.dot(DRAG_DIR, st[0, 3:6]))

    assert J == pytest.approx(drag(wl.omega), rel=1e-12)
    h = 1e-6
    fd = (drag(wl.omega + h) - drag(wl.omega - h)) / (2 * h)
    assert gO == pytest.approx(fd, rel=1e-5), (gO, fd)


def test_face_steady_drag_adjoint():
    """dDrag/domega of the converged channel past a sphere (velocity inlet,
    pressure outlet) from the steady adjoint, against central differences of
    converged FP64 runs."""
    def converged(omega):
        lat = _face_channel("regularized", omega=omega, shape=(20, 10, 10)).lattice("fp64")
        lat.collide_and_stream(12000)
        return lat

    omega = 1.2
    lat = converged(omega)
    J, _, gO, _ = lat.adjoint_steady(iterations=6000, want_force=False, drag=DRAG_DIR)
    _, _, gO2, _ = lat.adjoint_steady(iterations=12000, want_force=False, drag=DRAG_DIR)
    assert gO2 == pytest.approx(gO, rel=1e-8)

    def drag(om):
        J2, _, _, _ = converged(om).adjoint_steady(iterations=0, want_force=False, drag=DRAG_DIR)
        return J2

    h = 1e-5
    fd = (drag(omega + h) - drag(omega - h)) / (2 * h)
    assert gO == pytest.approx(fd, rel=1e-5), (gO, fd)


def test_face_adjoint_fp32_tracks_fp64():
    wl = _face_channel("regularized")
    g = {}
    for prec in ("fp64", "fp32"):
        lat = wl.lattice(prec)
        lat.collide_and_stream(3)
        lat.adjoint_forward(30, 6)
        J, _, gO, _ = lat.adjoint_backward(drag=DRAG_DIR, want_force=False)
        g[prec] = (J, gO)
    assert g["fp32"][0] == pytest.approx(g["fp64"][0], rel=1e-4)
    assert g["fp32"][1] == pytest.approx(g["fp64"][1], rel=1e-3)


# ---------------------------------------------------------------- edges and corners

def _velocity_box(shape=(12, 10, 9), omega=1.7, seed=7, precision="fp64", lid_only=False):
    """setVelocityConditionOnBlockBoundaries over the whole box (regularized
    velocity faces, external velocity edges and corners, all with stored
    wall velocities), BGK next to the walls and a Guo-forced core; or
    (lid_only) a box driven by its top face's velocity whose x = nx-1 face is
    a regularized pressure outlet at rho = 1 (which fixes the mass, so that
    the steady state is unique; the edges around it read the outlet's
    computed velocity)."""
    from palabos_gb300 import DeviceLattice3D
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    lat = DeviceLattice3D(nx, ny, nz, omega, precision)
    lat.set_velocity_condition_on_block_boundaries()
    force = np.zeros(shape + (3,))
    if not lid_only:
        lat.define_dynamics((2, nx - 3, 2, ny - 3, 2, nz - 3), N.GUO)
        force[2:-2, 2:-2, 2:-2] = 1e-5 + 1e-6 * rng.standard_normal((nx - 4, ny - 4, nz - 4, 3))
        lat.set_external_vector(None, force)
        u = 0.02 * rng.standard_normal(shape + (3,))
    else:
        u = np.zeros(shape + (3,))
        u[:, :, -1, 0] = 0.04
    lat.set_boundary_velocity(None, u)
    if lid_only:
        outlet = (nx - 1, nx - 1, 1, ny - 2, 1, nz - 2)
        lat.add_pressure_boundary(outlet, 0, +1)
        lat.set_boundary_density(outlet, 1.0)      # after the velocities: the density shares their slot
    if lid_only:
        lat.initialize_at_equilibrium(None, 1.0, (0.0, 0.0, 0.0))
    else:
        rho = 1.0 + 0.01 * rng.standard_normal(shape)
        lat.initialize_at_equilibrium(None, rho, 0.01 * rng.standard_normal(shape + (3,)))
    lat.initialize()
    return lat, force


@pytest.mark.parametrize("K", [1, 4])
def test_edge_corner_adjoint_matches_tangent_linear(K):
    """Faces, edges and corners of a velocity box: the reverse of the edge and
    corner processors (finite differences over the neighbours) with the rest
    of the step, against the dual-number run, for a force direction on the
    Guo core and omega; the domain continues bit for bit like a plain run."""
    lat, force = _velocity_box()
    lat.collide_and_stream(2)
    f0 = lat.receive()
    T = 16
    rng = np.random.default_rng(21)
    w = rng.standard_normal(lat.shape + (3,))
    dF = np.zeros_like(force)
    dF[2:-2, 2:-2, 2:-2] = rng.standard_normal(force[2:-2, 2:-2, 2:-2].shape)
    J_t, dJ = lat.tangent_linear(T, dF, 0.6, weights=w)
    lat.adjoint_forward(T, K)
    J, gF, gO, _ = lat.adjoint_backward(weights=w)
    assert J == pytest.approx(J_t, rel=1e-13) and J != 0.0
    adj = float(np.sum(gF * dF)) + gO * 0.6
    assert adj == pytest.approx(dJ, rel=1e-9), (adj, dJ)
    plain, _ = _velocity_box()
    plain.collide_and_stream(2)
    assert np.array_equal(plain.receive(), f0)
    plain.collide_and_stream(T)
    assert np.array_equal(lat.receive(), plain.receive())


def test_edge_corner_adjoint_matches_finite_differences():
    """dJ/domega and dJ/dF against central differences of the domain's own
    FP64 steps (the fused kernels and the edge and corner processors, bit for
    bit the reference's arithmetic)."""
    T = 12
    w = np.random.default_rng(4).standard_normal((12, 10, 9, 3))

    def objective(omega, force_delta=None):
        lat, force = _velocity_box()          # the same initial state (initialize() depends on omega)
        lat.set_params(omega)
        if force_delta is not None:
            lat.set_external_vector(None, force + force_delta)
        lat.collide_and_stream(T)
        J, _, _, _ = lat.adjoint_steady(weights=w, iterations=0, want_force=False)
        return J

    lat, force = _velocity_box()
    lat.adjoint_forward(T, 3)
    J, gF, gO, _ = lat.adjoint_backward(weights=w)
    assert J == pytest.approx(objective(1.7), rel=1e-13)
    h = 1e-6
    fd = (objective(1.7 + h) - objective(1.7 - h)) / (2 * h)
    assert gO == pytest.approx(fd, rel=1e-5), (gO, fd)
    for cell, d in (((3, 4, 4), 0), ((6, 2, 5), 2), ((9, 7, 2), 1)):
        e = np.zeros_like(force)
        e[cell + (d,)] = 1e-7
        fd = (objective(1.7, e) - objective(1.7, -e)) / 2e-7
        assert gF[cell + (d,)] == pytest.approx(fd, rel=1e-5, abs=1e-9 * abs(gO)), (cell, d, gF[cell + (d,)], fd)


def test_edge_corner_steady_adjoint():
    """Lid-driven box with a pressure outlet at steady state: d(sum w . u)/domega
    from the steady adjoint against central differences of converged FP64
    runs.  (In a box closed by velocity conditions alone the mass level is a
    neutral mode that the transient sets, which a steady adjoint cannot see.)"""
    w = np.random.default_rng(9).standard_normal((10, 8, 8, 3))

    def converged(omega):
        lat, _ = _velocity_box((10, 8, 8), omega=omega, lid_only=True)
        lat.collide_and_stream(8000)
        return lat

    lat = converged(1.3)
    J, _, gO, _ = lat.adjoint_steady(weights=w, iterations=4000, want_force=False)
    _, _, gO2, _ = lat.adjoint_steady(weights=w, iterations=8000, want_force=False)
    assert gO2 == pytest.approx(gO, rel=1e-8)
    h = 1e-5

    def J_at(om):
        return converged(om).adjoint_steady(weights=w, iterations=0, want_force=False)[0]

    fd = (J_at(1.3 + h) - J_at(1.3 - h)) / (2 * h)
    assert gO == pytest.approx(fd, rel=1e-5), (gO, fd)


def test_edge_corner_adjoint_fp32_tracks_fp64():
    w = np.random.default_rng(3).standard_normal((12, 10, 9, 3))
    g = {}
    for prec in ("fp64", "fp32"):
        lat, _ = _velocity_box(precision=prec)
        lat.adjoint_forward(20, 5)
        J, gF, gO, _ = lat.adjoint_backward(weights=w)
        g[prec] = (J, gF, gO)
    assert g["fp32"][0] == pytest.approx(g["fp64"][0], rel=1e-4)
    assert np.abs(g["fp32"][1] - g["fp64"][1]).max() <= 2e-3 * np.abs(g["fp64"][1]).max()
    assert g["fp32"][2] == pytest.approx(g["fp64"][2], rel=2e-3)
