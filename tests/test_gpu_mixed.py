"""Reduced-precision storage forms (FP32 compute; FP32 / BF16 / FP16 f-bar
storage) against the reference's FP64 golden results.

These forms do not reproduce the reference bit for bit; the bound is on the
largest population error relative to the largest |f-bar| of the case, with
the tolerance of each storage type written here (about twice the largest
error measured on a GB300 over these cases: FP32 6.1e-6, FP16 8.9e-4, BF16
8.5e-3, BF16 with stochastic rounding 1.2e-2).  They run through the same C
ABI and the same interior-row kernels as production runs: the paired
(two-cell) kernel of the 2-byte forms where rows have an even length, the
one-cell kernel otherwise.
"""
import numpy as np
import pytest

import goldens
from palabos_gb300 import lattice_from_description

pytestmark = pytest.mark.gpu

# max |f - f_ref| / max |f_ref| after the case's steps
TOL = {"fp32": 1.5e-5, "fp16": 2e-3, "bf16": 1.5e-2, "bf16sr": 2.5e-2}
CASES = ["periodic_bgk", "cavity_bb_lid", "channel_sphere", "guo_channel", "regvel_faces",
         "zhpress_faces", "incbgk_nodyn", "mebb_walls", "velocity_box"]


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp16", "bf16sr"])
@pytest.mark.parametrize("name", CASES)
def test_reduced_precision_tracks_reference(name, precision):
    g, meta = goldens.load(name)
    lat = lattice_from_description(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"],
                                   g["flags"], g["bcval"], g["force"], meta.get("rho0", 1.0),
                                   meta.get("bb_rho", 0.0), precision)
    lat.send(g["f_init"])
    lat.collide_and_stream(meta["nsteps"] - 1)
    lat.collide_and_stream(1, stats=True)
    f = lat.receive()
    ref = g["f_final"]
    err = np.abs(f - ref).max() / np.abs(ref).max()
    assert err < TOL[precision], err
    st = lat.internal_statistics()
    assert np.isfinite(st["raw"]).all()
    e, rho = lat.reduce()
    assert e == pytest.approx(float(g["energy"]), rel=50 * TOL[precision])


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp16"])
@pytest.mark.parametrize("name", ["external_periodic_bgk", "external_mebb_periodic"])
def test_reduced_precision_external_form(name, precision):
    """The external rho-bar/j form in the reduced storage forms (fields in
    FP32) against the reference's FP64 result."""
    g, meta = goldens.load(name)
    lat = lattice_from_description(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"],
                                   g["flags"], g["bcval"], g["force"], meta.get("rho0", 1.0),
                                   meta.get("bb_rho", 0.0), precision)
    lat.send(g["f_init"])
    lat.set_rhobar_j(g["rho_bar0"], g["j0"])
    lat.collide_and_stream_external(meta["nsteps"], recompute=True)
    f = lat.receive()
    ref = g["f_final"]
    err = np.abs(f - ref).max() / np.abs(ref).max()
    assert err < TOL[precision], err


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_row_kernels_agree_across_row_lengths(precision):
    """nz = 32 (the paired kernel for BF16, the one-cell kernel for FP32) and
    nz = 33 (the one-cell kernel) give the same physics on a flow that
    depends only on y."""
    from palabos_gb300 import DeviceLattice3D
    out = []
    for nz in (32, 33):
        lat = DeviceLattice3D(16, 12, nz, 1.7, precision)
        lat.periodicity(1, 1, 1)
        z = np.arange(nz)
        u = np.zeros((16, 12, nz, 3))
        u[..., 0] = 0.03 * np.sin(2 * np.pi * np.arange(12) / 12)[None, :, None]
        lat.initialize_at_equilibrium(None, np.ones((16, 12, nz)), u)
        lat.collide_and_stream(20)
        f = lat.receive()
        out.append(f[:, :, :8].astype(np.float64))   # depends only on y
    assert np.abs(out[0] - out[1]).max() < TOL[precision] * 0.03 + 1e-7


def test_taylor_green_velocity_error_of_storage_forms():
    """Small Taylor-Green vortex (64^3, 400 steps, omega close to 2): relative
    velocity L2 error against the FP64 path of FP32 storage (measured 1.2e-5)
    below 1e-4, FP16 storage (measured 1.2e-3) below 1e-2, BF16 storage below
    2e-1, ordered by storage precision; kinetic energy of FP32 storage within
    1e-4 of FP64 at every sampled time."""
    from palabos_gb300.accuracy import taylor_green_study
    r = taylor_green_study(n=64, steps=400, every=100, slab=16)
    f = r["forms"]
    print({p: v["vel_l2_rel"] for p, v in f.items()})
    assert f["fp32"]["vel_l2_rel"] < 1e-4, f
    assert f["fp16"]["vel_l2_rel"] < 1e-2, f
    assert f["bf16"]["vel_l2_rel"] < 2e-1, f
    assert f["bf16sr"]["vel_l2_rel"] < 2e-1, f
    assert f["fp32"]["vel_l2_rel"] < f["fp16"]["vel_l2_rel"] < f["bf16"]["vel_l2_rel"]
    assert f["fp32"]["ke_rel_max"] < 1e-4, f
    assert 0.0 < r["ke_decay_fp64"] < 1.0


def test_compute_velocity_and_density_match_reductions():
    """computeVelocity / computeDensity fields average to computeAverageEnergy /
    computeAverageDensity."""
    g, meta = goldens.load("channel_sphere")
    lat = lattice_from_description(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"],
                                   g["flags"], g["bcval"], g["force"])
    lat.send(g["f_init"])
    lat.collide_and_stream(9)
    u = lat.compute_velocity()
    rho = lat.compute_density()
    e, d = lat.reduce()
    assert 0.5 * np.mean(np.sum(u * u, axis=-1)) == pytest.approx(e, rel=1e-12)
    # BounceBack(rho=0) cells report density 0 and rho-bar -1: the averages agree
    assert np.mean(rho) == pytest.approx(d, rel=1e-12)


def test_fp32_reproduces_the_reference_single_precision_regression():
    """The reference's own regression test runs its 3D cavity (regularized
    velocity on faces, edges and corners, 20x31x42, 30 steps) in double and in
    single precision and prints the same five digits for both
    (jlabos/src/testing/test_cylinder.py:92-97).  The FP32 form gives the
    published energy to the precision the FP64 reference does (3e-3 relative)
    and the FP64 average density within 1e-7."""
    import lbcases
    import oracle as O
    e_pub, _ = lbcases.DOCTEST_CAVITY[(20, 31, 42)]
    s = lbcases.doctest_cavity(20, 31, 42)
    lat = lattice_from_description(s.nx, s.ny, s.nz, s.periodic, s.omega, s.flags, s.bcval, s.force, s.rho0,
                                   s.bb_rho, "fp32")
    lat.send(s.f0)
    lat.initialize()
    lat.collide_and_stream(s.nsteps)
    e, rho = lat.reduce()
    ol = O.OracleLattice(s.nx, s.ny, s.nz, s.periodic, s.omega, s.flags, s.bcval, s.force, s.rho0, s.bb_rho)
    oe, orho = ol.reduce(ol.run(ol.initialize(s.f0), s.nsteps)[0])
    assert abs(round(e, 10) / e_pub - 1) < 3e-3
    assert e == pytest.approx(oe, rel=1e-3)
    assert abs(rho - orho) <= 1e-7
