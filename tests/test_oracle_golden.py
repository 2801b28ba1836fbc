"""The CPU oracle against golden vectors produced by the unmodified reference.

The goldens were generated by tests/golden/make_golden.py, which drives the
reference's own MultiBlockLattice3D construction API and collideAndStream().
Populations must agree bit for bit; reductions to summation rounding.
"""
import hashlib

import numpy as np
import pytest

import goldens
import lbcases
import oracle as O


@pytest.mark.parametrize("name", goldens.case_names())
def test_oracle_matches_reference(name):
    g, meta = goldens.load(name)
    if meta.get("options", 0) & lbcases.OPT_SPARSE:
        return _check_sparse(g, meta, with_drag=name != "sparse_unsealed_channel")
    lat = O.OracleLattice.from_golden(g, meta)
    if meta.get("options", 0) & lbcases.OPT_EXTERNAL_RHOJ:
        f, rb, j, stats = lat.run_external(g["f_init"], g["rho_bar0"], g["j0"], meta["nsteps"])
        assert np.array_equal(rb, g["rho_bar_final"]) and np.array_equal(j, g["j_final"])
    else:
        f, stats = lat.run(g["f_init"], meta["nsteps"])
    ref = g["f_final"]
    assert np.array_equal(f.reshape(ref.shape), ref), \
        f"max |diff| = {np.abs(f.reshape(ref.shape) - ref).max()}"
    e, rho = lat.reduce(f)
    assert e == pytest.approx(float(g["energy"]), rel=1e-12, abs=0)
    assert rho == pytest.approx(float(g["density"]), rel=1e-12, abs=0)
    gs = g["stats"]
    ok, worst = goldens.stats_close(stats[gs[:, 0].astype(int) - 1, :6], gs[:, 1:])
    assert ok, worst


def sparse_flags(g, meta):
    """Cell kinds of a sparse case: cells outside every block kept by
    computeSparseManagement are not part of the lattice."""
    keep = O.sparse_blocks(g["sparse"], meta["blocks"])
    mask = O.sparse_cell_mask(g["flags"].shape, meta["blocks"], keep)
    flags = g["flags"].copy()
    flags[~mask] = lbcases.NONE
    return flags, mask


def _check_sparse(g, meta, with_drag=True):
    """Populations of the compared cells bit for bit (the fluid a bounce-back
    seal keeps away from the dropped blocks, or the cells further from them
    than one cell per step); the drag where the obstacle is among them."""
    flags, mask = sparse_flags(g, meta)
    assert np.array_equal(mask, g["in_lattice"].astype(bool))   # the reference's block selection
    lat = O.OracleLattice(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"], flags,
                          g["bcval"], g["force"], meta.get("rho0", 1.0), meta.get("bb_rho", 0.0))
    f, stats = lat.run(g["f_init"], meta["nsteps"])
    cmp = g["compare"].astype(bool)
    assert cmp.any() and np.array_equal(f[cmp], g["f_final"][cmp])
    if with_drag:
        gs = g["stats"]
        ok, worst = goldens.stats_close(stats[gs[:, 0].astype(int) - 1, 3:6], gs[:, 4:7])   # drag
        assert ok, worst


@pytest.mark.parametrize("name", goldens.case_names())
def test_oracle_initialize_matches_reference(name):
    """Completing the boundary faces of the raw initial state reproduces the
    reference's state after lattice.initialize()."""
    g, meta = goldens.load(name)
    spec = lbcases.case_by_name(name)
    if meta.get("options", 0) & lbcases.OPT_SPARSE:
        return   # f_init holds zeros outside the lattice; the run itself is checked above
    if meta.get("options", 0) & lbcases.OPT_NO_INITIALIZE:
        assert np.array_equal(spec.f0, g["f_init"])
        return
    lat = O.OracleLattice.from_golden(g, meta)
    f0 = lat.initialize(spec.f0)
    assert np.array_equal(f0.reshape(g["f_init"].shape), g["f_init"])


def test_multiblock_equals_single_block():
    """The reference's multi-block decomposition does not change a single bit of
    the populations, so one global addressing scheme reproduces it."""
    for a, b in [("periodic_bgk", "periodic_bgk_multiblock"),
                 ("cavity_bb_lid", "cavity_bb_lid_multiblock"),
                 ("channel_sphere", "channel_sphere_multiblock"),
                 ("velocity_box", "velocity_box_multiblock")]:
        ga, _ = goldens.load(a)
        gb, _ = goldens.load(b)
        assert np.array_equal(ga["f_final"], gb["f_final"])


@pytest.mark.slow
def test_oracle_cavity64_full_size():
    """The lid-driven cavity at full size (64^3, 1000 steps) against the
    reference's fingerprint: sha256 of every population bit, plus energy."""
    fp = goldens.load_fingerprint("cavity64")
    s = lbcases.case_cavity64()
    lat = O.OracleLattice(s.nx, s.ny, s.nz, s.periodic, s.omega, s.flags, s.bcval, s.force,
                          s.rho0, s.bb_rho)
    f0 = lat.initialize(s.f0)
    assert hashlib.sha256(f0.tobytes()).hexdigest() == fp["sha256_f_init"]
    f, stats = lat.run(f0, s.nsteps)
    assert hashlib.sha256(f.tobytes()).hexdigest() == fp["sha256_f_final"]
    e, rho = lat.reduce(f)
    assert e == pytest.approx(fp["energy"], rel=1e-12)
    assert e == pytest.approx(7.114849642596e-06, rel=1e-12)


@pytest.mark.parametrize("shape", sorted(lbcases.DOCTEST_CAVITY))
def test_oracle_reproduces_published_cavity_regression(shape):
    """The reference's own 3D cavity regression values (regularized velocity
    conditions on faces, edges and corners; 30 steps from rest).  They were
    printed to five significant digits by an older build: the density agrees
    to one unit of the last printed digit, the energy to 3e-3 relative, which
    is also how far the reference built from these sources lies from them."""
    e_pub, rho_pub = lbcases.DOCTEST_CAVITY[shape]
    s = lbcases.doctest_cavity(*shape)
    lat = O.OracleLattice(s.nx, s.ny, s.nz, s.periodic, s.omega, s.flags, s.bcval, s.force,
                          s.rho0, s.bb_rho)
    f, _ = lat.run(lat.initialize(s.f0), s.nsteps)
    e, rho = lat.reduce(f)
    assert abs(round(e, 10) / e_pub - 1) < 3e-3
    assert abs(round(rho, 10) - rho_pub) <= 1.5e-7
