"""CUDA path against the reference's golden vectors and the CPU oracle.

FP64: populations bit for bit (the FP64 kernels are compiled without FMA
contraction and keep the reference's operand order), reductions within 1e-12
relative (they are summed in a different order), through the C ABI.
"""
import hashlib

import numpy as np
import pytest

import goldens
import lbcases
import oracle as O
from palabos_gb300 import lattice_from_description

pytestmark = pytest.mark.gpu


def _lat(g, meta, precision="fp64"):
    return lattice_from_description(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"],
                                    g["flags"], g["bcval"], g["force"], meta.get("rho0", 1.0),
                                    meta.get("bb_rho", 0.0), precision)


@pytest.mark.parametrize("name", [n for n in goldens.case_names() if not n.startswith("sparse_")])
def test_fp64_matches_reference(name):
    g, meta = goldens.load(name)
    lat = _lat(g, meta)
    lat.send(g["f_init"])
    external = bool(meta.get("options", 0) & lbcases.OPT_EXTERNAL_RHOJ)
    if external:
        lat.set_rhobar_j(g["rho_bar0"], g["j0"])
    gs = g["stats"]
    recorded = {int(s): k for k, s in enumerate(gs[:, 0])}
    for step in range(1, meta["nsteps"] + 1):
        take = step in recorded
        if external:
            lat.collide_and_stream_external(1, recompute=True, stats=take)
        else:
            lat.collide_and_stream(1, stats=take)
        if take:
            st = lat.internal_statistics()["raw"][:6]
            ok, worst = goldens.stats_close(st, gs[recorded[step], 1:])
            assert ok, (step, worst, st, gs[recorded[step], 1:])
    f = lat.receive()
    ref = g["f_final"]
    assert np.array_equal(f, ref), f"max |diff| {np.abs(f - ref).max():.3e}"
    e, rho = lat.reduce()
    assert e == pytest.approx(float(g["energy"]), rel=1e-12, abs=0)
    assert rho == pytest.approx(float(g["density"]), rel=1e-12, abs=0)
    if external:
        rb, j = lat.get_rhobar_j()
        assert np.array_equal(rb, g["rho_bar_final"]) and np.array_equal(j, g["j_final"])


@pytest.mark.parametrize("name", ["periodic_bgk", "channel_sphere", "velocity_box", "guo_channel"])
def test_external_form_with_own_moments_equals_collide_and_stream(name):
    """collideExternal with the fields BoxRhoBarJfunctional3D computed from
    the same populations is the ordinary collision: the external form, with
    the fields refreshed every step, reproduces the ordinary steps -- except
    for boundary cells, whose fields the functional reads before their
    completion, and Guo cells, whose generic external route rounds
    differently; those are compared against the oracle's external form."""
    g, meta = goldens.load(name)
    lat = _lat(g, meta)
    lat.send(g["f_init"])
    lat.compute_rhobar_j()
    rb0, j0 = lat.get_rhobar_j()
    k = min(meta["nsteps"], 12)
    lat.collide_and_stream_external(k, recompute=True, stats=True)
    ol = O.OracleLattice.from_golden(g, meta)
    ref, rbr, jr, st = ol.run_external(g["f_init"], rb0, j0, k)
    assert np.array_equal(lat.receive(), ref.reshape(lat.receive().shape))
    rb, j = lat.get_rhobar_j()
    assert np.array_equal(rb, rbr) and np.array_equal(j, jr)
    ok, worst = goldens.stats_close(lat.internal_statistics()["raw"][:6], st[k - 1, :6])
    assert ok, worst
    if name == "periodic_bgk":
        std, _ = ol.run(g["f_init"], k)
        assert np.array_equal(lat.receive(), std.reshape(lat.receive().shape))


def test_external_form_needs_fields():
    from palabos_gb300 import DeviceLattice3D, PlbGpuError
    lat = DeviceLattice3D(8, 8, 8, 1.5)
    with pytest.raises(PlbGpuError) as e:
        lat.collide_and_stream_external(1)
    assert e.value.code == -5
    import ctypes
    v = np.zeros(4 * 10)   # a 2x2x2 box needs 4 * 8 values
    rc = lat.lib.plbgpu_set_rhobar_j(lat.ctx.h, lat.handle, 0, 1, 0, 1, 0, 1,
                                     v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), v.size)
    assert rc == -1


@pytest.mark.parametrize("name", ["cavity_bb_lid", "channel_sphere", "regpress_faces", "zhvel_faces",
                                  "velocity_box", "doctest_cavity20"])
def test_initialize_completes_faces_like_reference(name):
    g, meta = goldens.load(name)
    spec = lbcases.case_by_name(name)
    lat = _lat(g, meta)
    lat.send(spec.f0)
    lat.initialize()
    assert np.array_equal(lat.receive(), g["f_init"])
    # and stepping from the lazily-completed state gives the reference's result
    lat.collide_and_stream(meta["nsteps"])
    assert np.array_equal(lat.receive(), g["f_final"])


@pytest.mark.parametrize("name", ["periodic_bgk", "channel_sphere", "guo_channel", "mebb_walls"])
def test_multistep_calls_and_odd_parity_transfers(name):
    """Many steps per call, receive after odd step counts, partial-box
    send/receive round trips on the AA-swapped state."""
    g, meta = goldens.load(name)
    lat = _lat(g, meta)
    lat.send(g["f_init"])
    ol = O.OracleLattice.from_golden(g, meta)
    k = 7
    lat.collide_and_stream(k)
    ref7, _ = ol.run(g["f_init"], k)
    assert np.array_equal(lat.receive(), ref7.reshape(lat.receive().shape))
    box = (1, meta["nx"] - 3, 2, meta["ny"] - 2, 0, meta["nz"] - 2)
    part = lat.receive(box)
    lat.send(part, box)   # odd parity: send must invert receive exactly
    lat.collide_and_stream(meta["nsteps"] - k)
    assert np.array_equal(lat.receive(), g["f_final"])


@pytest.mark.parametrize("precision", ["fp64", "fp32", "bf16", "bf16sr"])
@pytest.mark.parametrize("name", ["velocity_box", "channel_sphere", "guo_channel", "zhpress_faces"])
def test_long_call_replays_steps_like_single_steps(name, precision):
    """A long collide_and_stream call replays its middle steps from a CUDA
    graph; the result and the parity equal those of one call per step, the
    statistics of its last step agree to the rounding of their summation (the
    per-block partial sums of the interior and border rows, which run on two
    streams, meet in FP64 atomic adds whose order varies from run to run)."""
    g, meta = goldens.load(name)
    n = 1 + 16 * 3 + 5
    runs = []
    for per_call in (n, 1):
        lat = _lat(g, meta, precision)
        lat.send(g["f_init"])
        for _ in range(n // per_call):
            lat.collide_and_stream(per_call, stats=True)
        runs.append((lat.receive(), lat.internal_statistics()["raw"]))
        lat.close()
    assert np.array_equal(runs[0][0], runs[1][0])
    ok, worst = goldens.stats_close(runs[0][1], runs[1][1])
    assert ok, worst


def test_velocity_condition_on_block_boundaries_sets_faces_edges_corners():
    """setVelocityConditionOnBlockBoundaries over a box: the kinds of the
    reference's instantiation, interior kinds left alone."""
    from palabos_gb300 import DeviceLattice3D, GUO
    lat = DeviceLattice3D(11, 10, 9, 1.5)
    lat.define_dynamics(None, GUO)
    lat.set_velocity_condition_on_block_boundaries()
    want = lbcases.velocity_box_kinds((11, 10, 9))
    want[want == lbcases.BGK] = GUO
    assert np.array_equal(lat.get_kinds(), want)
    inner = DeviceLattice3D(12, 12, 12, 1.5)
    inner.set_velocity_condition_on_block_boundaries((2, 8, 3, 9, 1, 10))
    k = inner.get_kinds()
    assert np.array_equal(k[2:9, 3:10, 1:11], lbcases.velocity_box_kinds((7, 7, 10)))
    assert (k[:2] == 0).all() and (k[9:] == 0).all()


def test_edge_without_inward_neighbours_is_reported_not_run():
    """An edge whose finite differences would leave a non-periodic domain is
    refused before any kernel reads it; made periodic, the same layout runs."""
    from palabos_gb300 import DeviceLattice3D, PlbGpuError, edge_kind
    lat = DeviceLattice3D(6, 6, 6, 1.5)
    # plane-0 edge with outward normals +y, +z placed at y = z = 0: the inward
    # neighbours y - 1 and z - 1 lie outside
    lat.define_dynamics((1, 4, 0, 0, 0, 0), edge_kind(0, 1, 1))
    with pytest.raises(PlbGpuError) as e:
        lat.collide_and_stream(1)
    assert e.value.code == -1 and "edge/corner cell" in str(e.value)
    with pytest.raises(PlbGpuError):
        lat.initialize()
    lat.periodicity(0, 1, 1)
    lat.collide_and_stream(2)
    assert np.isfinite(lat.receive()).all()


def test_cavity64_full_size_matches_reference_fingerprint():
    """The 64^3 lid-driven cavity at full size, 1000 steps, every bit."""
    fp = goldens.load_fingerprint("cavity64")
    s = lbcases.case_cavity64()
    lat = lattice_from_description(s.nx, s.ny, s.nz, s.periodic, s.omega, s.flags, s.bcval, s.force)
    lat.send(s.f0)
    lat.initialize()
    assert hashlib.sha256(np.ascontiguousarray(lat.receive()).tobytes()).hexdigest() == fp["sha256_f_init"]
    for k in range(10):
        lat.collide_and_stream(100, stats=True)
        st = lat.internal_statistics()["raw"][:6]
        ok, worst = goldens.stats_close(st, np.asarray(fp["stats"][k][1:]))
        assert ok, (k, worst)
    f = np.ascontiguousarray(lat.receive())
    assert hashlib.sha256(f.tobytes()).hexdigest() == fp["sha256_f_final"]
    assert lat.compute_average_energy() == pytest.approx(7.114849642596e-06, rel=1e-12)


def test_coprocessor_form_matches_block_lattice():
    """plbgpu_cp_*: the reference's CoProcessor3D calls (1 = success) on a
    non-periodic BGK block, against the oracle's BlockLattice3D semantics."""
    import ctypes
    from palabos_gb300 import default_context
    ctx = default_context()
    lib = ctx.lib
    nx, ny, nz, omega = 9, 7, 6, 1.3
    h = ctypes.c_int()
    assert lib.plbgpu_cp_add_domain(ctx.h, nx, ny, nz, omega, ctypes.byref(h)) == 1
    rng = np.random.default_rng(5)
    f0 = lbcases.initial_state((nx, ny, nz), rng)
    data = np.ascontiguousarray(f0).tobytes()
    assert lib.plbgpu_cp_send(ctx.h, h.value, 0, nx - 1, 0, ny - 1, 0, nz - 1, data, len(data)) == 1
    for _ in range(5):
        assert lib.plbgpu_cp_collide_and_stream(ctx.h, h.value) == 1
    out = ctypes.create_string_buffer(len(data))
    assert lib.plbgpu_cp_receive(ctx.h, h.value, 0, nx - 1, 0, ny - 1, 0, nz - 1, out, len(data)) == 1
    got = np.frombuffer(out.raw, np.float64).reshape(nx, ny, nz, 19)
    ol = O.OracleLattice(nx, ny, nz, (0, 0, 0), omega, np.zeros((nx, ny, nz), np.uint8))
    ref, _ = ol.run(f0, 5)
    assert np.array_equal(got, ref)
    # wrong byte count: failure code 0, not a crash
    assert lib.plbgpu_cp_send(ctx.h, h.value, 0, nx - 1, 0, ny - 1, 0, nz - 1, data, len(data) - 8) == 0
    assert lib.plbgpu_cp_collide_and_stream(ctx.h, 12345) == 0


def test_coprocessor_form_single_precision():
    """plbgpu_cp_*_f32: CoProcessor3D<float> -- an FP32 domain exchanging 19
    floats per cell -- against the oracle's FP64 BlockLattice3D run of the same
    block, to FP32 rounding."""
    import ctypes
    from palabos_gb300 import default_context
    ctx = default_context()
    lib = ctx.lib
    nx, ny, nz, omega = 9, 7, 16, 1.3
    h = ctypes.c_int()
    assert lib.plbgpu_cp_add_domain_f32(ctx.h, nx, ny, nz, omega, ctypes.byref(h)) == 1
    f0 = lbcases.initial_state((nx, ny, nz), np.random.default_rng(6)).astype(np.float32)
    data = np.ascontiguousarray(f0).tobytes()
    assert lib.plbgpu_cp_send_f32(ctx.h, h.value, 0, nx - 1, 0, ny - 1, 0, nz - 1, data, len(data)) == 1
    for _ in range(5):
        assert lib.plbgpu_cp_collide_and_stream(ctx.h, h.value) == 1
    out = ctypes.create_string_buffer(len(data))
    assert lib.plbgpu_cp_receive_f32(ctx.h, h.value, 0, nx - 1, 0, ny - 1, 0, nz - 1, out, len(data)) == 1
    got = np.frombuffer(out.raw, np.float32).reshape(nx, ny, nz, 19)
    ol = O.OracleLattice(nx, ny, nz, (0, 0, 0), omega, np.zeros((nx, ny, nz), np.uint8))
    ref, _ = ol.run(f0.astype(np.float64), 5)
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()
    # FP32 records: a byte count of doubles is not a whole number of cells here
    assert lib.plbgpu_cp_send_f32(ctx.h, h.value, 0, nx - 1, 0, ny - 1, 0, nz - 1, data, len(data) - 4) == 0


def test_equilibrium_initialization_matches_oracle_formula():
    """initializeAtEquilibrium: f-bar = t_i (rhoBar + 3 c.j + invRho(4.5 (c.j)^2 - 1.5 j^2)), 0 on walls."""
    nx, ny, nz = 6, 5, 4
    from palabos_gb300 import DeviceLattice3D, BOUNCEBACK
    lat = DeviceLattice3D(nx, ny, nz, 1.2)
    lat.define_dynamics((0, 0, 0, ny - 1, 0, nz - 1), BOUNCEBACK)
    rng = np.random.default_rng(9)
    rho = 1 + 0.01 * rng.standard_normal((nx, ny, nz))
    u = 0.05 * rng.standard_normal((nx, ny, nz, 3))
    lat.initialize_at_equilibrium(None, rho, u)
    got = lat.receive()
    ref = lbcases.equilibrium(rho, u)
    ref[0] = 0.0
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-17)


def test_error_paths_leave_context_usable():
    from palabos_gb300 import DeviceLattice3D, PlbGpuError
    lat = DeviceLattice3D(4, 4, 4, 1.0)
    with pytest.raises(PlbGpuError):
        lat.send(np.zeros(10))
    with pytest.raises(PlbGpuError):
        lat.define_dynamics((0, 9, 0, 0, 0, 0), 0)
    with pytest.raises(PlbGpuError):
        lat.define_dynamics(None, 77)
    with pytest.raises(PlbGpuError):
        lat.internal_statistics()   # nothing gathered yet
    lat.collide_and_stream(3, stats=True)
    assert lat.internal_statistics()["count"] == 64


@pytest.mark.parametrize("precision", ["fp64", "fp32", "bf16"])
def test_diverged_state_is_reported_and_cleared(precision):
    """A NaN planted on the host in one fluid cell's populations (sent through
    plbgpu_send) reaches the next statistics step's block sums: synchronize
    reports PLBGPU_ERR_STATE once, and the domain keeps working once a finite
    state is sent again."""
    from palabos_gb300 import DeviceLattice3D, PlbGpuError
    from palabos_gb300 import native as N
    lat = DeviceLattice3D(12, 10, 16, 1.2, precision)
    lat.periodicity(1, 1, 1)
    f = np.zeros((12, 10, 16, 19))
    lat.send(f)
    lat.collide_and_stream(2, stats=True)
    lat.ctx.synchronize()                       # finite state: nothing reported
    bad = f.copy()
    bad[5, 4, 7, 3] = np.nan
    lat.send(bad)
    lat.collide_and_stream(1, stats=False)      # no statistics: not looked at yet
    lat.ctx.synchronize()
    lat.collide_and_stream(1, stats=True)
    with pytest.raises(PlbGpuError) as e:
        lat.ctx.synchronize()
    assert e.value.code == -5 and "non-finite" in str(e.value)
    lat.ctx.synchronize()                       # reported once, then cleared
    lat.send(f)
    lat.collide_and_stream(3, stats=True)
    st = lat.internal_statistics()
    assert st["count"] == 12 * 10 * 16 and np.isfinite(st["avRhoBar"])


def test_sparse_lattice_matches_reference_and_oracle():
    """A sparse lattice (computeSparseManagement over a 4x3x3 regular
    distribution): the kept blocks are the reference's; the fluid sealed off
    by bounce-back matches the reference bit for bit, drag included; every
    cell of the lattice, the statistics and the reductions match the oracle
    run with the same sparse semantics (outside of the kept blocks = outside
    of the domain)."""
    g, meta = goldens.load("sparse_sealed_channel")
    lat = lattice_from_description(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"],
                                   g["flags"], g["bcval"], g["force"], sparse=(g["sparse"], meta["blocks"]))
    kinds = lat.get_kinds()
    assert np.array_equal(kinds != 255, g["in_lattice"].astype(bool))
    lat.send(g["f_init"])
    gs = g["stats"]
    recorded = {int(s): k for k, s in enumerate(gs[:, 0])}
    for step in range(1, meta["nsteps"] + 1):
        take = step in recorded
        lat.collide_and_stream(1, stats=take)
        if take:
            ok, worst = goldens.stats_close(lat.internal_statistics()["raw"][3:6], gs[recorded[step], 4:7])
            assert ok, (step, worst)
    f = lat.receive()
    cmp = g["compare"].astype(bool)
    assert np.array_equal(f[cmp], g["f_final"][cmp])
    # the oracle with the same kinds
    ol = O.OracleLattice(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"], kinds, g["bcval"],
                         g["force"])
    ref, st = ol.run(g["f_init"], meta["nsteps"])
    assert np.array_equal(f, ref.reshape(f.shape))
    ok, worst = goldens.stats_close(lat.internal_statistics()["raw"][:6], st[-1, :6])
    assert ok, worst
    e, rho = lat.reduce()
    oe, orho = ol.reduce(ref)
    assert e == pytest.approx(oe, rel=1e-12) and rho == pytest.approx(orho, rel=1e-12)


def test_sparse_lattice_without_seal_counts_the_band_next_to_dropped_blocks():
    """Fluid touching dropped blocks directly (no bounce-back seal).  The
    reference gives each kept block an envelope layer facing the dropped
    blocks whose cells collide and stream within that block; the GPU treats
    a neighbour in a dropped block like the domain edge.  After n steps the two
    differ exactly in the kept cells within n cells (chessboard distance) of a
    dropped block -- every one of them differs, none beyond -- and the GPU
    equals the oracle (the same domain-edge rule) on every cell."""
    from scipy.ndimage import distance_transform_cdt
    g, meta = goldens.load("sparse_unsealed_channel")
    lat = lattice_from_description(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"],
                                   g["flags"], g["bcval"], g["force"], sparse=(g["sparse"], meta["blocks"]))
    kinds = lat.get_kinds()
    inl = g["in_lattice"].astype(bool)
    assert np.array_equal(kinds != 255, inl)
    lat.send(g["f_init"])
    lat.collide_and_stream(meta["nsteps"], stats=True)
    f = lat.receive()
    dist = distance_transform_cdt(inl, metric="chessboard")
    far = inl & (dist > meta["nsteps"])
    band = inl & (dist <= meta["nsteps"])
    assert far.sum() > 0
    assert np.array_equal(f[far], g["f_final"][far])
    differ = np.any(f != g["f_final"], axis=-1) & inl
    assert not (differ & far).any()
    assert differ.sum() == band.sum() == 2160      # 2592 kept cells, 432 beyond the band
    ol = O.OracleLattice(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"], kinds, g["bcval"],
                         g["force"])
    ref, _ = ol.run(g["f_init"], meta["nsteps"])
    assert np.array_equal(f, ref.reshape(f.shape))

