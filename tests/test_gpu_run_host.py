"""plbgpu_run_host: send, nsteps steps and receive in one call, the host
transfers overlapped with ramps of x-slab steps at both ends.  The state must
be bit for bit that of plbgpu_send + plbgpu_collide_and_stream +
plbgpu_receive, and the statistics records those of the same steps (summed in
another order: 1e-12 relative).  The cases cover both parities of the first
and the last step, periodic and walled x, faces pending, ramps cut short by
statistics steps, and whole-domain steps between the ramps."""
import numpy as np
import pytest

from palabos_gb300 import native as N
from palabos_gb300 import workloads

pytestmark = pytest.mark.gpu


def _sequential(lat, f0, nsteps, every):
    lat.send(f0)
    recs, t = [], 0
    while t < nsteps:
        nxt = t
        while nxt < nsteps and not (every and ((nxt + 1) % every == 0 or nxt == nsteps - 1)):
            nxt += 1
        if nxt == nsteps:
            lat.collide_and_stream(nsteps - t)
            break
        lat.collide_and_stream(nxt - t + 1, stats=True)
        recs.append(lat.internal_statistics()["raw"].copy())
        t = nxt + 1
    return lat.receive(), np.array(recs).reshape(-1, 7)


def _pinned(a):
    """A copy of a in page-locked host memory, which the GPU addresses
    directly on any system (ordinary memory only on a GB300)."""
    torch = pytest.importorskip("torch")
    p = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
    p[...] = a
    return p


def _case(name):
    if name == "channel":                     # faces at the x ends, momentum exchange, walls
        return workloads.channel_sphere((24, 12, 12), (8.2, 5.6, 6.3), 2.5, 0.05, 1.8)
    if name == "periodic":                    # periodic x: slab 0 waits for the last slab
        return workloads.forced_channel((20, 10, 12), omega=1.6, seed=4, sigma=1e-4, drive=1e-3)
    raise KeyError(name)


@pytest.mark.parametrize("precision", ["fp64", "fp32", "bf16", "fp16"])
@pytest.mark.parametrize("warm", [0, 1])          # 0: the first step is odd (plain send); 1: even (slab inserts)
@pytest.mark.parametrize("name", ["channel", "periodic"])
def test_run_host_equals_send_steps_receive(name, warm, precision):
    wl = _case(name)
    a, b = wl.lattice(precision), wl.lattice(precision)
    a.collide_and_stream(3 + warm)
    b.collide_and_stream(3 + warm)
    f0 = a.receive()
    fin, fout = _pinned(f0), _pinned(np.zeros_like(f0))
    for nsteps, every in ((7, 3), (6, 0), (2, 1), (23, 10)):
        got, st = a.run_host(fin, nsteps, every, out=fout)
        ref, st_ref = _sequential(b, f0, nsteps, every)
        assert np.array_equal(got, ref), (nsteps, every, np.abs(got - ref).max())
        assert st.shape == st_ref.shape
        np.testing.assert_allclose(st, st_ref, rtol=1e-12, atol=1e-15)
        # both continue from the same state and parity
        a.collide_and_stream(1)
        b.collide_and_stream(1)
        assert np.array_equal(a.receive(), b.receive())


def test_run_host_without_overlap_paths(monkeypatch):
    """One step, and a context whose transfers go through the staging buffer
    (no direct host pointers), give the sequential result."""
    from palabos_gb300.lattice import Context
    monkeypatch.setenv("PLBGPU_STAGED_TRANSFERS", "1")
    staged = Context()
    wl = _case("channel")
    a, b = wl.lattice("fp64", ctx=staged), wl.lattice("fp64")
    f0 = a.receive()
    got, _ = a.run_host(f0, 1)
    ref, _ = _sequential(b, f0, 1, 0)
    assert np.array_equal(got, ref)
    out = np.empty_like(f0)
    got2, st = a.run_host(got, 4, 2, out=out)
    ref2, st_ref = _sequential(b, ref, 4, 2)
    assert got2 is out and np.array_equal(got2, ref2)
    np.testing.assert_allclose(st, st_ref, rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("pinned", [False, True])
def test_run_host_in_place_buffer(pinned):
    wl = _case("periodic")
    a, b = wl.lattice("fp64"), wl.lattice("fp64")
    f = a.receive()
    ref, _ = _sequential(b, f.copy(), 5, 0)
    if pinned:
        f = _pinned(f)
    got, _ = a.run_host(f, 5, 0, out=f)      # the same buffer in and out
    assert got is f and np.array_equal(f, ref)


def test_run_host_narrow_domain():
    """Two slabs of two planes (nx = 4), walled x: each slab's neighbour is
    the other one."""
    wl = workloads.forced_channel((4, 6, 10), omega=1.3, seed=8, sigma=1e-4, drive=1e-3)
    wl.periodic = (0, 0, 0)
    wl.kinds[0] = wl.kinds[-1] = N.BOUNCEBACK
    a, b = wl.lattice("fp32"), wl.lattice("fp32")
    f0 = a.receive()
    got, st = a.run_host(_pinned(f0), 9, 4, out=_pinned(f0))
    ref, st_ref = _sequential(b, f0, 9, 4)
    assert np.array_equal(got, ref)
    np.testing.assert_allclose(st, st_ref, rtol=1e-12, atol=1e-15)


def test_run_host_stochastic_rounding_tracks_sequential():
    """BF16 with stochastic rounding hashes the slot's device address into its
    random bits, so two lattices agree only to the rounding."""
    wl = _case("channel")
    a, b = wl.lattice("bf16sr"), wl.lattice("bf16sr")
    a.collide_and_stream(4)
    b.collide_and_stream(4)
    f0 = a.receive()
    got, st = a.run_host(f0, 6, 3)
    ref, st_ref = _sequential(b, f0, 6, 3)
    assert np.abs(got - ref).max() <= 0.03 * np.abs(ref).max()
    assert st.shape == st_ref.shape == (2, 7)
    np.testing.assert_allclose(st[:, 6], st_ref[:, 6])          # the cells counted
    np.testing.assert_allclose(st[:, 0], st_ref[:, 0], atol=1e-3)
