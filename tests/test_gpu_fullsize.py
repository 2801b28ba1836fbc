"""The benchmarked configurations at their full sizes, FP64, against the
oracle (the reference's arithmetic restated in C, bit-identical to the
reference on every golden case): populations bit for bit, the per-step
statistics and the momentum-exchange drag within 1e-12.

  channel past a sphere  256x128x128, regularized parabolic inlet, regularized
                         pressure outlet, bounce-back walls, momentum-exchange
                         sphere r=16, omega 1.8: 1000 steps, drag every 100
                         (MultiBlockLattice3D::collideAndStream,
                         multiBlock/multiBlockLattice3D.hh:318-357; drag
                         boundaryCondition/bounceBackModels.hh:100-136)
  Taylor-Green vortex    512^3 periodic, u0 0.04, Re 1600: 20 steps

The oracle runs on all host threads of the GPU machine.  The 512^3 case holds
two FP64 states on the host (2 x 20.4 GB) and is skipped when the host has
less memory available than that.
"""
import os

import numpy as np
import pytest

import oracle as O
from palabos_gb300 import workloads

pytestmark = pytest.mark.gpu

REL = 1e-12


def _mem_available_bytes():
    try:
        with open("/proc/meminfo") as fh:
            for line in fh:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def _close(a, b, rel=REL, abs_=1e-15):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return bool(np.all(np.abs(a - b) <= rel * np.abs(b) + abs_))


def test_channel_sphere_full_size_1000_steps_matches_oracle():
    wl = workloads.channel_sphere((256, 128, 128), omega=1.8)
    lat = wl.lattice("fp64")                      # rest state, lattice.initialize()
    ol = O.OracleLattice(*wl.shape, wl.periodic, wl.omega, wl.kinds, wl.bcval)
    O.set_threads(O.max_threads())
    f = ol.initialize(np.zeros(wl.shape + (19,)))
    for chunk in range(10):
        lat.collide_and_stream(100, stats=True)
        f, stats = ol.run(f, 100, with_stats=True, inplace=True)
        got = lat.internal_statistics()
        ref = stats[-1]
        assert got["count"] == int(ref[6])
        assert _close(got["drag"], ref[3:6]), (chunk, got["drag"], ref[3:6])
        assert _close([got["avRhoBar"], got["avUSqr"], got["maxUSqr"]], ref[0:3], abs_=1e-18), (chunk, got, ref)
    out = np.empty(wl.shape + (19,))
    lat.receive(out=out)
    assert np.array_equal(out, f), f"max |diff| {np.abs(out - f).max():.3e}"
    e, d = lat.compute_average_energy(), lat.compute_average_density()
    e_ref, d_ref = ol.reduce(f)
    assert _close([e, d], [e_ref, d_ref], abs_=1e-18)
    # the drag has built up (the flow is not at rest any more)
    assert abs(ref[3]) > 1e-4
    lat.close()


def test_taylor_green_512_fp64_20_steps_matches_oracle():
    n = 512
    state = n ** 3 * 19 * 8
    if _mem_available_bytes() < 2.5 * state:
        pytest.skip(f"needs {2.5 * state / 2**30:.0f} GiB of host memory for two FP64 512^3 states")
    wl = workloads.taylor_green(n)
    lat = wl.lattice("fp64", slab=8)
    f = np.empty((n, n, n, 19))
    lat.receive(out=f)                             # the initial state, bit for bit the GPU's
    ol = O.OracleLattice(n, n, n, wl.periodic, wl.omega, wl.kinds)
    O.set_threads(O.max_threads())
    lat.collide_and_stream(20, stats=True)
    f, stats = ol.run(f, 20, with_stats=True, inplace=True)
    got = lat.internal_statistics()
    assert got["count"] == n ** 3
    # the average rho-bar of the vortex is a sum of 1.3e8 terms of either sign
    # that cancels to ~1e-17: summation order alone moves it by ~1e-16
    assert abs(got["avRhoBar"] - stats[-1, 0]) <= 1e-15
    assert _close([got["avUSqr"], got["maxUSqr"]], stats[-1, 1:3])
    buf = np.empty((8, n, n, 19))
    for x0 in range(0, n, 8):
        lat.receive((x0, x0 + 7, 0, n - 1, 0, n - 1), out=buf)
        if not np.array_equal(buf, f[x0:x0 + 8]):
            raise AssertionError(f"slab x={x0}..{x0 + 7}: max |diff| {np.abs(buf - f[x0:x0 + 8]).max():.3e}")
    lat.close()
