"""The allocation-free reduction entry point, checked against plbgpu_reduce.

plbgpu_reduce_noalloc is for callers that cannot call cudaMalloc themselves
(for example applications with their own device-memory pool or a fixed
device-memory budget): they pass their own device arrays
and result buffer, and the entry point keeps its scratch in a static device
array instead of allocating.  Here the caller-owned device memory comes from
torch; the lattice itself is built with the regular C ABI, and both entry
points must agree on the average energy and density.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ROWS = 262144
ERR_ARG = -1


def _lattice(nx, ny, nz, seed):
    import lbcases
    from palabos_gb300 import (DeviceLattice3D, BOUNCEBACK, MOMENTUM_EXCHANGE, NODYNAMICS, INCBGK)
    lat = DeviceLattice3D(nx, ny, nz, 1.7, "fp64", rho0=1.05, bb_rho=1.0)
    kinds = np.zeros((nx, ny, nz), np.uint8)
    kinds[:, 0, :] = BOUNCEBACK
    kinds[:, -1, :] = BOUNCEBACK
    kinds[3:6, 3:6, 2:5] = MOMENTUM_EXCHANGE
    kinds[nx - 3, 2, 1] = NODYNAMICS
    kinds[: nx // 3, ny // 2:, :] = np.where(kinds[: nx // 3, ny // 2:, :] == 0, INCBGK,
                                             kinds[: nx // 3, ny // 2:, :])
    lat.periodicity(True, False, True)
    lat.set_kinds(kinds)
    lat.initialize_momentum_exchange()
    rng = np.random.default_rng(seed)
    lat.send(lbcases.initial_state((nx, ny, nz), rng, u_amp=0.04))
    return lat, kinds


def _device_inputs(lat, kinds, torch, pad):
    """Caller-owned device copies: 19 FP64 planes `stride` apart, and the kinds."""
    f = lat.receive()                       # natural order, [x][y][z][19]
    n = f.shape[0] * f.shape[1] * f.shape[2]
    stride = n + pad
    planes = np.zeros((19, stride))
    planes[:, :n] = f.reshape(n, 19).T
    d_pop = torch.from_numpy(planes).cuda()
    d_kinds = torch.from_numpy(np.ascontiguousarray(kinds).reshape(-1)).cuda()
    return d_pop, d_kinds, stride


def _noalloc(lib, d_pop, stride, d_kinds, shape, lat, d_out):
    nx, ny, nz = shape
    return lib.plbgpu_reduce_noalloc(d_pop.data_ptr(), stride, d_kinds.data_ptr(), nx, ny, nz,
                                     lat.bb_rho, lat.rho0, d_out.data_ptr(), None)


def test_noalloc_matches_allocating_reduction_twice_in_a_row():
    torch = pytest.importorskip("torch")
    from palabos_gb300 import native
    lib = native.load()
    shape = (14, 11, 9)
    lat, kinds = _lattice(*shape, seed=21)
    d_out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")

    for call, pad in enumerate((0, 37)):
        lat.collide_and_stream(5 + call)            # odd then even parity on the device side
        want_e, want_rho = lat.reduce()
        d_pop, d_kinds, stride = _device_inputs(lat, kinds, torch, pad)
        torch.cuda.synchronize()
        assert _noalloc(lib, d_pop, stride, d_kinds, shape, lat, d_out) == 0
        torch.cuda.synchronize()
        got_e, got_rho = d_out.cpu().tolist()
        assert got_e == pytest.approx(want_e, rel=1e-12, abs=0), (call, got_e, want_e)
        assert got_rho == pytest.approx(want_rho, rel=1e-12, abs=0), (call, got_rho, want_rho)

    # the fixed summation order makes repeated calls bit-identical
    first = d_out.clone()
    assert _noalloc(lib, d_pop, stride, d_kinds, shape, lat, d_out) == 0
    torch.cuda.synchronize()
    assert torch.equal(first, d_out)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from palabos_gb300 import native
    lib = native.load()
    d = torch.zeros(4, dtype=torch.float64, device="cuda")
    k = torch.zeros(4, dtype=torch.uint8, device="cuda")
    nx, ny = 1024, MAX_ROWS // 1024 + 1           # nx * ny > scratch rows
    rc = lib.plbgpu_reduce_noalloc(d.data_ptr(), nx * ny, k.data_ptr(), nx, ny, 1, 0.0, 1.0, d.data_ptr(), None)
    assert rc == ERR_ARG
    rc = lib.plbgpu_reduce_noalloc(None, 4, k.data_ptr(), 1, 1, 1, 0.0, 1.0, d.data_ptr(), None)
    assert rc == ERR_ARG
