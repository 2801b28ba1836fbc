"""The slab schedule of plbgpu_run_host (plbgpu_run_host_plan, host logic
only), executed on a one-dimensional model of the in-place (AA) layout with
the library's slot rules, against the plain order: insert every cell, step
the whole domain nsteps times, extract every cell.

Model (three velocities along x, which is all that x-slabs see of D3Q19:
every population crosses at most one plane per step):
  even parity: population i of cell x sits in slot (x, i);
  odd parity:  population i of cell x sits in slot (x - c_i, opp(i)), or in
               (x, i) when x - c_i is outside a walled domain;
  a step at parity p reads the cell's populations at parity p and writes
  f*_i where population i of cell x + c_i is read at the other parity (back
  into the cell, as opp(i), when x + c_i is outside a walled domain).
Each slot then belongs to one cell at each parity, which is what lets slabs
step separately.  The slots start as NaN, so a step that reads a slot no
insert or step wrote yet poisons the result, and a step or receive issued
out of order reads a stale value: either way the states differ."""
import ctypes
import itertools

import numpy as np
import pytest

from palabos_gb300 import native as N

C = np.array([0, 1, -1])
OPP = np.array([0, 2, 1])
SEND, STEP, RECEIVE, WHOLE = 0, 1, 2, 3
ERR_ARG = -1   # PLBGPU_ERR_ARG


def _plan(nx, periodic, nsteps, stats_every, precision):
    lib = N.load()
    width = ctypes.c_int()
    count = ctypes.c_size_t()
    assert lib.plbgpu_run_host_plan(nx, periodic, nsteps, stats_every, precision, ctypes.byref(width), None, 0,
                                    ctypes.byref(count)) == N.OK
    ops = (ctypes.c_int * (3 * count.value))()
    assert lib.plbgpu_run_host_plan(nx, periodic, nsteps, stats_every, precision, None, ops, len(ops),
                                    ctypes.byref(count)) == N.OK
    return width.value, np.array(ops, dtype=np.int64).reshape(-1, 3)


class AALine:
    def __init__(self, nx, periodic):
        self.nx, self.periodic = nx, periodic
        self.slots = np.full((nx, 3), np.nan)

    def _wrap(self, x):
        return x % self.nx if self.periodic else x

    def _inside(self, x):
        return self.periodic or (0 <= x < self.nx)

    def slot(self, odd, x, i):
        if not odd:
            return x, i
        s = x - C[i]
        if self._inside(s):
            return self._wrap(s), OPP[i]
        return x, i

    def insert(self, odd, x, f):
        for i in range(3):
            self.slots[self.slot(odd, x, i)] = f[i]

    def extract(self, odd, x):
        return np.array([self.slots[self.slot(odd, x, i)] for i in range(3)])

    def step(self, odd, x):
        f = self.extract(odd, x)
        # a nonlinear, cell-dependent collision: any mixing shows misordering
        rho = f.sum()
        fs = f + 0.3 * (rho / 3.0 - f) + 0.01 * np.sin(rho + x) * C
        for i in range(3):
            y = x + C[i]
            if self._inside(y):
                self.slots[self.slot(not odd, self._wrap(y), i)] = fs[i]
            else:
                self.slots[self.slot(not odd, x, OPP[i])] = fs[i]


def _run_plain(nx, periodic, nsteps, odd0, f0):
    m = AALine(nx, periodic)
    for x in range(nx):
        m.insert(odd0, x, f0[x])
    for t in range(nsteps):
        for x in range(nx):
            m.step(odd0 ^ (t & 1), x)
    return np.array([m.extract(odd0 ^ (nsteps & 1), x) for x in range(nx)])


def _run_plan(nx, periodic, nsteps, odd0, f0, width, ops):
    m = AALine(nx, periodic)
    out = np.full((nx, 3), np.nan)
    slab = lambda j: range(j * width, min(nx, (j + 1) * width))
    for kind, j, t in ops:
        if kind == SEND:
            for x in slab(j):
                m.insert(odd0, x, f0[x])
        elif kind == STEP:
            for x in slab(j):
                m.step(odd0 ^ (t & 1), x)
        elif kind == RECEIVE:
            for x in slab(j):
                out[x] = m.extract(odd0 ^ (nsteps & 1), x)
        else:
            for s in range(j, t):
                for x in range(nx):
                    m.step(odd0 ^ (s & 1), x)
    return out


def _check_structure(nx, periodic, nsteps, stats_every, width, ops):
    nslab = (nx + width - 1) // width
    kinds = ops[:, 0]
    assert (kinds == WHOLE).sum() == 1
    w = int(np.flatnonzero(kinds == WHOLE)[0])
    first, end = ops[w, 1], ops[w, 2]
    assert 1 <= first <= end <= nsteps - 1
    # every slab sent once, in order, before the steps between; received once, after them
    assert list(ops[kinds == SEND, 1]) == list(range(nslab))
    assert np.all(np.flatnonzero(kinds == SEND) < w)
    assert sorted(ops[kinds == RECEIVE, 1]) == list(range(nslab))
    assert np.all(np.flatnonzero(kinds == RECEIVE) > w)
    # each slab takes the ramp steps exactly once, in order
    steps = ops[kinds == STEP]
    for j in range(nslab):
        mine = list(steps[steps[:, 1] == j, 2])
        assert mine == list(range(first)) + list(range(end, nsteps))
    # at most one statistics step in each ramp
    stats_at = [stats_every > 0 and ((t + 1) % stats_every == 0 or t == nsteps - 1) for t in range(nsteps)]
    assert sum(stats_at[:first]) <= 1 and sum(stats_at[end:]) <= 1


CASES = list(itertools.product([4, 5, 7, 16, 33, 40], [0, 1], [2, 3, 5, 8, 13], [0, 1, 3, 100], [N.FP64, N.FP32]))


@pytest.mark.parametrize("nx,periodic,nsteps,stats_every,precision", CASES)
def test_run_host_plan_orders_slabs_like_the_whole_domain(nx, periodic, nsteps, stats_every, precision):
    width, ops = _plan(nx, periodic, nsteps, stats_every, precision)
    _check_structure(nx, periodic, nsteps, stats_every, width, ops)
    rng = np.random.default_rng(nx * 1000 + nsteps * 10 + periodic)
    f0 = rng.uniform(0.1, 1.0, (nx, 3))
    for odd0 in (False, True):
        ref = _run_plain(nx, periodic, nsteps, odd0, f0)
        got = _run_plan(nx, periodic, nsteps, odd0, f0, width, ops)
        assert not np.isnan(ref).any()
        assert np.array_equal(got, ref), (odd0, np.nanmax(np.abs(got - ref)))


def test_run_host_plan_ramps():
    """FP64 takes ramps of two steps, the other forms three; a statistics step
    at every step leaves ramps of one."""
    _, ops = _plan(256, 0, 20, 100, N.FP64)
    w = ops[ops[:, 0] == WHOLE][0]
    assert (w[1], w[2]) == (2, 18)
    _, ops = _plan(256, 0, 20, 100, N.FP32)
    w = ops[ops[:, 0] == WHOLE][0]
    assert (w[1], w[2]) == (3, 17)
    _, ops = _plan(256, 0, 20, 1, N.FP64)
    w = ops[ops[:, 0] == WHOLE][0]
    assert (w[1], w[2]) == (1, 19)


def test_run_host_plan_rejects_bad_arguments():
    lib = N.load()
    count = ctypes.c_size_t()
    assert lib.plbgpu_run_host_plan(3, 0, 5, 0, 0, None, None, 0, ctypes.byref(count)) == ERR_ARG
    assert lib.plbgpu_run_host_plan(16, 0, 1, 0, 0, None, None, 0, ctypes.byref(count)) == ERR_ARG
    assert lib.plbgpu_run_host_plan(16, 0, 5, -1, 0, None, None, 0, ctypes.byref(count)) == ERR_ARG
    assert lib.plbgpu_run_host_plan(16, 0, 5, 0, 9, None, None, 0, ctypes.byref(count)) == ERR_ARG
    assert lib.plbgpu_run_host_plan(16, 0, 5, 0, 0, None, None, 0, ctypes.byref(count)) == N.OK
    small = (ctypes.c_int * 3)()
    assert lib.plbgpu_run_host_plan(16, 0, 5, 0, 0, None, small, 3, ctypes.byref(count)) == ERR_ARG
