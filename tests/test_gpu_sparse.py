"""Sparse domains stepped through row lists: the rows whose 3x3 neighbourhood of
rows lies entirely in kept blocks take the interior-row kernels (uniform
neighbour offsets; the 128-bit kernel for the 2-byte forms), the other live
rows the general kernel, and rows of dropped blocks nothing.

The geometry is a voxelized sphere in a periodic box with a body force, flow
outside the sphere, 8^3 blocks: the blocks deep inside the sphere hold neither
fluid nor wall and are dropped (computeSparseManagement,
offLattice/makeSparse3D.hh:107-160).  FP64 must equal the oracle (which steps
every cell with the general rule) bit for bit; the reduced forms must equal
their one-cell kernels bit for bit.
"""
import os

import numpy as np
import pytest

import oracle as O
from palabos_gb300 import Context, DeviceLattice3D, meshes, voxel
from palabos_gb300 import native as N

pytestmark = pytest.mark.gpu

SHAPE = (48, 40, 48)
BLOCKS = (6, 5, 6)


def _geometry():
    tri = meshes.sphere((23.6, 19.7, 24.2), 17.3, 2000)
    flags = voxel.voxelize(tri, SHAPE)
    kinds = voxel.kinds_from_flags(flags, "outside", fluid=N.GUO)
    keep = O.sparse_blocks((kinds != N.NODYNAMICS).astype(np.int32), BLOCKS)
    live = O.sparse_cell_mask(SHAPE, BLOCKS, keep)
    return kinds, keep, live


def _lattice(kinds, precision, ctx=None):
    lat = DeviceLattice3D(*SHAPE, 1.7, precision, ctx)
    lat.periodicity(1, 1, 1)
    lat.set_kinds(kinds)
    lat.select_sparse_blocks((kinds != N.NODYNAMICS).astype(np.int32), BLOCKS)
    force = np.zeros(SHAPE + (3,))
    force[..., 0] = 2e-5
    force[..., 1] = -1e-5
    lat.set_external_vector(None, force)
    return lat, force


def _initial(live):
    rng = np.random.default_rng(41)
    t = np.asarray([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    f = 1e-3 * rng.standard_normal(SHAPE + (19,)) * t[None, None, None]
    f[~live] = 0.0
    return f


def test_sparse_row_lists_fp64_match_oracle():
    kinds, keep, live = _geometry()
    assert 0 < keep.sum() < keep.size
    lat, force = _lattice(kinds, "fp64")
    f0 = _initial(live)
    lat.send(f0)
    lat.collide_and_stream(11, stats=True)
    got = lat.receive()
    st = lat.internal_statistics()
    flags = kinds.copy()
    flags[~live] = N.NONE
    ol = O.OracleLattice(*SHAPE, (1, 1, 1), 1.7, flags, None, force)
    ref, stats = ol.run(f0, 11)
    assert np.array_equal(got[live], ref[live])
    assert (got[~live] == 0).all()
    assert st["count"] == int(stats[-1, 6])
    np.testing.assert_allclose(st["raw"][:3], stats[-1, :3], rtol=1e-12, atol=1e-17)


def _run_form(kinds, live, precision, form):
    old = os.environ.get("PLBGPU_ROW_KERNEL")
    if form:
        os.environ["PLBGPU_ROW_KERNEL"] = form
    else:
        os.environ.pop("PLBGPU_ROW_KERNEL", None)
    try:
        ctx = Context(0)
    finally:
        if old is None:
            os.environ.pop("PLBGPU_ROW_KERNEL", None)
        else:
            os.environ["PLBGPU_ROW_KERNEL"] = old
    lat, _ = _lattice(kinds, precision, ctx)
    lat.send(_initial(live))
    lat.collide_and_stream(9)
    f = lat.receive()
    lat.close()
    ctx.close()
    return f


@pytest.mark.parametrize("precision", ["bf16", "fp16", "fp32"])
def test_sparse_row_lists_reduced_forms_match_one_cell_kernel(precision):
    kinds, _, live = _geometry()
    f_fast = _run_form(kinds, live, precision, None)
    f_cell = _run_form(kinds, live, precision, "cell")
    assert np.isfinite(f_fast).all()
    assert np.array_equal(f_fast, f_cell)
