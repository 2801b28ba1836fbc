"""Sparse domains stepped through tile lists: the tiles (up to 32 cells of a
row) whose 3x3 neighbourhood of rows lies entirely in kept blocks, one cell
beyond each end included, take the interior-row kernels (uniform neighbour
offsets); the other live tiles of interior rows take the one-cell row kernel
with each cell's mask of neighbours in dropped blocks; the live tiles of the
domain's border rows the general kernel; cells of dropped blocks nothing.

The geometry is a voxelized sphere in a box with a body force, flow outside
the sphere: the blocks deep inside the sphere hold neither fluid nor wall and
are dropped (computeSparseManagement, offLattice/makeSparse3D.hh:107-160).
Two boxes: periodic with rows of one 48-cell tile, and periodic in x and y
only with rows of a 64-cell and a 36-cell tile.  FP64 must equal the oracle
(which steps every cell with the general rule) bit for bit; the reduced forms
must equal their one-cell kernels bit for bit, for every interior-row kernel.
"""
import os

import numpy as np
import pytest

import oracle as O
from palabos_gb300 import Context, DeviceLattice3D, meshes, voxel
from palabos_gb300 import native as N

pytestmark = pytest.mark.gpu

# (shape, blocks, periodicity, sphere centre, radius)
BOXES = {
    "periodic_48": ((48, 40, 48), (6, 5, 6), (1, 1, 1), (23.6, 19.7, 24.2), 17.3),
    "walled_z_100": ((40, 36, 100), (5, 4, 10), (1, 1, 0), (19.6, 17.7, 51.2), 16.3),
}


def _geometry(box):
    shape, blocks, _, centre, radius = BOXES[box]
    tri = meshes.sphere(centre, radius, 2000)
    flags = voxel.voxelize(tri, shape)
    kinds = voxel.kinds_from_flags(flags, "outside", fluid=N.GUO)
    keep = O.sparse_blocks((kinds != N.NODYNAMICS).astype(np.int32), blocks)
    live = O.sparse_cell_mask(shape, blocks, keep)
    return kinds, keep, live


def _lattice(box, kinds, precision, ctx=None):
    shape, blocks, per, _, _ = BOXES[box]
    lat = DeviceLattice3D(*shape, 1.7, precision, ctx)
    lat.periodicity(*per)
    lat.set_kinds(kinds)
    lat.select_sparse_blocks((kinds != N.NODYNAMICS).astype(np.int32), blocks)
    force = np.zeros(shape + (3,))
    force[..., 0] = 2e-5
    force[..., 1] = -1e-5
    lat.set_external_vector(None, force)
    return lat, force


def _initial(box, live):
    shape = BOXES[box][0]
    rng = np.random.default_rng(41)
    t = np.asarray([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    f = 1e-3 * rng.standard_normal(shape + (19,)) * t[None, None, None]
    f[~live] = 0.0
    return f


@pytest.mark.parametrize("box", sorted(BOXES))
def test_sparse_tile_lists_fp64_match_oracle(box):
    shape, _, per, _, _ = BOXES[box]
    kinds, keep, live = _geometry(box)
    assert 0 < keep.sum() < keep.size
    lat, force = _lattice(box, kinds, "fp64")
    f0 = _initial(box, live)
    lat.send(f0)
    lat.collide_and_stream(11, stats=True)
    got = lat.receive()
    st = lat.internal_statistics()
    flags = kinds.copy()
    flags[~live] = N.NONE
    ol = O.OracleLattice(*shape, per, 1.7, flags, None, force)
    ref, stats = ol.run(f0, 11)
    assert np.array_equal(got[live], ref[live])
    assert (got[~live] == 0).all()
    assert st["count"] == int(stats[-1, 6])
    np.testing.assert_allclose(st["raw"][:3], stats[-1, :3], rtol=1e-12, atol=1e-17)


def _run_form(box, kinds, live, precision, form):
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
    lat, _ = _lattice(box, kinds, precision, ctx)
    lat.send(_initial(box, live))
    lat.collide_and_stream(9)
    f = lat.receive()
    lat.close()
    ctx.close()
    return f


@pytest.mark.parametrize("form", [None, "vec8", "vec4", "vec2"])
@pytest.mark.parametrize("precision", ["bf16", "fp16", "fp32"])
@pytest.mark.parametrize("box", sorted(BOXES))
def test_sparse_tile_lists_reduced_forms_match_one_cell_kernel(box, precision, form):
    if form and precision == "fp32":
        pytest.skip("the vector kernels are forms of the 2-byte storage types")
    kinds, _, live = _geometry(box)
    f_fast = _run_form(box, kinds, live, precision, form)
    f_cell = _run_form(box, kinds, live, precision, "cell")
    assert np.isfinite(f_fast).all()
    assert np.array_equal(f_fast, f_cell)
