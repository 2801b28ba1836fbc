"""GPU voxelizer against the reference's own voxel flags
(tests/golden/voxel_reference.npz) and the oracle's restatement of its
voxelize() (flood fill with segment crossings), and the voxelized-domain
pipeline (kinds, sparse blocks) against the oracle's block selection."""
import os

import numpy as np
import pytest

import oracle as O
from palabos_gb300 import DeviceLattice3D, PlbGpuError, meshes, voxel
from palabos_gb300 import native as N
from voxcases import CASES, WIDTHS

pytestmark = pytest.mark.gpu

VOXEL_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "voxel_reference.npz")


@pytest.mark.parametrize("width", WIDTHS)
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_voxelizer_matches_oracle(name, width):
    make, shape = CASES[name]
    tri = make()
    assert np.array_equal(voxel.voxelize(tri, shape, width), O.voxelize(tri, shape, width))


@pytest.mark.parametrize("width", WIDTHS)
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_voxelizer_matches_reference(name, width):
    """The reference's own voxel flags of the same meshes."""
    g = np.load(VOXEL_GOLDEN)
    tri, shape = g[f"{name}__tri"], tuple(g[f"{name}__shape"])
    assert np.array_equal(voxel.voxelize(tri, shape, width), g[f"{name}__w{width}"])


def test_gpu_voxelizer_counts_edge_touches_as_touches():
    """A thin box with half-integer faces: diagonal neighbour segments of the
    reference's flood pass exactly through its edges, and counting such a
    touch as a crossing (the reference merges equal-distance crossings) marks
    cells beyond the box inside.  The GPU counts crossings watertightly and
    gives the box itself."""
    shape, lo, hi = (34, 12, 28), (3.5, 4.25, 5.5), (30.5, 5.75, 22.5)
    flags = voxel.voxelize(meshes.cuboid(lo, hi, (5, 1, 3)), shape)
    X, Y, Z = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
    box = (X > lo[0]) & (X < hi[0]) & (Y > lo[1]) & (Y < hi[1]) & (Z > lo[2]) & (Z < hi[2])
    assert np.array_equal(np.isin(flags, (voxel.INSIDE, voxel.INNER_BORDER)), box)


@pytest.mark.parametrize("width", (0, 1))
def test_gpu_voxelizer_finely_meshed_faces_on_lattice_planes(width):
    """A cuboid whose faces lie on lattice planes, every face cut into 20x20
    squares: each lattice line in its y and z faces runs along some forty
    facets parallel to x, whose on-surface cells form one run however many
    facets cover them.  The GPU gives exactly the flags of the same box meshed
    with two triangles per face, on which it equals the oracle (the
    reference's flood).  On the subdivided mesh the oracle itself does not: its
    flood meets facet edges head-on along many diagonal neighbour segments and
    merges the equal-distance crossings there (the edge-touch defect of the
    reference's flood), misplacing some 700 cells."""
    shape = (26, 24, 28)
    fine = voxel.voxelize(meshes.cuboid((5, 6, 4), (20, 18, 22), (20, 20, 20)), shape, width)
    coarse_tri = meshes.cuboid((5, 6, 4), (20, 18, 22), (1, 1, 1))
    assert np.array_equal(fine, voxel.voxelize(coarse_tri, shape, width))
    assert np.array_equal(fine, O.voxelize(coarse_tri, shape, width))


def test_gpu_voxelizer_large_sphere_matches_geometry():
    """256^3 box, 20480 facets: the inside set equals the analytic sphere
    away from the surface, and the border layers are one cell thick."""
    n, c, r = 256, np.array([127.6, 128.3, 126.9]), 90.4
    flags = voxel.voxelize(meshes.sphere(c, r, 20000), (n, n, n))
    x = np.arange(n, dtype=float)
    d2 = ((x[:, None, None] - c[0]) ** 2 + (x[None, :, None] - c[1]) ** 2 + (x[None, None, :] - c[2]) ** 2)
    d = np.sqrt(d2)
    inside = np.isin(flags, (voxel.INSIDE, voxel.INNER_BORDER))
    far = np.abs(d - r) > 0.2      # the facets stay within 0.2 cell of this sphere
    assert np.array_equal(inside[far], (d < r)[far])
    assert not np.isin(flags[np.abs(d - r) > 2.0], (voxel.INNER_BORDER, voxel.OUTER_BORDER)).any()


def test_voxelized_domain_kinds_and_sparse_blocks():
    shape = (64, 48, 48)
    # two disjoint chambers (a union of overlapping closed meshes is not a
    # closed surface: the overlap would count as outside)
    boxes = [((2.3, 2.6, 2.7), (61.4, 13.3, 13.2)), ((2.4, 20.2, 2.5), (13.6, 45.3, 13.4))]
    tri = meshes.merge(*[meshes.cuboid(lo, hi) for lo, hi in boxes])
    lat = DeviceLattice3D(*shape, 1.0)
    flags, kinds, keep = voxel.voxelized_domain(lat, tri, flow="inside", blocks=(4, 3, 3))
    # the boxes themselves (the flood's diagonal segments would touch their
    # edges exactly: x = 2.3 and y = 13.3 share a fractional part)
    X, Y, Z = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
    inside = np.zeros(shape, bool)
    for lo, hi in boxes:
        inside |= (X > lo[0]) & (X < hi[0]) & (Y > lo[1]) & (Y < hi[1]) & (Z > lo[2]) & (Z < hi[2])
    assert np.array_equal(np.isin(flags, (voxel.INSIDE, voxel.INNER_BORDER)), inside)
    assert np.array_equal(kinds, voxel.kinds_from_flags(flags, "inside"))
    assert np.array_equal(keep, O.sparse_blocks((kinds != N.NODYNAMICS).astype(np.int32), (4, 3, 3)))
    assert 0 < keep.sum() < keep.size        # the chambers leave blocks out
    lat.collide_and_stream(4)                 # the sparse lattice steps


def test_voxelizer_rejects_bad_input():
    tri = meshes.sphere((8.2, 8.3, 8.1), 4.0, 80)
    with pytest.raises(PlbGpuError):
        voxel.voxelize(tri, (0, 16, 16))
    with pytest.raises(PlbGpuError):
        voxel.voxelize(tri, (16, 16, 16), border_width=-1)
    bad = tri.copy()
    bad[0, 0, 0] = np.nan
    with pytest.raises(PlbGpuError):
        voxel.voxelize(bad, (16, 16, 16))
    # 40 thin slabs stacked along x: 80 crossings on every line through them
    slabs = meshes.merge(*[meshes.cuboid((2.2 + 2 * i, 2.5, 2.5), (2.7 + 2 * i, 9.5, 9.5)) for i in range(40)])
    with pytest.raises(PlbGpuError):
        voxel.voxelize(slabs, (90, 12, 12))
    assert voxel.voxelize(tri, (16, 16, 16)).shape == (16, 16, 16)   # the context still works
