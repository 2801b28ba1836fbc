"""Mesh generators and the oracle's restatement of the reference voxelizer,
against the reference's own voxel flags (tests/golden/voxel_reference.npz,
made by tests/golden/make_voxel_golden.py from oracle/_ref/plb_voxel) and
against geometry whose answer is known: analytic spheres and boxes.
"""
import os

import numpy as np
import pytest

import voxcases

import oracle as O
from palabos_gb300 import meshes, voxel
from palabos_gb300 import native as N


def _signed_volume(tri):
    return float(np.sum(np.einsum("ij,ij->i", tri[:, 0], np.cross(tri[:, 1], tri[:, 2])))) / 6.0


def _closed(tri):
    """Every edge is shared by exactly two triangles, in opposite directions."""
    edges = {}
    for t in np.round(tri, 12):
        for a, b in ((0, 1), (1, 2), (2, 0)):
            key = (tuple(t[a]), tuple(t[b]))
            edges[key] = edges.get(key, 0) + 1
    return all(edges.get((b, a), 0) == n for (a, b), n in edges.items())


def test_meshes_are_closed_and_point_outwards():
    s = meshes.sphere((10.3, 11.1, 9.7), 6.4, 500)
    assert len(s) >= 500 and _closed(s)
    assert _signed_volume(s) == pytest.approx(4 / 3 * np.pi * 6.4 ** 3, rel=0.02)
    c = meshes.cuboid((1.5, 2.0, 3.25), (9.5, 7.0, 8.25), (2, 3, 1))
    assert _closed(c)
    assert _signed_volume(c) == pytest.approx(8.0 * 5.0 * 5.0, rel=1e-12)
    assert _signed_volume(meshes.merge(s, c)) == pytest.approx(_signed_volume(s) + _signed_volume(c))


def _grid(shape):
    return np.meshgrid(*(np.arange(n, dtype=float) for n in shape), indexing="ij")


def test_oracle_voxelizer_sphere_matches_geometry():
    shape, c, r = (32, 34, 30), (15.3, 16.7, 14.1), 9.2
    flags = O.voxelize(meshes.sphere(c, r, 320), shape)
    X, Y, Z = _grid(shape)
    d = np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2)
    inside = np.isin(flags, (voxel.INSIDE, voxel.INNER_BORDER))
    # the facets stay within 0.5 cell of the sphere of this size and resolution
    far = np.abs(d - r) > 0.5
    assert np.array_equal(inside[far], (d < r)[far])
    assert set(np.unique(flags)) == {voxel.OUTSIDE, voxel.OUTER_BORDER, voxel.INSIDE, voxel.INNER_BORDER}


@pytest.mark.parametrize("lo,hi", [((5.5, 6.25, 4.75), (20.5, 18.25, 22.75)), ((5, 6, 4), (20, 18, 22))])
def test_oracle_voxelizer_box_is_exact(lo, hi):
    """Fractional faces, and faces through cell centres (which count as
    inside: the reference shifts the surface outward along its normal)."""
    shape = (28, 26, 30)
    flags = O.voxelize(meshes.cuboid(lo, hi, (3, 2, 4)), shape)
    X, Y, Z = _grid(shape)
    inside = ((X >= lo[0]) & (X <= hi[0]) & (Y >= lo[1]) & (Y <= hi[1]) & (Z >= lo[2]) & (Z <= hi[2]))
    assert np.array_equal(np.isin(flags, (voxel.INSIDE, voxel.INNER_BORDER)), inside)


@pytest.mark.parametrize("width", [0, 1, 2])
def test_oracle_border_layers(width):
    """DetectBorderLineFunctional3D: a border cell has a cell of the other
    side within `width` (box neighbourhood), a bulk cell has none."""
    shape = (20, 21, 19)
    flags = O.voxelize(meshes.cuboid((5.5, 6.5, 4.5), (13.5, 14.5, 12.5)), shape, width)
    inside = np.isin(flags, (voxel.INSIDE, voxel.INNER_BORDER))
    padded = np.pad(inside, width, constant_values=False)
    padded_out = np.pad(~inside, width, constant_values=False)
    near_in = np.zeros(shape, bool)
    near_out = np.zeros(shape, bool)
    for dx in range(-width, width + 1):
        for dy in range(-width, width + 1):
            for dz in range(-width, width + 1):
                sl = tuple(slice(width + d, width + d + n) for d, n in zip((dx, dy, dz), shape))
                near_in |= padded[sl]
                near_out |= padded_out[sl]
    assert np.array_equal(flags == voxel.OUTER_BORDER, ~inside & near_in)
    assert np.array_equal(flags == voxel.INNER_BORDER, inside & near_out)


def test_oracle_voxelizer_two_bodies():
    shape = (40, 30, 30)
    flags = O.voxelize(meshes.merge(meshes.sphere((11.2, 15.3, 14.6), 6.1, 320),
                                    meshes.cuboid((23.5, 8.5, 9.5), (33.5, 21.5, 19.5))), shape)
    assert not np.isin(flags[:, :, :2], (voxel.INSIDE, voxel.INNER_BORDER)).any()
    assert np.isin(flags[11, 15, 14], (voxel.INSIDE,)) and flags[28, 15, 14] == voxel.INSIDE
    assert flags[20, 15, 14] == voxel.OUTSIDE and flags[18, 15, 14] == voxel.OUTER_BORDER


def test_kinds_from_flags():
    flags = np.array([voxel.OUTSIDE, voxel.OUTER_BORDER, voxel.INNER_BORDER, voxel.INSIDE])
    assert list(voxel.kinds_from_flags(flags, "outside")) == [N.BGK, N.BGK, N.BOUNCEBACK, N.NODYNAMICS]
    assert list(voxel.kinds_from_flags(flags, "inside", N.GUO)) == [N.NODYNAMICS, N.BOUNCEBACK, N.GUO, N.GUO]
    with pytest.raises(ValueError):
        voxel.kinds_from_flags(flags, "around")


@pytest.mark.parametrize("binary", [True, False])
def test_stl_round_trip_and_lattice_units(tmp_path, binary):
    tri = meshes.sphere((0.1, -0.2, 0.05), 0.4, 80)
    path = tmp_path / "s.stl"
    meshes.write_stl(path, tri, binary=binary)
    back = meshes.read_stl(path)
    assert back.shape == tri.shape
    assert np.allclose(back, tri, atol=1e-6 if binary else 0.0)
    lu, origin, dx = meshes.to_lattice_units(back, 40, 0, layer=3)
    assert lu[..., 0].min() == pytest.approx(3.0) and lu[..., 0].max() == pytest.approx(43.0)
    assert dx == pytest.approx(np.ptp(back[..., 0]) / 40)
    assert np.allclose(origin + dx * lu.reshape(-1, 3), back.reshape(-1, 3))
    flags = O.voxelize(lu, (50, 50, 50))
    assert np.isin(flags[23, 23, 23], (voxel.INSIDE,))


VOXEL_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "voxel_reference.npz")


@pytest.mark.parametrize("width", voxcases.WIDTHS)
@pytest.mark.parametrize("name", sorted(voxcases.CASES))
def test_oracle_voxelizer_matches_reference(name, width):
    """The restated flood gives the reference's voxel flags cell for cell:
    spheres (generic and integer centres, vertices on cell centres), boxes
    with fractional and integer faces, two bodies, a thin slab."""
    g = np.load(VOXEL_GOLDEN)
    tri, shape = g[f"{name}__tri"], tuple(g[f"{name}__shape"])
    assert np.array_equal(O.voxelize(tri, shape, width), g[f"{name}__w{width}"])


def test_reference_flood_misreads_edge_touches():
    """The reference on a thin box whose edges lie exactly on the flood's
    diagonal neighbour segments: it merges the two equal-distance crossings
    of such a touch into one, flips the flag and marks cells wrongly, so its
    inside set is not the box (the GPU counts the touch as no crossing and
    gives the box, tests/test_gpu_voxel.py)."""
    g = np.load(VOXEL_GOLDEN)
    lo, hi, _, shape = voxcases.EDGE_TOUCH
    X, Y, Z = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
    box = (X > lo[0]) & (X < hi[0]) & (Y > lo[1]) & (Y < hi[1]) & (Z > lo[2]) & (Z < hi[2])
    inside = np.isin(g["edge_touch__w1"], (3, 4))
    assert (inside != box).sum() > 0


PLB_VOXEL = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "plb_voxel")


def _awkward_facets():
    """A sphere plus facets the reference's reader treats specially: stored
    normals opposite to the vertex order, a repeated vertex, collinear
    vertices, and a 1e-6 edge (dropped at FLT precision, kept at DBL)."""
    tri = meshes.sphere((4.1, 3.7, 5.2), 2.5, 80)
    extra = np.array([[[3.0, 3.0, 3.0], [3.0, 3.0, 3.0], [4.0, 3.0, 3.0]],
                      [[1.0, 1.0, 1.0], [2.0, 2.0, 2.0], [3.0, 3.0, 3.0]],
                      [[3.0, 4.0, 5.0], [3.000001, 4.0, 5.0], [3.0, 5.0, 5.0]]])
    tri = np.concatenate([tri, extra])
    cn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    nrm = cn / np.maximum(np.linalg.norm(cn, axis=1, keepdims=True), 1e-300)
    nrm[::7] *= -1.0
    return tri, nrm


def _write(path, tri, nrm, binary):
    if binary:
        rec = np.zeros(len(tri), np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("attr", "<u2")]))
        rec["n"], rec["v"] = nrm, tri
        with open(path, "wb") as f:
            f.write(b"binary".ljust(80, b" ") + np.uint32(len(tri)).tobytes() + rec.tobytes())
    else:
        lines = ["solid awkward"]
        for t, n in zip(tri, nrm):
            lines += ["  facet normal " + " ".join(repr(float(x)) for x in n), "    outer loop"]
            lines += ["      vertex " + " ".join(repr(float(x)) for x in v) for v in t]
            lines += ["    endloop", "  endfacet"]
        with open(path, "w") as f:
            f.write("\n".join(lines + ["endsolid awkward", ""]))


@pytest.mark.skipif(not os.path.exists(PLB_VOXEL), reason="reference driver not built (needs the reference sources)")
@pytest.mark.parametrize("precision", ["flt", "dbl"])
@pytest.mark.parametrize("binary", [True, False])
def test_read_stl_matches_reference_reader(binary, precision, tmp_path):
    """read_stl gives the triangles the reference's TriangleSet(fname,
    precision) reads from the same file: same order and values, facets with
    reversed normals reoriented, degenerate facets dropped."""
    import subprocess
    tri, nrm = _awkward_facets()
    path, out = str(tmp_path / "m.stl"), str(tmp_path / "r")
    _write(path, tri, nrm, binary)
    subprocess.run([PLB_VOXEL, "--stl", path, precision, out], check=True, capture_output=True)
    data = open(out, "rb").read()
    assert data[:8] == b"PLBTRI01"
    n = int(np.frombuffer(data, "<i4", 1, 8)[0])
    ref = np.frombuffer(data, "<f8", n * 9, 12).reshape(n, 3, 3)
    got = meshes.read_stl(path, precision)
    assert got.shape == ref.shape and np.array_equal(got, ref)


@pytest.mark.skipif(not os.path.exists(PLB_VOXEL), reason="reference driver not built (needs the reference sources)")
@pytest.mark.parametrize("binary", [True, False])
def test_written_stl_scales_like_reference(binary, tmp_path):
    """Files written by write_stl are read by the reference (ASCII included:
    its reader's ASCII test looks for the first "endfacet" in a fixed window),
    and to_lattice_units gives the triangles of the reference's
    DEFscaledMesh(set, resolution, referenceDirection, margin, extraLayer)
    bit for bit."""
    import subprocess
    tri = meshes.merge(meshes.sphere((4.1, 3.7, 5.2), 2.5, 320), meshes.cuboid((7.3, 1.2, 2.2), (9.9, 4.4, 8.1)))
    path, out = str(tmp_path / "m.stl"), str(tmp_path / "r")
    meshes.write_stl(path, tri, binary=binary)
    for res, direction, margin, extra in [(40, 0, 0, 0), (64, 1, 2, 1), (33, 2, 3, 0)]:
        subprocess.run([PLB_VOXEL, "--scale", path, str(res), str(direction), str(margin), str(extra), out],
                       check=True, capture_output=True)
        data = open(out, "rb").read()
        n = int(np.frombuffer(data, "<i4", 1, 8)[0])
        ref = np.frombuffer(data, "<f8", n * 9, 12).reshape(n, 3, 3)
        got = meshes.to_lattice_units(meshes.read_stl(path, "dbl"), res, direction, margin + extra)[0]
        assert got.shape == ref.shape and np.array_equal(got, ref)
