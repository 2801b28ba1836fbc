"""Closed triangle meshes for the voxelizer, in lattice coordinates.

Counterparts of the reference's generators constructSphere and
constructCuboid (offLattice/triangleSetGenerator.h:43-70): a sphere as a
subdivided icosahedron projected on the sphere, a cuboid with each face split
into a grid of triangle pairs.  Every triangle is returned as its three
vertices, ordered so that the normal (v1 - v0) x (v2 - v0) points out of the
body, as the reference's voxelizer assumes.  Meshes are plain arrays
(t, 3, 3) of float64.
"""
from __future__ import annotations

import numpy as np


def _icosahedron():
    p = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0],
                  [0, -1, p], [0, 1, p], [0, -1, -p], [0, 1, -p],
                  [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    return v / np.linalg.norm(v, axis=1, keepdims=True), f


def sphere(center, radius, min_triangles=500):
    """Sphere of the given centre and radius with at least min_triangles
    triangles (20 * 4^k)."""
    v, f = _icosahedron()
    while len(f) < min_triangles:
        verts = list(v)
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        v, f = np.array(verts), np.array(nf, np.int64)
    tri = np.asarray(center, np.float64) + radius * v[f]
    # orient outwards
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    flip = np.einsum("ij,ij->i", n, tri.mean(axis=1) - np.asarray(center, np.float64)) < 0
    tri[flip] = tri[flip][:, ::-1]
    return tri


def cuboid(lower, upper, segments=(1, 1, 1)):
    """Axis-aligned box [lower, upper] with segments[a] divisions along axis a."""
    lo = np.asarray(lower, np.float64)
    hi = np.asarray(upper, np.float64)
    out = []
    for axis in range(3):
        u, w = (axis + 1) % 3, (axis + 2) % 3
        nu, nw = segments[u], segments[w]
        us = np.linspace(lo[u], hi[u], nu + 1)
        ws = np.linspace(lo[w], hi[w], nw + 1)
        for side, val in ((-1, lo[axis]), (1, hi[axis])):
            for i in range(nu):
                for j in range(nw):
                    q = []
                    for a, b in ((i, j), (i + 1, j), (i + 1, j + 1), (i, j + 1)):
                        p = np.zeros(3)
                        p[axis], p[u], p[w] = val, us[a], ws[b]
                        q.append(p)
                    # (u, w) counter-clockwise seen from +axis: normal +axis
                    t1, t2 = [q[0], q[1], q[2]], [q[0], q[2], q[3]]
                    if side < 0:
                        t1, t2 = t1[::-1], t2[::-1]
                    out += [t1, t2]
    return np.array(out, np.float64)


def merge(*meshes):
    """One mesh from several (the reference's TriangleSet::append)."""
    return np.concatenate([np.asarray(m, np.float64).reshape(-1, 3, 3) for m in meshes])


def read_stl(path, precision="flt"):
    """Triangles (t, 3, 3) of an ASCII or binary STL file as the reference's
    TriangleSet(fname, precision) reads them (offLattice/triangleSet.hh:70-345):
    vertices in file order, except that a facet whose vertex order disagrees
    with its stored normal gets its last two vertices swapped, and a facet
    with an edge or an area within 2 eps of zero is dropped
    (checkForDegenerateTrianglesAndFixOrientationNoAbort, :498-548), eps = 10x
    the machine epsilon of `precision`, "flt" (the constructor's default) or
    "dbl" (core/globalDefs.h:104-126)."""
    with open(path, "rb") as f:
        data = f.read()
    tri = nrm = None
    if len(data) >= 84:
        count = int(np.frombuffer(data, "<u4", 1, 80)[0])
        if 84 + 50 * count == len(data):
            rec = np.frombuffer(data, np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("attr", "<u2")]), count, 84)
            tri, nrm = rec["v"].astype(np.float64), rec["n"].astype(np.float64)
    if tri is None:
        text = data.decode("ascii", errors="replace").split()
        verts = [text[i + 1:i + 4] for i, w in enumerate(text) if w == "vertex"]
        norms = [text[i + 1:i + 4] for i, w in enumerate(text) if w == "normal"]
        if not verts or len(verts) % 3 or len(norms) * 3 != len(verts):
            raise ValueError(f"{path}: not an STL file")
        tri = np.array(verts, np.float64).reshape(-1, 3, 3)
        nrm = np.array(norms, np.float64).reshape(-1, 3)
    eps = 10.0 * float(np.finfo(np.float32 if precision == "flt" else np.float64).eps)

    def norm(v):
        return np.sqrt((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2])

    v01, v02, v12 = tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0], tri[:, 2] - tri[:, 1]
    cn = np.stack([v01[:, 1] * v02[:, 2] - v01[:, 2] * v02[:, 1],
                   v01[:, 2] * v02[:, 0] - v01[:, 0] * v02[:, 2],
                   v01[:, 0] * v02[:, 1] - v01[:, 1] * v02[:, 0]], axis=1)
    keep = (norm(v01) > 2 * eps) & (norm(v02) > 2 * eps) & (norm(v12) > 2 * eps) & (norm(cn) > 2 * eps)
    dot = (cn[:, 0] * nrm[:, 0] + cn[:, 1] * nrm[:, 1]) + cn[:, 2] * nrm[:, 2]
    tri = tri.copy()
    tri[dot < 0] = tri[dot < 0][:, [0, 2, 1]]
    return tri[keep]


def write_stl(path, triangles, binary=True):
    """Write triangles (t, 3, 3) as a binary (or ASCII) STL file.  ASCII
    vertices are written in the shortest text that reads back to the same
    double, and the first facet is kept short: the reference's reader takes a
    file for ASCII only if "endfacet" appears within the 256 bytes after byte
    80 (offLattice/triangleSet.hh:120-160, PLB_CBUFSIZ)."""
    tri = np.asarray(triangles, np.float64).reshape(-1, 3, 3)
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-300)
    if binary:
        rec = np.zeros(len(tri), np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("attr", "<u2")]))
        rec["n"], rec["v"] = n, tri
        with open(path, "wb") as f:
            f.write(b"\0" * 80 + np.uint32(len(tri)).tobytes() + rec.tobytes())
        return
    with open(path, "w") as f:
        f.write("solid mesh\n")
        for t, nn in zip(tri, n):
            f.write(f"facet normal {nn[0]:.6e} {nn[1]:.6e} {nn[2]:.6e}\nouter loop\n")
            for v in t:
                f.write("vertex " + " ".join(repr(float(x)) for x in v) + "\n")
            f.write("endloop\nendfacet\n")
        f.write("endsolid mesh\n")


def to_lattice_units(triangles, resolution, reference_direction=0, layer=0):
    """The reference's DEFscaledMesh(set, resolution, referenceDirection,
    margin, extraLayer) scaling (toLatticeUnits,
    offLattice/triangularSurfaceMesh.hh:1552-1575; triangleBoundary3D.hh:
    272-300): the bounding box's low corner moves to the origin, the extent
    along reference_direction becomes `resolution` cells, then everything
    shifts by `layer` (margin + extraLayer) cells on every axis.  Returns the
    mesh, the physical position of the lattice origin and dx."""
    tri = np.asarray(triangles, np.float64).reshape(-1, 3, 3)
    lo = tri.reshape(-1, 3).min(axis=0)
    hi = tri.reshape(-1, 3).max(axis=0)
    scale = float(resolution) / (hi[reference_direction] - lo[reference_direction])
    dx = 1.0 / scale
    out = (tri - lo) * scale + float(layer)
    return out, lo - float(layer) * dx, dx
