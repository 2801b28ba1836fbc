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
