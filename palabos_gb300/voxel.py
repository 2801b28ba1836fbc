"""Voxelized geometry: voxel flags of a closed triangle mesh on the GPU, and the
lattice kinds and sparse blocks a flow domain takes from them.

voxelize() is the reference's voxelize(mesh, domain, borderWidth)
(offLattice/voxelizer.hh:106-141) through plbgpu_voxelize; the flags are
OUTSIDE, OUTER_BORDER, INSIDE, INNER_BORDER (voxelizer.h:36-56).
voxelized_domain() follows the use VoxelizedDomain3D
(offLattice/triangleBoundary3D.h:362-367) and computeSparseManagement
(offLattice/makeSparse3D.hh:107-160) are put to: the flow runs on one side
of the surface, the border layer on the other side of it becomes bounce-back
walls, the rest of that side no-dynamics, and with `blocks` the lattice keeps
only the blocks that hold fluid.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native as N
from .lattice import default_context

UNDETERMINED, OUTSIDE, OUTER_BORDER, INSIDE, INNER_BORDER = 0, 1, 2, 3, 4


def voxelize(triangles, shape, border_width=1, ctx=None):
    """Voxel flags (nx, ny, nz) int32 of the closed mesh `triangles` (t, 3, 3)
    in lattice coordinates, outward normals; the box's outer layer is
    outside."""
    ctx = ctx or default_context()
    tri = np.ascontiguousarray(triangles, np.float64).reshape(-1, 9)
    nx, ny, nz = map(int, shape)
    flags = np.zeros(nx * ny * nz, np.int32)
    N.check(ctx.h, ctx.lib.plbgpu_voxelize(ctx.h, tri.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), tri.shape[0],
                                           nx, ny, nz, int(border_width),
                                           flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), flags.size))
    return flags.reshape(nx, ny, nz)


def kinds_from_flags(flags, flow="outside", fluid=N.BGK):
    """Cell kinds of a flow on one side of the surface: `flow` = "outside"
    (around a body) or "inside" (in a vessel).  Fluid cells get `fluid`, the
    border layer beyond the surface bounce-back, the rest of that side
    no-dynamics."""
    flags = np.asarray(flags)
    if flow == "outside":
        is_fluid = (flags == OUTSIDE) | (flags == OUTER_BORDER)
        wall = flags == INNER_BORDER
    elif flow == "inside":
        is_fluid = (flags == INSIDE) | (flags == INNER_BORDER)
        wall = flags == OUTER_BORDER
    else:
        raise ValueError("flow is 'outside' or 'inside'")
    kinds = np.full(flags.shape, N.NODYNAMICS, np.uint8)
    kinds[is_fluid] = fluid
    kinds[wall] = N.BOUNCEBACK
    return kinds


def voxelized_domain(lattice, triangles, flow="outside", border_width=1, fluid=N.BGK, blocks=None):
    """Voxelize `triangles` on the lattice's box, set the kinds of a flow on
    the `flow` side, and with `blocks` = (bx, by, bz) drop the blocks that
    hold neither fluid nor wall (computeSparseManagement over the fluid and
    wall cells).  Returns (flags, kinds, keep or None)."""
    flags = voxelize(triangles, lattice.shape, border_width, lattice.ctx)
    kinds = kinds_from_flags(flags, flow, fluid)
    lattice.set_kinds(kinds)
    keep = None
    if blocks is not None:
        keep = lattice.select_sparse_blocks((kinds != N.NODYNAMICS).astype(np.int32), blocks)
    return flags, kinds, keep
