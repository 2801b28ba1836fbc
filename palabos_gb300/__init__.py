"""GB300-native D3Q19 lattice Boltzmann hot path with the Palabos construction API.

The compute path is libplbgpu.so (hand-written CUDA for sm_103a) behind the C
ABI in include/plbgpu.h; this package is a thin Python front end over it.
"""
from .native import (BGK, GUO, INCBGK, BOUNCEBACK, MOMENTUM_EXCHANGE, NODYNAMICS, REG_VELOCITY,
                     REG_PRESSURE, ZOUHE_VELOCITY, ZOUHE_PRESSURE, VELOCITY_EDGE, VELOCITY_CORNER, FP64,
                     FP32, BF16, FP16, face_kind, edge_kind, corner_kind, PlbGpuError)
from .lattice import Context, DeviceLattice3D, default_context, lattice_from_description
from . import meshes, voxel

__all__ = ["BGK", "GUO", "INCBGK", "BOUNCEBACK", "MOMENTUM_EXCHANGE", "NODYNAMICS", "REG_VELOCITY",
           "REG_PRESSURE", "ZOUHE_VELOCITY", "ZOUHE_PRESSURE", "VELOCITY_EDGE", "VELOCITY_CORNER", "FP64",
           "FP32", "BF16", "FP16", "face_kind", "edge_kind", "corner_kind", "PlbGpuError", "Context",
           "DeviceLattice3D", "default_context", "lattice_from_description", "meshes", "voxel"]
