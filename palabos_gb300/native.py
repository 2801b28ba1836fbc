"""ctypes binding of libplbgpu.so (include/plbgpu.h).

The library is built in-tree by palabos_gb300/build.py.  There is no CPU
fallback: if the shared library cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "_lib", "libplbgpu.so")
HEADER = os.path.join(ROOT, "include", "plbgpu.h")

OK = 0
ERRORS = {-1: "PLBGPU_ERR_ARG", -2: "PLBGPU_ERR_HANDLE", -3: "PLBGPU_ERR_CUDA",
          -4: "PLBGPU_ERR_NOMEM", -5: "PLBGPU_ERR_STATE"}

FP64, FP32, BF16, FP16, BF16_SR = 0, 1, 2, 3, 4
PRECISIONS = {"fp64": FP64, "fp32": FP32, "bf16": BF16, "fp16": FP16, "bf16sr": BF16_SR}

BGK, GUO, INCBGK, BOUNCEBACK, MOMENTUM_EXCHANGE, NODYNAMICS = 0, 1, 2, 3, 4, 5
REG_VELOCITY, REG_PRESSURE, ZOUHE_VELOCITY, ZOUHE_PRESSURE = 6, 12, 18, 24
VELOCITY_EDGE, VELOCITY_CORNER, NKINDS = 30, 42, 50
NONE = 255   # not part of the lattice (sparse domains)
BLOCKS = {"lattice": 0, "forced_lattice": 1, "density": 2, "velocity": 3, "rho_bar": 4, "j": 5}


def face_kind(family: int, direction: int, orientation: int) -> int:
    """Kind of a face boundary: family + 2*direction + (orientation > 0)."""
    return family + 2 * direction + (1 if orientation > 0 else 0)


def edge_kind(plane: int, normal1: int, normal2: int) -> int:
    """External velocity edge along axis `plane`; normal1 is along (plane+1)%3,
    normal2 along (plane+2)%3 (addExternalVelocityEdge{plane}{N|P}{N|P})."""
    return VELOCITY_EDGE + 4 * plane + 2 * (normal1 > 0) + (normal2 > 0)


def corner_kind(x_normal: int, y_normal: int, z_normal: int) -> int:
    """External velocity corner (addExternalVelocityCorner{N|P}{N|P}{N|P})."""
    return VELOCITY_CORNER + 4 * (x_normal > 0) + 2 * (y_normal > 0) + (z_normal > 0)


class PlbGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)
_c_u8_p = ctypes.POINTER(ctypes.c_uint8)
_vp = ctypes.c_void_p
_i = ctypes.c_int
_l = ctypes.c_long
_d = ctypes.c_double
_sz = ctypes.c_size_t
BOX = [_i] * 6
LBOX = [_l] * 6

SIGNATURES = {
    "plbgpu_create": [_i, ctypes.POINTER(_vp)],
    "plbgpu_destroy": [_vp],
    "plbgpu_launch_count": [_vp, ctypes.POINTER(ctypes.c_ulonglong)],
    "plbgpu_get_stream": [_vp, ctypes.POINTER(_vp)],
    "plbgpu_measure_fp64_rate": [_vp, _c_dbl_p],
    "plbgpu_synchronize": [_vp],
    "plbgpu_add_domain": [_vp, _i, _i, _i, _i, _c_int_p],
    "plbgpu_remove_domain": [_vp, _i],
    "plbgpu_domain_info": [_vp, _i, _c_int_p, _c_int_p, _c_int_p, _c_int_p, ctypes.POINTER(ctypes.c_ulonglong)],
    "plbgpu_set_periodicity": [_vp, _i, _i, _i, _i],
    "plbgpu_set_params": [_vp, _i, _d, _d, _d],
    "plbgpu_define_dynamics": [_vp, _i, *BOX, _i],
    "plbgpu_set_kinds": [_vp, _i, *BOX, _c_u8_p, _sz],
    "plbgpu_get_kinds": [_vp, _i, *BOX, _c_u8_p, _sz],
    "plbgpu_set_velocity_condition_on_block_boundaries": [_vp, _i, *BOX],
    "plbgpu_add_boundary": [_vp, _i, *BOX, _i],
    "plbgpu_add_processor": [_vp, _i, ctypes.c_char_p, ctypes.POINTER(_l), ctypes.c_char_p, _l,
                             ctypes.POINTER(_l), _i],
    "plbgpu_clear_processors": [_vp, _i],
    "plbgpu_processor_count": [_vp, _i, _c_int_p],
    "plbgpu_get_processor": [_vp, _i, _i, ctypes.c_char_p, _sz, ctypes.POINTER(_l), ctypes.c_char_p, _sz,
                             ctypes.POINTER(_l), ctypes.POINTER(_l), _i, _c_int_p],
    "plbgpu_load_processors": [_vp, _i, ctypes.c_char_p],
    "plbgpu_compute_rhobar_j": [_vp, _i],
    "plbgpu_set_rhobar_j": [_vp, _i, *BOX, _c_dbl_p, _sz],
    "plbgpu_get_rhobar_j": [_vp, _i, *BOX, _c_dbl_p, _sz],
    "plbgpu_collide_and_stream_external": [_vp, _i, _i, _i, _i],
    "plbgpu_select_sparse_blocks": [_vp, _i, ctypes.POINTER(ctypes.c_int32), _sz, _i, _i, _i, _c_u8_p, _sz],
    "plbgpu_save_binary_block": [_vp, _i, _i, ctypes.c_char_p, _i],
    "plbgpu_load_binary_block": [_vp, _i, _i, ctypes.c_char_p, _i],
    "plbgpu_save_state": [_vp, _i, _i, ctypes.c_char_p],
    "plbgpu_load_state": [_vp, _i, _i, ctypes.c_char_p],
    "plbgpu_save_state_dynamic": [_vp, _i, _i, ctypes.c_char_p],
    "plbgpu_load_state_dynamic": [_vp, _i, _i, ctypes.c_char_p],
    "plbgpu_set_boundary_velocity": [_vp, _i, *BOX, _d, _d, _d],
    "plbgpu_set_boundary_velocity_field": [_vp, _i, *BOX, _c_dbl_p, _sz],
    "plbgpu_set_boundary_density": [_vp, _i, *BOX, _d],
    "plbgpu_set_boundary_density_field": [_vp, _i, *BOX, _c_dbl_p, _sz],
    "plbgpu_set_force": [_vp, _i, *BOX, _d, _d, _d],
    "plbgpu_set_force_field": [_vp, _i, *BOX, _c_dbl_p, _sz],
    "plbgpu_initialize_momentum_exchange": [_vp, _i],
    "plbgpu_initialize_at_equilibrium": [_vp, _i, *BOX, _d, _d, _d, _d],
    "plbgpu_initialize_at_equilibrium_field": [_vp, _i, *BOX, _c_dbl_p, _sz],
    "plbgpu_initialize": [_vp, _i],
    "plbgpu_send": [_vp, _i, *BOX, _c_dbl_p, _sz],
    "plbgpu_receive": [_vp, _i, *BOX, _c_dbl_p, _sz],
    "plbgpu_send_f32": [_vp, _i, *BOX, ctypes.POINTER(ctypes.c_float), _sz],
    "plbgpu_receive_f32": [_vp, _i, *BOX, ctypes.POINTER(ctypes.c_float), _sz],
    "plbgpu_collide_and_stream": [_vp, _i, _i, _i],
    "plbgpu_run_host": [_vp, _i, _c_dbl_p, _c_dbl_p, _sz, _i, _i, _c_dbl_p, _sz],
    "plbgpu_run_host_plan": [_i, _i, _i, _i, _i, _c_int_p, _c_int_p, _sz, ctypes.POINTER(ctypes.c_size_t)],
    "plbgpu_get_stats": [_vp, _i, _c_dbl_p],
    "plbgpu_reduce": [_vp, _i, *BOX, _c_dbl_p, _c_dbl_p],
    "plbgpu_compute_velocity": [_vp, _i, *BOX, _c_dbl_p, _sz],
    "plbgpu_compute_density": [_vp, _i, *BOX, _c_dbl_p, _sz],
    "plbgpu_time_steps": [_vp, _i, _i, _i, ctypes.POINTER(ctypes.c_float)],
    "plbgpu_cp_add_domain": [_vp, _l, _l, _l, _d, _c_int_p],
    "plbgpu_cp_send": [_vp, _i, *LBOX, ctypes.c_char_p, _sz],
    "plbgpu_cp_receive": [_vp, _i, *LBOX, ctypes.c_char_p, _sz],
    "plbgpu_cp_collide_and_stream": [_vp, _i],
    "plbgpu_cp_add_domain_f32": [_vp, _l, _l, _l, _d, _c_int_p],
    "plbgpu_cp_send_f32": [_vp, _i, *LBOX, ctypes.c_char_p, _sz],
    "plbgpu_cp_receive_f32": [_vp, _i, *LBOX, ctypes.c_char_p, _sz],
    "plbgpu_voxelize": [_vp, _c_dbl_p, _sz, _i, _i, _i, _i, ctypes.POINTER(ctypes.c_int32), _sz],
    "plbgpu_adjoint_forward": [_vp, _i, _i, _i],
    "plbgpu_adjoint_interval": [_vp, _i, _c_int_p],
    "plbgpu_adjoint_backward": [_vp, _i, _c_dbl_p, _sz, _c_dbl_p, _c_dbl_p, _sz, _c_dbl_p,
                                ctypes.POINTER(ctypes.c_float)],
    "plbgpu_tangent_linear": [_vp, _i, _i, _c_dbl_p, _sz, _d, _c_dbl_p, _sz, _c_dbl_p, _c_dbl_p],
    "plbgpu_adjoint_backward_weighted": [_vp, _i, _c_dbl_p, _sz, _c_dbl_p, _c_dbl_p, _sz, _c_dbl_p,
                                         ctypes.POINTER(ctypes.c_float)],
    "plbgpu_tangent_linear_weighted": [_vp, _i, _i, _c_dbl_p, _sz, _d, _c_dbl_p, _sz, _c_dbl_p, _c_dbl_p],
    "plbgpu_adjoint_steady_weighted": [_vp, _i, _i, _c_dbl_p, _sz, _c_dbl_p, _c_dbl_p, _sz, _c_dbl_p,
                                       ctypes.POINTER(ctypes.c_float)],
    "plbgpu_adjoint_backward_drag": [_vp, _i, _c_dbl_p, _c_dbl_p, _c_dbl_p, _sz, _c_dbl_p,
                                     ctypes.POINTER(ctypes.c_float)],
    "plbgpu_tangent_linear_drag": [_vp, _i, _i, _c_dbl_p, _sz, _d, _c_dbl_p, _c_dbl_p, _c_dbl_p],
    "plbgpu_adjoint_steady_drag": [_vp, _i, _i, _c_dbl_p, _c_dbl_p, _c_dbl_p, _sz, _c_dbl_p,
                                   ctypes.POINTER(ctypes.c_float)],
    "plbgpu_reduce_noalloc": [_vp, ctypes.c_longlong, _vp, _i, _i, _i, _d, _d, _vp, _vp],
}

_lib = None


def header_symbols() -> list[str]:
    """Every function the C header declares."""
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(plbgpu_\w+)\s*\(", text, re.M)))


def load(path: str = LIB_PATH):
    """Load libplbgpu.so.  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m palabos_gb300.build` "
                           "(the GPU path has no CPU fallback)")
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _i
    lib.plbgpu_last_error.argtypes = [_vp]
    lib.plbgpu_last_error.restype = ctypes.c_char_p
    _lib = lib
    return lib


def check(ctx, rc):
    if rc != OK:
        msg = load().plbgpu_last_error(ctx).decode() if ctx else ""
        raise PlbGpuError(rc, msg)
    return rc
