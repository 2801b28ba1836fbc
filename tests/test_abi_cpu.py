"""Host-only checks of the C ABI: the library loads and exports every symbol
the header declares, and the Python signatures cover the header."""
import ctypes
import os
import subprocess

import pytest

from palabos_gb300 import native as N


def test_library_exports_every_header_symbol():
    lib = N.load()
    missing = [s for s in N.header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_signatures_cover_header():
    declared = set(N.header_symbols())
    bound = set(N.SIGNATURES) | {"plbgpu_last_error"}
    assert declared == bound, (declared - bound, bound - declared)


def test_create_without_gpu_fails_cleanly():
    """No GPU here: plbgpu_create must return an error code, not crash."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = N.load()
    h = ctypes.c_void_p()
    rc = lib.plbgpu_create(0, ctypes.byref(h))
    assert rc in (-1, -3)
    assert not h.value


def test_null_context_arguments_are_rejected():
    lib = N.load()
    assert lib.plbgpu_synchronize(None) == -1
    assert lib.plbgpu_destroy(None) == -1
    assert lib.plbgpu_collide_and_stream(None, 0, 1, 0) == -1
    assert lib.plbgpu_cp_add_domain(None, 4, 4, 4, 1.0, None) == 0
