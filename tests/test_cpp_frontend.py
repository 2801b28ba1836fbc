"""The C++ host side: the case driver built on include/plbgpu.hpp (GPU) and
the Palabos co-processor adapter compiled against the reference (CPU)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import goldens
import lbcases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "tests", "cpp", "_build", "plb_case_gpu")
REFERENCE = os.environ.get("PALABOS_REFERENCE", "/root/reference")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cavity_bb_lid", "channel_sphere", "guo_channel", "zhpress_faces",
                                  "incbgk_nodyn", "mebb_walls", "velocity_box", "velocity_box_noinit",
                                  "doctest_cavity20"])
def test_cpp_driver_reproduces_reference_golden(name):
    """Same case file in, same result file out as the reference driver:
    populations bit for bit, reductions to summation rounding."""
    assert os.path.exists(DRIVER), "build() compiles the C++ driver"
    spec = lbcases.case_by_name(name)
    g, _ = goldens.load(name)
    with tempfile.TemporaryDirectory() as tmp:
        cpath, rpath = os.path.join(tmp, "c"), os.path.join(tmp, "r")
        lbcases.write_case_file(spec, cpath)
        subprocess.run([DRIVER, cpath, rpath], check=True)
        res = lbcases.read_result_file(rpath, spec)
    assert np.array_equal(res["f_init"], g["f_init"])
    assert np.array_equal(res["f_final"], g["f_final"])
    ok, worst = goldens.stats_close(res["stats"][:, 1:], g["stats"][:, 1:])
    assert ok, worst
    assert res["energy"] == pytest.approx(float(g["energy"]), rel=1e-12)
    assert res["density"] == pytest.approx(float(g["density"]), rel=1e-12)


@pytest.mark.slow
def test_coprocessor_adapter_compiles_against_reference():
    """plbgpu::GpuD3Q19CoProcessor3D<double> derives from the reference's
    plb::CoProcessor3D<double> and links with the reference library."""
    lib = os.path.join(ROOT, "oracle", "_ref", "libplb.a")
    if not os.path.isdir(os.path.join(REFERENCE, "src")) or not os.path.exists(lib):
        pytest.skip("reference sources / library not present")
    gpu_lib = os.path.join(ROOT, "palabos_gb300", "_lib")
    src = os.path.join(REFERENCE, "src")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "adapter")
        subprocess.run(["g++", "-std=c++11", "-O1", "-w", "-I", src, "-I", os.path.join(src, "externalLibraries"),
                        "-I", os.path.join(src, "externalLibraries", "tinyxml"), "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "coprocessor_adapter_check.cpp"), lib,
                        "-L", gpu_lib, "-lplbgpu", f"-Wl,-rpath,{gpu_lib}", "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    assert "addDomain=0 context=no" in out or "addDomain=1 context=yes" in out
    assert "energy=" in out
