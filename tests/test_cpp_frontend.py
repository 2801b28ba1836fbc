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


@pytest.mark.gpu
def test_cpp_run_host_matches_send_steps_receive():
    """plbgpu::Lattice3D::runHost against send + collideAndStream + receive
    from C++ (tests/cpp/run_host_check.cpp): bit for bit, statistics records
    to summation rounding."""
    exe = os.path.join(ROOT, "tests", "cpp", "_build", "run_host_check")
    assert os.path.exists(exe), "build() compiles the C++ check"
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    kv = dict(t.split("=") for t in out.split()[1:])
    assert float(kv["maxabs"]) > 1e-3, out
    assert float(kv["maxdiff"]) == 0.0, out
    assert float(kv["statsrel"]) <= 1e-12, out
    assert kv["records"] == "3/3", out


@pytest.mark.slow
def test_coprocessor_adapter_runs_reference_coprocessor_path():
    """plbgpu::GpuD3Q19CoProcessor3D<T> (include/plbgpu_coprocessor3d.hh)
    registered as the reference's default co-processor and driven through the
    reference's own wiring -- initiateCoProcessors, transferToCoProcessors,
    MultiBlockLattice3D::collideAndStream, transferFromCoProcessors
    (coProcessors/coProcessorCommunication3D.hh:34-125) -- on a 2x2x1-block
    BGK lattice, against the reference's example co-processor
    (D3Q19ExampleCoProcessor3D).  The device calls go to a CPU stand-in built
    on the oracle (tests/cpp/fake_plbgpu_cp.cpp); the GPU's co-processor calls
    are checked against the same oracle on the GPU.  T = double is bit for
    bit, T = float (FP32 records) to FP32 rounding."""
    lib = os.path.join(ROOT, "oracle", "_ref", "libplb.a")
    orc = os.path.join(ROOT, "oracle", "_build")
    if not os.path.isdir(os.path.join(REFERENCE, "src")) or not os.path.exists(lib):
        pytest.skip("reference sources / library not present")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    src = os.path.join(REFERENCE, "src")
    inc = ["-I", src, "-I", os.path.join(src, "externalLibraries"), "-I",
           os.path.join(src, "externalLibraries", "tinyxml"), "-I", os.path.join(ROOT, "include")]
    with tempfile.TemporaryDirectory() as tmp:
        fake = os.path.join(tmp, "fake.o")
        drv = os.path.join(tmp, "e2e.o")
        exe = os.path.join(tmp, "e2e")
        subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-c",
                        os.path.join(ROOT, "tests", "cpp", "fake_plbgpu_cp.cpp"), "-o", fake], check=True)
        subprocess.run(["g++", "-std=c++11", "-O1", "-w", *inc, "-c",
                        os.path.join(ROOT, "tests", "cpp", "coprocessor_e2e.cpp"), "-o", drv], check=True)
        subprocess.run(["g++", drv, fake, lib, "-L", orc, "-lplboracle", f"-Wl,-rpath,{orc}", "-o", exe],
                       check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    rows = {}
    for line in out.splitlines():
        kv = dict(t.split("=") for t in line.split()[1:])
        rows[line.split()[0]] = kv
    assert rows["double"]["domains"] == "4/4" and rows["float"]["domains"] == "4/4", out
    assert float(rows["double"]["maxabs"]) > 1e-3, out          # the flow is not trivial
    assert float(rows["double"]["maxdiff"]) == 0.0, out
    assert float(rows["float"]["maxdiff"]) <= 1e-6 * float(rows["float"]["maxabs"]), out
