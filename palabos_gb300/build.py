"""Build the CUDA library libplbgpu.so in-tree (palabos_gb300/_lib/).

nvcc for sm_103a only; the translation units (host API, FP64 kernels, one unit
per reduced storage type, the allocation-free reduction, the adjoint) compile
in parallel.  The FP64 kernels and the host API are compiled with
--fmad=false so that the FP64 path rounds every multiply and add separately,
exactly like the reference built without FMA contraction; the mixed-precision
kernels use FMA.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIB_DIR, "libplbgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-I", os.path.join(ROOT, "include")]
# (source, fmad)
# Storage forms: (name, fmad).  Per form, the time-step kernels of each AA
# parity (the costliest code) and the rest of its launcher table are separate
# units; longest first.
FORMS = [("fp64", False), ("fp32", True), ("bf16", True), ("fp16", True), ("bf16sr", True)]
UNITS = ([(f"step_{f}_{p}.cu", fm) for f, fm in FORMS for p in ("even", "odd")]
         + [(f"step_{f}.cu", fm) for f, fm in FORMS]
         + [("adjoint.cu", False), ("api.cu", False), ("noalloc.cu", False), ("checkpoint.cu", False), ("voxelizer.cu", False),
            ("pipe_rate.cu", False)])


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libplbgpu")
    return p


def _headers_mtime() -> float:
    m = 0.0
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def _compile(src: str, fmad: bool, extra: list[str], force: bool) -> str:
    obj = os.path.join(OBJ, src.replace(".cu", ".o"))
    srcp = os.path.join(CSRC, src)
    if (not force and os.path.exists(obj)
            and os.path.getmtime(obj) >= max(os.path.getmtime(srcp), _headers_mtime())):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, f"--fmad={'true' if fmad else 'false'}", *extra, "-c", srcp, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, ptxas_verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    with cf.ThreadPoolExecutor(max_workers=min(len(UNITS), max(4, os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], extra, force), UNITS))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv))
