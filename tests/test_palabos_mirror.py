"""plbgpu::describe() (include/plbgpu_palabos3d.hh) reads a lattice built
through the reference's own API and must recover exactly the kinds, boundary
values, forces and populations the parity cases were built from.  The
reference driver calls it on every case when PLB_DESCRIBE is set (host code
only; no GPU is involved)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import goldens
import lbcases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "plb_case")

NAMES = [n for n in goldens.case_names() if not n.startswith("sparse_")]


def _describe(spec):
    with tempfile.TemporaryDirectory() as tmp:
        cpath, rpath, dpath = (os.path.join(tmp, x) for x in ("case", "res", "desc"))
        lbcases.write_case_file(spec, cpath)
        subprocess.run([DRIVER, cpath, rpath], check=True, env=dict(os.environ, PLB_DESCRIBE=dpath))
        data = open(dpath, "rb").read()
    n = spec.nx * spec.ny * spec.nz
    shape = (spec.nx, spec.ny, spec.nz)
    off = 0
    kinds = np.frombuffer(data, np.uint8, n, off).reshape(shape)
    off += n
    bcval = np.frombuffer(data, np.float64, 3 * n, off).reshape(shape + (3,))
    off += 24 * n
    force = np.frombuffer(data, np.float64, 3 * n, off).reshape(shape + (3,))
    off += 24 * n
    f = np.frombuffer(data, np.float64, 19 * n, off).reshape(shape + (19,))
    off += 152 * n
    omega, bb_rho = np.frombuffer(data, np.float64, 2, off)
    return kinds, bcval, force, f, omega, bb_rho


@pytest.mark.skipif(not os.path.exists(DRIVER), reason="reference driver not built (needs the reference sources)")
@pytest.mark.parametrize("name", NAMES)
def test_describe_recovers_case(name):
    spec = lbcases.case_by_name(name)
    g, meta = goldens.load(name)
    kinds, bcval, force, f, omega, bb_rho = _describe(spec)
    assert np.array_equal(kinds, spec.flags)
    vel = ((kinds >= 6) & (kinds < 12)) | ((kinds >= 18) & (kinds < 24)) | (kinds >= 30)
    press = ((kinds >= 12) & (kinds < 18)) | ((kinds >= 24) & (kinds < 30))
    assert np.array_equal(bcval[vel], spec.bcval[vel])
    assert np.array_equal(bcval[press][:, 0], spec.bcval[press][:, 0])
    if spec.forced:
        assert np.array_equal(force, spec.force)
    assert np.array_equal(f, g["f_init"])
    assert omega == spec.omega
    if np.isin(kinds, (lbcases.BB, lbcases.MEBB)).any():
        assert bb_rho == spec.bb_rho
