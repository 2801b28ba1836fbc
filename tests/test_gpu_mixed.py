"""Reduced-precision storage forms (FP32 compute; FP32 / BF16 / FP16 f-bar
storage) against the reference's FP64 golden results.

These forms do not reproduce the reference bit for bit; the bound is on the
largest population error relative to the largest |f-bar| of the case, with
the tolerance of each storage type written here.  They run through the same
C ABI, including the staged (bulk-copy) row kernel of the 2- and 4-byte forms.
"""
import numpy as np
import pytest

import goldens
from palabos_gb300 import lattice_from_description

pytestmark = pytest.mark.gpu

# max |f - f_ref| / max |f_ref| after the case's steps
TOL = {"fp32": 2e-5, "fp16": 1e-2, "bf16": 6e-2}
CASES = ["periodic_bgk", "cavity_bb_lid", "channel_sphere", "guo_channel", "regvel_faces",
         "zhpress_faces", "incbgk_nodyn", "mebb_walls"]


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp16"])
@pytest.mark.parametrize("name", CASES)
def test_reduced_precision_tracks_reference(name, precision):
    g, meta = goldens.load(name)
    lat = lattice_from_description(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"],
                                   g["flags"], g["bcval"], g["force"], meta.get("rho0", 1.0),
                                   meta.get("bb_rho", 0.0), precision)
    lat.send(g["f_init"])
    lat.collide_and_stream(meta["nsteps"] - 1)
    lat.collide_and_stream(1, stats=True)
    f = lat.receive()
    ref = g["f_final"]
    err = np.abs(f - ref).max() / np.abs(ref).max()
    assert err < TOL[precision], err
    st = lat.internal_statistics()
    assert np.isfinite(st["raw"]).all()
    e, rho = lat.reduce()
    assert e == pytest.approx(float(g["energy"]), rel=50 * TOL[precision])


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_staged_rows_match_unstaged_geometry(precision):
    """nz a multiple of the 16-byte copy granule (staged row kernel) and nz odd
    (register row kernel) must give the same physics on the same flow."""
    from palabos_gb300 import DeviceLattice3D
    out = []
    for nz in (32, 33):
        lat = DeviceLattice3D(16, 12, nz, 1.7, precision)
        lat.periodicity(1, 1, 1)
        z = np.arange(nz)
        u = np.zeros((16, 12, nz, 3))
        u[..., 0] = 0.03 * np.sin(2 * np.pi * np.arange(12) / 12)[None, :, None]
        lat.initialize_at_equilibrium(None, np.ones((16, 12, nz)), u)
        lat.collide_and_stream(20)
        f = lat.receive()
        out.append(f[:, :, :8].astype(np.float64))   # depends only on y
    assert np.abs(out[0] - out[1]).max() < TOL[precision] * 0.03 + 1e-7
