"""saveState / loadState files (parallelIO) through the C ABI: the GPU writes
exactly the oracle's restatement of the format (which the reference itself
loads, tests/test_checkpoint_format.py), and reads the reference's own
multi-component states."""
import os

import numpy as np
import pytest

import goldens
import oracle as O
from palabos_gb300 import DeviceLattice3D, PlbGpuError, lattice_from_description

pytestmark = pytest.mark.gpu

STATES = ["state_periodic_bgk_multiblock", "state_guo_periodic_multiblock"]


def _lat(g, meta):
    return lattice_from_description(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"],
                                    g["flags"], g["bcval"], g["force"], meta.get("rho0", 1.0),
                                    meta.get("bb_rho", 0.0))


@pytest.mark.parametrize("name", STATES)
def test_save_state_matches_format(name, tmp_path):
    g, meta = goldens.load(name)
    lat = _lat(g, meta)
    lat.send(g["f_init"])
    lat.collide_and_stream(meta["nsteps"])
    what = "forced_lattice" if meta["forced"] else "lattice"
    base = str(tmp_path / "s")
    lat.save_state(base, what)
    recs = g["f_final"] if not meta["forced"] else np.concatenate([g["f_final"], g["force"]], axis=-1)
    plb, dat = O.state_files(recs.reshape(-1, recs.shape[-1]), g["f_final"].shape[:3], recs.shape[-1],
                             "BlockLattice3D", "ForcedD3Q19" if meta["forced"] else "D3Q19", base + ".dat")
    assert open(base + ".plb").read() == plb
    assert open(base + ".dat", "rb").read() == dat


@pytest.mark.parametrize("name", STATES)
def test_load_reference_state(name, tmp_path):
    """The reference wrote one component per block; the loader places each."""
    g, meta = goldens.load(name)
    plb = str(g["state_plb"])
    dat_path = str(tmp_path / "ref.dat")
    with open(dat_path, "wb") as f:
        f.write(bytes(g["state_dat"]))
    import re
    plb = re.sub(r"<File>[^<]*</File>", f"<File> {dat_path} </File>", plb)
    with open(tmp_path / "ref.plb", "w") as f:
        f.write(plb)
    lat = _lat(g, meta)
    lat.load_state(str(tmp_path / "ref.plb"), "forced_lattice" if meta["forced"] else "lattice")
    assert np.array_equal(lat.receive(), g["f_final"])


def test_state_round_trip_and_refusals(tmp_path):
    lat = DeviceLattice3D(9, 7, 5, 1.4)
    lat.periodicity(1, 1, 1)
    rng = np.random.default_rng(3)
    f = 1e-3 * rng.standard_normal((9, 7, 5, 19))
    lat.send(f)
    lat.collide_and_stream(3)
    ref = lat.receive()
    lat.save_state(str(tmp_path / "a"))
    other = DeviceLattice3D(9, 7, 5, 1.4)
    other.load_state(str(tmp_path / "a.plb"))
    assert np.array_equal(other.receive(), ref)
    with pytest.raises(PlbGpuError):
        DeviceLattice3D(9, 7, 6, 1.4).load_state(str(tmp_path / "a.plb"))       # another size
    with pytest.raises(PlbGpuError):
        other.load_state(str(tmp_path / "a.plb"), "forced_lattice")             # 19 values, not 22
    text = open(tmp_path / "a.plb").read().replace("False", "True")
    with open(tmp_path / "b.plb", "w") as fh:
        fh.write(text)
    with pytest.raises(PlbGpuError):
        other.load_state(str(tmp_path / "b.plb"))                               # dynamic content
