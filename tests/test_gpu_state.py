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


# ---------------------------------------------------------------- dynamic content

import re

DSTATES = ["dstate_channel_sphere_multiblock", "dstate_velocity_box", "dstate_zhpress_faces",
           "dstate_guo_channel", "dstate_incbgk_nodyn"]


def _what(meta):
    return "forced_lattice" if meta["forced"] else "lattice"


def _recs(g, meta, key):
    return g[key] if not meta["forced"] else np.concatenate([g[key], g["force"]], axis=-1)


def _masks(g, meta):
    return O.OracleLattice.from_golden(g, meta).mebb_masks().reshape(meta["nx"], meta["ny"], meta["nz"])


def _reference_files(g, tmp_path):
    dat_path = str(tmp_path / "ref.dat")
    with open(dat_path, "wb") as f:
        f.write(bytes(g["dstate_dat"]))
    plb = re.sub(r"<File>[^<]*</File>", f"<File> {dat_path} </File>", str(g["dstate_plb"]))
    with open(tmp_path / "ref.plb", "w") as f:
        f.write(plb)
    return str(tmp_path / "ref.plb")


@pytest.mark.parametrize("name", DSTATES)
def test_save_state_dynamic_matches_format(name, tmp_path):
    """plbgpu_save_state_dynamic writes exactly the restated format (which the
    reference loads and continues bit for bit, tests/test_checkpoint_format.py)."""
    g, meta = goldens.load(name)
    lat = _lat(g, meta)
    lat.send(g["f_init"])
    lat.collide_and_stream(meta["nsteps"])
    base = str(tmp_path / "s")
    lat.save_state_dynamic(base, _what(meta))
    recs = _recs(g, meta, "f_final")
    plb, dat = O.dynamic_state_files(g["flags"], g["bcval"], _masks(g, meta), recs, recs.shape[-1],
                                     "ForcedD3Q19" if meta["forced"] else "D3Q19", base + ".dat", meta["omega"],
                                     meta.get("rho0", 1.0), meta.get("bb_rho", 0.0))
    assert open(base + ".plb").read() == plb
    assert open(base + ".dat", "rb").read() == dat


@pytest.mark.parametrize("name", DSTATES)
def test_load_reference_dynamic_state(name, tmp_path):
    """The reference's state (one component per block) into a blank lattice
    of the same size: kinds, wall values, parameters and populations come
    from the file, and the next steps equal the oracle's."""
    g, meta = goldens.load(name)
    lat = DeviceLattice3D(meta["nx"], meta["ny"], meta["nz"], 1.0)
    lat.periodicity(*meta["periodic"])
    lat.load_state_dynamic(_reference_files(g, tmp_path), _what(meta))
    assert np.array_equal(lat.get_kinds(), g["flags"])
    assert np.array_equal(lat.receive(), g["f_final"])
    lat.collide_and_stream(3)
    ol = O.OracleLattice.from_golden(g, meta)
    ref, _ = ol.run(np.ascontiguousarray(g["f_final"]).copy(), 3)
    assert np.array_equal(lat.receive(), ref.reshape(g["f_final"].shape))


def test_static_load_of_dynamic_state_takes_populations_only(tmp_path):
    name = "dstate_channel_sphere_multiblock"
    g, meta = goldens.load(name)
    lat = DeviceLattice3D(meta["nx"], meta["ny"], meta["nz"], 1.0)
    before = lat.get_kinds()
    lat.load_state(_reference_files(g, tmp_path))
    assert np.array_equal(lat.get_kinds(), before)
    lat2 = _lat(g, meta)
    lat2.load_state(str(tmp_path / "ref.plb"))
    assert np.array_equal(lat2.receive(), g["f_final"])


def test_dynamic_state_round_trip_and_refusals(tmp_path):
    g, meta = goldens.load("dstate_velocity_box")
    lat = _lat(g, meta)
    lat.send(g["f_init"])
    lat.collide_and_stream(5)
    ref = lat.receive()
    lat.save_state_dynamic(str(tmp_path / "a"))
    other = DeviceLattice3D(meta["nx"], meta["ny"], meta["nz"], 1.7)
    other.load_state_dynamic(str(tmp_path / "a.plb"))
    assert np.array_equal(other.get_kinds(), g["flags"])
    assert np.array_equal(other.receive(), ref)
    lat.collide_and_stream(4)
    other.collide_and_stream(4)
    assert np.array_equal(other.receive(), lat.receive())
    with pytest.raises(PlbGpuError):
        DeviceLattice3D(meta["nx"], meta["ny"], meta["nz"] + 1, 1.0).load_state_dynamic(str(tmp_path / "a.plb"))
    lat.save_state(str(tmp_path / "s"))
    with pytest.raises(PlbGpuError):
        other.load_state_dynamic(str(tmp_path / "s.plb"))                   # static content
    # two omegas: the GPU lattice holds one
    dat = open(tmp_path / "a.dat", "rb").read()
    om = np.float64(meta["omega"]).tobytes()
    bad = dat.replace(om, np.float64(1.2345).tobytes(), 1)
    with open(tmp_path / "a.dat", "wb") as f:
        f.write(bad)
    with pytest.raises(PlbGpuError):
        other.load_state_dynamic(str(tmp_path / "a.plb"))
    assert np.array_equal(other.get_kinds(), g["flags"])                     # nothing changed


def test_sparse_dynamic_state(tmp_path):
    """The reference's state of a sparse lattice (one component per kept
    block) loads into the GPU's sparse domain on the same blocks; the GPU's
    save writes the cells outside the lattice as NoDynamics with zero
    populations, as restated (the reference skips them when loading)."""
    g, meta = goldens.load("sparse_dstate_sealed_channel")
    shape = (meta["nx"], meta["ny"], meta["nz"])
    lat = lattice_from_description(*shape, meta["periodic"], meta["omega"], g["flags"], g["bcval"], g["force"],
                                   sparse=(g["sparse"], meta["blocks"]))
    ref_plb = _reference_files(g, tmp_path)
    lat.load_state_dynamic(ref_plb)
    inside = g["in_lattice"].astype(bool)
    kinds = lat.get_kinds()
    assert np.array_equal(kinds[inside], g["flags"][inside]) and (kinds[~inside] == 255).all()
    f = lat.receive()
    assert np.array_equal(f[inside], g["f_final"][inside]) and not f[~inside].any()
    base = str(tmp_path / "s")
    lat.save_state_dynamic(base)
    ol = O.OracleLattice(*shape, meta["periodic"], meta["omega"], kinds, g["bcval"], g["force"], meta["rho0"],
                         meta["bb_rho"])
    plb, dat = O.dynamic_state_files(kinds, g["bcval"], ol.mebb_masks().reshape(shape), f, 19, "D3Q19",
                                     base + ".dat", meta["omega"], meta["rho0"], meta["bb_rho"])
    assert open(base + ".plb").read() == plb
    assert open(base + ".dat", "rb").read() == dat
    with pytest.raises(PlbGpuError):   # a dense lattice: the kept blocks do not cover it
        DeviceLattice3D(*shape, 1.0).load_state_dynamic(ref_plb)
