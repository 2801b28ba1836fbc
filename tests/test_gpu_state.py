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


# ---------------------------------------------------------------- data-processor list

def _processor_section(plb_text):
    a, b = plb_text.find("        <Processor"), plb_text.rfind("</Processor>\n")
    return "" if a < 0 else plb_text[a:b + len("</Processor>\n")]


def _planar_runs(flags, kind, direction):
    """The case builder's maximal one-kind runs: along z for x and y faces,
    along x for z faces (the wrapped boundary processors need a planar box)."""
    nx, ny, nz = flags.shape
    runs = []
    if direction != 2:
        for x in range(nx):
            for y in range(ny):
                z = 0
                while z < nz:
                    if flags[x, y, z] != kind:
                        z += 1
                        continue
                    z1 = z
                    while z1 + 1 < nz and flags[x, y, z1 + 1] == kind:
                        z1 += 1
                    runs.append((x, x, y, y, z, z1))
                    z = z1 + 1
    else:
        for y in range(ny):
            for z in range(nz):
                x = 0
                while x < nx:
                    if flags[x, y, z] != kind:
                        x += 1
                        continue
                    x1 = x
                    while x1 + 1 < nx and flags[x1 + 1, y, z] == kind:
                        x1 += 1
                    runs.append((x, x1, y, y, z, z))
                    x = x1 + 1
    return runs


def _replay_boundary_calls(lat, flags):
    """The boundary-condition calls that built the case in the reference:
    faces kind by kind over their planar runs, then every edge and corner
    cell on its own."""
    from palabos_gb300 import native as N
    for k in range(N.REG_VELOCITY, N.VELOCITY_EDGE):
        for run in _planar_runs(flags, k, ((k - N.REG_VELOCITY) % 6) // 2):
            lat.add_boundary(run, k)
    for k in range(N.VELOCITY_EDGE, N.NKINDS):
        for x, y, z in np.argwhere(flags == k):
            lat.add_boundary((x, x, y, y, z, z), k)


@pytest.mark.parametrize("name", DSTATES)
def test_saved_description_carries_the_reference_processor_list(name, tmp_path):
    """The lattice built by the same boundary-condition calls as the
    reference's case saves the reference's <Processor> list byte for byte
    (names, domains, data, levels, block ids, ids), static and dynamic."""
    g, meta = goldens.load(name)
    ref = _processor_section(str(g["dstate_plb"]))
    lat = _lat(g, meta)
    _replay_boundary_calls(lat, g["flags"])
    assert len(lat.processors()) == ref.count("<Processor")
    lat.save_state_dynamic(str(tmp_path / "d"), _what(meta))
    assert _processor_section(open(tmp_path / "d.plb").read()) == ref
    lat.save_state(str(tmp_path / "s"), _what(meta))
    assert _processor_section(open(tmp_path / "s.plb").read()) == ref


@pytest.mark.parametrize("name", ["dstate_velocity_box", "dstate_zhpress_faces"])
def test_processor_list_read_from_a_reference_description(name, tmp_path):
    """readXmlProcessors: the list read from the reference's description is
    saved again unchanged; a load of the state leaves the list alone."""
    g, meta = goldens.load(name)
    ref_plb = _reference_files(g, tmp_path)
    lat = _lat(g, meta)
    lat.load_state_dynamic(ref_plb, _what(meta))
    assert lat.processors() == []
    lat.load_processors(ref_plb)
    lat.save_state_dynamic(str(tmp_path / "d"), _what(meta))
    assert _processor_section(open(tmp_path / "d.plb").read()) == _processor_section(str(g["dstate_plb"]))
    first = lat.processors()[0]
    assert first["name"] == "WrappedLocalBoundary3D_%TD" and first["data"] == "0 0 " and first["blocks"] == (0,)


def test_block_boundaries_record_the_reference_processors(tmp_path):
    """setVelocityConditionOnBlockBoundaries over a 6x5x4 box: six faces,
    twelve edges, eight corners, in the reference's order and boxes."""
    lat = DeviceLattice3D(6, 5, 4, 1.2)
    lat.set_velocity_condition_on_block_boundaries()
    p = lat.processors()
    assert [r["name"] for r in p[:6]] == ["WrappedLocalBoundary3D_%TD"] * 6
    assert p[0]["domain"] == (0, 0, 1, 3, 1, 2) and p[5]["domain"] == (1, 4, 1, 3, 3, 3)
    assert [r["name"] for r in p[6:10]] == [f"OuterVelocityEdge_%TD_0_{a}_{b}" for a in (-1, 1) for b in (-1, 1)]
    assert p[6]["domain"] == (1, 4, 0, 0, 0, 0) and p[9]["domain"] == (1, 4, 4, 4, 3, 3)
    assert p[11]["domain"] == (5, 5, 1, 3, 0, 0)          # plane y: z negative, x positive
    assert p[14]["domain"] == (0, 0, 0, 0, 1, 2) and p[16]["domain"] == (5, 5, 0, 0, 1, 2)   # plane z: x, y sides
    assert [r["name"] for r in p[18:]] == [f"OuterVelocityCorner3D_%TD_{x}_{y}_{z}"
                                           for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)]
    assert p[25]["domain"] == (5, 5, 4, 4, 3, 3)
    lat.save_state(str(tmp_path / "s"))
    text = open(tmp_path / "s.plb").read()
    assert text.count("<Processor id=") == 26 and "OuterVelocityCorner3D_double_D3Q19_1_1_1" in text
    lat.clear_processors()
    lat.add_processor("Custom_%TD", (0, 1, 0, 1, 0, 1), data="", level=1, blocks=())
    lat.save_state(str(tmp_path / "t"), "forced_lattice")
    assert _processor_section(open(tmp_path / "t.plb").read()) == (
        "        <Processor>\n            <Name> Custom_double_ForcedD3Q19 </Name>\n"
        "            <Domain> 0 1 0 1 0 1 </Domain>\n            <Data></Data>\n            <Level> 1 </Level>\n"
        "            <Blocks></Blocks>\n        </Processor>\n")
