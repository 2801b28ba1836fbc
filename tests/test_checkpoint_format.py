"""The binary-block checkpoint format (saveBinaryBlock) against files the
reference itself wrote: the oracle's restatement of the format reproduces
them byte for byte from the golden populations."""
import numpy as np
import pytest

import goldens
import oracle as O

CASES = ["binary_channel_sphere", "binary_guo_periodic_multiblock"]


@pytest.mark.parametrize("name", CASES)
def test_lattice_block_format(name):
    g, meta = goldens.load(name)
    f = g["f_final"]
    recs = f.reshape(-1, 19)
    if meta["forced"]:
        recs = np.concatenate([recs, g["force"].reshape(-1, 3)], axis=1)
    assert O.binary_block(recs) == bytes(g["binary_lattice"])


@pytest.mark.parametrize("name", CASES)
def test_velocity_block_format(name):
    g, meta = goldens.load(name)
    lat = O.OracleLattice.from_golden(g, meta)
    u = lat.velocity(g["f_final"])
    assert O.binary_block(u.reshape(-1, 3)) == bytes(g["binary_velocity"])


def test_header_forms():
    # 8-byte count: 12 characters with one '='; 4-byte count: 8 characters with '=='
    a = O.binary_block(np.zeros((2, 19)))
    b = O.binary_block(np.zeros((2, 19)), enforce_uint=True)
    assert a[:12].endswith(b"=") and b[:8].endswith(b"==") and a[12:] == b[8:]


# ---------------------------------------------------------------- saveState / parallelIO

import os
import re
import subprocess
import tempfile

import lbcases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "plb_case")
STATES = ["state_periodic_bgk_multiblock", "state_guo_periodic_multiblock"]


def state_components(plb):
    boxes = [tuple(map(int, m.split())) for m in re.findall(r"<Component[^>]*>([^<]*)</Component>", plb)]
    offsets = list(map(int, re.search(r"<Offsets>([^<]*)</Offsets>", plb).group(1).split()))
    return boxes, offsets


def records(g, meta):
    recs = g["f_final"]
    if meta["forced"]:
        recs = np.concatenate([recs, g["force"]], axis=-1)
    return recs


@pytest.mark.parametrize("name", STATES)
def test_reference_state_layout(name):
    """The reference's .dat is each component's records, x-major, in
    component order, at the offsets its description gives."""
    g, meta = goldens.load(name)
    plb = str(g["state_plb"])
    dat = bytes(g["state_dat"])
    boxes, offsets = state_components(plb)
    recs = records(g, meta)
    start = 0
    for (x0, x1, y0, y1, z0, z1), end in zip(boxes, offsets):
        part = np.ascontiguousarray(recs[x0:x1 + 1, y0:y1 + 1, z0:z1 + 1]).tobytes()
        assert dat[start:end] == part
        start = end
    assert start == len(dat)
    assert f"<cellDim> {recs.shape[-1]} </cellDim>" in plb


@pytest.mark.skipif(not os.path.exists(DRIVER), reason="reference driver not built (needs the reference sources)")
@pytest.mark.parametrize("name", STATES)
def test_reference_loads_single_component_state(name):
    """A state written the way plbgpu_save_state writes it (one component,
    oracle.state_files) is loaded by the reference's own parallelIO::load and
    continues the reference's trajectory bit for bit."""
    spec = lbcases.case_by_name(name)
    g, meta = goldens.load(name)
    f_init = g["f_init"]
    recs = f_init if not meta["forced"] else np.concatenate([f_init, g["force"]], axis=-1)
    with tempfile.TemporaryDirectory() as tmp:
        plb, dat = O.state_files(recs.reshape(-1, recs.shape[-1]), f_init.shape[:3], recs.shape[-1],
                                 "BlockLattice3D", "ForcedD3Q19" if meta["forced"] else "D3Q19",
                                 os.path.join(tmp, "s.dat"))
        with open(os.path.join(tmp, "s.plb"), "w") as f:
            f.write(plb)
        with open(os.path.join(tmp, "s.dat"), "wb") as f:
            f.write(dat)
        spec.options &= ~lbcases.OPT_SAVE_STATE
        cpath, rpath = os.path.join(tmp, "c"), os.path.join(tmp, "r")
        lbcases.write_case_file(spec, cpath)
        subprocess.run([DRIVER, cpath, rpath], check=True,
                       env=dict(os.environ, PLB_LOAD_STATE=os.path.join(tmp, "s.plb")))
        res = lbcases.read_result_file(rpath, spec)
    assert np.array_equal(res["f_init"], f_init)
    assert np.array_equal(res["f_final"], g["f_final"])


# ---------------------------------------------------------------- states with dynamic content

DSTATES = ["dstate_channel_sphere_multiblock", "dstate_velocity_box", "dstate_zhpress_faces",
           "dstate_guo_channel", "dstate_incbgk_nodyn", "sparse_dstate_sealed_channel"]
SINGLE_COMPONENT = DSTATES[1:5]


def _kinds(g):
    """The case's kinds, 255 outside the lattice of a sparse case."""
    kinds = g["flags"].copy()
    if "in_lattice" in g:
        kinds[~g["in_lattice"].astype(bool)] = 255
    return kinds


def _shape(meta):
    return (meta["nx"], meta["ny"], meta["nz"])


def _velocity_kind(k):
    return 6 <= k < 12 or 18 <= k < 24 or k >= 30


def _density_kind(k):
    return 12 <= k < 18 or 24 <= k < 30


def _masks(g, meta, kinds=None):
    if kinds is None:
        return O.OracleLattice.from_golden(g, meta).mebb_masks().reshape(_shape(meta))
    ol = O.OracleLattice(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"], kinds, g["bcval"],
                         g["force"], meta["rho0"], meta["bb_rho"])
    return ol.mebb_masks().reshape(_shape(meta))


@pytest.mark.parametrize("name", DSTATES)
def test_reference_dynamic_state_decodes(name):
    """parallelIO::save(lattice, base, true) as the reference wrote it: every
    cell's dynamics chain decodes to the case's kind, wall values and
    parameters, and its static values are the final populations."""
    g, meta = goldens.load(name)
    st = O.read_dynamic_state(str(g["dstate_plb"]), bytes(g["dstate_dat"]), _shape(meta))
    kinds = _kinds(g)
    assert np.array_equal(st["kinds"], kinds)   # a sparse state holds the kept blocks only
    vel = np.vectorize(_velocity_kind)(kinds)
    den = np.vectorize(_density_kind)(kinds)
    assert np.array_equal(st["bc"][vel], g["bcval"][vel])
    assert np.array_equal(st["bc"][den][:, 0], g["bcval"][den][:, 0])
    inside = kinds != 255
    assert np.array_equal(st["records"][inside], records(g, meta).reshape(st["records"].shape)[inside])
    assert st["omegas"] == {meta["omega"]}
    if (kinds == 2).any():
        assert st["inv_rho0s"] == {1.0 / meta["rho0"]}
    if np.isin(kinds, (3, 4, 5)).any():
        assert st["rhos"] == {meta["bb_rho"]}
    mebb = kinds == 4
    if mebb.any():
        assert np.array_equal(st["masks"][mebb], _masks(g, meta, kinds)[mebb])


@pytest.mark.parametrize("name", SINGLE_COMPONENT)
def test_dynamic_state_writer_reproduces_reference_bytes(name):
    """With the reference's own dynamics ids, the restated writer gives the
    reference's data file byte for byte and its DynamicsDict."""
    g, meta = goldens.load(name)
    ref_plb, ref_dat = str(g["dstate_plb"]), bytes(g["dstate_dat"])
    ids = {n: i for i, n in O.read_dynamic_state(ref_plb, ref_dat, _shape(meta))["names"].items()}
    plb, dat = O.dynamic_state_files(g["flags"], g["bcval"], _masks(g, meta), records(g, meta), 22 if meta["forced"] else 19,
                                     "ForcedD3Q19" if meta["forced"] else "D3Q19", "x.dat", meta["omega"],
                                     meta["rho0"], meta["bb_rho"], ids=ids)
    assert dat == ref_dat
    dd = re.search(r"<DynamicsDict>.*?</DynamicsDict>", plb, re.S).group(0)
    assert dd == re.search(r"<DynamicsDict>.*?</DynamicsDict>", ref_plb, re.S).group(0)


@pytest.mark.skipif(not os.path.exists(DRIVER), reason="reference driver not built (needs the reference sources)")
@pytest.mark.parametrize("name", ["dstate_channel_sphere_multiblock", "dstate_velocity_box", "dstate_zhpress_faces",
                                  "dstate_incbgk_nodyn", "sparse_dstate_sealed_channel"])
def test_reference_loads_dynamic_state(name):
    """A state written the way plbgpu_save_state_dynamic writes it (one
    component, the library's own ids) is loaded by the reference's
    parallelIO::load(plb, lattice, true) into a lattice built with other
    parameters (omega, wall velocities and densities, rho0); the regenerated
    dynamics carry the state's and the run continues the reference's
    trajectory bit for bit."""
    spec = lbcases.case_by_name(name)
    g, meta = goldens.load(name)
    cd = 22 if meta["forced"] else 19
    recs = g["f_init"] if not meta["forced"] else np.concatenate([g["f_init"], g["force"]], axis=-1)
    with tempfile.TemporaryDirectory() as tmp:
        kinds = _kinds(g)
        plb, dat = O.dynamic_state_files(kinds, g["bcval"], _masks(g, meta, kinds), recs, cd,
                                         "ForcedD3Q19" if meta["forced"] else "D3Q19", os.path.join(tmp, "s.dat"),
                                         meta["omega"], meta["rho0"], meta["bb_rho"])
        with open(os.path.join(tmp, "s.plb"), "w") as f:
            f.write(plb)
        with open(os.path.join(tmp, "s.dat"), "wb") as f:
            f.write(dat)
        spec.options &= ~lbcases.OPT_SAVE_DYNAMIC_STATE
        spec.omega = 1.1
        spec.bcval = np.where(spec.bcval != 0, 0.5 * spec.bcval + 0.25, 0.0)
        spec.rho0 = 1.07
        cpath, rpath = os.path.join(tmp, "c"), os.path.join(tmp, "r")
        lbcases.write_case_file(spec, cpath)
        subprocess.run([DRIVER, cpath, rpath], check=True,
                       env=dict(os.environ, PLB_LOAD_DYNAMIC_STATE=os.path.join(tmp, "s.plb")))
        res = lbcases.read_result_file(rpath, spec)
    assert np.array_equal(res["f_init"], g["f_init"])
    # A sparse lattice's blocks keep envelope cells facing the dropped blocks,
    # which are in no state and collide with the lattice's own background
    # dynamics: the fluid sealed off from them is compared.
    cmp = g["compare"].astype(bool) if "compare" in g else np.ones(g["flags"].shape, bool)
    assert np.array_equal(res["f_final"][cmp], g["f_final"][cmp])


@pytest.fixture(scope="module")
def dynstate_check(tmp_path_factory):
    """tests/cpp/dynstate_check.cpp built with the host compiler."""
    import shutil
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("cpp") / "dynstate_check")
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "dynstate_check.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("name", DSTATES)
def test_library_state_codec_reencodes_reference_bytes(name, dynstate_check, tmp_path):
    """The library's own C++ codec (palabos_gb300/csrc/dynstate.h) decodes
    every cell of the reference's state and, under the state's ids, encodes
    it back to the same bytes."""
    g, meta = goldens.load(name)
    plb, dat = tmp_path / "s.plb", tmp_path / "s.dat"
    plb.write_text(str(g["dstate_plb"]))
    dat.write_bytes(bytes(g["dstate_dat"]))
    out = subprocess.run([dynstate_check, str(plb), str(dat), str(meta["nx"]), str(meta["ny"]), str(meta["nz"])],
                         capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.startswith("ok "), out.stdout


@pytest.mark.parametrize("damage", ["truncated", "unknown_id", "bad_run", "extra_bytes"])
def test_library_state_codec_rejects_damaged_states(damage, dynstate_check, tmp_path):
    """A damaged state is reported as an error, not read past its end: a
    truncated data file, a dynamics id missing from the DynamicsDict, a run
    whose count exceeds the dynamics' values, bytes beyond the last cell."""
    g, meta = goldens.load("dstate_velocity_box")
    plb, dat = str(g["dstate_plb"]), bytearray(bytes(g["dstate_dat"]))
    if damage == "truncated":
        dat = dat[:len(dat) // 2]
    elif damage == "unknown_id":
        dat[4:8] = (9999).to_bytes(4, "little")          # id of the first cell's outer dynamics
    elif damage == "bad_run":
        dat[16:20] = (1000).to_bytes(4, "little")        # count of its first run of values
    else:
        dat += b"\0" * 8
    (tmp_path / "s.plb").write_text(plb)
    (tmp_path / "s.dat").write_bytes(bytes(dat))
    out = subprocess.run([dynstate_check, str(tmp_path / "s.plb"), str(tmp_path / "s.dat"), str(meta["nx"]),
                          str(meta["ny"]), str(meta["nz"])], capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and out.stdout.startswith("FAIL"), (out.returncode, out.stdout)
