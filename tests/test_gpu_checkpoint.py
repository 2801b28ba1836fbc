"""Binary-block checkpoints through the C ABI: files byte-identical to the
ones the reference wrote (saveBinaryBlock of the lattice, computeDensity and
computeVelocity), and load round trips.  Records are built and base64-encoded
on the device in slabs of x-planes; the multi-slab case checks the carry of
partial base64 groups across slabs against the oracle's encoding."""
import os

import numpy as np
import pytest

import goldens
import lbcases
import oracle as O
from palabos_gb300 import DeviceLattice3D, PlbGpuError, lattice_from_description

pytestmark = pytest.mark.gpu

CASES = ["binary_channel_sphere", "binary_guo_periodic_multiblock"]


def _lat(g, meta, precision="fp64"):
    return lattice_from_description(meta["nx"], meta["ny"], meta["nz"], meta["periodic"], meta["omega"],
                                    g["flags"], g["bcval"], g["force"], meta.get("rho0", 1.0),
                                    meta.get("bb_rho", 0.0), precision)


def _read(path):
    with open(path, "rb") as f:
        return f.read()


@pytest.mark.parametrize("name", CASES)
def test_saved_blocks_match_reference_files(name, tmp_path):
    g, meta = goldens.load(name)
    lat = _lat(g, meta)
    lat.send(g["f_init"])
    lat.collide_and_stream(meta["nsteps"])
    kind = "forced_lattice" if meta["forced"] else "lattice"
    for what, key in ((kind, "binary_lattice"), ("density", "binary_density"), ("velocity", "binary_velocity")):
        p = str(tmp_path / what)
        lat.save_binary_block(p, what)
        assert _read(p) == bytes(g[key]), what


@pytest.mark.parametrize("name", CASES)
def test_load_reference_file(name, tmp_path):
    g, meta = goldens.load(name)
    lat = _lat(g, meta)
    p = str(tmp_path / "ref")
    with open(p, "wb") as f:
        f.write(bytes(g["binary_lattice"]))
    lat.load_binary_block(p, "forced_lattice" if meta["forced"] else "lattice")
    assert np.array_equal(lat.receive(), g["f_final"])


@pytest.mark.parametrize("odd", [False, True])
def test_multi_slab_round_trip(tmp_path, odd):
    """A domain larger than one 32 MB slab, saved after an odd or even number
    of steps: the text equals the oracle's encoding of the received state, and
    loading it into a fresh domain restores every bit."""
    # 98 x 97 cells x 152 B = 1,444,912 B per plane: 23 planes per 32 MB slab, so the
    # slab boundaries fall 2 and 1 bytes into a base64 group (3 slabs)
    shape = (64, 98, 97)
    rng = np.random.default_rng(11)
    lat = DeviceLattice3D(*shape, 1.6)
    lat.periodicity(1, 1, 1)
    lat.send(lbcases.initial_state(shape, rng))
    lat.collide_and_stream(3 if odd else 2)
    f = lat.receive()
    p = str(tmp_path / "big")
    lat.save_binary_block(p)
    assert _read(p) == O.binary_block(f.reshape(-1, 19))
    for uint in (False, True):
        q = str(tmp_path / f"big{uint}")
        lat.save_binary_block(q, enforce_uint=uint)
        other = DeviceLattice3D(*shape, 1.6)
        other.load_binary_block(q, enforce_uint=uint)
        assert np.array_equal(other.receive(), f)


def test_external_fields_round_trip(tmp_path):
    g, meta = goldens.load("external_periodic_bgk")
    lat = _lat(g, meta)
    lat.set_rhobar_j(g["rho_bar0"], g["j0"])
    for what in ("rho_bar", "j"):
        lat.save_binary_block(str(tmp_path / what), what)
    assert _read(str(tmp_path / "rho_bar")) == O.binary_block(g["rho_bar0"].reshape(-1, 1))
    assert _read(str(tmp_path / "j")) == O.binary_block(g["j0"].reshape(-1, 3))
    other = _lat(g, meta)
    other.load_binary_block(str(tmp_path / "rho_bar"), "rho_bar")
    other.load_binary_block(str(tmp_path / "j"), "j")
    rb, j = other.get_rhobar_j()
    assert np.array_equal(rb, g["rho_bar0"]) and np.array_equal(j, g["j0"])


def test_bad_files_are_refused(tmp_path):
    lat = DeviceLattice3D(6, 5, 4, 1.5)
    good = str(tmp_path / "good")
    lat.save_binary_block(good)
    small = DeviceLattice3D(6, 5, 3, 1.5)
    with pytest.raises(PlbGpuError) as e:
        small.load_binary_block(good)              # byte count of another domain
    assert e.value.code == -1
    bad = str(tmp_path / "bad")
    text = bytearray(_read(good))
    text[40] = ord("*")
    with open(bad, "wb") as f:
        f.write(bytes(text))
    with pytest.raises(PlbGpuError):
        lat.load_binary_block(bad)                 # not base64
    with pytest.raises(PlbGpuError):
        lat.load_binary_block(good, "density")     # derived data cannot be loaded
    with pytest.raises(PlbGpuError):
        lat.load_binary_block(str(tmp_path / "missing"))
    lat.collide_and_stream(1)                      # the context stays usable
