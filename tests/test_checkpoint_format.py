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
