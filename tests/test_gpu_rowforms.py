"""The interior-row kernels of the 2-byte storage forms against the one-cell
kernel (PLBGPU_ROW_KERNEL=cell), bit for bit: the default paired kernel (two
cells per thread) and the vector kernels (palabos_gb300/csrc/vecrow.cuh:
eight, four or two cells per thread, 128-, 64- or 32-bit population words).

All run the same FP32 collision on the same stored values, so every stored
population must be identical; the cases reach every path of the vector
kernels' streaming:

  rows of 1, 2, 12 and 64 eight-cell segments (a whole row in one lane, rows
  inside a warp, rows straddling warp boundaries, rows spanning two warps) and
  of 1 and 33 two-cell segments (rows whose length is no multiple of eight,
  which only the two-cell vector kernel and the paired kernel take);
  periodic and non-periodic z (the wrap and the domain-edge reflection at the
  row ends); bounce-back, momentum exchange, Guo force, regularized and
  Zou/He faces inside interior rows (pending face completion); both AA
  parities; statistics steps; the external rho-bar/j form.
"""
import os

import numpy as np
import pytest

import lbcases as C
from palabos_gb300 import Context, lattice_from_description
from palabos_gb300 import native as N

pytestmark = pytest.mark.gpu


def _context(form):
    """A context whose interior rows run `form` ("cell", "vec8", "vec4",
    "vec2" or "default")."""
    old = os.environ.get("PLBGPU_ROW_KERNEL")
    if form != "default":
        os.environ["PLBGPU_ROW_KERNEL"] = form
    else:
        os.environ.pop("PLBGPU_ROW_KERNEL", None)
    try:
        return Context(0)
    finally:
        if old is None:
            os.environ.pop("PLBGPU_ROW_KERNEL", None)
        else:
            os.environ["PLBGPU_ROW_KERNEL"] = old


def _periodic(shape, seed):
    flags, bcval, force, _ = C.empty(shape)
    f0 = C.initial_state(shape, np.random.default_rng(seed))
    return dict(shape=shape, periodic=(1, 1, 1), omega=1.7, flags=flags, bcval=bcval, force=None, f0=f0)


def _walled_z(shape, seed):
    """Periodic x and y, bounce-back planes at z = 0 and z = nz-1, Guo-forced
    fluid with a few bounce-back and momentum-exchange cells inside."""
    rng = np.random.default_rng(seed)
    flags, bcval, force, _ = C.empty(shape)
    flags[:] = N.GUO
    flags[:, :, 0] = flags[:, :, -1] = N.BOUNCEBACK
    inner = rng.random(shape) < 0.04
    inner[:, :, 0] = inner[:, :, -1] = False
    flags[inner] = N.BOUNCEBACK
    flags[rng.random(shape) < 0.02] = N.MOMENTUM_EXCHANGE
    force[..., 0] = 1e-5
    force += 1e-6 * rng.standard_normal(force.shape)
    f0 = C.initial_state(shape, rng)
    return dict(shape=shape, periodic=(1, 1, 0), omega=1.4, flags=flags, bcval=bcval, force=force, f0=f0)


def _faces_z(shape, seed, family):
    """Non-periodic box: bounce-back walls at x and y ends, velocity (or
    pressure) faces of `family` on the z = 0 and z = nz-1 planes of the
    interior rows."""
    rng = np.random.default_rng(seed)
    flags, bcval, force, _ = C.empty(shape)
    flags[0] = flags[-1] = N.BOUNCEBACK
    flags[:, 0] = flags[:, -1] = N.BOUNCEBACK
    for o, z in ((-1, 0), (1, shape[2] - 1)):
        sl = (slice(1, -1), slice(1, -1), z)
        flags[sl] = N.face_kind(family, 2, o)
        if family in (N.REG_VELOCITY, N.ZOUHE_VELOCITY):
            bcval[sl + (2,)] = -0.02 * o
            bcval[sl + (0,)] = 0.01 * rng.standard_normal(bcval[sl + (0,)].shape)
        else:
            bcval[sl + (0,)] = 1.0 + 0.002 * rng.standard_normal(bcval[sl + (0,)].shape)
    f0 = C.initial_state(shape, rng, u_amp=0.02, rho_amp=0.003)
    return dict(shape=shape, periodic=(0, 0, 0), omega=1.6, flags=flags, bcval=bcval, force=None, f0=f0)


def _cavity(shape, seed):
    s = C.cavity(shape, 0.05, 1.85, 1, "cavity", np.random.default_rng(seed))
    return dict(shape=shape, periodic=(0, 0, 0), omega=s.omega, flags=s.flags, bcval=s.bcval, force=None, f0=s.f0)


def _channel(shape, seed):
    s = C.channel_sphere(shape, (shape[0] // 3, shape[1] // 2, shape[2] // 2), 3.0, 0.05, 1.8, 1, "channel",
                         np.random.default_rng(seed))
    return dict(shape=shape, periodic=(0, 0, 0), omega=s.omega, flags=s.flags, bcval=s.bcval, force=None, f0=s.f0)


CASES = {
    "periodic_rows_of_64_segments": lambda: _periodic((6, 5, 512), 11),
    "periodic_rows_of_12_segments": lambda: _periodic((7, 6, 96), 12),
    "walled_z_rows_of_1_segment": lambda: _walled_z((9, 7, 8), 13),
    "walled_z_rows_of_12_segments": lambda: _walled_z((6, 7, 96), 14),
    "periodic_rows_of_1_pair": lambda: _periodic((6, 5, 2), 21),
    "walled_z_rows_of_33_pairs": lambda: _walled_z((6, 7, 66), 22),
    "regularized_velocity_faces_in_rows": lambda: _faces_z((8, 7, 24), 15, N.REG_VELOCITY),
    "zouhe_pressure_faces_in_rows": lambda: _faces_z((8, 7, 40), 16, N.ZOUHE_PRESSURE),
    "cavity_lid_in_rows": lambda: _cavity((10, 9, 96), 17),
    "channel_past_sphere": lambda: _channel((24, 12, 16), 18),
}


def _run(case, precision, form, steps, external=False):
    ctx = _context(form)
    nx, ny, nz = case["shape"]
    lat = lattice_from_description(nx, ny, nz, case["periodic"], case["omega"], case["flags"], case["bcval"],
                                   case["force"], precision=precision, ctx=ctx)
    lat.send(case["f0"])
    if external:
        lat.compute_rhobar_j()
        lat.collide_and_stream_external(steps, recompute=True, stats=True)
    else:
        lat.initialize()
        lat.collide_and_stream(steps - 1)
        lat.collide_and_stream(1, stats=True)
    f = lat.receive()
    st = lat.internal_statistics()
    lat.close()
    ctx.close()
    return f, st


@pytest.mark.parametrize("precision", ["bf16", "fp16"])
@pytest.mark.parametrize("form", ["default", "vec8", "vec4", "vec2"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_row_kernels_equal_one_cell_rows(name, form, precision):
    case = CASES[name]()
    steps = 9   # both AA parities, ending on an odd step
    f_vec, st_vec = _run(case, precision, form, steps)
    f_cell, st_cell = _run(case, precision, "cell", steps)
    assert np.isfinite(f_vec).all()
    if not np.array_equal(f_vec, f_cell):
        bad = np.argwhere(f_vec != f_cell)
        raise AssertionError(f"{len(bad)} populations differ, first at {bad[:4].tolist()}")
    assert st_vec["count"] == st_cell["count"]
    np.testing.assert_allclose(st_vec["raw"][:3], st_cell["raw"][:3], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(st_vec["drag"], st_cell["drag"], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("precision", ["bf16", "fp16"])
@pytest.mark.parametrize("form", ["default", "vec8", "vec4", "vec2"])
def test_row_kernels_external_form_equal_one_cell_rows(form, precision):
    case = _periodic((8, 6, 64), 19)
    f_vec, _ = _run(case, precision, form, 7, external=True)
    f_cell, _ = _run(case, precision, "cell", 7, external=True)
    assert np.array_equal(f_vec, f_cell)


@pytest.mark.parametrize("form", ["default", "vec8", "vec2"])
def test_row_kernels_stochastic_rounding_track_one_cell_rows(form):
    """BF16 with stochastic rounding draws its random bits from different
    addresses in the kernels, so the states agree only to the rounding."""
    case = _periodic((7, 6, 96), 20)
    f_vec, _ = _run(case, "bf16sr", form, 9)
    f_cell, _ = _run(case, "bf16sr", "cell", 9)
    scale = np.abs(f_cell).max()
    assert np.abs(f_vec - f_cell).max() <= 0.03 * scale
