"""Synthetic workloads with the shapes, sizes and value distributions of the
reference's benchmark configurations (deterministic, seeded).

  cavity(n)            lid-driven cavity, bounce-back on 5 walls, regularized lid
  channel_sphere()     channel past a momentum-exchange sphere, regularized inlet/outlet
  taylor_green(n)      periodic Taylor-Green vortex, Re = 1600 with L = 1/k
  forced_channel()     Guo-forced periodic-x channel with a seeded per-cell force field
  sphere_packing(n)    periodic random packing of bounce-back spheres, porosity 0.4

Each builder returns the cell kinds and the per-cell values the C ABI takes
(face values, Guo force, initial rho/u) plus omega.  Cell kinds follow
include/plbgpu.h.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import native as N


@dataclasses.dataclass
class Workload:
    name: str
    shape: tuple
    omega: float
    periodic: tuple
    kinds: np.ndarray
    bcval: np.ndarray | None = None      # (nx, ny, nz, 3): velocity, or density in component 0
    force: np.ndarray | None = None      # (nx, ny, nz, 3) Guo force
    rho_u: object = None                 # callable(x0, x1) -> (rho, u) for the slab of x in [x0, x1]

    def lattice(self, precision="fp64", ctx=None, slab=16):
        """A device lattice initialized at equilibrium with rho_u (rest if None)."""
        from .lattice import lattice_from_description
        nx, ny, nz = self.shape
        lat = lattice_from_description(nx, ny, nz, self.periodic, self.omega, self.kinds, self.bcval,
                                       self.force, precision=precision, ctx=ctx)
        if self.rho_u is None:
            lat.initialize_at_equilibrium(None, 1.0, (0.0, 0.0, 0.0))
        else:
            for x0 in range(0, nx, slab):
                x1 = min(nx, x0 + slab) - 1
                rho, u = self.rho_u(x0, x1)
                lat.initialize_at_equilibrium((x0, x1, 0, ny - 1, 0, nz - 1), rho, u)
        lat.initialize()
        return lat


def cavity(n=64, lid_u=0.02, re=100.0):
    """Lid-driven cavity, n^3, nu = lid_u * n / Re, omega = 1/(3 nu + 1/2)."""
    kinds = np.zeros((n, n, n), np.uint8)
    bc = np.zeros((n, n, n, 3))
    for sl in [(0, slice(None), slice(None)), (-1, slice(None), slice(None)),
               (slice(None), 0, slice(None)), (slice(None), -1, slice(None)),
               (slice(None), slice(None), 0)]:
        kinds[sl] = N.BOUNCEBACK
    kinds[1:-1, 1:-1, -1] = N.face_kind(N.REG_VELOCITY, 2, +1)
    bc[1:-1, 1:-1, -1, 0] = lid_u
    kinds[0, :, -1] = kinds[-1, :, -1] = kinds[:, 0, -1] = kinds[:, -1, -1] = N.BOUNCEBACK
    nu = lid_u * n / re
    return Workload("cavity", (n, n, n), 1.0 / (3.0 * nu + 0.5), (0, 0, 0), kinds, bc)


def channel_sphere(shape=(256, 128, 128), center=(64, 64, 64), radius=16, u_max=0.05, omega=1.8):
    """Channel past a sphere: parabolic regularized inlet at x=0, regularized pressure rho=1
    at x=nx-1, bounce-back channel walls, momentum-exchange sphere."""
    nx, ny, nz = shape
    kinds = np.zeros(shape, np.uint8)
    bc = np.zeros(shape + (3,))
    kinds[:, 0, :] = kinds[:, -1, :] = kinds[:, :, 0] = kinds[:, :, -1] = N.BOUNCEBACK
    kinds[0, 1:-1, 1:-1] = N.face_kind(N.REG_VELOCITY, 0, -1)
    kinds[-1, 1:-1, 1:-1] = N.face_kind(N.REG_PRESSURE, 0, +1)
    yy = (np.arange(ny) - 0.5) / (ny - 1)
    zz = (np.arange(nz) - 0.5) / (nz - 1)
    prof = 16.0 * u_max * (yy[:, None] * (1 - yy[:, None])) * (zz[None, :] * (1 - zz[None, :]))
    bc[0, 1:-1, 1:-1, 0] = prof[1:-1, 1:-1]
    bc[-1, 1:-1, 1:-1, 0] = 1.0
    x = np.arange(nx)[:, None, None]
    y = np.arange(ny)[None, :, None]
    z = np.arange(nz)[None, None, :]
    sphere = ((x - center[0]) ** 2 + (y - center[1]) ** 2 + (z - center[2]) ** 2 <= radius * radius)
    kinds[sphere & (kinds == N.BGK)] = N.MOMENTUM_EXCHANGE
    return Workload("channel_sphere", shape, omega, (0, 0, 0), kinds, bc)


def taylor_green(n=512, u0=0.04, re=1600.0):
    """Taylor-Green vortex: u = u0 (sin kx cos ky cos kz, -cos kx sin ky cos kz, 0),
    k = 2 pi / n, p = (u0^2/16)(cos 2kx + cos 2ky)(cos 2kz + 2), rho = 1 + 3p;
    Re = u0 / (k nu), i.e. the length scale is 1/k."""
    k = 2.0 * math.pi / n
    nu = u0 / (k * re)
    omega = 1.0 / (3.0 * nu + 0.5)

    def rho_u(x0, x1):
        x = np.arange(x0, x1 + 1, dtype=np.float64)[:, None, None] * k
        y = np.arange(n, dtype=np.float64)[None, :, None] * k
        z = np.arange(n, dtype=np.float64)[None, None, :] * k
        shape = (x1 - x0 + 1, n, n)
        u = np.zeros(shape + (3,))
        u[..., 0] = u0 * np.sin(x) * np.cos(y) * np.cos(z)
        u[..., 1] = -u0 * np.cos(x) * np.sin(y) * np.cos(z)
        p = (u0 * u0 / 16.0) * (np.cos(2 * x) + np.cos(2 * y)) * (np.cos(2 * z) + 2.0)
        return np.broadcast_to(1.0 + 3.0 * p, shape).copy(), u

    kinds = np.zeros((n, n, n), np.uint8)
    return Workload("taylor_green", (n, n, n), omega, (1, 1, 1), kinds, rho_u=rho_u)


def forced_channel(shape=(128, 64, 64), omega=1.6, seed=1234, sigma=1e-6, drive=1e-5):
    """Guo-forced channel (the adjoint's forward model): periodic x, bounce-back walls at y and z ends,
    Guo-forced BGK with F ~ N(0, sigma^2) i.i.d. per component plus (drive, 0, 0)."""
    rng = np.random.default_rng(seed)
    kinds = np.full(shape, N.GUO, np.uint8)
    kinds[:, 0, :] = kinds[:, -1, :] = kinds[:, :, 0] = kinds[:, :, -1] = N.BOUNCEBACK
    force = sigma * rng.standard_normal(shape + (3,))
    force[..., 0] += drive
    return Workload("forced_channel", shape, omega, (1, 0, 0), kinds, force=force)


def sphere_packing(n=384, porosity=0.68, rmin=6.0, rmax=12.0, seed=77, force=1e-6, omega=1.0,
                   max_attempts=400000):
    """Sphere packing: periodic box, seeded non-overlapping spheres with radius
    U[rmin, rmax] placed by random sequential addition until the porosity
    (fluid fraction) falls to the target or the attempts run out, as
    bounce-back cells; Guo force along x in every cell (only the fluid uses
    it).  Non-overlapping random addition jams near a solid fraction of 0.38,
    and the rejections multiply well before that: at n = 384 the default
    0.68 takes a little over 3 x 10^5 attempts (porosity 0.72 after 10^5),
    and 0.65 is not reached in 4 x 10^5.  Overlap tests use a grid of
    buckets of side 2 rmax."""
    rng = np.random.default_rng(seed)
    solid = np.zeros((n, n, n), bool)
    nb = max(1, int(n // (2 * rmax)))
    side = n / nb
    buckets = {}
    target = (1.0 - porosity) * n ** 3
    filled = 0
    attempts = 0
    while filled < target and attempts < max_attempts:
        attempts += 1
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(0, n, size=3)
        b = (c // side).astype(int) % nb
        ok = True
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for c2, r2 in buckets.get(((b[0] + dx) % nb, (b[1] + dy) % nb, (b[2] + dz) % nb), ()):
                        d = np.abs(c - c2)
                        d = np.minimum(d, n - d)
                        if d[0] * d[0] + d[1] * d[1] + d[2] * d[2] < (r + r2) ** 2:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if not ok:
            continue
        buckets.setdefault(tuple(b), []).append((c, r))
        lo = np.floor(c - r).astype(int)
        hi = np.ceil(c + r).astype(int)
        ax = [np.arange(lo[a], hi[a] + 1) for a in range(3)]
        X, Y, Z = np.meshgrid(*ax, indexing="ij")
        m = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 <= r * r
        ix, iy, iz = np.mod(X[m], n), np.mod(Y[m], n), np.mod(Z[m], n)
        filled += int((~solid[ix, iy, iz]).sum())
        solid[ix, iy, iz] = True
    kinds = np.where(solid, N.BOUNCEBACK, N.GUO).astype(np.uint8)
    f = np.zeros((n, n, n, 3))
    f[..., 0] = force
    # omega = 1 (nu = 1/6) by default: the configuration fixes the force, not the viscosity
    return Workload("sphere_packing", (n, n, n), omega, (1, 1, 1), kinds, force=f)


def permeability(mean_ux, force, omega):
    """Darcy permeability k = nu <u_x> / F of a body-forced periodic medium:
    <u_x> the superficial velocity (mean over all cells, walls counted as 0),
    F the force density, nu = (1/omega - 1/2) / 3."""
    return (1.0 / omega - 0.5) / 3.0 * mean_ux / force


def permeability_derivative(mean_ux, d_mean_ux_domega, force, omega):
    """dk/domega from <u_x> and its derivative d<u_x>/domega."""
    nu = (1.0 / omega - 0.5) / 3.0
    return (-1.0 / (3.0 * omega * omega) * mean_ux + nu * d_mean_ux_domega) / force
