"""Accuracy of the reduced-precision storage forms on the Taylor-Green vortex.

Runs the FP64 form (the reference-exact path) and the FP32-compute forms with
FP32, BF16 (round to nearest and stochastic rounding) and FP16 f-bar storage
side by side on the same periodic
Taylor-Green vortex, and reports for each form

  vel_l2_rel   ||u - u_fp64||_2 / ||u_fp64||_2 over all cells at the end,
  ke_rel_max   max over the sampled times of |E - E_fp64| / E_fp64(0),
  ke_final     the average kinetic energy (computeAverageEnergy) at the end,

with E the average energy per cell.  The FP64 form itself matches the
reference CPU path bit for bit (tests/test_gpu_parity.py), so it is the
oracle here.
"""
from __future__ import annotations

import time

import numpy as np

from . import workloads
from .lattice import DeviceLattice3D


def taylor_green_study(n=512, steps=5000, forms=("fp32", "bf16", "fp16", "bf16sr"), every=500, slab=8, ctx=None):
    wl = workloads.taylor_green(n)
    names = ("fp64",) + tuple(forms)
    lats = {}
    for p in names:
        lat = DeviceLattice3D(n, n, n, wl.omega, p, ctx)
        lat.periodicity(1, 1, 1)
        for x0 in range(0, n, slab):
            x1 = min(n, x0 + slab) - 1
            rho, u = wl.rho_u(x0, x1)
            lat.initialize_at_equilibrium((x0, x1, 0, n - 1, 0, n - 1), rho, u)
        lats[p] = lat
    energy = {p: [lats[p].compute_average_energy()] for p in names}
    times = [0]
    seconds = {p: 0.0 for p in names}
    done = 0
    while done < steps:
        k = min(every, steps - done)
        for p in names:
            seconds[p] += lats[p].time_steps(k) / 1e3
            energy[p].append(lats[p].compute_average_energy())
        done += k
        times.append(done)
    # velocity-field error, slab by slab
    num = {p: 0.0 for p in forms}
    den = 0.0
    for x0 in range(0, n, slab):
        box = (x0, min(n, x0 + slab) - 1, 0, n - 1, 0, n - 1)
        ref = lats["fp64"].compute_velocity(box)
        den += float(np.sum(ref * ref))
        for p in forms:
            d = lats[p].compute_velocity(box) - ref
            num[p] += float(np.sum(d * d))
    e0 = energy["fp64"][0]
    out = {"n": n, "steps": steps, "omega": wl.omega, "times": times,
           "energy_fp64": energy["fp64"], "mlups": {}, "forms": {}}
    for p in names:
        out["mlups"][p] = round(n ** 3 * steps / seconds[p] / 1e6, 1)
    for p in forms:
        ke = np.asarray(energy[p])
        kr = np.asarray(energy["fp64"])
        out["forms"][p] = {
            "vel_l2_rel": float(np.sqrt(num[p] / den)),
            "ke_rel_max": float(np.max(np.abs(ke - kr)) / e0),
            "ke_final": float(ke[-1]),
        }
    out["ke_final_fp64"] = float(energy["fp64"][-1])
    out["ke_decay_fp64"] = float(energy["fp64"][-1] / e0)
    for lat in lats.values():
        lat.close()
    return out


def _mean_flux(lat, n, slab=16):
    """Mean x-velocity over all cells (walls count as 0): the superficial velocity."""
    s = 0.0
    for x0 in range(0, n, slab):
        s += float(np.sum(lat.compute_velocity((x0, min(n, x0 + slab) - 1, 0, n - 1, 0, n - 1))[..., 0]))
    return s / n ** 3


def permeability_study(n=384, steps=20000, forms=("fp32", "bf16"), every=1000, adjoint_iterations=(3000,),
                       force=1e-6, seed=77, ctx=None):
    """Permeability of the sphere packing (periodic n^3 box, Guo force along
    x, bounce-back spheres) in the FP64 form and the reduced-precision forms:
    k = nu <u_x> / F after `steps` steps, with the flux history every `every`
    steps, the MLUPS of each form, and dk/domega from the steady adjoint of
    the converged state (FP64 and FP32; one entry per iteration count, so the
    convergence of the adjoint sum shows)."""
    wl = workloads.sphere_packing(n=n, seed=seed, force=force)
    blocks = n // 32
    fluid = wl.kinds != 3
    kept = int(fluid[:blocks * 32, :blocks * 32, :blocks * 32]
               .reshape(blocks, 32, blocks, 32, blocks, 32).any(axis=(1, 3, 5)).sum()) if blocks else 0
    out = {"n": n, "steps": steps, "omega": wl.omega, "force": force, "porosity": float(fluid.mean()),
           "blocks_32": blocks ** 3, "blocks_32_with_fluid": kept, "forms": {}}
    w = None
    for p in ("fp64",) + tuple(forms):
        lat = wl.lattice(p, ctx)
        seconds, history, done = 0.0, [], 0
        while done < steps:
            k = min(every, steps - done)
            seconds += lat.time_steps(k) / 1e3
            done += k
            history.append(_mean_flux(lat, n))
        flux = history[-1]
        r = {"mean_ux": flux, "k": workloads.permeability(flux, force, wl.omega),
             "flux_history": history, "mlups": round(n ** 3 * steps / seconds / 1e6, 1)}
        if p in ("fp64", "fp32"):
            if w is None:
                w = np.zeros((n, n, n, 3))
                w[..., 0] = 1.0 / n ** 3
            r["adjoint"] = []
            for it in adjoint_iterations:
                J, _, g, ms = lat.adjoint_steady(w, it, want_force=False)
                r["adjoint"].append({"iterations": it, "mean_ux": J, "d_mean_ux_domega": g,
                                     "dk_domega": workloads.permeability_derivative(J, g, force, wl.omega),
                                     "ms_per_iteration": round(ms / max(it, 1), 4)})
        out["forms"][p] = r
        lat.close()
    k64 = out["forms"]["fp64"]["k"]
    for p in forms:
        out["forms"][p]["k_rel_err"] = abs(out["forms"][p]["k"] - k64) / abs(k64)
    return out
