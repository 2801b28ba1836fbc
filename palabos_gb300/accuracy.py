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
