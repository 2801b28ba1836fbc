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


def drag_gradient_study(shape=(256, 128, 128), steps=10000, precisions=("fp64", "fp32"), fd_h=1e-4, ctx=None):
    """dD_x/domega of the channel past a sphere (regularized parabolic inlet,
    regularized pressure outlet, bounce-back walls, momentum-exchange sphere
    r = shape[1] / 8, omega 1.8): D the momentum-exchange drag of the state
    after `steps` steps from rest, through the checkpointed adjoint (the
    checkpoint interval the library picks from free memory), against a
    central difference of two FP64 runs.  Reports the cost of the recording
    and of the backward sweep per step against a plain step."""
    from . import workloads
    nx, ny, nz = shape
    wl = workloads.channel_sphere(shape, (nx / 4, ny / 2, nz / 2), ny / 8, 0.05, 1.8)
    e = np.array([1.0, 0.0, 0.0])
    out = {"shape": list(shape), "steps": steps, "omega": wl.omega, "forms": {}}
    for p in precisions:
        lat = wl.lattice(p, ctx)
        f0 = lat.receive()
        fwd_ms = lat.time_steps(100) / 100
        lat.send(f0)
        t0 = time.perf_counter()
        K = lat.adjoint_forward(steps, 0)
        rec_s = time.perf_counter() - t0
        J, _, g, ms = lat.adjoint_backward(drag=e, want_force=False)
        out["forms"][p] = {"drag_x": J, "d_drag_x_domega": g, "K": K,
                           "forward_step_ms": round(fwd_ms, 4), "record_ms_per_step": round(rec_s * 1e3 / steps, 4),
                           "backward_ms_per_step": round(ms / steps, 4),
                           "backward_over_forward": round(ms / steps / fwd_ms, 3)}
        lat.close()
    if fd_h:
        vals = []
        for om in (wl.omega + fd_h, wl.omega - fd_h):
            w2 = workloads.channel_sphere(shape, (nx / 4, ny / 2, nz / 2), ny / 8, 0.05, om)
            lat = w2.lattice("fp64", ctx)
            lat.collide_and_stream(steps)
            J2, _, _, _ = lat.adjoint_steady(iterations=0, want_force=False, drag=e)
            vals.append(J2)
            lat.close()
        fd = (vals[0] - vals[1]) / (2 * fd_h)
        out["fd_fp64"] = {"h": fd_h, "d_drag_x_domega": fd}
        for p in precisions:
            out["forms"][p]["rel_err_vs_fd"] = abs(out["forms"][p]["d_drag_x_domega"] - fd) / abs(fd)
    return out
