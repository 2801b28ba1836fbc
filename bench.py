"""Benchmark of the D3Q19 collide-and-stream hot path on GB300.

Workload (the configuration the metric is quoted on that fits one GPU):
channel flow past a sphere, D3Q19 BGK, 256x128x128, regularized parabolic
velocity inlet at x=0 (u_max 0.05), regularized pressure outlet rho=1 at
x=255, bounce-back channel walls, momentum-exchange bounce-back sphere of
radius 16 at (64,64,64), omega 1.8; the momentum-exchange drag is reduced in
FP64 every 100 steps.  Synthetic, deterministic geometry; the flow starts at
rest.  One benchmark step = one collide-and-stream time step of the whole
lattice.  The lattice state (637 MB in FP64) is larger than the 129 MB L2, so
no explicit flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  `value` = MLUPS of the FP64 form with the
state resident in HBM; `e2e` = the same metric through the C ABI with host
buffers (the FP64 state in pinned host memory allocated before the timed
region -- sent at the start, drag read back every 100 steps, state received at
the end into the same buffer, all inside the timed region, in one
plbgpu_run_host call that overlaps the send with the first step and the
receive with the last; on a GB300 the transfer kernels read and write the host
buffer directly over NVLink-C2C; `e2e.sequential` times plbgpu_send,
plbgpu_collide_and_stream and plbgpu_receive one after another and
`e2e.pageable` repeats both with an ordinary numpy array).  The FP64 form is bound by the
FP64 pipe, not by HBM: its `roofline` compares the algorithmic FP64 adds and
multiplies per second with the pipe rate the library measures in the same run
(plbgpu_measure_fp64_rate), and carries the HBM fraction beside it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MLUPS & %HBM roofline: FP64 plain vs FP32/BF16-store at stated L2 err; adjoint/fwd"
SHAPE = (256, 128, 128)
OMEGA = 1.8
STATS_EVERY = 100
FALLBACK_HBM_GBS = 6800.0
# Algorithmic bytes per cell and step (AA pattern: every population read once
# and written once, plus the one-byte cell kind).
B_CELL = {"fp64": 305, "fp32": 153, "bf16": 77, "fp16": 77, "bf16sr": 77}
# Algorithmic FP64 adds and multiplies of one BGK collision in the reference's
# operand order (dynamicsTemplates3D.h:2289-2366, momentTemplates3D.h:351-365):
# moments 37 adds, 1 / (rho-bar + 1) one add and one division, collision 137.
FP64_OPS_BGK = 176


def workload_geometry():
    """Cell kinds and face values of the channel (palabos_gb300.workloads.channel_sphere)."""
    from palabos_gb300 import workloads
    wl = workloads.channel_sphere(SHAPE, omega=OMEGA)
    return wl.kinds, wl.bcval


def build_lattice(precision, ctx=None):
    from palabos_gb300 import workloads
    wl = workloads.channel_sphere(SHAPE, omega=OMEGA)
    return wl.lattice(precision, ctx), wl.kinds


def algorithmic_bytes(kinds, precision):
    from palabos_gb300 import native as N
    cells = kinds.size
    faces = int(((kinds >= N.REG_VELOCITY) & (kinds < N.VELOCITY_EDGE)).sum())
    mebb = int((kinds == N.MOMENTUM_EXCHANGE).sum())
    # cells that run a BGK collision (bulk, faces, edges, corners)
    colliding = int(((kinds == N.BGK) | (kinds == N.GUO) | (kinds == N.INCBGK)
                     | ((kinds >= N.REG_VELOCITY) & (kinds < N.NKINDS))).sum())
    # faces also read their 3 FP64 boundary values
    return cells * B_CELL[precision] + faces * 24, dict(cells=cells, faces=faces, mebb=mebb, colliding=colliding)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def load_traffic(kernel_key):
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(kernel_key)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ distributed

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ CPU baseline

def cpu_baseline(steps_cap=None, seconds=15.0):
    """The oracle (plain-C restatement of the reference path) on the host
    cores, on the same workload, all OpenMP threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    kinds, bc = workload_geometry()
    lat = O.OracleLattice(*SHAPE, (0, 0, 0), OMEGA, kinds, bc)
    f = lat.initialize(np.zeros(SHAPE + (19,)))
    threads = O.max_threads()
    O.set_threads(threads)
    f, _ = lat.run(f, 1, with_stats=False)   # warm-up
    t0 = time.perf_counter()
    f, _ = lat.run(f, 1, with_stats=False)
    one = time.perf_counter() - t0
    n = max(1, int(seconds / max(one, 1e-6)))
    if steps_cap:
        n = min(n, steps_cap)
    t0 = time.perf_counter()
    f, _ = lat.run(f, n, with_stats=True)
    dt = time.perf_counter() - t0
    cells = kinds.size
    return {"value": round(cells * n / dt / 1e6, 3), "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"{n} collide-and-stream steps of the full 256x128x128 lattice with statistics "
                      f"({dt:.1f} s on {threads} OpenMP threads)"}


def run_reference(args):
    ws, rank, local = dist_env()
    dist = init_dist(ws)
    if rank != 0:
        barrier(dist)
        return
    budget = 60.0
    cb = cpu_baseline(seconds=budget / max(args.steps, 1) * args.steps)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "MLUPS", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "channel_sphere_256x128x128_bgk_fp64", "shape": list(SHAPE),
                       "omega": OMEGA, "drag_every": STATS_EVERY},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    barrier(dist)


# ------------------------------------------------------------------ GPU arm

def adjoint_cost(ctx, T=2000, K=100, precisions=("fp64", "fp32")):
    """Guo-forced 128x64x64 channel (periodic x, bounce-back walls),
    omega 1.6, force N(0, 1e-12) + 1e-5 x-drive (seed 1234); target velocity
    from a forward run with a second force field (seed 5678); objective
    1/2 sum |u(T) - u*|^2, checkpoint every K steps.  Reports the device time
    per time step of the forward recording and of the backward sweep
    (recomputation included) against one fused forward step; "all_states"
    repeats the sweep with the interval the library picks from free device
    memory (K = 1 keeps every state: no recomputation)."""
    from palabos_gb300 import workloads
    out = {"workload": "forced_channel_128x64x64_guo", "T": T, "K": K}
    for prec in precisions:
        tgt = workloads.forced_channel(seed=5678).lattice(prec, ctx)
        tgt.collide_and_stream(T)
        u_target = tgt.compute_velocity()
        tgt.close()
        wl = workloads.forced_channel(seed=1234)
        lat = wl.lattice(prec, ctx)
        f0 = lat.receive()
        fwd_ms = time_form(lat, 200, 10) / 200
        lat.send(f0)
        t0 = time.perf_counter()
        lat.adjoint_forward(T, K)
        rec_s = time.perf_counter() - t0
        J, gF, gO, back_ms = lat.adjoint_backward(u_target)
        out[prec] = {"forward_step_ms": round(fwd_ms, 5),
                     "record_ms_per_step": round(rec_s * 1e3 / T, 5),
                     "backward_ms_per_step": round(back_ms / T, 5),
                     "adjoint_step_over_forward_step": round(back_ms / T / fwd_ms, 3),
                     "objective": J, "grad_omega": gO, "grad_force_l2": float(np.sqrt(np.sum(gF * gF)))}
        lat.send(f0)
        used = lat.adjoint_forward(T, 0)
        J1, gF1, gO1, back1 = lat.adjoint_backward(u_target, want_force=False)
        out[prec]["all_states"] = {"K": used, "backward_ms_per_step": round(back1 / T, 5),
                                   "adjoint_step_over_forward_step": round(back1 / T / fwd_ms, 3),
                                   "grad_omega": gO1}
        lat.close()
    return out


def time_form(lat, steps, warmup):
    lat.collide_and_stream(warmup, stats=False)
    lat.ctx.synchronize()
    return lat.time_steps(steps, stats=False)


def sparse_throughput(n=256, radius=110.0, block=16, steps=200, precisions=("fp64", "fp32", "bf16"), ctx=None):
    """Flow outside a voxelized sphere in a periodic n^3 box (Guo force along
    x), blocks of block^3 cells: the blocks deep inside the sphere hold
    neither fluid nor wall and leave the lattice (computeSparseManagement).
    MLUPS over the cells of the kept blocks, against the same geometry with
    every block kept (the sphere's interior as no-dynamics cells)."""
    from palabos_gb300 import DeviceLattice3D, meshes, voxel
    from palabos_gb300 import native as N
    shape = (n, n, n)
    c = (n / 2 - 0.37, n / 2 + 0.21, n / 2 - 0.13)
    flags = voxel.voxelize(meshes.sphere(c, radius, 20000), shape, ctx=ctx)
    kinds = voxel.kinds_from_flags(flags, "outside", fluid=N.GUO)
    blocks = (n // block,) * 3
    out = {"workload": f"sphere_exterior_{n}^3_r{radius:g}_blocks{block}^3", "steps": steps}
    for prec in precisions:
        res = {}
        for sparse in (False, True):
            lat = DeviceLattice3D(n, n, n, 1.7, prec, ctx)
            lat.periodicity(1, 1, 1)
            lat.set_kinds(kinds)
            kept = n ** 3
            if sparse:
                keep = lat.select_sparse_blocks((kinds != N.NODYNAMICS).astype(np.int32), blocks)
                kept = int(keep.sum()) * block ** 3
                res["kept_blocks"] = f"{int(keep.sum())}/{keep.size}"
            lat.set_external_vector(None, np.array([1e-6, 0.0, 0.0]))
            lat.initialize_at_equilibrium(None, 1.0, (0.0, 0.0, 0.0))
            lat.collide_and_stream(10)
            ms = lat.time_steps(steps) / steps
            res["sparse_mlups_kept" if sparse else "dense_mlups"] = round(kept / (ms * 1e-3) / 1e6, 1)
            res["sparse_ms" if sparse else "dense_ms"] = round(ms, 4)
            lat.close()
        out[prec] = res
    return out


def cavity_throughput(n=64, steps=1000, precisions=("fp64", "fp32", "bf16", "fp16"), ctx=None):
    """The lid-driven cavity (bounce-back on five walls, regularized velocity lid
    u = (0.02, 0, 0), Re 100, from rest): MLUPS of `steps` steps per storage form."""
    from palabos_gb300 import workloads
    wl = workloads.cavity(n)
    out = {"workload": f"lid_driven_cavity_{n}^3_re100", "steps": steps}
    for prec in precisions:
        lat = wl.lattice(prec, ctx)
        lat.collide_and_stream(10)
        ms = lat.time_steps(steps) / steps
        out[prec] = {"mlups": round(n ** 3 / (ms * 1e-3) / 1e6, 1), "ms_per_step": round(ms, 5)}
        lat.close()
    return out


def run_gpu(args):
    ws, rank, local = dist_env()
    dist = init_dist(ws)
    from palabos_gb300 import Context
    ctx = Context(local)
    peak, peak_src = load_peaks()

    head = args.precision
    lat, kinds = build_lattice(head, ctx)
    bytes_step, counts = algorithmic_bytes(kinds, head)
    cells = counts["cells"]
    K, W = args.steps, args.warmup

    # warm-up, then the timed region: K steps, drag reduced every 100 steps
    for _ in range(W):
        lat.collide_and_stream(1, stats=False)
    ctx.synchronize()
    launches0 = ctx.launch_count()
    barrier(dist)
    with ClockSampler(local) as clk:
        ms_total = 0.0
        done = 0
        while done < K:
            chunk = min(STATS_EVERY, K - done)
            ms_total += lat.time_steps(chunk, stats=(chunk == STATS_EVERY))
            done += chunk
        ctx.synchronize()
    launches = ctx.launch_count() - launches0
    barrier(dist)
    t_max = max_over_ranks(dist, ms_total)
    value = ws * cells * K / (t_max * 1e-3) / 1e6
    drag = lat.internal_statistics()["drag"].tolist() if K >= STATS_EVERY else None

    # dominant kernel alone: average launch duration of the fused step kernel
    k_ms = time_form(lat, min(K, 400), 10) / min(K, 400)
    achieved = bytes_step / (k_ms * 1e-3) / 1e9
    traffic = load_traffic(f"stepKernel_{head}_channel_sphere")
    fp64_rate = ctx.fp64_rate() if head == "fp64" else None

    # e2e through the C ABI with host buffers: the FP64 state in pinned host
    # memory (allocated and touched before the timed region), sent at the
    # start, drag read every 100 steps, state received into the same buffer at
    # the end; then the same with an ordinary pageable array
    e2e_steps = K
    state_bytes = cells * 19 * 8   # the ABI exchanges FP64 f-bar
    nread = (e2e_steps + STATS_EVERY - 1) // STATS_EVERY

    def e2e_run(f_host):
        lat.receive(out=f_host)
        barrier(dist)
        t0 = time.perf_counter()
        lat.send(f_host)
        t_sent = time.perf_counter()
        done = 0
        while done < e2e_steps:
            chunk = min(STATS_EVERY, e2e_steps - done)
            lat.collide_and_stream(chunk, stats=True)
            lat.internal_statistics()      # drag to the host (synchronizes)
            done += chunk
        t_recv = time.perf_counter()
        lat.receive(out=f_host)
        t1 = time.perf_counter()
        e2e_s = max_over_ranks(dist, t1 - t0)
        return (round(ws * cells * e2e_steps / e2e_s / 1e6, 2), round(state_bytes / (t_sent - t0) / 1e9, 1),
                round(state_bytes / (t1 - t_recv) / 1e9, 1))

    def e2e_overlapped(f_host):
        # plbgpu_run_host: the same send, K steps with the drag every 100
        # steps and receive in one call; the send overlaps the first step and
        # the receive the last, slab by slab
        lat.receive(out=f_host)
        barrier(dist)
        t0 = time.perf_counter()
        _, recs = lat.run_host(f_host, e2e_steps, STATS_EVERY, out=f_host)
        t1 = time.perf_counter()
        assert len(recs) == nread
        return round(ws * cells * e2e_steps / max_over_ranks(dist, t1 - t0) / 1e6, 2)

    try:
        import torch
        pinned = torch.empty(SHAPE + (19,), dtype=torch.float64, pin_memory=True).numpy()
        pinned[...] = 0.0
        host_kind = "pinned"
    except Exception:   # no torch or no pinned allocation: pageable only
        pinned, host_kind = np.zeros(SHAPE + (19,)), "pageable"
    v_seq, h2d, d2h = e2e_run(pinned)
    v_e2e = e2e_overlapped(pinned)
    pageable = np.zeros(SHAPE + (19,))
    v_pg_seq, h2d_pg, d2h_pg = e2e_run(pageable)
    v_pg = e2e_overlapped(pageable)
    e2e = {"value": v_e2e, "unit": "MLUPS",
           "h2d_bytes_per_step": round(state_bytes / e2e_steps, 1),
           "d2h_bytes_per_step": round((state_bytes + 56 * nread) / e2e_steps, 1),
           "host_memory": host_kind,
           "sequential": {"value": v_seq, "h2d_gbs": h2d, "d2h_gbs": d2h},
           "pageable": {"value": v_pg, "sequential": v_pg_seq, "h2d_gbs": h2d_pg, "d2h_gbs": d2h_pg},
           "note": f"FP64 state in {host_kind} host memory, sent once and received once per run of K steps "
                   "through plbgpu_run_host (x-slabs copied over NVLink-C2C by a copy kernel on a few SMs, the send "
                   "overlapped with a ramp of the first two steps and the receive with a ramp of the last two); "
                   "drag read every 100 steps; 'sequential' = plbgpu_send, plbgpu_collide_and_stream "
                   "and plbgpu_receive called one after another; 'pageable' repeats both with an ordinary "
                   "numpy array"}
    del pinned, pageable
    lat.close()

    # the other storage forms on the same workload (kernel-only rate)
    forms = {head: {"mlups": round(cells / (k_ms * 1e-3) / 1e6, 1), "bytes_per_cell": B_CELL[head],
                    "hbm_frac": round(achieved / peak, 4)}}
    if not args.skip_forms:
        for prec in [p for p in ("fp64", "fp32", "bf16", "fp16", "bf16sr") if p != head]:
            l2, _ = build_lattice(prec, ctx)
            n = min(K, 400)
            ms = time_form(l2, n, 10) / n
            b, _ = algorithmic_bytes(kinds, prec)
            forms[prec] = {"mlups": round(cells / (ms * 1e-3) / 1e6, 1), "bytes_per_cell": B_CELL[prec],
                           "hbm_frac": round(b / (ms * 1e-3) / 1e9 / peak, 4)}
            l2.close()
        # accuracy of each storage form against FP64 on the Taylor-Green vortex (u0 0.04,
        # Re 1600) at 256^3 for 2500 steps: with u0 and Re fixed, the viscous time of the
        # 512^3 x 5000-step configuration
        from palabos_gb300.accuracy import taylor_green_study
        tg = taylor_green_study(n=256, steps=2500, every=500, slab=16, ctx=ctx)
        for prec, acc in tg["forms"].items():
            forms[prec]["taylor_green_256_2500steps"] = {k: round(v, 9) for k, v in acc.items()}
        met = sorted(p for p, a in tg["forms"].items() if a["vel_l2_rel"] <= 1e-3)
        forms["accuracy_bound"] = {"criterion": "velocity L2 <= 1e-3 relative to FP64, Taylor-Green 256^3 x 2500",
                                   "meets": met, "fails": sorted(set(tg["forms"]) - set(met))}
        # the benchmark's own quantity: the momentum-exchange drag after the full
        # 10000 steps of the channel, FP32 storage against FP64
        drag = {}
        for prec in ("fp64", "fp32"):
            l2, _ = build_lattice(prec, ctx)
            l2.collide_and_stream(9999)
            l2.collide_and_stream(1, stats=True)
            drag[prec] = l2.internal_statistics()["drag"].tolist()
            l2.close()
        ref = np.asarray(drag["fp64"])
        forms["drag_channel_10000_steps"] = {
            "fp64": drag["fp64"], "fp32": drag["fp32"],
            "fp32_rel_err": float(np.linalg.norm(np.asarray(drag["fp32"]) - ref) / np.linalg.norm(ref))}

    adjoint = None if args.skip_adjoint else adjoint_cost(ctx)

    kernel_name = (f"rowStepKernel+edgeRowStepKernel<{head}>: one fused collide+stream+faces step, AA pattern"
                   if head in ("fp64", "fp32") else
                   f"pairRowStepKernel+edgeRowStepKernel<{head}>: one fused collide+stream+faces step, AA pattern")
    hbm = {"achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
           "traffic": traffic, "traffic_source": "committed ncu capture (profiles/ncu_traffic.json), "
                                                 "scaled from the row kernel by cells; not measured in this run",
           "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)", "bytes_per_launch": bytes_step}
    if head == "fp64":
        ops_step = FP64_OPS_BGK * counts["colliding"]
        fp64_achieved = ops_step / (k_ms * 1e-3) / 1e12
        fp64_peak = fp64_rate / 1e12
        roofline = {"bound": "fp64", "achieved": round(fp64_achieved, 4), "peak": round(fp64_peak, 4),
                    "unit": "TFLOP/s", "frac": round(fp64_achieved / fp64_peak, 4), "traffic": traffic,
                    "kernel": kernel_name,
                    "ops_per_launch": ops_step,
                    "ops_per_cell": f"{FP64_OPS_BGK} FP64 adds and multiplies per colliding cell "
                                    f"({counts['colliding']} of {cells} cells collide)",
                    "peak_source": "measured in this run: plbgpu_measure_fp64_rate (independent DMUL/DADD chains, "
                                   "every SM, CUDA events)",
                    "hbm": hbm}
    else:
        roofline = {"bound": "hbm", **{k: hbm[k] for k in ("achieved", "peak", "unit", "frac", "traffic")},
                    "kernel": kernel_name, **{k: hbm[k] for k in ("traffic_source", "peak_source",
                                                                   "bytes_per_launch")}}

    if rank == 0:
        clocks = clk.summary()
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "MLUPS", "n_gpus": ws, "steps": K,
            "warmup": W, "ms_per_step": round(t_max / K, 5), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if head == "fp64" else "f32", "data": "synthetic",
            "config": {"workload": f"channel_sphere_256x128x128_bgk_{head}", "shape": list(SHAPE), "omega": OMEGA,
                       "storage": head,
                       "inlet": "regularized velocity, parabolic u_max=0.05", "outlet": "regularized pressure rho=1",
                       "obstacle": "momentum-exchange bounce-back sphere r=16 at (64,64,64)",
                       "drag_every": STATS_EVERY, "cells": cells, "faces": counts["faces"],
                       "mebb_cells": counts["mebb"], "l2": "state (637 MB) larger than L2, no flush",
                       "parallelism": f"replicas{ws}"},
            "roofline": roofline,
            "forms": forms,
            "adjoint": adjoint,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clocks,
            "drag_last": drag,
        }
        if not args.skip_cpu:
            line["cpu_baseline"] = cpu_baseline()
        print(json.dumps(line), flush=True)
    barrier(dist)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-forms", action="store_true")
    ap.add_argument("--skip-adjoint", action="store_true")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32", "bf16", "fp16", "bf16sr"])
    ap.add_argument("--accuracy", action="store_true",
                    help="run only the Taylor-Green accuracy study (512^3, 5000 steps) and print its JSON")
    ap.add_argument("--accuracy-n", type=int, default=512)
    ap.add_argument("--accuracy-steps", type=int, default=5000)
    ap.add_argument("--permeability", action="store_true",
                    help="run only the sphere-packing permeability study (384^3, 20000 steps) and print its JSON")
    ap.add_argument("--permeability-n", type=int, default=384)
    ap.add_argument("--permeability-steps", type=int, default=20000)
    ap.add_argument("--permeability-adjoint", type=int, nargs="+", default=[3000])
    ap.add_argument("--drag-gradient", action="store_true",
                    help="run only the channel-past-a-sphere drag-gradient study (256x128x128, 10000 steps)")
    ap.add_argument("--drag-gradient-steps", type=int, default=10000)
    ap.add_argument("--sparse", action="store_true",
                    help="run only the sparse-domain throughput study (voxelized sphere exterior, 256^3)")
    ap.add_argument("--cavity", action="store_true",
                    help="run only the lid-driven cavity throughput study (64^3, 1000 steps per storage form)")
    ap.add_argument("--cavity-n", type=int, default=64)
    ap.add_argument("--sparse-steps", type=int, default=200)
    ap.add_argument("--sparse-precisions", nargs="+", default=["fp64", "fp32", "bf16"],
                    choices=["fp64", "fp32", "bf16", "fp16", "bf16sr"])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.accuracy:
        from palabos_gb300 import Context
        from palabos_gb300.accuracy import taylor_green_study
        ctx = Context(dist_env()[2])
        r = taylor_green_study(n=args.accuracy_n, steps=args.accuracy_steps, every=500, slab=8, ctx=ctx)
        print(json.dumps({"study": "taylor_green_storage_forms", **r}))
        return
    if args.drag_gradient:
        from palabos_gb300 import Context
        from palabos_gb300.accuracy import drag_gradient_study
        ctx = Context(dist_env()[2])
        r = drag_gradient_study(steps=args.drag_gradient_steps, ctx=ctx)
        print(json.dumps({"study": "channel_sphere_drag_gradient", **r}))
        return
    if args.cavity:
        from palabos_gb300 import Context
        ctx = Context(dist_env()[2])
        print(json.dumps({"study": "lid_driven_cavity", **cavity_throughput(n=args.cavity_n, ctx=ctx)}))
        return
    if args.sparse:
        from palabos_gb300 import Context
        ctx = Context(dist_env()[2])
        r = sparse_throughput(steps=args.sparse_steps, precisions=tuple(args.sparse_precisions), ctx=ctx)
        print(json.dumps({"study": "sparse_sphere_exterior", **r}))
        return
    if args.permeability:
        from palabos_gb300 import Context
        from palabos_gb300.accuracy import permeability_study
        ctx = Context(dist_env()[2])
        r = permeability_study(n=args.permeability_n, steps=args.permeability_steps,
                               adjoint_iterations=tuple(args.permeability_adjoint), ctx=ctx)
        print(json.dumps({"study": "sphere_packing_permeability", **r}))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
