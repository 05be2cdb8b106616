#!/usr/bin/env python
"""Throughput benchmark of the GB300 time-advance path (prints one JSON line).

Workload: the supersonic isothermal-wall channel 192 x 128 x 160 (reference axes: mx = 128
wall-normal, my = 160 spanwise, mz = 192 streamwise; stretched walls, constant-mass-flux
body force), 8th-order stencils (S = V = 4), Wray low-storage RK3, plain FP64.
A "step" is one RK3 time step of the whole grid (3 stages); the metric is
Mpoint-steps/s = grid points x steps / second, summed over ranks (replicas only: the
path is not sharded across GPUs, each rank advances its own channel).

  value       device-resident state, CUDA events on the solver's stream around K steps
  e2e         the same through the C ABI with pinned host buffers: copy the five fields
              in, advance K steps, copy them out (host wall clock)
  roofline    the RHS + stage-update kernel (dominant kernel): its event-timed average
              launch against the FP64 pipe (measured live) and against HBM
  cpu_baseline  the CPU oracle (the reference's algorithm restated, OpenMP) on the host
              cores, on the same full channel (whole RK3 steps for ~12 s)
  fp32_rhs    the same workload with the RHS in FP32 (state/accumulation FP64)
  pair_rhs    the same workload with the RHS in FP32-pair (~48-bit) arithmetic, and its
              largest state difference from the FP64 run after the same steps
  batched     48 Taylor-Green boxes of uneven size (seeded), FP32 RHS / FP64 state, in the
              execution mode the autotuner picks (one persistent launch per RK stage for the
              whole ensemble, or every member's step graph on concurrent streams), graph
              replay; the other mode is timed beside it
  serving     Poisson-arrival "advance N steps" requests (Taylor-Green 32^3-192^3 and
              64x48x64 channels, N in [50, 500]) under a 150 GB budget: p50/p99 latency and
              aggregate Mpoint-steps/s per arrival rate, 100 requests per rate, rates swept
              from light load to past the batch's capacity

--impl reference times the CPU port of the reference's path (the reference itself only
has a GPU path) on all host cores, on the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

METRIC = "Mpoint-steps/s"
PEAKS_FILE = os.path.join(REPO, "MEASURED_PEAKS.json")
TRAFFIC_FILE = os.path.join(REPO, "profiles", "rhs_kernel_channel_traffic.txt")
TRAFFIC_FILE_FP32 = os.path.join(REPO, "profiles", "rhs_kernel_channel_fp32_traffic.txt")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["channel", "tgv", "precision", "batch"], default="channel")
    ap.add_argument("--batch-members", type=int, default=48,
                    help="batch workload: the first N members of the 48-member ensemble")
    ap.add_argument("--batch-mode", choices=["tuned", "persistent", "concurrent"], default="tuned",
                    help="batch workload: execution mode (tuned: the autotuner's pick)")
    ap.add_argument("--t-end", type=float, default=10.0, help="precision study: end time")
    ap.add_argument("--precision", choices=["fp64", "fp32", "pair"], default="fp64")
    ap.add_argument("--no-extras", action="store_true", help="skip fp32/cpu/e2e side measurements")
    ap.add_argument("--grid", default=None, help="override the grid as MX,MY,MZ (profiling of smaller cases)")
    ap.add_argument("--serve-requests", type=int, default=100, help="requests per arrival rate in the serving leg")
    ap.add_argument("--serve-rates", default="2,4,8,16", help="arrival rates (requests/s) of the serving leg")
    return ap.parse_args()


def workload(name: str, precision: str, grid=None):
    from cudanavierstokes_gb300.params import PREC_FP32_RHS, PREC_FP64, PREC_PAIR_RHS, channel_params, tgv_params
    prec = {"fp32": PREC_FP32_RHS, "pair": PREC_PAIR_RHS}.get(precision, PREC_FP64)
    if grid:
        mx, my, mz = (int(v) for v in grid.split(","))
        base = channel_params(mx, my, mz, precision=prec) if name == "channel" else tgv_params(mx, precision=prec)
        base = base.copy(my=my, mz=mz)
        return base, f"{name} {mx}x{my}x{mz} (reference axes), 8th order S=V=4, Wray RK3"
    if name == "channel":
        p = channel_params(128, 160, 192, precision=prec)
        desc = ("supersonic isothermal-wall channel 192x128x160 (reference axes mx=128 wall-normal, my=160 span, "
                "mz=192 stream), Ma 1.5, Re 3000, 8th order S=V=4, Wray RK3")
    else:
        p = tgv_params(64, precision=prec)
        desc = "Taylor-Green vortex 64^3, Ma 0.1, Re 1600, 8th order S=V=4, Wray RK3"
    return p, desc


def initial_state(p, x=None):
    from cudanavierstokes_gb300.initial import channel_fields, tgv_fields
    if p.periodic_x:
        return tgv_fields(p)
    return channel_fields(p, x, seed=0)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.remove(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        loaded = [v for v in sm if mx and v >= 0.5 * max(mx)] or sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max((num(r[3]) or 0) for r in rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def allreduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else torch.device("cpu")
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_sample(p, steps_min: int = 2, seconds: float = 12.0):
    """Time the CPU oracle on the full workload grid on all host cores, whole RK3 steps until
    `seconds` have passed: returns Mpoint-steps/s, threads, text."""
    from oracle import oracle as orc
    q = p.copy(precision=0)
    orc.set_threads(os.cpu_count() or 1)
    o = orc.Oracle(q)
    o.set_state(*initial_state(q, o.grid()["x"]))
    o.run(1)                       # warm-up step
    n, t0 = 0, time.perf_counter()
    while n < steps_min or time.perf_counter() - t0 < seconds:
        o.run(1)
        n += 1
    dt = time.perf_counter() - t0
    pts = q.npoints
    return pts * n / dt / 1e6, orc.max_threads(), (f"{n} RK3 steps of the full {q.mx}x{q.my}x{q.mz} workload grid "
                                                    f"({pts} points, FP64, same physics and stencils), {dt:.1f} s")


def run_batched(args, stream_ptr, members=48, mode_req="tuned", with_other=True):
    """The batched ensemble of 48 Taylor-Green boxes of uneven size (or its first `members`) in FP32-RHS mode,
    in the execution mode and launch shape the autotuner picks (or the mode requested, at
    full residency); the other mode is timed beside it for the record."""
    import torch
    from cudanavierstokes_gb300.batch import Batch
    from cudanavierstokes_gb300.workloads import ensemble, ensemble_fields
    mem = ensemble(48, seed=0)[:members]
    bt = Batch(precision=1)
    bt.set_stream(stream_ptr)
    total_steps = 2 * args.warmup + 2 * args.steps + 128
    for p, ph in mem:
        bt.add(p, ensemble_fields(p, ph), max_steps=total_steps)
    tuned_ms = None
    if mode_req == "tuned":
        tuned_ms = bt.tune(2)
    else:
        bt.set_mode(0 if mode_req == "persistent" else 1)
        bt.set_shape(128, 32)   # full residency: clamped to the kernel's co-residency limit
    stream = torch.cuda.ExternalStream(stream_ptr)

    def timed():
        bt.step(args.warmup)
        info0 = bt.info()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        bt.step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), bt.info()["launches"] - info0["launches"]

    mode, shape = bt.mode(), bt.shape()
    ms, launches = timed()
    pts = bt.info()["points"]
    names = {0: "persistent (one cooperative launch per RK stage for all members)",
             1: "concurrent (members' step graphs on 16 streams)"}
    out = {"value": pts * args.steps / (ms * 1e-3) / 1e6, "unit": "Mpoint-steps/s", "members": bt.info()["count"],
           "points": pts, "ms_per_step": ms / args.steps, "mode": names[mode],
           "launch_shape": {"threads": shape[0], "blocks_per_sm": shape[1]} if mode == 0 else None,
           "tune_ms_per_step": tuned_ms, "kernel_launches_timed": launches,
           "workload": "48 Taylor-Green boxes, edge in {32,48,64,96,128}, Re log-U[400,3200], Ma U[0.1,0.8], "
                       "seeded phases (seed 0), 8th order, Wray RK3, FP32 RHS / FP64 state"}
    if not with_other:
        bt.close()
        return out
    # the other execution mode on the same members
    other = 1 - mode
    bt.set_mode(other)
    if other == 0:
        bt.set_shape(128, 32)   # full residency: clamped to the kernel's co-residency limit
    oms, _ = timed()
    out["other_mode"] = {"mode": names[other], "value": pts * args.steps / (oms * 1e-3) / 1e6,
                         "ms_per_step": oms / args.steps}
    if mode == 1:
        out["why_mode"] = ("the persistent kernel runs the standalone point bodies over all members with the "
                           "members' parameters from a kernel-argument table (uniform per member loop), but "
                           "with compile-time stencil weights scaled by each member's spacings (+7 % on the RHS) "
                           "and a grid barrier after each phase; the concurrent mode's standalone kernels keep "
                           "premultiplied weights as constant-bank operands (profiles/batch_stage_persistent_fp32.md)")
    if other == 0:
        out["other_mode"]["launch_shape"] = {"threads": 128, "blocks_per_sm": bt.shape()[1]}
    bt.close()
    return out


def run_serving(args):
    """The serving workload: Poisson arrivals of advance-N-steps requests, continuous batching.
    The requests' initial fields are generated once per (kind, grid) before the clock starts
    and shared by the requests of that grid (the work of a request does not depend on its
    field values: N steps of its grid)."""
    import threading
    from cudanavierstokes_gb300.server import Server
    from cudanavierstokes_gb300.workloads import request_fields, serving_requests
    rates = [float(r) for r in args.serve_rates.split(",") if r]
    res = []
    pool = {}
    for rate in rates:
        reqs = serving_requests(args.serve_requests, rate, seed=1)
        fields = []
        for (_, p, kind, _, sd) in reqs:
            key = (kind, p.mx, p.my, p.mz)
            if key not in pool:
                pool[key] = [np.ascontiguousarray(a) for a in request_fields(p, kind, sd)]
            fields.append(pool[key])
        srv = Server(precision=1, hbm_budget_bytes=150 * 10**9)
        ids = []
        t0 = time.perf_counter()

        def submit():
            for (ta, p, kind, n, sd), f in zip(reqs, fields):
                dt = ta - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                ids.append(srv.submit(p, f, n))
        th = threading.Thread(target=submit)
        th.start()
        th.join()
        for i in list(ids):
            srv.wait(i, timeout_s=900, fetch=False)
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        offered = sum(p.npoints * n for (_, p, _, n, _) in reqs) / reqs[-1][0] / 1e6
        res.append({"rate_per_s": rate, "requests": len(reqs), "p50_s": st["p50_s"], "p99_s": st["p99_s"],
                    "max_s": st["max_s"], "value": st["point_steps"] / wall / 1e6, "unit": "Mpoint-steps/s",
                    "offered": offered, "busy_value": st["point_steps"] / max(st["busy_seconds"], 1e-9) / 1e6,
                    "batch_steps": st["batch_steps"], "wall_s": wall})
    return {"rates": res, "workload": "Poisson arrivals, N ~ U[50,500] steps, Taylor-Green 32^3-192^3 (Re, Ma as "
                                      "the ensemble) and 64x48x64 channels (25 %), FP32 RHS, 150 GB HBM budget; "
                                      "'offered' = the requests' point-steps / their arrival span"}


def ke_series(p, fields, t_end, chunk=250):
    """Run to t_end logging, every step, the state's time and <u.u>, <rho|u|^2>/2 (the
    bulk diagnostic is evaluated on the state at the start of each step); near t_end single
    steps, with the device's viscous dissipation <tau_ij du_i/dx_j> of the states on either
    side of t_end, interpolated linearly to t_end."""
    from cudanavierstokes_gb300 import Solver
    s = Solver(p.copy(check_bulk=1))
    s.copy_field_in(*fields)
    t_prev, ts, k1, k2 = 0.0, [], [], []
    dt = None
    t0 = time.perf_counter()
    diss = []
    while t_prev < t_end:
        # chunks that stay short of t_end (dt drifts slowly), then single steps across it
        n = chunk if dt is None else min(chunk, int(0.98 * (t_end - t_prev) / dt) - 1)
        single = n < 2
        if single:
            diss.append((t_prev, s.dissipation()["eps"]))
        lg = s.run(1 if single else n)
        tt = np.concatenate([[t_prev], lg["time"][:-1]])
        ts.append(tt); k1.append(lg["par1"]); k2.append(lg["par2"])
        dt = float(lg["time"][-1] - tt[-1])
        t_prev = float(lg["time"][-1])
    diss.append((t_prev, s.dissipation()["eps"]))
    lg = s.run(3)   # samples beyond t_end for the cubic through the 4 around it
    ts.append(np.concatenate([[t_prev], lg["time"][:-1]])); k1.append(lg["par1"]); k2.append(lg["par2"])
    wall = time.perf_counter() - t0
    (ta, ea), (tb, eb) = diss[-2], diss[-1]
    eps_end = ea + (eb - ea) * (t_end - ta) / (tb - ta)
    out = dict(t=np.concatenate(ts), ke=np.concatenate(k1), ke_rho=np.concatenate(k2), wall=wall,
               steps=int(sum(len(a) for a in ts)), eps_viscous=eps_end)
    s.close()
    return out


def at_time(t, y, t0):
    """Value and derivative at t0 of the cubic through the 4 samples around t0."""
    i = int(np.searchsorted(t, t0))
    sl = slice(max(i - 2, 0), max(i - 2, 0) + 4)
    c = np.polyfit(t[sl] - t0, y[sl], 3)
    return float(c[-1]), float(c[-2])


def run_precision(args):
    """The precision study: Taylor-Green to t_end, FP32 RHS (or, with --precision pair, the
    FP32-pair RHS; FP64 state, accumulation, T/p recovery, reductions in both) against
    all-FP64; relative error of <u.u>, <rho|u|^2>/2, of the dissipation rate eps = -dK/dt at
    t_end (K = <rho|u|^2>/2) and of the viscous dissipation <tau_ij du_i/dx_j> at t_end
    (cns_dissipation)."""
    from cudanavierstokes_gb300.initial import tgv_fields
    from cudanavierstokes_gb300.params import PREC_FP32_RHS, PREC_PAIR_RHS, tgv_params
    n = int(args.grid.split(",")[0]) if args.grid else 128
    mode, prec, dtype = (("pair_rhs", PREC_PAIR_RHS, "f32x2-rhs/f64-state vs f64") if args.precision == "pair"
                         else ("fp32_rhs", PREC_FP32_RHS, "f32-rhs/f64-state vs f64"))
    p64 = tgv_params(n)
    f = tgv_fields(p64)
    r64 = ke_series(p64, f, args.t_end)
    r32 = ke_series(p64.copy(precision=prec), f, args.t_end)
    res = {"eps_viscous": {"fp64": r64["eps_viscous"], mode: r32["eps_viscous"],
                           "rel_err": abs(r32["eps_viscous"] - r64["eps_viscous"]) / abs(r64["eps_viscous"])}}
    for key in ("ke", "ke_rho"):
        a, da = at_time(r64["t"], r64[key], args.t_end)
        b, db = at_time(r32["t"], r32[key], args.t_end)
        res[key] = {"fp64": a, mode: b, "rel_err": abs(b - a) / abs(a),
                    "eps_fp64": -da, "eps_" + mode: -db, "eps_rel_err": abs(db - da) / abs(da)}
    what = "FP32-pair RHS" if prec == PREC_PAIR_RHS else "FP32 RHS"
    line = {"metric": f"kinetic-energy relative error at t_end, {what} vs FP64", "value": res["ke_rho"]["rel_err"],
            "unit": "relative", "higher_is_better": False, "dtype": dtype,
            "data": "synthetic", "config": {"workload": f"Taylor-Green {n}^3, Ma 0.1, Re 1600, Pr 0.71, S=V=4, "
                                                        "Wray RK3, CFL 0.5", "t_end": args.t_end},
            "ke_uu": res["ke"], "ke_rho": res["ke_rho"], "eps_viscous": res["eps_viscous"],
            "fp64": {"steps": r64["steps"], "wall_s": r64["wall"],
                     "Mpoint_steps_per_s": p64.npoints * r64["steps"] / r64["wall"] / 1e6},
            mode: {"steps": r32["steps"], "wall_s": r32["wall"],
                   "Mpoint_steps_per_s": p64.npoints * r32["steps"] / r32["wall"] / 1e6}}
    print(json.dumps(line), flush=True)


def read_profile_summary(path=TRAFFIC_FILE):
    """Key: value lines of a committed ncu summary of the RHS kernel (FP64 channel by default)."""
    try:
        with open(path) as f:
            return {k.strip(): v.strip() for k, v in (line.split(":", 1) for line in f if ":" in line)}
    except Exception:
        return {}


def read_traffic(N: int, fp32: bool = False):
    """Per-launch DRAM bytes of the RHS kernel from the committed ncu summary of its precision
    (scaled to this grid by points if the capture was taken on a smaller case)."""
    kv = read_profile_summary(TRAFFIC_FILE_FP32 if fp32 else TRAFFIC_FILE)
    try:
        return float(kv["dram_bytes_per_launch"]) * N / float(kv["points"])
    except Exception:
        return None


def run_reference(args, world, rank):
    """CPU port of the reference path (the oracle) on all host cores, rank 0 only, on the
    full workload grid: W untimed steps, then K timed steps."""
    if rank != 0:
        return
    from oracle import oracle as orc
    p, desc = workload(args.workload, "fp64", args.grid)
    orc.set_threads(os.cpu_count() or 1)
    o = orc.Oracle(p)
    o.set_state(*initial_state(p, o.grid()["x"]))
    for _ in range(args.warmup):
        o.run(1)
    t0 = time.perf_counter()
    o.run(args.steps)
    dt = time.perf_counter() - t0
    v = p.npoints * args.steps / dt / 1e6
    cores = orc.max_threads()
    sample = (f"{args.steps} RK3 steps of the full {p.mx}x{p.my}x{p.mz} workload grid ({p.npoints} points, FP64) "
              f"per timed region, CPU restatement of the reference kernels (OpenMP, {cores} threads)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mpoint-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": desc, "grid": [p.mx, p.my, p.mz], "points": p.npoints, "precision": "fp64",
                       "parallelism": "replicas x1"},
            "cpu_baseline": {"value": v, "unit": "Mpoint-steps/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "Mpoint-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def hbm_peak_gbs():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json, of measured)"
    except Exception:
        return 6800.0, "fallback (of fallback)"


def fp32_roofline(N, S, V, ph, fp32_peak):
    """Roofline object of the FP32-RHS RHS + stage kernel: algorithmic bytes (FP64 state and
    FP32 RK register in and out, 160 B/point) against the measured HBM bandwidth, with the
    FP32 algorithmic flops against the live FP32 FMA peak and the ncu DRAM traffic beside."""
    from cudanavierstokes_gb300 import roofline as rf
    rhs_s = ph["rhs_ms"] * 1e-3
    hbm_peak, hbm_src = hbm_peak_gbs()
    ach = rf.RHS_KERNEL_BYTES * N / rhs_s / 1e9
    tf = rf.fused_rhs_kernel_flops(S, V) * N / rhs_s / 1e12
    kv = read_profile_summary(TRAFFIC_FILE_FP32)
    out = {"bound": "hbm", "kernel": "k_rhs<float> (FP32 RHS x/y/z + body force + sponge + FP64 RK stage update + "
           "next-stage state recovery)", "achieved": ach, "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak,
           "peak_source": hbm_src, "traffic": read_traffic(N, fp32=True), "launch_ms": ph["rhs_ms"],
           "bytes_per_point": rf.RHS_KERNEL_BYTES, "flops_per_point": rf.fused_rhs_kernel_flops(S, V),
           "fp32": {"achieved": tf, "peak": fp32_peak, "unit": "TFLOP/s", "frac": tf / fp32_peak,
                    "peak_source": "measured live (FMA-chain probe, cns_probe_fma_peak)"},
           "phase_ms": ph}
    executed = {k: float(v) for k, v in kv.items() if k.endswith(("_per_point", "_pct"))}
    if executed:
        out["executed"] = dict(executed, source="ncu --set full, profiles/rhs_kernel_channel_fp32.md")
    return out


def run_gb300(args, world, rank, local):
    import numpy as np
    import torch

    from cudanavierstokes_gb300 import Solver, native
    from cudanavierstokes_gb300 import roofline as rf

    torch.cuda.set_device(local)
    p, desc = workload(args.workload, args.precision, args.grid)
    N = p.npoints
    s = Solver(p, device=local)
    stream = torch.cuda.Stream(device=local)
    s.set_stream(stream.cuda_stream)
    fields = initial_state(p, s.grid()["x"])
    s.copy_field_in(*fields)
    s.run(args.warmup, logs=False)

    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    l0 = s.kernel_launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.run(args.steps, logs=False)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    launches = s.kernel_launches - l0
    ms = allreduce_max(e0.elapsed_time(e1), world)
    value = world * N * args.steps / (ms * 1e-3) / 1e6

    # dominant kernel (RHS + stage update), event-timed per launch on the solver's stream
    ph = s.time_phases(6)
    S, V = p.stencil_size, p.stencil_visc
    rhs_s = ph["rhs_ms"] * 1e-3
    ach_tf = rf.fused_rhs_kernel_flops(S, V) * N / rhs_s / 1e12
    ach_gbs = rf.RHS_KERNEL_BYTES * N / rhs_s / 1e9
    t64 = native.ctypes.c_double()
    fp64_peak = args.precision in ("fp64", "pair")
    native.check(native.lib().cns_probe_fma_peak(local, 1 if fp64_peak else 0, 2000 if fp64_peak else 20000,
                                                 native.ctypes.byref(t64)))
    hbm_peak, hbm_src = hbm_peak_gbs()
    traffic = read_traffic(N, fp32=args.precision == "fp32")
    roof = {"bound": "fp64" if args.precision == "fp64" else "fp32", "kernel": "k_rhs (RHS x/y/z + body force + "
            "sponge + RK stage update)", "achieved": ach_tf, "peak": t64.value, "unit": "TFLOP/s",
            "frac": ach_tf / t64.value, "peak_source": "measured live (FMA-chain probe, cns_probe_fma_peak)",
            "traffic": traffic, "launch_ms": ph["rhs_ms"],
            "flops_per_point": rf.fused_rhs_kernel_flops(S, V), "bytes_per_point": rf.RHS_KERNEL_BYTES,
            "hbm": {"achieved": ach_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": ach_gbs / hbm_peak,
                    "peak_source": hbm_src},
            "phase_ms": ph}
    kv = read_profile_summary()
    if args.precision == "fp32":
        roof = fp32_roofline(N, S, V, ph, t64.value)
    if args.precision == "pair":
        # FP64-equivalent rate of the reference's operation count against the FP64 pipe: the
        # pair arithmetic runs on the FP32 pipe, so frac > 1 is past what FP64 can reach
        roof["bound"] = "fp32 issue (pair arithmetic)"
        roof["peak_source"] = "the FP64 pipe peak, measured live (FMA-chain probe): FP64-equivalent comparison"
        roof["traffic"] = None
    if args.precision == "fp64" and "fp64_inst_per_point" in kv:
        # the algorithmic count above is the reference's operation structure; the kernel
        # executes fewer FP64 instructions (shared flux products, lambda/mu), so the
        # algorithmic rate can exceed the pipe peak; the pipe utilisation is measured by ncu
        roof["executed"] = {"fp64_inst_per_point": float(kv["fp64_inst_per_point"]),
                            "fp64_pipe_active": float(kv["fp64_pipe_active_pct"]) / 100.0,
                            "source": "ncu --set full, profiles/rhs_kernel_channel_fp64.md"}

    line = {"metric": METRIC, "value": value, "unit": "Mpoint-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": {"fp64": "f64", "fp32": "f32-rhs/f64-state", "pair": "f32x2-rhs/f64-state"}[args.precision],
            "data": "synthetic",
            "config": {"workload": desc, "grid": [p.mx, p.my, p.mz], "points": N,
                       "precision": args.precision, "parallelism": f"replicas x{world}",
                       "l2": "no flush: the working set (~1.3 GB of fields) is 10x the 129 MB L2"},
            "gpu_launches": launches, "clocks": clk, "roofline": roof}

    if not args.no_extras and rank == 0:
        # end to end through the C ABI with pinned host buffers
        pinned = [torch.empty(p.shape, dtype=torch.float64, pin_memory=True).numpy() for _ in range(5)]
        outs = [torch.empty(p.shape, dtype=torch.float64, pin_memory=True).numpy() for _ in range(5)]
        for a, f in zip(pinned, fields):
            a[...] = f
        s.copy_field_in(*pinned)
        s.run(1, logs=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.copy_field_in(*pinned)
        s.run(args.steps, logs=False)
        s.copy_field_out(outs)
        t_e2e = time.perf_counter() - t0
        line["e2e"] = {"value": N * args.steps / t_e2e / 1e6, "unit": "Mpoint-steps/s",
                       "h2d_bytes_per_step": 5 * 8 * N / args.steps, "d2h_bytes_per_step": 5 * 8 * N / args.steps,
                       "what": f"cns_copy_field(0) of 5 pinned host fields + cns_run({args.steps}) + "
                               "cns_copy_field(1), host wall clock"}
        if not all(np.isfinite(o).all() for o in outs):
            line["e2e"]["error"] = "non-finite state"
        s.close()
        # FP32-RHS variant of the same workload
        if args.precision == "fp64":
            p32, _ = workload(args.workload, "fp32", args.grid)
            s32 = Solver(p32, device=local)
            s32.set_stream(stream.cuda_stream)
            s32.copy_field_in(*fields)
            s32.run(args.warmup, logs=False)
            torch.cuda.synchronize()
            e0.record(stream)
            s32.run(args.steps, logs=False)
            e1.record(stream)
            torch.cuda.synchronize()
            ms32 = e0.elapsed_time(e1)
            ph32 = s32.time_phases(6)
            t32 = native.ctypes.c_double()
            native.check(native.lib().cns_probe_fma_peak(local, 0, 20000, native.ctypes.byref(t32)))
            line["fp32_rhs"] = {"value": N * args.steps / (ms32 * 1e-3) / 1e6, "unit": "Mpoint-steps/s",
                                "ms_per_step": ms32 / args.steps, "phase_ms": ph32,
                                "speedup_vs_fp64": (ms / ms32),
                                "roofline": fp32_roofline(N, S, V, ph32, t32.value)}
            s32.close()
            # FP32-pair RHS variant: its rate, and its largest state difference from an FP64
            # run of the same steps from the same start (both fresh solvers)
            pp, _ = workload(args.workload, "pair", args.grid)
            states = []
            for q in (p, pp):
                sq = Solver(q, device=local)
                sq.set_stream(stream.cuda_stream)
                sq.copy_field_in(*fields)
                sq.run(args.steps, logs=False)
                states.append(sq.copy_field_out())
                sq.close()
            diff = max(float(np.abs(a - b).max() / np.abs(b).max()) for a, b in zip(states[1], states[0]))
            sp = Solver(pp, device=local)
            sp.set_stream(stream.cuda_stream)
            sp.copy_field_in(*fields)
            sp.run(args.warmup, logs=False)
            torch.cuda.synchronize()
            e0.record(stream)
            sp.run(args.steps, logs=False)
            e1.record(stream)
            torch.cuda.synchronize()
            msp = e0.elapsed_time(e1)
            line["pair_rhs"] = {"value": N * args.steps / (msp * 1e-3) / 1e6, "unit": "Mpoint-steps/s",
                                "ms_per_step": msp / args.steps, "phase_ms": sp.time_phases(6),
                                "speedup_vs_fp64": ms / msp,
                                "max_rel_state_diff_vs_fp64": diff,
                                "diff_after_steps": args.steps}
            sp.close()
        # batched ensemble and serving (FP32 RHS / FP64 state)
        line["batched"] = run_batched(args, stream.cuda_stream)
        line["batched"]["vs_plain_fp64"] = line["batched"]["value"] / value
        line["serving"] = run_serving(args)
        # CPU baseline (oracle) on the host cores
        v, cores, sample = cpu_sample(p)
        line["cpu_baseline"] = {"value": v, "unit": "Mpoint-steps/s", "cores": cores, "kind": "port",
                                "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_batch_only(args):
    """The batched ensemble alone (for profiling the batch kernels): one JSON line."""
    import torch
    from cudanavierstokes_gb300.batch import Batch  # noqa: F401  (loads the library)
    torch.cuda.init()
    stream = torch.cuda.Stream()
    res = run_batched(args, stream.cuda_stream, members=args.batch_members, mode_req=args.batch_mode,
                      with_other=False)
    print(json.dumps({"metric": "Mpoint-steps/s", "value": res["value"], "unit": "Mpoint-steps/s", "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
                      "higher_is_better": True, "dtype": "f32-rhs/f64-state", "data": "synthetic",
                      "config": {"workload": res["workload"], "members": res["members"], "points": res["points"],
                                 "mode": res["mode"], "launch_shape": res["launch_shape"]}}))


def main():
    args = parse_args()
    world, rank, local = dist_setup()
    if args.workload == "precision":
        if rank == 0:
            run_precision(args)
    elif args.workload == "batch":
        if rank == 0:
            run_batch_only(args)
    elif args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gb300(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
