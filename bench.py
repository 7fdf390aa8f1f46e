#!/usr/bin/env python
"""Throughput of the explicit P1 shallow-water step on one GB300 per rank.

A bench step is one SSP-RK3 time step (COMPUTE_DT + three forward-Euler
stages with the FCT limiter, SOURCES/main.f90:61-91) over the whole mesh.
Default workload: the 4M-node wet/dry basin (jittered-lattice Delaunay mesh
of [0,10]^2, 2000x2000 points, 32 Gaussian bumps, circular dam, Manning
n = 0.03), mixed FP32/FP64 precision, compared with the plain FP64 GPU step
after the same number of steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU (torchrun): every rank advances its own replica of the workload
(the step has no data-parallel exchange for one mesh; independent meshes are
replicas), so the scaling is weak.  Rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from dataclasses import replace
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "shallow-water-eric_gb300"))
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

T_START = time.perf_counter()


def log(msg):
    print(f"[bench +{time.perf_counter() - T_START:7.1f}s] {msg}", file=sys.stderr, flush=True)


METRIC = "mesh-node RK-stage updates/s, mixed vs FP64 at matched L1 error; HBM GB/s"
UNIT = "node-stage updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=2000, help="lattice points per side of the wet/dry basin")
    ap.add_argument("--cpu-n", type=int, default=500, help="lattice size of the CPU baseline sample")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--profile-steps", type=int, default=3)
    ap.add_argument("--no-fp64", action="store_true")
    return ap.parse_args()


# ------------------------------------------------------------------ helpers
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def b_alg(n, nnz, precision, S=3):
    """Compulsory bytes of one stage: N (3 S_u + S_z + S_m + 4) + nnz (4 + 2 S_c)."""
    if precision == 1:
        su = 8 + 4 * (S - 1)
        return n * (3 * su + 4 + 8 + 4) + nnz * (4 + 2 * 4)
    return n * (3 * 8 * S + 8 + 8 + 4) + nnz * (4 + 2 * 8)


def make_case(n):
    from swe import cases as C
    return C.bump_basin_case(n=n, nsteps=200)


def cpu_baseline(n, steps, warm=1):
    """FP64 oracle (row-parallel OpenMP, every host core) on a bounded sample."""
    import oracle
    case = make_case(n)
    o = oracle.Oracle(case.mesh["jj"], case.mesh["rr"])
    o.set_params(oracle.Params(*case.params.fields()))
    o.set_bath(case.bath)
    for comp, js, vals in case.dirichlet:
        o.set_dirichlet(comp, js, vals)
    u = case.u0.copy(order="F")
    t = 0.0
    for _ in range(warm):
        t = o.rk3_step(u, t)
    t0 = time.perf_counter()
    for _ in range(steps):
        t = o.rk3_step(u, t)
    el = time.perf_counter() - t0
    N = case.mesh["rr"].shape[1]
    return N * 3 * steps / el, N, el


# ------------------------------------------------------------------ arms
def run_reference(args, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    value, N, el = cpu_baseline(args.cpu_n, args.steps, warm=args.warmup)
    sample = (f"{args.steps} SSP-RK3 steps of the {args.cpu_n}x{args.cpu_n}-point wet/dry basin ({N} nodes), "
              f"FP64 restatement (oracle), OpenMP over rows")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "wetdry_basin", "nodes": N, "precision": "fp64"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def timed_run(upd, u0, steps, warmup, dist, sampler=None):
    import torch
    upd.upload(u0)
    upd.set_time(0.0, 1e30)
    if warmup:
        upd.rk3_steps(warmup)
    upd.upload(u0)
    upd.set_time(0.0, 1e30)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    if sampler:
        sampler.start()
    t0 = time.perf_counter()
    _, dt, n = upd.rk3_steps(steps)
    wall = time.perf_counter() - t0
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    dev_ms = upd.last_device_ms
    launches = upd.last_launch_count
    if dist:
        t = torch.tensor([dev_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms = float(t.item())
        dist.barrier()
    return dict(dev_ms=dev_ms, wall_s=wall, steps=n, launches=launches, clocks=clocks, last_dt=float(dt[0]))


def run_ours(args, rank, world, dist):
    import torch
    from swe.update import from_case

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    case = make_case(args.n)
    N = case.mesh["rr"].shape[1]
    log(f"mesh ready: {N} nodes")
    upd = from_case(case, precision=1)
    log("mixed context ready")
    nnz = upd.sizes()[1]
    lump = upd.lumped
    u0 = case.u0
    mass0 = float(np.sum(lump * u0[0]))
    sampler = ClockSampler(dev)
    r = timed_run(upd, u0, args.steps, args.warmup, dist, sampler)
    log(f"mixed timed run: {r['dev_ms']:.1f} ms for {r['steps']} steps")
    u_mix = upd.download()
    mass_mix = float(upd.total_mass()[0])
    value = world * N * 3 * r["steps"] / (r["dev_ms"] / 1e3)
    prof = upd.profile_kernels(args.profile_steps)
    stage_ms = prof["node"] + prof["low"] + prof["fct"] + prof["update"]
    step_kernel_ms = prof["dt"] + 3 * stage_ms
    peak, peak_kind = peaks()
    balg = b_alg(N, nnz, 1)
    achieved = balg / (stage_ms / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "traffic_per_node_stage.json"
    if tf.exists():
        d = json.loads(tf.read_text())
        if "mixed_bytes_per_node_stage" in d:
            traffic = d["mixed_bytes_per_node_stage"] * N

    # e2e through the C ABI with pinned host buffers: per step, H2D of the
    # state, one time step, D2H of the new state
    S = u0.shape[0]
    hin = torch.empty(S * N, dtype=torch.float64, pin_memory=True)
    hout = torch.empty(S * N, dtype=torch.float64, pin_memory=True)
    hin.copy_(torch.from_numpy(np.ascontiguousarray(u0.ravel(order="F"))))
    upd.set_time(0.0, 1e30)
    upd.upload_ptr(hin.data_ptr())
    upd.rk3_steps(1)
    upd.download_ptr(hout.data_ptr())
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        upd.upload_ptr(hin.data_ptr())
        upd.rk3_steps(1)
        upd.download_ptr(hout.data_ptr())
        hin, hout = hout, hin
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * N * 3 * args.e2e_steps / e2e_s
    upd.close()

    log(f"e2e done: {e2e_s:.2f} s")
    fp64 = None
    if not args.no_fp64:
        u64 = from_case(case, precision=0)
        r64 = timed_run(u64, u0, args.steps, min(args.warmup, 3), dist)
        u_ref = u64.download()
        prof64 = u64.profile_kernels(1)
        stage64 = prof64["node"] + prof64["low"] + prof64["fct"] + prof64["update"]
        v64 = world * N * 3 * r64["steps"] / (r64["dev_ms"] / 1e3)
        w = lump
        l1 = float(np.sum(w * np.abs(u_mix[0] - u_ref[0])) / np.sum(w * np.abs(u_ref[0])))
        fp64 = {"value": v64, "ms_per_step": r64["dev_ms"] / r64["steps"], "steps": r64["steps"],
                "stage_kernels_ms": {k: round(v, 4) for k, v in prof64.items()},
                "roofline_frac": b_alg(N, nnz, 0) / (stage64 / 1e3) / 1e9 / peak,
                "l1_rel_h_mixed_vs_fp64": l1,
                "max_abs_h_mixed_vs_fp64": float(np.max(np.abs(u_mix[0] - u_ref[0])))}
        u64.close()
        log(f"fp64 timed run: {r64['dev_ms']:.1f} ms")

    if rank != 0:
        return
    cpu = None
    if world == 1:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        cv, cN, cel = cpu_baseline(args.cpu_n, args.cpu_steps)
        cpu = {"value": cv, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": "port",
               "sample": f"{args.cpu_steps} SSP-RK3 steps of the {args.cpu_n}x{args.cpu_n}-point wet/dry basin "
                         f"({cN} nodes, {cel:.1f} s), FP64 restatement, OpenMP over rows"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["dev_ms"] / r["steps"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded jittered-lattice Delaunay mesh, Gaussian-bump bathymetry)",
        "config": {"workload": "wetdry_basin_4M" if args.n == 2000 else f"wetdry_basin_{args.n}x{args.n}",
                   "nodes": N, "nnz": nnz, "precision": "mixed (FP32 bulk, FP64 h/limiter)",
                   "steps_timed": r["steps"], "replicas": world,
                   "l2": "working set larger than L2 (no flush)", "manning_n": 0.03, "cfl": 0.25},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "unit_of_work": "one RK stage (k_node+k_low+k_fct+k_update), algorithmic bytes "
                                     f"{balg / N:.1f} B/node"},
        "stage_kernels_ms": {k: round(v, 4) for k, v in prof.items()},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": S * N * 8, "d2h_bytes_per_step": S * N * 8},
        "cpu_baseline": cpu,
        "clocks": r["clocks"],
        "gpu_launches": r["launches"],
        "fp64": fp64,
        "speedup_mixed_vs_fp64": (value / fp64["value"]) if fp64 else None,
        "mass_rel_drift_mixed": (mass_mix - mass0) / mass0,
        "min_h_mixed": float(u_mix[0].min()),
        "kernel_time_share_of_step": step_kernel_ms / (r["dev_ms"] / r["steps"]),
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if args.impl == "reference":
        return run_reference(args, rank)
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    try:
        run_ours(args, rank, world, dist)
    finally:
        if dist:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
