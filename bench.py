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
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=2000, help="lattice points per side of the wet/dry basin")
    ap.add_argument("--parity-steps", type=int, default=15,
                    help="steps of the oracle leg on the same mesh (CPU baseline and full-size parity); 0 skips it")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--profile-steps", type=int, default=3)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--workload", choices=["wetdry", "thacker", "batch", "dam", "sgn"], default="wetdry",
                    help="wetdry (default line) or one of the other workloads, printed as extra JSON lines")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--batch-subset", type=int, default=64,
                    help="instances of the batched ensemble (the first ones of its seed) in the default line; 0 skips")
    ap.add_argument("--sgn-nx", type=int, default=10001)
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


def design_bytes(n, nnz):
    """Bytes per node that each mixed stage kernel reads and writes once per
    launch in the four-sweep design (3-component systems), with e the
    off-diagonal entries per row (16-bit position, c_ij or (d, mu), |c|lambda
    per entry): k_dt 25 + 14e; k_low 65 + 18e, plus 4e in stage 1 (it reads
    k_dt's |c|lambda); k_fct 37 + 10e; k_update 78 + 10e, plus 24 in stages 2
    and 3 (u0); k_node 21 + 4e in stages 2 and 3.  Averaged per stage like
    swe_profile_kernels' times."""
    e = (nnz - n) / n
    return {"dt": 25 + 14 * e, "node": (21 + 4 * e) * 2 / 3, "low": 65 + 18 * e + 4 * e / 3,
            "fct": 37 + 10 * e, "update": 78 + 10 * e + 16}


def make_case(n):
    from swe import cases as C
    return C.bump_basin_case(n=n, nsteps=200)


def oracle_for(case):
    import oracle
    o = oracle.Oracle(case.mesh["jj"], case.mesh["rr"])
    o.set_params(oracle.Params(*case.params.fields()))
    o.set_bath(case.bath)
    for comp, js, vals in case.dirichlet:
        o.set_dirichlet(comp, js, vals)
    return o


def oracle_steps(case, steps, warm=0):
    """The FP64 oracle (row-parallel OpenMP over every host core) advancing
    the workload's own initial state: returns (state, node-stage/s, s)."""
    o = oracle_for(case)
    u = case.u0.copy(order="F")
    t = 0.0
    for _ in range(warm):
        t = o.rk3_step(u, t)
    t0 = time.perf_counter()
    for _ in range(steps):
        t = o.rk3_step(u, t)
    el = time.perf_counter() - t0
    N = case.mesh["rr"].shape[1]
    return u, N * 3 * steps / el, el


def host_cpu():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith(("model name", "cpu part")):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def workload_config(args, N, nnz, steps):
    return {"workload": "wetdry_basin_4M" if args.n == 2000 else f"wetdry_basin_{args.n}x{args.n}",
            "nodes": N, "nnz": nnz, "steps_timed": steps, "replicas": int(os.environ.get("WORLD_SIZE", "1")),
            "l2": "working set larger than L2 (no flush)", "manning_n": 0.03, "cfl": 0.25}


# ------------------------------------------------------------------ arms
def run_reference(args, rank):
    """The reference's CPU implementation of the step (the FP64 restatement:
    no Fortran compiler exists here or on the GPU machine) on the same workload as
    the GPU arm: the same mesh, W untimed then K timed SSP-RK3 steps."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    case = make_case(args.n)
    N = case.mesh["rr"].shape[1]
    log(f"reference arm: mesh ready ({N} nodes)")
    o = oracle_for(case)
    nnz = len(o.matrices()["ja"])
    u = case.u0.copy(order="F")
    t = 0.0
    for _ in range(args.warmup):
        t = o.rk3_step(u, t)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t = o.rk3_step(u, t)
    el = time.perf_counter() - t0
    value = N * 3 * args.steps / el
    cores = int(os.environ["OMP_NUM_THREADS"])
    sample = (f"{args.steps} timed SSP-RK3 steps (after {args.warmup} untimed) of the full workload, {N} nodes, "
              f"FP64 restatement of the reference step (oracle), OpenMP over rows, {cores} threads, {host_cpu()}")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, N, nnz, args.steps), "precision": "fp64",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
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


def parity_leg(args, case, N, world):
    """Oracle leg on the same mesh, outside every timed region: the FP64
    oracle runs --parity-steps steps of the workload (timed: the CPU
    baseline); the FP64 and mixed GPU paths run the same steps from the same
    initial state and are compared with it."""
    from swe.update import from_case
    k = args.parity_steps
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    u_orc, v_orc, el = oracle_steps(case, k)
    log(f"oracle leg: {k} steps in {el:.1f} s")
    out = {"steps": k}
    for prec in (0, 1):
        upd = from_case(case, precision=prec)
        upd.upload(case.u0)
        upd.set_time(0.0, 1e30)
        upd.rk3_steps(k)
        u = upd.download()
        lump = upd.lumped
        upd.close()
        if prec == 0:
            # bit for bit except Manning friction's pow (CUDA's and the C
            # library's differ by an ulp): held to 1e-12 relative
            scale = np.abs(u_orc).max(axis=1, keepdims=True) + 1e-300
            out["fp64_bit_exact_vs_oracle"] = bool(np.array_equal(u, u_orc))
            out["fp64_max_rel_diff_vs_oracle"] = float((np.abs(u - u_orc) / scale).max())
        else:
            w = lump
            out["l1_rel_h_mixed_vs_oracle"] = float(np.sum(w * np.abs(u[0] - u_orc[0])) / np.sum(w * np.abs(u_orc[0])))
            out["max_abs_h_mixed_vs_oracle"] = float(np.abs(u[0] - u_orc[0]).max())
            out["min_h_mixed"] = float(u[0].min())
    cores = int(os.environ["OMP_NUM_THREADS"])
    cpu = {"value": v_orc, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"{k} SSP-RK3 steps of the same workload ({N} nodes, {el:.1f} s), FP64 restatement of the "
                     f"reference step (oracle), OpenMP over rows, {cores} threads, {host_cpu()}"}
    return out, cpu


def batched_leg(args):
    """C4 in the default line: the first --batch-subset instances of the
    batched dam-break ensemble (seed 2; node counts log-uniform in [2e3, 2e5])
    in one batched context (one launch per kernel for all instances,
    per-instance dt), against the same meshes looped one context at a time
    with the batched context's launch shapes; the same steps."""
    from swe import cases as C
    from swe.update import Update, from_case
    cases = C.batch_instances(n_inst=args.batch_subset, precision=1)
    NT = sum(c.mesh["rr"].shape[1] for c in cases)
    log(f"batched leg: {len(cases)} instances, {NT} nodes")
    upd = Update(batch=[(c.mesh, c.bath, c.params) for c in cases])
    for b, c in enumerate(cases):
        for comp, js, vals in c.dirichlet:
            upd.set_dirichlet(comp, js, vals, inst=b)
    u0 = [c.u0 for c in cases]
    upd.upload(u0); upd.set_time(0.0, 1e30); upd.rk3_steps(args.warmup)
    upd.upload(u0); upd.set_time(0.0, 1e30)
    _, _, n = upd.rk3_steps(args.steps)
    batched_ms = upd.last_device_ms
    spec = upd.tuning.split("autotuned ", 1)[-1]
    got = upd.download_split()
    upd.close()
    loop_ms, same = 0.0, True
    for b, c in enumerate(cases):
        s = from_case(c, precision=1)
        s.set_tuning(spec)
        s.upload(c.u0); s.set_time(0.0, 1e30); s.rk3_steps(args.warmup)
        s.upload(c.u0); s.set_time(0.0, 1e30)
        s.rk3_steps(args.steps)
        loop_ms += s.last_device_ms
        same = same and np.array_equal(s.download(), got[b])
        s.close()
    vb = NT * 3 * n / (batched_ms / 1e3)
    vl = NT * 3 * n / (loop_ms / 1e3)
    return {"workload": f"batched_dam_breaks_first_{len(cases)}_of_512", "instances": len(cases), "nodes": NT,
            "steps": n, "batched_node_stage_per_s": vb, "looped_single_instance_node_stage_per_s": vl,
            "batched_over_looped": vb / vl, "batched_equals_looped_bitwise": bool(same),
            "launch_shapes": "autotuned on the batched context, the same for the looped contexts"}


def run_ours(args, rank, world, dist):
    import torch
    from swe.update import from_case

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    case = make_case(args.n)
    N = case.mesh["rr"].shape[1]
    log(f"mesh ready: {N} nodes")
    t_setup = time.perf_counter()
    upd = from_case(case, precision=1)
    setup_s = time.perf_counter() - t_setup
    log(f"mixed context ready ({setup_s:.2f} s: device assembly, Morton order, layout, upload)")
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
    tuning = upd.tuning
    prof = upd.profile_kernels(args.profile_steps)
    stage_ms = prof["node"] + prof["low"] + prof["fct"] + prof["update"]
    step_kernel_ms = prof["dt"] + 3 * stage_ms
    peak, peak_kind = peaks()
    balg = b_alg(N, nnz, 1)
    achieved = balg / (stage_ms / 1e3) / 1e9
    kernel_bw = {k: {"ms": round(prof[k], 4), "design_bytes_per_node": round(b, 1),
                     "gbs": round(b * N / (prof[k] / 1e3) / 1e9, 1)}
                 for k, b in design_bytes(N, nnz).items() if prof.get(k)}
    traffic = None
    tf = ROOT / "profiles" / "traffic_per_node_stage.json"
    if tf.exists():
        d = json.loads(tf.read_text())
        if "mixed_bytes_per_node_stage" in d:
            traffic = d["mixed_bytes_per_node_stage"] * N

    # e2e through the C ABI with pinned host buffers: per step, one
    # swe_rk3_steps_host call (H2D of the state, one time step, D2H of the
    # new state, one synchronisation)
    S = u0.shape[0]
    hin = torch.empty(S * N, dtype=torch.float64, pin_memory=True)
    hout = torch.empty(S * N, dtype=torch.float64, pin_memory=True)
    hin.copy_(torch.from_numpy(np.ascontiguousarray(u0.ravel(order="F"))))
    upd.set_time(0.0, 1e30)
    upd.rk3_steps_host_ptr(hin.data_ptr(), hout.data_ptr(), 1)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        upd.rk3_steps_host_ptr(hin.data_ptr(), hout.data_ptr(), 1)
        hin, hout = hout, hin
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * N * 3 * args.e2e_steps / e2e_s
    # the same through three calls per step (swe_upload, swe_rk3_steps,
    # swe_download), each synchronising
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        upd.upload_ptr(hin.data_ptr())
        upd.rk3_steps(1)
        upd.download_ptr(hout.data_ptr())
        hin, hout = hout, hin
    e2e3_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e3_s], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e3_s = float(t.item())
    e2e3_value = world * N * 3 * args.e2e_steps / e2e3_s
    # host state in and out every 10 steps (the state crossing the link once
    # per output frame, as main.f90 writes frames every few steps)
    calls10 = max(1, args.e2e_steps // 10)
    t0 = time.perf_counter()
    for _ in range(calls10):
        upd.rk3_steps_host_ptr(hin.data_ptr(), hout.data_ptr(), 10)
        hin, hout = hout, hin
    e2e10_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e10_s], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e10_s = float(t.item())
    e2e10_value = world * N * 3 * 10 * calls10 / e2e10_s
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

    # the spec precision split (FP64 depth update, limiter and limited
    # depth sum over the same FP32 fluxes) on the same workload and steps
    split = None
    if not args.no_fp64:
        us = from_case(case, precision=2)
        rs = timed_run(us, u0, args.steps, min(args.warmup, 3), dist)
        u_s = us.download()
        prof_s = us.profile_kernels(1)
        vs = world * N * 3 * rs["steps"] / (rs["dev_ms"] / 1e3)
        split = {"value": vs, "ms_per_step": rs["dev_ms"] / rs["steps"], "steps": rs["steps"],
                 "stage_kernels_ms": {k: round(v, 4) for k, v in prof_s.items()},
                 "speed_vs_default_mixed": vs / value}
        if fp64:
            w = lump
            split["l1_rel_h_vs_fp64"] = float(np.sum(w * np.abs(u_s[0] - u_ref[0])) / np.sum(w * np.abs(u_ref[0])))
        us.close()
        log(f"precision split timed run: {rs['dev_ms']:.1f} ms")

    if rank != 0:
        return
    parity, cpu = None, None
    if world == 1 and args.parity_steps > 0:
        parity, cpu = parity_leg(args, case, N, world)
    batched = None
    if world == 1 and args.batch_subset > 0:
        batched = batched_leg(args)
        log(f"batched leg: {batched['batched_over_looped']:.2f}x looped")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["dev_ms"] / r["steps"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (double-float depth)",
        "data": "synthetic (seeded jittered-lattice Delaunay mesh, Gaussian-bump bathymetry)",
        "config": workload_config(args, N, nnz, r["steps"]),
        "precision": "mixed (FP32 arithmetic, double-float depth)",
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "unit_of_work": "one RK stage (k_node+k_low+k_fct+k_update), algorithmic bytes "
                                     f"{balg / N:.1f} B/node"},
        "stage_kernels_ms": {k: round(v, 4) for k, v in prof.items()},
        "kernel_design_bandwidth": kernel_bw,
        "setup_s": round(setup_s, 3),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": S * N * 8, "d2h_bytes_per_step": S * N * 8,
                "api": "swe_rk3_steps_host (one call per step)", "three_calls_value": e2e3_value,
                "ten_steps_per_call_value": e2e10_value},
        "cpu_baseline": cpu,
        "clocks": r["clocks"],
        "gpu_launches": r["launches"],
        "fp64": fp64,
        "speedup_mixed_vs_fp64": (value / fp64["value"]) if fp64 else None,
        "precision_split": split,
        "parity_vs_oracle": parity,
        "batched": batched,
        "mass_rel_drift_mixed": (mass_mix - mass0) / mass0,
        "min_h_mixed": float(u_mix[0].min()),
        "kernel_time_share_of_step": step_kernel_ms / (r["dev_ms"] / r["steps"]),
        "tuning": tuning,
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- other workloads
def _run_case(case, precision, steps=None):
    """Advance a case on the GPU; returns (state, node-stage/s, steps run, upd)."""
    from swe.update import from_case
    upd = from_case(case, precision=precision)
    upd.upload(case.u0)
    tf = case.tfinal if steps is None else 1e30
    upd.set_time(0.0, tf)
    n = steps if steps is not None else 10 ** 9
    _, _, k = upd.rk3_steps(min(n, 3))          # warm-up (graph build, autotune)
    upd.upload(case.u0)
    upd.set_time(0.0, tf)
    total_ms, done = 0.0, 0
    while done < n:
        chunk = min(n - done, 400)
        t, dt, k = upd.rk3_steps(chunk)
        total_ms += upd.last_device_ms
        done += k
        if k < chunk:
            break
    N = case.mesh["rr"].shape[1]
    return upd.download(), N * 3 * done / (total_ms / 1e3), done, upd


def run_thacker(args):
    """Thacker paraboloid, one period, FP64 and mixed per mesh spacing: analytic
    L1 error of h (quadrature at Gauss points, like compute_errors), rates, and
    the mixed-vs-FP64 difference.  Three set-ups: "film" is the current
    reference initial state (+htiny everywhere, condlim.f90:440) with its
    htiny = 1e-4 max_water_h = 4e-4 (max_water_h = hL = 4 for type 5);
    "no_film" the revision that produced the recorded runs, same htiny;
    "htiny_dx2" film-free with htiny = 4e-4 (spacing/0.05)^2, proportional
    to the lumped mass as in the reference's commented-out choice
    (main.f90:64-65).  A fixed htiny leaves an htiny-wide shoreline layer
    whose error does not fall under refinement."""
    import oracle
    from swe import cases as C, mesh as M
    from swe.lib import SweError
    rows = []
    for mode in ("film", "no_film", "htiny_dx2"):
        prev = None
        for hsp in (0.2, 0.1, 0.05, 0.025, 0.0125):
            mesh = C.thacker_mesh(hsp)
            film = mode == "film"
            case = C.thacker_case(mesh, periods=1.0, cfl=0.3, film=film)
            if mode == "htiny_dx2":
                ht = 4e-4 * (hsp / 0.05) ** 2
                rr = mesh["rr"]
                u0 = np.asfortranarray(np.vstack([C.thacker_sol(k, rr, 0.0, ht, 9.81, False) for k in (1, 2, 3)]))
                js = M.dirichlet_nodes(mesh["jjs"], mesh["sides"], [1, 2, 3, 4])
                bc = [(k - 1, js, C.thacker_sol(k, rr[:, js - 1], 0.0, ht, 9.81, False)) for k in (1, 2, 3)]
                case = replace(case, params=replace(case.params, htiny=ht), u0=u0, dirichlet=bc,
                               exact=lambda k, r, t, ht=ht: C.thacker_sol(k, r, t, ht, 9.81, False))
            o = oracle.Oracle(mesh["jj"], mesh["rr"])
            rj, rg = o.gauss()
            lump = o.matrices()["lumped"]
            out = {}
            try:
                for prec in (0, 1):
                    u, v, n, upd = _run_case(replace(case, params=replace(case.params, precision=prec)), prec)
                    tfin = float(upd.rk3_steps(0)[0][0])
                    upd.close()
                    ex = case.exact(1, rg, tfin)
                    err = o.norms(u[0], ex)[0] / o.norms(np.zeros(o.np), ex)[0]
                    out[prec] = (u, v, n, err)
            except SweError as e:
                # the reference STOPs as well (check_hmin) on such meshes
                rows.append({"spacing": hsp, "setup": mode, "nodes": o.np,
                             "stopped": f"{'FP64' if prec == 0 else 'mixed'} run: {e}"})
                log(f"thacker h={hsp} {mode}: stopped ({e})")
                prev = None
                continue
            u64, v64, n64, e64 = out[0]
            umx, vmx, nmx, emx = out[1]
            dmx = float(np.sum(lump * np.abs(umx[0] - u64[0])) / np.sum(lump * np.abs(u64[0])))
            rate = None if prev is None else math.log(prev / e64) / math.log(2.0)
            prev = e64
            rows.append({"spacing": hsp, "setup": mode, "htiny": case.params.htiny, "nodes": o.np, "steps": n64,
                         "l1_fp64": e64, "l1_mixed": emx, "rate_fp64": rate, "mixed_vs_fp64_l1": dmx,
                         "fp64_node_stage_per_s": v64, "mixed_node_stage_per_s": vmx})
            log(f"thacker h={hsp} {mode}: N={o.np} L1 fp64={e64:.4e} mixed={emx:.4e} diff={dmx:.2e}")
    print(json.dumps({"workload": "thacker_paraboloid_one_period", "rows": rows}), flush=True)


def run_batch(args):
    """Batched ensemble of dam breaks: one batched context (one launch per
    kernel for all instances, per-instance dt) versus looping single-instance
    contexts over the same meshes."""
    from swe import cases as C
    from swe.update import Update, from_case
    cases = C.batch_instances(n_inst=args.batch_count, precision=1)
    NT = sum(c.mesh["rr"].shape[1] for c in cases)
    log(f"batch meshes ready: {len(cases)} instances, {NT} nodes")
    items = [(c.mesh, c.bath, c.params) for c in cases]
    upd = Update(batch=items)
    for b, c in enumerate(cases):
        for comp, js, vals in c.dirichlet:
            upd.set_dirichlet(comp, js, vals, inst=b)
    u0 = [c.u0 for c in cases]
    upd.upload(u0); upd.set_time(0.0, 1e30); upd.rk3_steps(args.warmup)
    upd.upload(u0); upd.set_time(0.0, 1e30)
    upd.rk3_steps(args.steps)
    batched_ms = upd.last_device_ms
    vb = NT * 3 * args.steps / (batched_ms / 1e3)
    tuning = upd.tuning
    upd.close()
    # one context per instance, default launch shapes (autotuning hundreds of
    # small contexts would dominate the run)
    loop_ms = 0.0
    prev = os.environ.get("SWE_AUTOTUNE")
    os.environ["SWE_AUTOTUNE"] = "0"
    for c in cases:
        s = from_case(c, precision=1)
        s.upload(c.u0); s.set_time(0.0, 1e30); s.rk3_steps(args.warmup)
        s.upload(c.u0); s.set_time(0.0, 1e30)
        s.rk3_steps(args.steps)
        loop_ms += s.last_device_ms
        s.close()
    if prev is None:
        os.environ.pop("SWE_AUTOTUNE", None)
    else:
        os.environ["SWE_AUTOTUNE"] = prev
    vl = NT * 3 * args.steps / (loop_ms / 1e3)
    print(json.dumps({"workload": f"batched_dam_breaks_{len(cases)}", "nodes": NT, "steps": args.steps,
                      "batched_node_stage_per_s": vb, "looped_single_instance_node_stage_per_s": vl,
                      "batched_over_looped": vb / vl, "tuning": tuning,
                      "looped_tuning": "default launch shapes"}), flush=True)


def solitary_peak(rr, h):
    """Crest of a wave travelling along x: position and height of the maximum
    of h on the channel's centre line, refined by the parabola through the
    largest nodal value and its two neighbours on that line."""
    ymid = 0.5 * (rr[1].min() + rr[1].max())
    yc = rr[1][np.argmin(np.abs(rr[1] - ymid))]
    line = np.where(np.abs(rr[1] - yc) < 1e-9)[0]
    line = line[np.argsort(rr[0][line])]
    x, y = rr[0][line], h[line]
    k = min(max(int(np.argmax(y)), 1), len(line) - 2)
    den = y[k - 1] - 2.0 * y[k] + y[k + 1]
    s = 0.5 * (y[k - 1] - y[k + 1]) / den if den != 0.0 else 0.0
    return float(x[k] + s * 0.5 * (x[k + 1] - x[k - 1])), float(y[k] - 0.25 * (y[k - 1] - y[k + 1]) * s)


def sgn_leg(case, steps):
    """One configuration of the SGN solitary wave: FP64, mixed and
    precision-split runs of `steps` steps from the exact wave, with their
    rates, the time and last dt reached, min / max h, relative L1(h) against
    FP64, the crest's amplitude and position against the exact travelling
    wave, and the FP64 run's own sensitivity (initial state perturbed by 1e-7
    relative, seeded)."""
    rr = case.mesh["rr"]
    names = {0: "fp64", 1: "mixed", 2: "mixed_f64_split"}
    res, out = {}, {"cfl": case.params.cfl, "lambda_sgn": case.params.lambda_sgn}
    for prec in (0, 1, 2):
        u, v, n, upd = _run_case(case, prec, steps)
        t, _, dt = upd.get_time()
        res[prec] = (u, float(t[0]))
        o = {"node_stage_per_s": v, "steps": n, "time": float(t[0]), "last_dt": float(dt[0]),
             "min_h": float(u[0].min()), "max_h": float(u[0].max())}
        if prec == 1:
            o["tuning"] = upd.tuning
            o["stage_kernels_ms"] = {k: round(x, 4) for k, x in upd.profile_kernels(3).items()}
        out[names[prec]] = o
        lump = upd.lumped
        upd.close()

    def l1(a, b):
        return float(np.sum(lump * np.abs(a - b)) / np.sum(lump * np.abs(b)))

    h1 = float(case.u0[0].min())
    for prec, (u, t) in res.items():
        xe, he = solitary_peak(rr, case.exact(1, rr, t))
        xp, hp = solitary_peak(rr, u[0])
        out[names[prec]]["crest_amplitude_rel_drift"] = (hp - h1) / (he - h1) - 1.0
        out[names[prec]]["crest_position_drift"] = xp - xe
        if prec:
            out[names[prec]]["l1_h_vs_fp64"] = l1(u[0], res[0][0][0])
    rng = np.random.default_rng(0)
    pert = replace(case, u0=np.asfortranarray(case.u0 * (1 + 1e-7 * rng.uniform(-1, 1, case.u0.shape))))
    u_p, _, _, upd = _run_case(pert, 0, steps)
    upd.close()
    out["fp64_sensitivity_l1_h_1e-7_perturbation"] = l1(u_p[0], res[0][0][0])
    return out


def run_single(args, which):
    from swe import cases as C
    if which == "sgn":
        # the channel of the solitary wave at the requested resolution, as
        # specified (CFL 0.1), and at the CFL that resolves the relaxation:
        # the reference's lambda_max (and so its dt) leaves out the speed of
        # the relaxation waves, which grows like lambda g h^3 / sqrt(m)
        mesh = None
        legs = {}
        for name, cfl in (("as_specified", 0.1), ("relaxation_resolved", 5e-4)):
            case = C.sgn_case(nx=args.sgn_nx, ny=max(3, int(round(2.0 / (100.0 / (args.sgn_nx - 1)))) + 1),
                              nsteps=1000, cfl=cfl, mesh=mesh)
            mesh = case.mesh
            log(f"sgn {name}: {mesh['rr'].shape[1]} nodes, cfl {cfl}")
            legs[name] = sgn_leg(case, args.steps)
        print(json.dumps({"workload": "sgn_solitary", "nodes": mesh["rr"].shape[1], "steps": args.steps, **legs}),
              flush=True)
        return
    case = C.dam_break_case(n=101, tfinal=0.2)
    log(f"{which}: {case.mesh['rr'].shape[1]} nodes")
    out = {"workload": case.name, "nodes": case.mesh["rr"].shape[1]}
    res = {}
    for prec in (0, 1):
        u, v, n, upd = _run_case(case, prec, None)
        res[prec] = u
        out[("fp64" if prec == 0 else "mixed") + "_node_stage_per_s"] = v
        out["steps"] = n
        lump = upd.lumped
        upd.close()
    out["mixed_vs_fp64_l1_h"] = float(np.sum(lump * np.abs(res[1][0] - res[0][0])) / np.sum(lump * np.abs(res[0][0])))
    out["min_h_mixed"] = float(res[1][0].min())
    # conditioning of the workload itself: the FP64 path from the initial
    # state perturbed by 1e-7 relative (seeded), after the same steps
    rng = np.random.default_rng(0)
    pert = replace(case, u0=np.asfortranarray(case.u0 * (1 + 1e-7 * rng.uniform(-1, 1, case.u0.shape))))
    u_p, _, n_p, upd = _run_case(pert, 0, None)
    upd.close()
    out["fp64_sensitivity_l1_h_1e-7_perturbation"] = float(np.sum(lump * np.abs(u_p[0] - res[0][0]))
                                                           / np.sum(lump * np.abs(res[0][0])))
    out["fp64_sensitivity_steps"] = n_p
    print(json.dumps(out), flush=True)


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
        if args.workload == "wetdry":
            run_ours(args, rank, world, dist)
        elif rank == 0:
            {"thacker": run_thacker, "batch": run_batch}.get(args.workload, lambda a: run_single(a, args.workload))(args)
    finally:
        if dist:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
