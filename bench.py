#!/usr/bin/env python
"""Throughput of the MPH-I time step on GB300 (particle-steps/s).

Workload (default): the 3D cube collapse of 100^3 fluid particles (l0 =
0.005 m) in a 3-layer wall tank around a 160x110x110 interior, gravity -9.8 in
z, dt = 5e-5 s, lambda*dt/(rho*l0^2) = 100, seeded +-0.01 l0 jitter:
1,297,696 particles.  Synthetic inputs generated here stand in for the case
files.  One step = the full reference step (sort, neighbours, explicit
physics, assembly, multigrid build, CR solve).

  value : particle-steps/s of the mixed form (FP32 CR + V-cycle, FP64 outer
          residual; --precision fp64 for the plain form) with the state
          resident in HBM, CUDA events on the case stream around K steps (the
          matrix alone is ~7 GB, far above L2); the line also carries the
          plain FP64 form's value on the same workload and the velocity
          difference of one step of each form from the same state
  e2e   : the same metric through the public API with pinned host buffers:
          every step uploads the particle state (mph_case_set_state) and reads
          back ids, types, positions and velocities (mph_get_fields)
  --impl reference : the CPU restatement of the reference (the oracle,
          OpenMP over all host cores) on a bounded sample of the workload
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [REPO, os.path.join(REPO, "oracle")]

from mphimplicit_gb300 import casegen  # noqa: E402

METRIC = "particle-steps/sec at <=1e-6 rel. err vs FP64 (mixed/batched vs plain GPU); p50/p99 step ms"
UNIT = "particle-steps/s"


def workload(name: str):
    if name == "cube3d_100":
        p, parts = casegen.cube_collapse_3d(100, seed=0)
        return 3, p, parts, "3D cube collapse, 100^3 fluid in a 3-layer tank around 160x110x110 (config 1)"
    m = re.match(r"cube3d_(\d+)$", name)
    if m:
        n = int(m.group(1))
        p, parts = casegen.cube_collapse_3d(n, seed=0)
        return 3, p, parts, f"3D cube collapse, {n}^3 fluid (config-1 geometry scaled)"
    if name == "dam2d_100":
        p, parts = casegen.square_drop_2d(1.0, seed=0)
        return 2, p, parts, "2D dam, 100x100 fluid in a 3-layer box around 200x150 (config 0)"
    raise SystemExit(f"unknown workload {name}")


def replica_throughput(units: float, seconds: float, dist=None, device="cpu"):
    """Whole-job throughput of independent replicas: the units every rank
    processed, summed, over the slowest rank's time (max over ranks)."""
    if dist is None:
        return units / seconds, seconds
    import torch
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(u.item()) / float(t.item()), float(t.item())


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` on the bench workload from the
    committed ncu summary (profiles/), or None."""
    path = os.path.join(REPO, "profiles", f"{kernel.split('+')[-1]}_cube3d_100.md")
    if not os.path.exists(path):
        return None
    m = re.search(r"dram_bytes_per_launch_full:\s*([0-9.eE+]+)", open(path).read())
    return float(m.group(1)) if m else None


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.f = tempfile.TemporaryFile(mode="w+")

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[2:6]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def spmv_bytes(prof, scal, dim, vb=8):
    """Algorithmic bytes of one block SpMV: every block once (D*D values of vb
    bytes + a column index), row lengths and slice pointers, x once, y
    written once (vb = 8 for the FP64 form, 4 for the FP32 inner solve)."""
    nf = int(scal["FluidParticleEnd"])
    blocks = scal["NonzeroCountA"] / (dim * dim)
    nsl = (nf + 31) // 32
    return blocks * (dim * dim * vb + 4) + nf * 4 + (nsl + 1) * 8 + 2 * dim * nf * vb


def pair_apply_bytes(prof, scal, dim, st=None):
    """Algorithmic bytes of one FP32 inner operator on the sliced pair terms
    (k_ct_apply32 + k_visc_pen32).  k_ct_apply32: column + D FP32 C values per
    transposed P-list slot, entry counts and slice pointers, s gathered once,
    t written.  k_visc_pen32: an 8-byte record per fluid slot (g = sqrt(f) e
    in FP16 and the neighbour's block-local index) and, unless the row
    block's neighbours are staged in shared memory, a 4-byte column (counted
    for no slot once any block is staged: a lower bound), column + D FP32
    lambda C per P-slot, the
    8-float diagonal / inertia record, row lengths, slice pointers and
    scales, s read once, t gathered once, y written; a staged block also reads
    its count and its distinct columns (4 bytes each; their s, which the block
    copies to shared memory, count as part of s read once)."""
    nf = int(scal["FluidParticleEnd"])
    n = int(scal["ParticleCount"])
    slots = scal["NonzeroCountA"] / (dim * dim)
    pslots = scal["NonzeroCountC"] / dim
    nsl, nct = (nf + 31) // 32, (n + 31) // 32
    st = st or {}
    staged = st.get("inner_local_blocks", 0) > 0
    col = 0 if staged else 4
    # P-slots and transposed slots: 16-byte records (D values, zero-padded in
    # 2-D, and the column or the block-local rank), counted as D * 4 + 4
    pcol = ctcol = 4
    ct = pslots * (dim * 4 + ctcol) + n * 4 + (nct + 1) * 8 + dim * nf * 4 + n * 4
    vp = slots * (8 + col) + pslots * (dim * 4 + pcol) + nf * (32 + 8) + 2 * (nsl + 1) * 8 + nsl * 4 \
        + 2 * dim * nf * 4 + n * 4
    if staged:
        vp += st["inner_local_cols"] * 4 + (st["inner_local_blocks"] + st["inner_gather_blocks"]) * 4
    return ct + vp


def assemble_bytes(prof, scal, dim):
    nf = int(scal["FluidParticleEnd"])
    n = int(scal["ParticleCount"])
    blocks = scal["NonzeroCountA"] / (dim * dim)
    return (blocks * (dim * dim * 8 + 4) + 4 * prof["nnb"] + 4 * prof["nnbP"] + 64 * n
            + dim * 8 * scal["NonzeroCountC"] / dim)


def cpu_sample(threads: int, steps: int = 1, fluid: int = 60, check_gpu: bool = False):
    """Time the oracle (OpenMP, `threads` threads) on the config-1 geometry
    scaled to `fluid`^3 fluid particles; optionally run the GPU engine on the
    same sample and report its velocity error against the oracle."""
    import oracle as orc
    orc.build_oracle()
    p, parts = casegen.cube_collapse_3d(fluid, seed=0)
    o = orc.Oracle(p, parts, 3, threads=threads)
    o.init()
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    out = {"value": parts.count * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"3D cube collapse {fluid}^3 fluid ({parts.count} particles), {steps} step(s) after the initial pass, "
                     f"{dt:.1f} s wall"}
    if check_gpu:
        from mphimplicit_gb300 import engine
        g = engine.Case(p, parts, 3)
        g.step(steps)
        vo = o.array("Velocity").reshape(-1, 3)[:g.fluid_count]
        vg = g.export("Velocity").reshape(-1, 3)[:g.fluid_count]
        ido, idg = o.array("ParticleIndex")[:g.fluid_count], g.export("ParticleIndex")[:g.fluid_count]
        vo, vg = vo[np.argsort(ido)], vg[np.argsort(idg)]
        out["gpu_err_vs_oracle"] = float(np.linalg.norm(vg - vo) / np.linalg.norm(vo))
        out["iters_oracle_gpu"] = [o.solve_stats()["iter"], g.solve_stats()["iter"]]
        g.close()
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    import oracle as orc
    orc.build_oracle()
    fluid = args.ref_fluid
    p, parts = casegen.cube_collapse_3d(fluid, seed=0)
    o = orc.Oracle(p, parts, 3, threads=threads)
    o.init()
    for _ in range(args.warmup):
        o.step(1)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.step(1)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = parts.count * args.steps / tot
    sample = (f"3D cube collapse {fluid}^3 fluid ({parts.count} particles; config-1 geometry scaled down), "
              f"{args.steps} timed steps after {args.warmup} warm-up steps")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "sample": sample, "threads": threads},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _vel_error_vs_fp64(engine, cases, prec_mixed, prec_fp64, tol_outer):
    """One step of each (params, parts, dim) in the mixed and the FP64 form
    from the same state: relative velocity error of the mixed result over the
    fluid particles (both forms keep the same particle order)."""
    errs = []
    for params, parts, dim in cases:
        out = []
        for prec in (prec_mixed, prec_fp64):
            g = engine.Case(params, parts, dim, precision=prec)
            if prec == prec_mixed:
                g.set_solver(tol_outer, 1e-3, 50)
            g.step(1)
            f = g.fields(("id", "type", "vel"))
            g.close()
            out.append(f)
        a, b = out
        assert np.array_equal(a["id"], b["id"])
        fl = b["type"] < 2
        errs.append(float(np.linalg.norm(a["vel"][fl] - b["vel"][fl]) / max(np.linalg.norm(b["vel"][fl]), 1e-300)))
    return errs


def _fp64_sequential_ms(engine, cases, prec_fp64):
    """Per-step time of each case run alone in the plain FP64 form (one warm-up
    step, one timed step, CUDA events on the legacy stream)."""
    import torch
    out = []
    for params, parts, dim in cases:
        g = engine.Case(params, parts, dim, precision=prec_fp64)
        g.step(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(torch.cuda.default_stream())
        g.step(1)
        e1.record(torch.cuda.default_stream())
        torch.cuda.synchronize()
        out.append(e0.elapsed_time(e1))
        g.close()
    return out


def run_ensemble(args, line_base):
    """Batched 2D ensemble (512 cases by default): every timed step advances
    every case once, all cases concurrently (mph_batch_step)."""
    import torch
    from mphimplicit_gb300 import engine, serving
    from mphimplicit_gb300.cabi import PRECISION_FP64, PRECISION_MIXED
    prec = PRECISION_MIXED if args.precision == "mixed" else PRECISION_FP64
    ens = casegen.ensemble_2d(args.cases, seed=1)
    cases = []
    for params, parts in ens:
        g = engine.Case(params, parts, 2, precision=prec)
        if prec == PRECISION_MIXED:
            g.set_solver(args.outer_tol, args.inner_tol, 50)
        cases.append(g)
    N = sum(g.count for g in cases)
    for _ in range(args.warmup):
        serving.batch_step(cases, 1, args.workers)
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    l0 = engine.launch_count()
    with Clocks(0) as clk:
        evs[0].record(torch.cuda.default_stream())
        for k in range(args.steps):
            serving.batch_step(cases, 1, args.workers)
            evs[k + 1].record(torch.cuda.default_stream())
        torch.cuda.synchronize()
    launches = engine.launch_count() - l0
    step_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    total_s = sum(step_ms) / 1000.0
    value = N * args.steps / total_s
    for g in cases:
        g.close()
    # plain FP64 form, one case after the other, on an evenly spaced sample
    idx = list(range(0, len(ens), max(1, len(ens) // args.sample)))[:args.sample]
    sample = [(ens[i][0], ens[i][1], 2) for i in idx]
    seq_ms = _fp64_sequential_ms(engine, sample, PRECISION_FP64)
    plain = sum(ens[i][1].count for i in idx) / (sum(seq_ms) / 1000.0)
    errs = _vel_error_vs_fp64(engine, sample[:4], PRECISION_MIXED, PRECISION_FP64, args.outer_tol) \
        if prec == PRECISION_MIXED else []
    line = dict(line_base)
    line.update({
        "value": value, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / args.steps,
        "dtype": "f64" if prec == PRECISION_FP64 else "f32-inner/f64-outer",
        "config": {"workload": "ensemble2d", "description": f"{len(ens)} independent 2D cases, fluid n x m, n,m ~ U[40,250] "
                   "(seed 1), mu log-uniform [0.01,1], gravity angle U[0,30], two fluid types in half (config 3); "
                   "one step = every case advanced once, all concurrently", "cases": len(ens), "particles": N,
                   "precision": args.precision, "workers": args.workers, "parallelism": "single",
                   "l2": "inputs larger than L2 (the cases' matrices total ~GBs)",
                   "p50_step_ms": float(np.percentile(step_ms, 50)), "p99_step_ms": float(np.percentile(step_ms, 99)),
                   "plain_fp64_sequential_value": plain,
                   "plain_fp64_sample": f"{len(idx)} evenly spaced cases, one step each, alone, FP64 form",
                   "speedup_vs_plain_fp64_sequential": value / plain,
                   "vel_rel_err_vs_fp64_per_step": errs},
        "gpu_launches": launches, "clocks": clk.summary(),
        "e2e": {"value": None, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    })
    print(json.dumps(line), flush=True)
    return 0


def run_serve(args, line_base):
    """Serving loop: Poisson arrivals (20 cases/s, seed 2) of 2D and 3D cases
    of 1e4..5e5 particles, admitted by device-memory footprint under a 150 GB
    budget, stepped concurrently; steps per case scaled by --serve-step-scale."""
    import threading
    import torch
    from mphimplicit_gb300 import engine, serving
    from mphimplicit_gb300.cabi import PRECISION_FP64, PRECISION_MIXED
    prec = PRECISION_MIXED if args.precision == "mixed" else PRECISION_FP64
    reqs = casegen.serving_requests(args.cases, seed=2, step_scale=args.serve_step_scale)
    srv = serving.Server(int(150e9), workers=args.workers)
    lock = threading.Lock()
    tickets = {}
    t0 = time.perf_counter()

    def submitter():
        for k, r in enumerate(reqs):
            dt = r["t"] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            t = srv.submit(r["params"], r["parts"], r["dim"], r["steps"], precision=prec, fields=("id",))
            with lock:
                tickets[t] = k

    th = threading.Thread(target=submitter)
    l0 = engine.launch_count()
    with Clocks(0) as clk:
        th.start()
        results = []
        while len(results) < len(reqs):
            results += srv.poll(wait_ms=100)
        th.join()
        torch.cuda.synchronize()
    launches = engine.launch_count() - l0
    stats = srv.stats()
    srv.close()
    bad = [r for r in results if r["status"] not in (0, 7)]
    if bad:
        raise SystemExit(f"served case failed: {bad[0]['error']}")
    first = min(r["submit_s"] for r in results)
    last = min(max(r["done_s"] for r in results), stats["elapsed_s"])
    span = max(r["done_s"] for r in results) - first
    psteps = sum(r["particles"] * r["steps"] for r in results)
    value = psteps / span
    step_ms = np.concatenate([r["step_ms"] for r in results])
    lat = np.array([r["done_s"] - r["submit_s"] for r in results])
    # plain FP64 form, the same requests one after the other (per-step time of
    # each request alone x its steps)
    sample = [(r["params"], r["parts"], r["dim"]) for r in reqs]
    seq_ms = _fp64_sequential_ms(engine, sample, PRECISION_FP64)
    seq_s = sum(ms / 1000.0 * r["steps"] for ms, r in zip(seq_ms, reqs))
    plain = psteps / seq_s
    errs = _vel_error_vs_fp64(engine, sample[:4], PRECISION_MIXED, PRECISION_FP64, args.outer_tol) \
        if prec == PRECISION_MIXED else []
    line = dict(line_base)
    line.update({
        "value": value, "steps": int(sum(r["steps"] for r in results)), "warmup": 0,
        "ms_per_step": float(np.mean(step_ms)), "dtype": "f64" if prec == PRECISION_FP64 else "f32-inner/f64-outer",
        "config": {"workload": "serve", "description": f"{len(reqs)} requests, Poisson arrivals 20/s (seed 2), 2D and 3D, "
                   "1e4..5e5 particles log-uniform, steps U[50,400] x step scale, 150 GB admission budget (config 4)",
                   "requests": len(reqs), "step_scale": args.serve_step_scale, "precision": args.precision,
                   "workers": args.workers, "parallelism": "single", "particle_steps": psteps, "span_s": span,
                   "l2": "inputs larger than L2",
                   "p50_step_ms": float(np.percentile(step_ms, 50)), "p99_step_ms": float(np.percentile(step_ms, 99)),
                   "p50_completion_s": float(np.percentile(lat, 50)), "p99_completion_s": float(np.percentile(lat, 99)),
                   "plain_fp64_sequential_value": plain,
                   "plain_fp64_sample": "every request alone in the FP64 form: one timed step x its step count",
                   "speedup_vs_plain_fp64_sequential": value / plain,
                   "vel_rel_err_vs_fp64_per_step": errs},
        "gpu_launches": launches, "clocks": clk.summary(),
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                "note": "requests are submitted from host memory and their fields returned to host buffers"},
    })
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="cube3d_100")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--inner-tol", type=float, default=1e-3,
                    help="mixed form: relative residual reduction of each FP32 inner solve")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-factored", action="store_true",
                    help="mixed form: assemble FP64 blocks instead of the factored FP64 operator")
    ap.add_argument("--extra-sweeps", type=int, default=0, help="mixed form: extra level-0 smoothing sweeps")
    ap.add_argument("--inner-blocks", type=int, default=-1, choices=[-1, 0, 1],
                    help="mixed form: inner operator on FP32 blocks (1) or sliced pair terms (0); -1 keeps the engine default")
    ap.add_argument("--no-fp64-leg", action="store_true", help="mixed form: skip the plain FP64 comparison run")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-fluid", type=int, default=60)
    ap.add_argument("--ref-fluid", type=int, default=50)
    ap.add_argument("--outer-tol", type=float, default=1e-6,
                    help="mixed form: FP64 outer relative residual (the reference's tolerance is 1e-6)")
    ap.add_argument("--cases", type=int, default=0, help="ensemble / serve: number of cases (0: 512 / 24)")
    ap.add_argument("--workers", type=int, default=64, help="ensemble / serve: host worker threads")
    ap.add_argument("--sample", type=int, default=16, help="ensemble: cases timed alone in the FP64 form")
    ap.add_argument("--serve-step-scale", type=float, default=0.1, help="serve: factor on each request's step count")
    args = ap.parse_args()
    if args.workload in ("ensemble2d", "serve") and args.cases <= 0:
        args.cases = 512 if args.workload == "ensemble2d" else 24

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    from mphimplicit_gb300 import build, engine
    from mphimplicit_gb300.cabi import PRECISION_FP64, PRECISION_MIXED
    if rank == 0 or world == 1:
        build.build()
    if dist:
        dist.barrier()
    if args.workload in ("ensemble2d", "serve"):
        base = {"metric": METRIC, "unit": UNIT, "n_gpus": world, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "data": "synthetic", "roofline": None, "cpu_baseline": None}
        return run_ensemble(args, base) if args.workload == "ensemble2d" else run_serve(args, base)
    dim, params, parts, desc = workload(args.workload)
    stream = torch.cuda.Stream()
    prec = PRECISION_MIXED if args.precision == "mixed" else PRECISION_FP64
    case = engine.Case(params, parts, dim, precision=prec, stream=stream.cuda_stream)
    if prec == PRECISION_MIXED:
        case.set_solver(args.outer_tol, args.inner_tol, 50)
        case.set_option("factored", 0 if args.no_factored else 1)
        case.set_option("mixed_extra_sweeps", args.extra_sweeps)
        if args.inner_blocks >= 0:
            case.set_option("inner_blocks", args.inner_blocks)
    N, Nf = case.count, case.fluid_count
    for _ in range(args.warmup):
        case.step(1)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    case.profile(True)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    iters = []
    l0 = engine.launch_count()
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        evs[0].record(stream)
        for k in range(args.steps):
            case.step(1)
            evs[k + 1].record(stream)
            iters.append(case.solve_stats()["iter"])
        torch.cuda.synchronize()
    launches = engine.launch_count() - l0
    if dist:
        dist.barrier()
    step_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    total_s = sum(step_ms) / 1000.0
    prof = case.profile_read()
    case.profile(False)
    scal = case.scalars()
    value, total_s = replica_throughput(N * args.steps, total_s, dist, "cuda")

    # end to end through the public API with host buffers (pinned)
    def pinned(shape, dt):
        return torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    fields = {"id": pinned((N,), torch.int32), "type": pinned((N,), torch.int32), "pos": pinned((N, 3), torch.float64),
              "vel": pinned((N, 3), torch.float64)}
    case.fields(out=fields)
    host = casegen.Particles(case.time(), parts.spacing, parts.domain_min, parts.domain_max, fields["type"], fields["pos"],
                             fields["vel"])
    ids = fields["id"]
    wc = case.export("WallCenter")
    vs = 2 if dim == 2 else 4
    h2d = N * (vs * 8 * 2 + 4 + 4)
    d2h = N * (vs * 8 * 2 + 4 + 4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if args.e2e_steps <= 0:
        t0 -= 1.0   # no end-to-end sample requested (profiling runs)
    for _ in range(args.e2e_steps):
        case.set_state(host, ids, wc)
        case.step(1)
        case.fields(out=fields)   # read back into the same pinned buffers
        host = casegen.Particles(case.time(), parts.spacing, parts.domain_min, parts.domain_max, fields["type"], fields["pos"],
                                 fields["vel"])
        wc = case.export("WallCenter")
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value = N * args.e2e_steps * world / e2e_s if args.e2e_steps > 0 else None

    # roofline of the dominant kernel (CUDA events on the case stream)
    peak, peak_kind = measured_peaks()
    vb = 4 if prec == PRECISION_MIXED else 8
    st = case.solve_stats()
    pairs = st.get("inner_form") == 2
    kern = {"spmv": ("k_ct_apply32+k_visc_pen32", lambda p_, s_, d_: pair_apply_bytes(p_, s_, d_, st)) if pairs else
                    ("k_spmv32" if vb == 4 else "k_spmv", lambda p_, s_, d_: spmv_bytes(p_, s_, d_, vb)),
            "assemble_a": ("k_assemble_cells", assemble_bytes)}
    dom = max(kern, key=lambda k: prof[f"kern_ms_{k}"])
    nlaunch = max(prof[f"kern_n_{dom}"], 1)
    avg_s = prof[f"kern_ms_{dom}"] / 1000.0 / nlaunch
    bytes_per = kern[dom][1](prof, scal, dim)
    achieved = bytes_per / avg_s / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": ncu_traffic(kern[dom][0]), "kernel": kern[dom][0], "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": bytes_per, "avg_launch_ms": avg_s * 1000.0, "launches": nlaunch}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_sample(os.cpu_count() or 1, 1, args.cpu_fluid, check_gpu=True)

    # the plain FP64 form on the same workload (for the mixed form's speed-up),
    # and one step of each form from the same state (velocity error)
    plain = None
    errs = []
    if prec == PRECISION_MIXED and not args.no_fp64_leg:
        case.close()
        f = engine.Case(params, parts, dim, precision=PRECISION_FP64, stream=stream.cuda_stream)
        for _ in range(args.warmup):
            f.step(1)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        ev[0].record(stream)
        for _ in range(args.steps):
            f.step(1)
        ev[1].record(stream)
        torch.cuda.synchronize()
        plain = N * args.steps / (ev[0].elapsed_time(ev[1]) / 1000.0)
        f.close()
        errs = _vel_error_vs_fp64(engine, [(params, parts, dim)], PRECISION_MIXED, PRECISION_FP64, args.outer_tol)

    stage_total = sum(prof[f"stage_ms_{s}"] for s in ("step_begin", "cellsort", "neighbors", "explicit", "assemble", "mg_build", "solve"))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == PRECISION_FP64 else "f32-inner/f64-outer", "data": "synthetic",
        "config": {"workload": args.workload, "description": desc, "dim": dim, "particles": N, "fluid": Nf,
                   "precision": args.precision, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs larger than L2 (the block matrix alone exceeds 129 MB by ~100x)",
                   "p50_step_ms": float(np.percentile(step_ms, 50)), "p99_step_ms": float(np.percentile(step_ms, 99)),
                   "cr_iterations": iters,
                   "inner_row_blocks": {"staged": st.get("inner_local_blocks"), "gathering": st.get("inner_gather_blocks"),
                                        "ct_blocks_staging_s": st.get("inner_ct_local_blocks"),
                                        "mean_distinct_cols": (st["inner_local_cols"] / st["inner_local_blocks"]
                                                               if st.get("inner_local_blocks") else None)},
                   "stage_ms_per_step": {s: prof[f"stage_ms_{s}"] / args.steps for s in
                                         ("step_begin", "cellsort", "neighbors", "explicit", "assemble", "mg_build", "solve")},
                   "stage_sum_ms_per_step": stage_total / args.steps,
                   "kernel_avg_ms": {k: (prof[f"kern_ms_{k}"] / prof[f"kern_n_{k}"] if prof[f"kern_n_{k}"] else None)
                                     for k in ("spmv", "vcycle", "assemble_a", "neighbors")},
                   "kernel_launches": {k: prof[f"kern_n_{k}"] for k in ("spmv", "vcycle", "assemble_a", "neighbors")},
                   "outer_tol": args.outer_tol if prec == PRECISION_MIXED else 1e-6,
                   "plain_fp64_value": plain,
                   "speedup_vs_plain_fp64": (value / plain) if plain else None,
                   "vel_rel_err_vs_fp64_per_step": errs},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": args.e2e_steps},
        "gpu_launches": launches,
        "roofline": roofline,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if prec != PRECISION_MIXED or args.no_fp64_leg:
        case.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
