"""Benchmark: batched library-build walker (the path's headline metric).

Workload (one "step"): 256 library entries, each a periodic box of 27-512
contracted Voronoi cells with (kio, rho, V) drawn log-uniform (kio 1-130 1/s,
rho 4.4e3-5.8e7 cells/uL, V 0.01-206 pL, 0.5 <= v_i <= 0.99), 1e5 fp32 walkers
per entry, dt = 0.01 ms, 4,600 steps, PGSE delta = 6 ms, Delta = 15/25/30/40 ms,
5 b values, 24 gradient directions; all entries in one persistent launch.
Metric: walker-steps/s over the whole job (all ranks).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

``--impl reference`` times the reference's CPU walk (the oracle's fp64
restatement of _walk_cpu, all host threads) on a bounded sample of the same
entries, with geometry built by the oracle alone.  Under torchrun each rank
walks its own 256 entries (weak scaling, no collective on the data path);
rank 0 prints one JSON line.

The secondary legs (rank 0, N = 1) measure the rest of the path's targets:
the plain one-entry-per-launch path and the served path on the same entries
(matched Monte Carlo error), the entries/h at <= 0.5 % signal error, the
library match on a walker-built 20,000-entry library (FP32, BF16 top-32 /
top-8, error against an FP64 oracle per result), the serving loop at and
below capacity, and a scaled large mixed workload.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "walker-steps/s"
CONFIG_NAME = "batched library build: 256 entries x 1e5 walkers x 4600 steps, 27-512 cells, 20 cols x 24 dirs"
# walk_f32_kernel DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum)
# per walker-step, from one ncu capture of 16 entries x 2e4 walkers x 4,600
# steps: 6.39 MB + 0 MB over 1.472e9 walker-steps
WALK_DRAM_BYTES_PER_WALKER_STEP = 6.39e6 / 1.472e9
SIGNAL_ERR = 0.005          # absolute standard error on S (normalised to b = 0)


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload_config(args, ws: int) -> dict:
    """The workload both arms measure (identical dict on the GPU and the reference line)."""
    return {"workload": CONFIG_NAME, "entries_per_gpu": args.entries, "walkers_per_entry": args.walkers,
            "n_steps": 4600, "dt_ms": 0.01, "columns": 20, "directions": 24, "cells": [27, 512],
            "kio_range": [1.0, 130.0], "rho_range": [4.4e3, 5.8e7], "V_range": [0.01, 206.0],
            "parallelism": f"replicas{ws}"}


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


# ---------------------------------------------------------------------------
# CPU legs: the oracle's restatement of the reference walk, geometry built by
# the oracle (no native code of the package is loaded by these legs)
# ---------------------------------------------------------------------------

def _pgse():
    """Step grid, (pair, b) columns and directions of the workload (host-only modules)."""
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.walker_gpu import pair_layout
    cfg = WL.batch_config(n_walkers=1)
    cols = S.build_columns(cfg)
    lay = pair_layout(cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    return cfg, (lay.jd, lay.jD, lay.js, lay.coef), cfg.direction_array()


def oracle_entries(n_entries: int, rank: int = 0):
    """(oracle geometry, p_p, walk key) of the first n entries of the workload, built by the oracle."""
    from oracle import geometry as OG
    from custom_madi_gb300 import workloads as WL
    cfg, _, _ = _pgse()
    trip = WL.batch_triplets(256, seed=1 + 1000 * rank)[:n_entries]
    out = []
    for i, (kio, rho, V, nc) in enumerate(trip):
        e = OG.periodic_ensemble(rho, V, nc, 1000 * rank + i)
        out.append((OG.oracle_geometry(e), OG.kio_to_pp(kio, e["mean_AV"], cfg.D0, cfg.ts), (0, 0x4D414449)))
    return out


def cpu_walk_rate(entries, budget_s: float, threads: int):
    """Oracle walker-steps/s on a bounded sample: every entry walked with the
    same walker count, sized from a short calibration run to about budget_s."""
    from oracle import oracle as O
    cfg, cols, dirs = _pgse()

    def walk(geo, pp, key, n):
        O.walk(geo, n_walkers=n, n_steps=cfg.n_steps, steps_per_h=cfg.steps_per_h, n_grid=cfg.n_grid,
               sigma=cfg.sigma, ts=cfg.ts, pp=pp, key=key, want_Y=False, columns=cols, dirs=dirs,
               n_threads=threads)
    n0 = max(threads * 4, 64)
    t0 = time.perf_counter()
    walk(*entries[0], n0)
    rate0 = n0 * cfg.n_steps / (time.perf_counter() - t0)
    per = max(threads, int(rate0 * budget_s / (cfg.n_steps * len(entries))))
    t0 = time.perf_counter()
    for e in entries:
        walk(*e, per)
    dt = time.perf_counter() - t0
    return per * len(entries) * cfg.n_steps / dt, f"{len(entries)} of the entries x {per} walkers x {cfg.n_steps} steps ({dt:.1f} s)"


def run_reference_arm(args, ws, rank):
    if rank != 0:
        return 0
    threads = len(os.sched_getaffinity(0))
    entries = oracle_entries(8)
    rates, sample = [], ""
    for i in range(args.warmup + args.steps):
        r, sample = cpu_walk_rate(entries, budget_s=args.ref_budget, threads=threads)
        if i >= args.warmup:
            rates.append(r)
    v = float(np.mean(rates))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "walker-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload_config(args, ws),
            "arm": "oracle: fp64 C restatement of the reference _walk_cpu (madi/walker_gpu.py:698-840), "
                   "geometry by the oracle's restatement of the ensemble build, all host threads",
            "cpu_baseline": {"value": v, "unit": "walker-steps/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "walker-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def build_workload(rank: int, n_entries: int, n_walkers: int, threads: int):
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.walker_gpu import WalkJob, kio_to_pp, _walk_seed
    cfg = WL.batch_config(n_walkers=n_walkers)
    trip = WL.batch_triplets(n_entries, seed=1 + 1000 * rank)
    t0 = time.perf_counter()
    ens = WL.build_ensembles(trip, cfg, seed=1000 * rank, threads=threads)
    t_build = time.perf_counter() - t0
    jobs = [WalkJob(e, kio_to_pp(t[0], e.mean_AV, cfg), _walk_seed(0, 0), n_walkers) for e, t in zip(ens, trip)]
    return cfg, ens, jobs, t_build


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--entries", type=int, default=256)
    ap.add_argument("--walkers", type=int, default=100_000)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--ref-budget", type=float, default=8.0)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-autotune", action="store_true", help="default launch shape (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop legs")
    ap.add_argument("--no-mixed", action="store_true", help="skip the large mixed workload")
    ap.add_argument("--no-match", action="store_true", help="skip the library-match leg")
    ap.add_argument("--no-refdesign", action="store_true", help="skip the reference-design plain leg")
    ap.add_argument("--serving-requests", type=int, default=200)
    args = ap.parse_args(argv)
    ws, rank, local = _dist()
    if args.impl == "reference":
        return run_reference_arm(args, ws, rank)

    import torch
    import torch.distributed as dist
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300.walker_gpu import LaunchConfig, WalkBatch, WalkGraph, pair_layout
    from custom_madi_gb300 import autotune
    from custom_madi_gb300.sharding import max_over_ranks

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=dev) if "device_id" in dist.init_process_group.__code__.co_varnames \
            else dist.init_process_group("nccl")
    threads = len(os.sched_getaffinity(0))
    cfg, ens, jobs, t_build = build_workload(rank, args.entries, args.walkers, threads)
    cols = S.build_columns(cfg)
    lay = pair_layout(cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    dirs = cfg.direction_array()
    launch = LaunchConfig() if args.no_autotune else autotune.choose(jobs, cfg, lay, dirs, device=dev)
    batch = WalkBatch(jobs, cfg, layout=lay, dirs=dirs, launch=launch, device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)   # > 129 MB L2
    stream = torch.cuda.current_stream(dev)
    graph = WalkGraph(batch)              # the whole batched launch as one CUDA graph
    for _ in range(args.warmup):
        flush.fill_(1)
        graph.replay()
    torch.cuda.synchronize(dev)
    counters = batch.counters_np().sum(axis=0)
    # ---- timed region (device-resident inputs) ----
    peaks, peak_kind = _peaks()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    ev = []
    with ClockSampler(local) as clk:
        t_wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            graph.replay()
            e1.record(stream)
            ev.append((e0, e1))
        torch.cuda.synchronize(dev)
        t_wall = time.perf_counter() - t_wall0
    if ws > 1:
        dist.barrier()
    dev_s = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    steps_per_run = sum(j.n_walkers for j in jobs) * cfg.n_steps
    t_max = max_over_ranks(dev_s)             # the slowest rank sets the job's time
    value = ws * steps_per_run * args.steps / t_max
    batched_results = batch.results()
    # ---- end to end: host geometry + job tables -> device -> walk -> host sums ----
    host = batch.host_mirror()
    e2e_t = []
    for i in range(0 if args.no_e2e else max(args.e2e_steps, 1) + 1):
        t0 = time.perf_counter()
        batch.run_from_host(host)
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(float(np.mean(e2e_t[1:])) if len(e2e_t) > 1 else float("nan"))
    e2e_val = steps_per_run / e2e_s * ws
    # ---- roofline (issue bound: lane-operations per walker-step) ----
    n_ws = max(int(counters[0]) * cfg.n_steps, 1)
    f_full = counters[3] / n_ws
    f_t1 = counters[4] / n_ws
    f_fp = counters[8] / n_ws
    k_mean = float(np.average([g.candidates_mean for g in batch.geoms]))
    nf_mean = float(np.average([g.facets_mean for g in batch.geoms]))
    # 255 RNG + move + Y, 34 label-cache test (sphere, three planes), 6 per facet
    # of a full facet pass, 25 per candidate of a voxel-grid pass
    ops_step = 255.0 + 34.0 + f_fp * 6.0 * nf_mean + f_full * 25.0 * k_mean
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    peak_ops = sm_count * 128 * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
    achieved = (steps_per_run * args.steps / dev_s) * ops_step / 1e12
    # DRAM bytes per launch: the ncu capture of the 16-entry case scaled by walker-steps
    traffic = WALK_DRAM_BYTES_PER_WALKER_STEP * steps_per_run
    line = {
        "metric": METRIC, "value": value, "unit": "walker-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_s / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, ws),
        "timing": {"l2": "flushed (256 MB write) between steps",
                   "launch": "one CUDA graph replay per step (zeroing + persistent walk)"},
        "launch": {"tile_walkers": batch.desc.tile_walkers, "grid_blocks": batch.desc.grid_blocks,
                   "min_blocks": batch.desc.min_blocks, "staged_smem_bytes": int(batch.desc.stage_smem)},
        "roofline": {"bound": "issue", "achieved": achieved, "peak": peak_ops, "unit": "Top/s",
                     "frac": achieved / peak_ops, "traffic": traffic,
                     "note": f"lane-ops per walker-step {ops_step:.1f} (255 RNG+move+Y, 34 label-cache test, "
                             f"6 x {nf_mean:.1f} facets x {f_fp:.3f} facet passes, 25 x {k_mean:.1f} candidates x "
                             f"{f_full:.4f} voxel-grid passes); peak = SMs x 128 lanes x sm_max_mhz ({peak_kind} clock); "
                             f"traffic scaled from the 16-entry ncu capture"},
        "e2e": {"value": e2e_val, "unit": "walker-steps/s", "h2d_bytes_per_step": int(host["h2d_bytes"]),
                "d2h_bytes_per_step": int(host["d2h_bytes"])},
        "gpu_launches": args.steps,
        "clocks": clk.summary(),
        "staged_fraction": batch.staged_fraction,
        "walker_counters": {"full_per_step": float(f_full), "tier1_per_step": float(f_t1),
                            "facet_pass_per_step": float(f_fp),
                            "fallback64": int(counters[5]), "escaped": int(counters[1]),
                            "classifier_error": int(counters[2])},
        "host_ensemble_build_s": t_build,
        "wall_s_timed": t_wall,
        "accuracy": accuracy(batched_results, jobs, len(dirs), dev_s / args.steps, value / ws, cfg.n_steps),
    }
    if rank == 0 and ws == 1 and not args.no_cpu:
        r, sample = cpu_walk_rate(oracle_entries(8), budget_s=args.cpu_budget, threads=threads)
        line["cpu_baseline"] = {"value": r, "unit": "walker-steps/s", "cores": threads, "kind": "port",
                                "sample": sample}
    del graph, host
    if rank == 0 and ws == 1 and not args.no_secondary:
        sec = {}
        sec["plain_vs_batched"] = plain_and_served(dev, cfg, jobs, lay, dirs, value, batch)
        del batch
        torch.cuda.empty_cache()
        if not args.no_refdesign:
            sec["reference_design_plain"] = reference_design_leg(dev, cfg, jobs, cols, value)
        torch.cuda.empty_cache()
        lib = None
        if not args.no_match:
            sec["match"], lib = match_leg(dev, threads)
        if not args.no_serving:
            sec["serving"] = serving_legs(dev, args.serving_requests, lib, threads)
        if not args.no_mixed:
            sec["mixed"] = mixed_leg(dev, lib, threads)
        sec["reduce_production_grid"] = reduce_leg(dev)
        line["secondary"] = sec
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def accuracy(results, jobs, n_dirs, step_s, rate, n_steps):
    """Signal error of the batch from its own sums, and entries/h at <= SIGNAL_ERR.

    Per walker the direction-averaged cos(phase) lies in [-1, 1] with mean S,
    so its variance is at most 1 - S^2 and the standard error of S over N
    walkers at most sqrt((1 - S^2) / N): a rigorous bound on the Monte Carlo
    error of every (column) signal, normalised to b = 0.
    """
    se_max, need = [], []
    for j, r in zip(jobs, results):
        Sv = r["cos"].sum(axis=1) / (n_dirs * j.n_walkers)
        var = np.maximum(1.0 - Sv ** 2, 0.0)
        se_max.append(float(np.sqrt(var.max() / j.n_walkers)))
        need.append(int(np.ceil(var.max() / SIGNAL_ERR ** 2 / 128.0)) * 128)
    n = len(jobs)
    return {"signal_err_bound": "SE(S) <= sqrt((1 - S^2) / N), absolute on S(b=0) = 1",
            "max_se_at_bench_walkers": max(se_max), "median_se_at_bench_walkers": float(np.median(se_max)),
            "entries_per_h_at_bench_walkers": 3600.0 * n / step_s,
            "all_entries_within_0p5pct": bool(max(se_max) <= SIGNAL_ERR),
            "walkers_needed_for_0p5pct": {"max": max(need), "median": int(np.median(need))},
            "entries_per_h_at_0p5pct": 3600.0 * rate / (float(np.mean(need)) * n_steps),
            "note": "entries/h at 0.5 %: the batch's walker-steps/s spent on each entry's own required "
                    "walker count (mean over the 256 entries)"}


def _host_geometry(ens, dev):
    """Pinned host copies of an ensemble's device geometry (re-uploaded per call by the plain path)."""
    g = ens.device(str(dev))
    bufs = [g.stage, g.seed_f64, *g.kd]
    return [(b, b.cpu().pin_memory()) for b in bufs]


def plain_and_served(dev, cfg, jobs, lay, dirs, batched_rate, batch):
    """The same entries (same walkers each: matched Monte Carlo error) three ways:
    batched (the headline), plain (the reference's launch structure,
    madi/walker_gpu.py:843-951: per entry geometry H2D, one non-persistent launch,
    synchronize, D2H of the sums), and served (all entries as requests to the
    serving loop at t = 0)."""
    import torch
    from custom_madi_gb300.serving import Server, SimRequest
    from custom_madi_gb300.walker_gpu import LaunchConfig, WalkBatch
    out = {"entries": len(jobs), "walkers_per_entry": int(jobs[0].n_walkers), "batched_walker_steps_per_s": batched_rate}
    host = [_host_geometry(j.ensemble, dev) for j in jobs]
    plain_lc = LaunchConfig(tile_walkers=128, persistent=False)
    # warm-up on one entry
    WalkBatch([jobs[0]], cfg, layout=lay, dirs=dirs, launch=plain_lc, device=dev).launch()
    torch.cuda.synchronize(dev)
    ref = batch.results()
    t0 = time.perf_counter()
    plain_res = []
    for j, hg in zip(jobs, host):
        for d, h in hg:
            d.copy_(h, non_blocking=True)
        b = WalkBatch([j], cfg, layout=lay, dirs=dirs, launch=plain_lc, device=dev)
        b.launch()
        plain_res.append(b.results()[0])            # synchronizes (D2H of the sums)
    t_plain = time.perf_counter() - t0
    steps = sum(j.n_walkers for j in jobs) * cfg.n_steps
    same = all(np.array_equal(a["cos_fixed"], b["cos_fixed"]) for a, b in zip(ref, plain_res))
    out.update({"plain_walker_steps_per_s": steps / t_plain, "plain_s": t_plain,
                "plain_identical_sums": bool(same),
                "batched_over_plain": batched_rate / (steps / t_plain)})
    srv = Server(cfg, lay, dirs, device=dev, n_slots=len(jobs), budget_bytes=16 << 30)
    reqs = [SimRequest(j.ensemble, j.pp, j.walk_seed, j.n_walkers, 0.0) for j in jobs]
    res = srv.run(reqs, realtime=True)
    served_same = all(np.array_equal(r.result["cos_fixed"], a["cos_fixed"]) for r, a in zip(res["records"], ref))
    out.update({"served_walker_steps_per_s": res["walker_steps_per_s"], "served_s": res["span_s"],
                "served_identical_sums": bool(served_same),
                "served_over_plain": res["walker_steps_per_s"] / (steps / t_plain),
                "note": "matched Monte Carlo error: every arm walks the same 1e5 walkers per entry; "
                        "sums are exact fixed point, so the arms are compared bit for bit"})
    return out


def reference_design_leg(dev, cfg, jobs, cols, batched_rate, n_entries=4):
    """The reference's GPU design for the same entries (madi/walker_gpu.py:
    520-695 kernels, :989-1063 launch): per entry the geometry H2D, one fp64
    walk launch (one thread per walker, exact KD rule every step, Y stored to
    HBM), the column reduction over the 3 axes, synchronize, D2H of the sums.
    Both kernels are this package's CUDA; the entries, walkers and Philox
    numbers are the batched arm's, so the Monte Carlo error is matched."""
    import torch
    from custom_madi_gb300 import _native as N
    from custom_madi_gb300.walker_gpu import WalkBatch
    sub = jobs[:n_entries]
    host = [_host_geometry(j.ensemble, dev) for j in sub]
    st = torch.cuda.current_stream(dev)
    jd, jD, js = (torch.from_numpy(np.asarray(a, np.int32)).to(dev) for a in (cols.j_delta, cols.j_Delta, cols.j_sum))
    pc = torch.from_numpy(np.asarray(cols.phase_coef, np.float64)).to(dev)
    cs = torch.empty(len(pc), dtype=torch.float64, device=dev)
    ss = torch.empty_like(cs)

    def one(j, hg):
        for d, h in hg:
            d.copy_(h, non_blocking=True)
        b = WalkBatch([j], cfg, out_mode=N.MADI_OUT_Y, precision=64, device=dev)
        b.launch()
        N.reduce_Y(b.Y, b.n_rows, cfg.n_grid, jd, jD, js, pc, cs, ss, st)
        r = b.results()[0]
        return cs.cpu().numpy(), r["counters"]

    one(sub[0], host[0])                            # warm-up
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    sums = [one(j, hg) for j, hg in zip(sub, host)]
    t = time.perf_counter() - t0
    steps = sum(j.n_walkers for j in sub) * cfg.n_steps
    rate = steps / t
    ok = all(c["escaped"] == 0 and c["classifier_error"] == 0 for _, c in sums)
    return {"entries": len(sub), "walkers_per_entry": int(sub[0].n_walkers), "s": t,
            "walker_steps_per_s": rate, "batched_over_reference_design": batched_rate / rate,
            "clean": bool(ok),
            "note": "the reference's GPU design (fp64, one thread per walker, exact KD rule every step, "
                    "Y stored, separate reduction), one entry per launch, as CUDA kernels of this package"}


def match_leg(dev, threads):
    """Library match on the walker-built 20,000 x 20 library: 1e6 Rician voxels
    (SNR 30), all 20 columns and a 2-Delta subset; FP32, BF16 top-32 and top-8
    timed on the device; each result's error against the FP64 oracle
    (madi/library.py:1444-1450) on the first 1e5 voxels."""
    import torch
    from oracle import oracle as O
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.fitters_gpu import match_device
    lib, params, info = WL.walker_library(threads=threads, device=dev)
    vox, truth = WL.rician_voxels(lib, n_vox=1_000_000, seed=3)
    out = {"library": {"entries": int(lib.shape[0]), "columns": int(lib.shape[1]), "source": "batched walker",
                       **info, "entries_per_h_walk": 3600.0 * info["entries"] / info["walk_s"]},
           "voxels": int(len(vox)), "snr": 30, "oracle_voxels": 100_000}
    L32 = torch.from_numpy(lib.astype(np.float32)).to(dev)
    M32 = torch.from_numpy(vox.astype(np.float32)).to(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(Mx, Lx, prec, topk=32):
        match_device(Mx[:4096], Lx, precision=prec, topk=topk)
        best, outv = None, None
        for _ in range(3):
            torch.cuda.synchronize(dev)
            e0.record()
            o = match_device(Mx, Lx, precision=prec, topk=topk, check=False)
            e1.record()
            o.check()
            t = e0.elapsed_time(e1)
            if best is None or t < best:
                best, outv = t, o
        return best, outv

    n_or = 100_000
    for name, cidx in (("all_columns", np.arange(lib.shape[1])), ("two_delta", WL.two_delta_columns())):
        cidx_t = torch.as_tensor(cidx, device=dev)
        Mx, Lx = M32[:, cidx_t].contiguous(), L32[:, cidx_t].contiguous()
        m64 = vox[:n_or][:, cidx].astype(np.float32).astype(np.float64)     # the fp32 inputs the GPU sees
        l64 = lib[:, cidx].astype(np.float32).astype(np.float64)
        t0 = time.perf_counter()
        i64, r64 = O.match_fixed(m64, l64, chunk=2000)
        t_cpu = time.perf_counter() - t0
        leg = {"columns": int(len(cidx)), "fp64_oracle_voxels_per_s": n_or / t_cpu}
        t32 = None
        for key, prec, k in (("fp32", "fp32", 32), ("bf16_top32", "bf16", 32), ("bf16_top8", "bf16", 8)):
            t, o = timed(Mx, Lx, prec, k)
            idx = o[0].cpu().numpy().astype(np.int64)
            res = o[1].cpu().numpy().astype(np.float64)
            sel = idx[:n_or]
            # FP64 residual of the chosen entry minus the FP64 best residual: the per-voxel
            # error of the chosen fit (0 where the index agrees)
            r_sel = np.sum((m64 - l64[sel]) ** 2, axis=1)
            excess = r_sel - r64
            rel = excess / np.maximum(r64, 1e-30)
            leg[key] = {"ms": t, "voxels_per_s": len(vox) / (t / 1e3),
                        "index_agreement_vs_fp64": float(np.mean(sel == i64)),
                        "excess_resid_fp64": {"median": float(np.median(excess)), "max": float(excess.max())},
                        "excess_resid_rel": {"median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99)),
                                             "max": float(rel.max())},
                        "reported_vs_fp64_resid_abs": {"median": float(np.median(np.abs(res[:n_or] - r_sel))),
                                                       "max": float(np.abs(res[:n_or] - r_sel).max())}}
            if key == "fp32":
                t32, i32 = t, idx
            else:
                leg[key]["speedup_vs_fp32"] = t32 / t
                leg[key]["index_agreement_vs_fp32"] = float(np.mean(idx == i32))
        leg["bf16_top32"]["tensor_tflops"] = 2.0 * len(vox) * lib.shape[0] * 32 / (leg["bf16_top32"]["ms"] / 1e3) / 1e12
        out[name] = leg
    return out, lib


def _serving_run(dev, cfg, lay, ens, trip, walkers, rate, lib, seed, fit_every=8, fit_voxels=100_000):
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.serving import FitRequest, Server, SimRequest, poisson_arrivals
    from custom_madi_gb300.walker_gpu import kio_to_pp
    arrivals = poisson_arrivals(len(trip), rate, seed=seed)
    vox = WL.rician_voxels(lib, n_vox=fit_voxels, seed=5)[0].astype(np.float32) if lib is not None else None
    reqs = []
    for i, ((kio, _r, _v, _n), e) in enumerate(zip(trip, ens)):
        reqs.append(SimRequest(e, kio_to_pp(kio, e.mean_AV, cfg), 1000 + i, int(walkers[i]), float(arrivals[i])))
        if vox is not None and i % fit_every == fit_every - 1:
            reqs.append(FitRequest(vox, "bf16", 32, arrival=float(arrivals[i])))
    srv = Server(cfg, lay, cfg.direction_array(), library=lib, device=dev, budget_bytes=16 << 30)
    out = srv.run(reqs, realtime=True)
    sims = [r for r in out["records"] if r.kind == "sim"]
    fits = [r for r in out["records"] if r.kind == "fit"]
    offered = float(walkers.sum() * cfg.n_steps / arrivals[-1])

    def pct(rs, q):
        return float(np.percentile([r.latency for r in rs], q)) if rs else None
    return {"arrival_rate_req_s": rate, "requests": len(reqs), "sim_requests": len(sims), "fit_requests": len(fits),
            "p50_latency_s": out["p50_s"], "p99_latency_s": out["p99_s"],
            "sim_p50_latency_s": pct(sims, 50), "sim_p99_latency_s": pct(sims, 99),
            "fit_p50_latency_s": pct(fits, 50), "fit_p99_latency_s": pct(fits, 99),
            "offered_walker_steps_per_s": offered, "served_walker_steps_per_s": out["walker_steps_per_s"],
            "offered_over_served": offered / out["walker_steps_per_s"], "span_s": out["span_s"],
            "launches": out["launches"],
            "mixed_launch_fraction": float(np.mean([len(x) > 1 for x in srv.launch_log])) if srv.launch_log else 0.0}


def serving_legs(dev, n_requests, lib, threads):
    """Serving: Poisson arrivals at 50 req/s (seed 2) of batched-build triplets
    with walkers log-uniform in [1e4, 1e6] and a 1e5-voxel fit every eighth
    request; then the same requests at 0.8x the served capacity of the first run."""
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.walker_gpu import pair_layout
    cfg = WL.batch_config()
    cols = S.build_columns(cfg)
    lay = pair_layout(cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    trip = WL.batch_triplets(n_requests, seed=2)
    t0 = time.perf_counter()
    ens = WL.build_ensembles(trip, cfg, seed=200, threads=threads)
    t_build = time.perf_counter() - t0
    rng = np.random.default_rng(2)
    walkers = np.exp(rng.uniform(np.log(1e4), np.log(1e6), n_requests)).astype(np.int64)
    a = _serving_run(dev, cfg, lay, ens, trip, walkers, 50.0, lib, seed=2)
    capacity = a["served_walker_steps_per_s"]
    rate = 0.8 * capacity / float(walkers.mean() * cfg.n_steps)
    b = _serving_run(dev, cfg, lay, ens, trip, walkers, rate, lib, seed=12)
    return {"workload": "Poisson arrivals, batched-build triplets, walkers log-uniform [1e4, 1e6], "
                        "1e5-voxel BF16 top-32 fit every eighth request",
            "host_ensemble_build_s": t_build,
            "at_50_req_s": {**a, "note": "offered load above capacity: the queue grows for the whole run, so "
                                         "latencies grow with the number of requests" if a["offered_over_served"] > 1
                            else "offered load below capacity"},
            "at_0p8_capacity": b}


def mixed_leg(dev, lib, threads, chunk_walkers=262_144, launch_walkers=622_592, launch=None):
    """Large mixed workload, scaled 1/100: 140 entries x 1e6 walkers (27-1024
    cells, batched-build ranges) submitted to the serving loop at t = 0, with
    fit requests of 1e4-1e6 voxels (log-uniform) arriving every 0.5 s; beside
    it the plain one-entry-per-launch path on the same 140 entries (per-entry
    rates range over 3x with the geometry, so a subset does not stand for the
    whole)."""
    import torch
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.serving import FitRequest, Server, SimRequest
    from custom_madi_gb300.walker_gpu import LaunchConfig, WalkBatch, WalkJob, kio_to_pp, pair_layout, _walk_seed
    cfg = WL.batch_config(n_walkers=1_000_000)
    cols = S.build_columns(cfg)
    lay = pair_layout(cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    dirs = cfg.direction_array()
    trip = WL.mixed_triplets(140, seed=4)
    t0 = time.perf_counter()
    ens = WL.build_ensembles(trip, cfg, seed=4000, threads=threads)
    t_build = time.perf_counter() - t0
    reqs = [SimRequest(e, kio_to_pp(t[0], e.mean_AV, cfg), _walk_seed(0, 0), 1_000_000, 0.0)
            for e, t in zip(ens, trip)]
    n_fit = 0
    if lib is not None:
        rng = np.random.default_rng(44)
        sizes = np.exp(rng.uniform(np.log(1e4), np.log(1e6), 40)).astype(np.int64)
        vox, _ = WL.rician_voxels(lib, n_vox=int(sizes.max()), seed=9)
        vox = vox.astype(np.float32)
        for i, n in enumerate(sizes):
            reqs.append(FitRequest(vox[:n], "bf16", 32, arrival=0.5 * (i + 1)))
        n_fit = len(sizes)
    # 1e6-walker entries: launches of four waves (~622k walkers) amortise each launch's tail
    srv = Server(cfg, lay, dirs, library=lib, device=dev, n_slots=len(ens), budget_bytes=32 << 30,
                 chunk_walkers=chunk_walkers, launch_walkers=launch_walkers, launch=launch)
    out = srv.run(reqs, realtime=True)
    sims = [r for r in out["records"] if r.kind == "sim"]
    fits = [r for r in out["records"] if r.kind == "fit"]
    sim_span = max(r.finish for r in sims)
    rate = out["walker_steps"] / sim_span
    # plain path on the same entries (same walkers: matched Monte Carlo error)
    plain_lc = LaunchConfig(tile_walkers=128, persistent=False)
    sub = [WalkJob(r.ensemble, r.pp, r.seed, r.n_walkers) for r in reqs if isinstance(r, SimRequest)]
    WalkBatch([sub[0]], cfg, layout=lay, dirs=dirs, launch=plain_lc, device=dev).launch()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for j in sub:
        b = WalkBatch([j], cfg, layout=lay, dirs=dirs, launch=plain_lc, device=dev)
        b.launch()
        b.results()
    t_plain = time.perf_counter() - t0
    plain_rate = len(sub) * 1_000_000 * cfg.n_steps / t_plain
    full_steps = 14_000 * 1_000_000 * cfg.n_steps
    return {"workload": "140 entries x 1e6 walkers (1/100 of 14,000), 27-1024 cells, fits of 1e4-1e6 voxels "
                        "every 0.5 s through the serving loop",
            "host_ensemble_build_s": t_build, "sim_walker_steps": out["walker_steps"], "sim_span_s": sim_span,
            "walker_steps_per_s": rate, "fit_requests": n_fit,
            "fit_p50_latency_s": float(np.percentile([r.latency for r in fits], 50)) if fits else None,
            "fit_p99_latency_s": float(np.percentile([r.latency for r in fits], 99)) if fits else None,
            "mixed_launch_fraction": float(np.mean([len(x) > 1 for x in srv.launch_log])) if srv.launch_log else 0.0,
            "plain_walker_steps_per_s": plain_rate, "plain_entries": len(sub), "served_over_plain": rate / plain_rate,
            "extrapolated_14000_entries_h": full_steps / rate / 3600.0,
            "extrapolated_14000_entries_plain_h": full_steps / plain_rate / 3600.0,
            "extrapolation": "time for 14,000 entries = 6.44e13 walker-steps at the measured rate "
                             "(host geometry builds overlap the walk and are not included)"}


def reduce_leg(dev):
    """Column reduction of stored Y at the reference's production grid: 31,125
    columns (1,245 (delta, Delta) pairs x 25 b), n_grid = 129 (T = 128 ms), 5e4
    walkers (one ensemble of the production configuration); Y is a synthetic
    Brownian trajectory integral of that shape.  The oracle's fp64 reduction
    times 64 of the walkers on one host thread."""
    import torch
    from oracle import oracle as O
    from custom_madi_gb300 import _native as N
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300.config import SimConfig
    cfg = SimConfig(ts=0.01)
    cols = S.build_columns(cfg)
    n, ng = 50_000, cfg.n_grid
    g = torch.Generator(device=dev).manual_seed(5)
    x = torch.cumsum(torch.randn((n, ng, 3), generator=g, device=dev, dtype=torch.float64) * 1.7, dim=1)
    Y = torch.cumsum(x, dim=1) * 1e-3
    jd, jD, js = (torch.from_numpy(np.asarray(a, np.int32)).to(dev) for a in (cols.j_delta, cols.j_Delta, cols.j_sum))
    pc = torch.from_numpy(np.asarray(cols.phase_coef, np.float64)).to(dev)
    cs = torch.empty(len(pc), dtype=torch.float64, device=dev)
    ss = torch.empty_like(cs)
    st = torch.cuda.current_stream(dev)
    N.reduce_Y(Y, n, ng, jd, jD, js, pc, cs, ss, st)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    for _ in range(3):
        e0.record(st)
        N.reduce_Y(Y, n, ng, jd, jD, js, pc, cs, ss, st)
        e1.record(st)
        torch.cuda.synchronize(dev)
        times.append(e0.elapsed_time(e1))
    t = min(times) / 1e3
    y64 = Y[:64].cpu().numpy()
    t0 = time.perf_counter()
    oc, _ = O.reduce(y64, cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    t_cpu = time.perf_counter() - t0
    terms = float(n) * len(pc) * 3
    return {"columns": int(len(pc)), "walkers": n, "n_grid": ng, "ms": t * 1e3,
            "walker_column_axis_terms_per_s": terms / t, "Y_bytes": int(Y.numel() * 8),
            "cpu_oracle_terms_per_s_1_thread": 64.0 * len(pc) * 3 / t_cpu,
            "note": "Y read once per block of 1,024 columns (31 blocks), fp64 sincos per term"}


if __name__ == "__main__":
    sys.exit(main())
