"""Launch-shape autotuner for the batched walker.

For a batch it times the candidate (tile_walkers, blocks_per_sm, register
budget, stage budget) shapes on a representative sub-batch (the first jobs,
enough tiles to fill every SM a few times, full walk length) with CUDA events
and keeps the fastest.  Winners are stored by the native cache
(``madi_autotune_load`` / ``madi_autotune_store``) keyed by (SM count, seed-count
bucket of the largest ensemble, stage-size bucket, output columns x
directions), so a repeated build pays nothing.  The cache file is
$MADI_AUTOTUNE_CACHE or ~/.cache/custom_madi_gb300/autotune.tsv.
"""

from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from . import _native as N
from .walker_gpu import LaunchConfig, PairLayout, WalkBatch, WalkJob

# (tile_walkers, blocks_per_sm (0 = occupancy), min_blocks register budget, stage budget bytes)
CANDIDATES = ((128, 0, 2, 0), (256, 0, 2, 0), (128, 0, 1, 0), (256, 0, 1, 0), (64, 0, 1, 0),
              (128, 0, 2, 48 * 1024), (256, 0, 1, 48 * 1024))
_lock = threading.Lock()


def cache_path() -> Path:
    p = os.environ.get("MADI_AUTOTUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "custom_madi_gb300" / "autotune.tsv"


def load(key: str) -> Optional[N.MadiLaunchShape]:
    """Stored shape for ``key`` or None."""
    sh = N.MadiLaunchShape()
    st = N.lib().madi_autotune_load(str(cache_path()).encode(), key.encode(), C.byref(sh))
    N.check(st, "madi_autotune_load")
    return sh if sh.tile_walkers > 0 else None


def store(key: str, tile_walkers: int, blocks_per_sm: int, min_blocks: int, stage_budget: int, rate: float) -> bool:
    sh = N.MadiLaunchShape(int(tile_walkers), int(blocks_per_sm), int(min_blocks), int(stage_budget), float(rate))
    st = N.lib().madi_autotune_store(str(cache_path()).encode(), key.encode(), C.byref(sh))
    return st == 0     # an unwritable cache only costs a re-tune next time


def key_for(jobs: Sequence[WalkJob], layout: PairLayout, n_dirs: int, sm_count: int) -> str:
    seeds = max(len(j.ensemble.classifier_seeds if j.ensemble.classifier_seeds is not None else j.ensemble.seeds)
                for j in jobs)
    bucket = int(2 ** np.ceil(np.log2(max(seeds, 2))))
    stage = max(j.ensemble.device().stage_bytes for j in jobs)
    sbucket = int(2 ** np.ceil(np.log2(max(stage, 1024))))
    return f"lib{N.lib_digest()}/sm{sm_count}/seeds{bucket}/stage{sbucket}/out{layout.n_pairs * layout.n_b}x{n_dirs}"


def _time(jobs, cfg, layout, dirs, lc, device, reps=2) -> float:
    import torch
    b = WalkBatch(jobs, cfg, layout=layout, dirs=dirs, launch=lc, device=device)
    b.launch()
    torch.cuda.synchronize(device)
    best = float("inf")
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        b.launch()
        e1.record()
        torch.cuda.synchronize(device)
        best = min(best, e0.elapsed_time(e1) / 1e3)
    steps = sum(j.n_walkers for j in jobs) * cfg.n_steps
    return steps / best


def choose(jobs: Sequence[WalkJob], cfg, layout: PairLayout, dirs, device=None, *, retune: bool = False,
           budget_tiles: Optional[int] = None) -> LaunchConfig:
    """Fastest LaunchConfig for this batch (cached)."""
    import torch
    device = torch.device(device or "cuda")
    sm = torch.cuda.get_device_properties(device).multi_processor_count
    n_dirs = len(dirs)
    key = key_for(jobs, layout, n_dirs, sm)
    with _lock:
        e = None if retune else load(key)
    if e is not None:
        return LaunchConfig(tile_walkers=int(e.tile_walkers), blocks_per_sm=int(e.blocks_per_sm),
                            min_blocks=int(e.min_blocks), stage_budget=int(e.stage_budget),
                            staged=bool(e.stage_budget))
    target = budget_tiles or sm * 8
    sub, tiles = [], 0
    for j in jobs:
        nw = min(j.n_walkers, 256 * max(1, (target - tiles)))
        sub.append(WalkJob(j.ensemble, j.pp, j.walk_seed, nw, j.walker_base))
        tiles += (nw + 255) // 256
        if tiles >= target:
            break
    results = {}
    for cand in CANDIDATES:
        tw, bps, mb, sb = cand
        lc = LaunchConfig(tile_walkers=tw, blocks_per_sm=bps, min_blocks=mb, stage_budget=sb, staged=bool(sb))
        try:
            results[cand] = _time(sub, cfg, layout, dirs, lc, device)
        except Exception:   # a shape the device cannot launch is simply not a candidate
            continue
    if not results:
        return LaunchConfig()
    (tw, bps, mb, sb), rate = max(results.items(), key=lambda kv: kv[1])
    with _lock:
        store(key, tw, bps, mb, sb, rate)
    return LaunchConfig(tile_walkers=tw, blocks_per_sm=bps, min_blocks=mb, stage_budget=sb, staged=bool(sb))
