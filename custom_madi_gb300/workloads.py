"""Named synthetic workloads (shapes and value ranges of the benchmark configurations).

* plain_config(): one 64-cell periodic box, rho = 2e5 cells/uL, v_i = 0.8
  (V = 4 pL), 1e4 walkers, dt = 0.01 ms, T = 46 ms, PGSE delta = 6 ms,
  Delta = 15/25/30/40 ms, b = 0/1000/2500/4000/6000 s/mm^2, 24 Fibonacci
  directions -> S[4 Delta, 5 b, 24 dir].
* batch_triplets(): 256 (kio, rho, V) drawn log-uniform from kio 1-130 1/s,
  rho 4.4e3-5.8e7 cells/uL, V 0.01-206 pL with 0.5 <= v_i <= 0.99 (the build's
  hard ceiling), periodic boxes of 27-512 cells, 1e5 walkers per entry.
* walker_library(): the 20,000 x 20 fitting library walked by the batched
  walker over the same (kio, rho, V) ranges: 2,000 (rho, V) geometries (64-cell
  periodic boxes) x 10 kio each, direction-averaged over 24 directions and
  normalised to b = 0 (S = 1 there exactly).
* mixed_triplets(): the large mixed workload's entries (cells 27-1024).
* match_library() / rician_voxels(): a 20,000 x 20 library of smooth
  direction-averaged decays normalised to b = 0 (kernel tests), and voxels
  drawn from a library with Rician noise at SNR 30.
"""

from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor
from dataclasses import replace
from typing import List, Optional, Tuple

import numpy as np

from .config import SimConfig, fibonacci_directions

PGSE = dict(ts=0.01, T_max_ms=46.0, small_deltas=[6.0], big_deltas=[15.0, 25.0, 30.0, 40.0],
            b_values=[0.0, 1000.0, 2500.0, 4000.0, 6000.0])


def plain_config(n_walkers: int = 10_000, directions: int = 24, **over) -> SimConfig:
    kw = dict(boundary_mode="periodic", n_cells=64, n_walkers=n_walkers, n_ensembles=1,
              geometry_validation_points=50_000, geometry_vi_tolerance=0.05,
              directions=fibonacci_directions(directions).tolist() if directions else None, **PGSE)
    kw.update(over)
    return SimConfig(**kw)


def batch_triplets(n: int = 256, seed: int = 1, vi_lo: float = 0.5, vi_hi: float = 0.99,
                   cells: Tuple[int, int] = (27, 512)) -> List[Tuple[float, float, float, int]]:
    """(kio, rho, V, n_cells) by rejection sampling of log-uniform (rho, V)."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        kio = float(np.exp(rng.uniform(np.log(1.0), np.log(130.0))))
        rho = float(np.exp(rng.uniform(np.log(4.4e3), np.log(5.8e7))))
        V = float(np.exp(rng.uniform(np.log(0.01), np.log(206.0))))
        nc = int(rng.integers(cells[0], cells[1] + 1))
        vi = rho * V * 1e-6
        if vi_lo <= vi <= vi_hi:
            out.append((kio, rho, V, nc))
    return out


def build_ensembles(triplets, cfg: SimConfig, seed: int = 0, threads: int = 8, verify_vi: bool = False,
                    measure_vi: bool = True):
    """One periodic ensemble per (kio, rho, V, n_cells), built on host threads."""
    from .ensemble import create_ensemble

    def one(i_t):
        i, (kio, rho, V, nc) = i_t
        c = replace(cfg, n_cells=int(nc))
        return create_ensemble(rho, V, c, seed=seed + i, verify_vi=verify_vi, measure_vi=measure_vi)
    with ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        return list(ex.map(one, enumerate(triplets)))


def batch_config(n_walkers: int = 100_000, directions: int = 24) -> SimConfig:
    return plain_config(n_walkers=n_walkers, directions=directions, geometry_validation_points=20_000,
                        geometry_vi_tolerance=0.1)


def match_library(n_lib: int = 20_000, seed: int = 3) -> Tuple[np.ndarray, np.ndarray]:
    """(lib [n_lib, 20] fp64, params [n_lib, 3]): bi-exponential decays over 4 Delta x 5 b.

    Columns are (Delta_i, b_j) pair-major; every row is 1 at b = 0.
    """
    rng = np.random.default_rng(seed)
    b = np.asarray(PGSE["b_values"]) * 1e-3            # ms/um^2
    Deltas = np.asarray(PGSE["big_deltas"])
    f = rng.uniform(0.3, 0.95, n_lib)[:, None, None]
    d_in = rng.uniform(0.1, 1.2, n_lib)[:, None, None]
    d_ex = rng.uniform(1.0, 3.0, n_lib)[:, None, None]
    tau = rng.uniform(20.0, 400.0, n_lib)[:, None, None]     # exchange-like Delta dependence
    x = np.exp(-Deltas[None, :, None] / tau)
    s = f * (x * np.exp(-b[None, None, :] * d_in) + (1 - x) * np.exp(-b[None, None, :] * d_ex)) \
        + (1 - f) * np.exp(-b[None, None, :] * d_ex)
    lib = s.reshape(n_lib, -1)
    lib /= lib[:, [0]]
    params = np.column_stack([rng.uniform(1, 130, n_lib), rng.uniform(4.4e3, 5.8e7, n_lib),
                              rng.uniform(0.01, 206, n_lib)])
    return lib, params


def rician_voxels(lib: np.ndarray, n_vox: int = 1_000_000, snr: float = 30.0, seed: int = 3):
    """(voxels [n_vox, F], truth index): |S0 s + sigma (n1 + i n2)|, S0 = 1, sigma = 1/snr."""
    rng = np.random.default_rng(seed + 1)
    idx = rng.integers(0, len(lib), n_vox)
    s = lib[idx]
    sig = 1.0 / snr
    v = np.sqrt((s + sig * rng.standard_normal(s.shape)) ** 2 + (sig * rng.standard_normal(s.shape)) ** 2)
    return v, idx


def two_delta_columns(seed: int = 3) -> np.ndarray:
    """Column indices of a random 2-Delta subset (10 of the 20 columns)."""
    rng = np.random.default_rng(seed + 2)
    d = np.sort(rng.choice(4, 2, replace=False))
    return np.concatenate([np.arange(5) + 5 * k for k in d])


def mixed_triplets(n: int = 140, seed: int = 4) -> List[Tuple[float, float, float, int]]:
    """Entries of the large mixed workload: batched-build ranges, 27-1024 cells."""
    return batch_triplets(n, seed=seed, cells=(27, 1024))


def walker_library(n_groups: int = 2000, kios_per_group: int = 10, n_walkers: int = 4096, seed: int = 3,
                   threads: int = 8, device=None, launch=None) -> Tuple[np.ndarray, np.ndarray, dict]:
    """(lib [n_groups * kios_per_group, 20] fp64, params [n, 3] (kio, rho, V), info).

    (rho, V) pairs are drawn like batch_triplets (log-uniform, 0.5 <= v_i <=
    0.99); each gets one 64-cell periodic geometry walked at kios_per_group kio
    values log-uniform in [1, 130] (the reference's kio sweep reuses a
    geometry: madi/library.py:483-520).  All walks run in one persistent launch;
    every entry is S averaged over 24 Fibonacci directions, 4 Delta x 5 b,
    pair-major, so S = 1 at b = 0.
    """
    import time
    from .walker_gpu import LaunchConfig, WalkBatch, WalkJob, _walk_seed, kio_to_pp, pair_layout
    from . import signal as S
    rng = np.random.default_rng(seed + 7)
    groups = batch_triplets(n_groups, seed=seed + 11)
    kios = np.sort(np.exp(rng.uniform(np.log(1.0), np.log(130.0), (n_groups, kios_per_group))), axis=1)
    cfg = batch_config(n_walkers=n_walkers)
    t0 = time.perf_counter()
    ens = build_ensembles([(1.0, r, v, 64) for _k, r, v, _n in groups], cfg, seed=seed * 100_000, threads=threads)
    t_host = time.perf_counter() - t0
    cols = S.build_columns(cfg)
    lay = pair_layout(cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    u = cfg.direction_array()
    jobs, params = [], []
    for g, e in enumerate(ens):
        for k in kios[g]:
            jobs.append(WalkJob(e, kio_to_pp(float(k), e.mean_AV, cfg), _walk_seed(seed, g), n_walkers))
            params.append((float(k), groups[g][1], groups[g][2]))
    import torch
    t0 = time.perf_counter()
    batch = WalkBatch(jobs, cfg, layout=lay, dirs=u, launch=launch or LaunchConfig(), device=device)
    batch.launch()
    torch.cuda.synchronize(batch.dev)
    t_walk = time.perf_counter() - t0
    res = batch.results()
    lib = np.stack([r["cos"].sum(axis=1) for r in res]) / float(len(u) * n_walkers)
    lib /= lib[:, [0]]
    cnt = batch.counters_np()
    if int(cnt[:, 1].sum()) or int(cnt[:, 2].sum()):
        raise RuntimeError("walker library: escaped walkers or classifier errors")
    info = {"entries": len(jobs), "geometries": len(ens), "walkers_per_entry": n_walkers,
            "walker_steps": len(jobs) * n_walkers * cfg.n_steps, "host_geometry_s": t_host,
            "walk_s": t_walk}
    return lib, np.asarray(params, np.float64), info
