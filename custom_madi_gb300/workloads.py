"""Named synthetic workloads (shapes and value ranges of the benchmark configurations).

* plain_config(): one 64-cell periodic box, rho = 2e5 cells/uL, v_i = 0.8
  (V = 4 pL), 1e4 walkers, dt = 0.01 ms, T = 46 ms, PGSE delta = 6 ms,
  Delta = 15/25/30/40 ms, b = 0/1000/2500/4000/6000 s/mm^2, 24 Fibonacci
  directions -> S[4 Delta, 5 b, 24 dir].
* batch_triplets(): 256 (kio, rho, V) drawn log-uniform from kio 1-130 1/s,
  rho 4.4e3-5.8e7 cells/uL, V 0.01-206 pL with 0.5 <= v_i <= 0.99 (the build's
  hard ceiling), periodic boxes of 27-512 cells, 1e5 walkers per entry.
* match_library() / rician_voxels(): a 20,000 x 20 library of smooth
  direction-averaged decays normalised to b = 0 and 1e6 voxels drawn from it
  with Rician noise at SNR 30.
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
