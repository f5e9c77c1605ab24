"""(delta, Delta, b) columns and the DWI signal of one library entry.

Mirrors ``madi/signal.py``: G_from_b (:38-45), ColumnGrid / build_columns
(:52-150, column = pair * n_b + b), _assemble (:157-195), compute_signals /
compute_signals_multi_kio (:198-248) and signals_to_flat (:261-264).

Finite-lobe phase: dM = Y(delta) + Y(Delta) - Y(Delta + delta) [um ms],
phase = gamma G dM 1e-9 [rad], S = <cos(phase)> (real part).  With
``cfg.directions`` the phase is taken along each unit direction u
(u . dM) and ``S_dir`` [n_pairs, n_b, n_dirs] is returned beside the
direction-averaged S; the 3-axis default reproduces the reference exactly.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Tuple

import numpy as np

from .config import GAMMA_RAD, SimConfig, grid_time_index
from .walker_gpu import ReducedResult, run_simulation_multi_kio_reduced, run_simulation_reduced


def G_from_b(b_s_mm2: float, delta_ms: float, Delta_ms: float) -> float:
    """Gradient amplitude [T/m] of a rectangular PGSE pair with b [s/mm^2], delta, Delta [ms]."""
    b = b_s_mm2 * 1e6
    d = delta_ms * 1e-3
    td = (Delta_ms - delta_ms / 3.0) * 1e-3
    if b <= 0 or td <= 0:
        return 0.0
    return float(np.sqrt(b / ((GAMMA_RAD * d) ** 2 * td)))


@dataclass
class ColumnGrid:
    delta_pairs: List[Tuple[float, float]]
    b_values: np.ndarray
    j_delta: np.ndarray
    j_Delta: np.ndarray
    j_sum: np.ndarray
    phase_coef: np.ndarray
    n_pairs: int
    n_b: int
    phase_model: str = "finite_lobe"
    narrow_snapshot_steps: Optional[np.ndarray] = None
    narrow_snapshot_index: Optional[np.ndarray] = None
    narrow_phase_coef: Optional[np.ndarray] = None
    narrow_tD_requested_ms: Optional[np.ndarray] = None
    narrow_tD_sampled_ms: Optional[np.ndarray] = None


def build_columns(cfg: Optional[SimConfig] = None, delta_pairs=None, b_values=None) -> ColumnGrid:
    """Column arrays for every (pair, b), pair-major; off-grid timings raise."""
    if cfg is None:
        cfg = SimConfig()
    pairs = list(delta_pairs) if delta_pairs is not None else cfg.delta_pairs()
    bvals = np.asarray(cfg.b_values if b_values is None else b_values, dtype=float)
    n_pairs, n_b = len(pairs), len(bvals)
    n = n_pairs * n_b
    jd = np.empty(n, np.int32)
    jD = np.empty(n, np.int32)
    js = np.empty(n, np.int32)
    pc = np.empty(n, np.float64)
    steps = np.empty(n, np.int32)
    npc = np.empty(n, np.float64)
    treq = np.empty(n, np.float64)
    tsam = np.empty(n, np.float64)
    for p, (d, D) in enumerate(pairs):
        a, b_, c = grid_time_index(d, cfg.h_ms), grid_time_index(D, cfg.h_ms), grid_time_index(D + d, cfg.h_ms)
        tD = float(D - d / 3.0)
        k = int(round(tD / cfg.ts))
        if k < 0 or k > cfg.n_steps:
            raise ValueError(f"narrow-pulse t_D={tD:g} ms lies outside the {cfg.T_max_ms:g} ms walk")
        for i, bv in enumerate(bvals):
            col = p * n_b + i
            jd[col], jD[col], js[col] = a, b_, c
            pc[col] = GAMMA_RAD * G_from_b(float(bv), d, D) * 1e-9
            steps[col] = k
            npc[col] = pc[col] * float(d)
            treq[col] = tD
            tsam[col] = k * cfg.ts
    if cfg.phase_model == "finite_lobe":
        ss = si = nc = rq = sm = None
    elif cfg.phase_model == "narrow_pulse":
        ss, si = np.unique(steps, return_inverse=True)
        nc, rq, sm = npc, treq, tsam
    else:
        raise ValueError(f"unknown phase_model {cfg.phase_model!r}")
    return ColumnGrid(pairs, bvals, jd, jD, js, pc, n_pairs, n_b, cfg.phase_model, ss, si, nc, rq, sm)


def _assemble(res: ReducedResult, columns: ColumnGrid) -> dict:
    n_eff = res.n_eff
    shape = (columns.n_pairs, columns.n_b)
    if len(res.ensemble_cos_means) != len(res.ensemble_sin_means):
        raise RuntimeError("reduction returned mismatched real/imaginary ensemble means")
    ens_S = ens_Si = None
    if res.ensemble_cos_means:
        ens_S = np.asarray(res.ensemble_cos_means, np.float64).reshape(len(res.ensemble_cos_means), *shape)
        ens_Si = np.asarray(res.ensemble_sin_means, np.float64).reshape(len(res.ensemble_sin_means), *shape)
    out = {
        "delta_pairs": columns.delta_pairs,
        "b_values": columns.b_values,
        "S": (res.cos_sum / n_eff).reshape(shape),
        "S_imag": (res.sin_sum / n_eff).reshape(shape),
        "ensemble_S": ens_S,
        "ensemble_S_imag": ens_Si,
        "phase_model": columns.phase_model,
        "n_eff": n_eff,
        "n_escaped": res.n_escaped,
        "kio_analytic_eq5": res.analytic_kio_eq5,
        "pp": res.mean_pp,
        "occupancy_fraction": res.occupancy_fraction,
        "geometry_stats": res.geometry_stats,
    }
    if res.cos_dir is not None:
        out["S_dir"] = (res.cos_dir / float(res.n_walkers)).reshape(*shape, -1)
        out["S_dir_imag"] = (res.sin_dir / float(res.n_walkers)).reshape(*shape, -1)
    return out


def compute_signals(rho: float, V: float, kio: float, cfg: Optional[SimConfig] = None,
                    columns: Optional[ColumnGrid] = None, seed: int = 0, verbose: bool = True) -> dict:
    if cfg is None:
        cfg = SimConfig()
    if columns is None:
        columns = build_columns(cfg)
    res = run_simulation_reduced(rho, V, kio, columns.j_delta, columns.j_Delta, columns.j_sum,
                                 columns.phase_coef, cfg, seed=seed, verbose=verbose,
                                 narrow_snapshot_steps=columns.narrow_snapshot_steps,
                                 narrow_snapshot_index=columns.narrow_snapshot_index,
                                 narrow_phase_coef=columns.narrow_phase_coef)
    return _assemble(res, columns)


def compute_signals_multi_kio(rho: float, V: float, kios: list, cfg: Optional[SimConfig] = None,
                              columns: Optional[ColumnGrid] = None, seed: int = 0, verbose: bool = True,
                              ensembles: Optional[list] = None) -> dict:
    if cfg is None:
        cfg = SimConfig()
    if columns is None:
        columns = build_columns(cfg)
    res = run_simulation_multi_kio_reduced(rho, V, kios, columns.j_delta, columns.j_Delta, columns.j_sum,
                                           columns.phase_coef, cfg, seed=seed, verbose=verbose,
                                           narrow_snapshot_steps=columns.narrow_snapshot_steps,
                                           narrow_snapshot_index=columns.narrow_snapshot_index,
                                           narrow_phase_coef=columns.narrow_phase_coef, ensembles=ensembles)
    return {k: _assemble(r, columns) for k, r in res.items()}


def compute_adc(b_values, signal_1d, b_adc: float = 1000.0) -> float:
    i = int(np.argmin(np.abs(np.asarray(b_values) - b_adc)))
    s = signal_1d[i]
    b = b_values[i] / 1e6
    if s <= 0 or b <= 0:
        return 0.0
    return float(-np.log(s) / b)


def signals_to_flat(result: dict) -> np.ndarray:
    return result["S"].ravel()
