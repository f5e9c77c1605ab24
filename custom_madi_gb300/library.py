"""MADI library: simulated signals indexed by (k_io, rho, V), and voxel matching.

Keeps the interface of ``madi/library.py``: LibraryEntry (:80-108), the
remediation log grid (:116-228), append keys and v_i filter (:231-264), the v5
diagnostics (:312-438), build_library_from_triplets / build_library (:445-670),
the npz schema writer / readers (:677-1160), nearest-column resolution and the
candidate matrix (:1167-1328), edge diagnostics (:1331-1395) and the MAP
matchers (:1402-1522).

GB300 differences: the builder walks every (rho, V) group x ensemble x k_io of
a build in one persistent launch per chunk (``max_jobs_per_launch``) instead
of one launch per ensemble and k_io; the matchers always run on the GPU
(``use_gpu=False`` raises) and accept ``precision="bf16"``.
"""

from __future__ import annotations

import json
import time
from collections import defaultdict
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import List, Mapping, Optional, Tuple

import numpy as np

from .config import (BVALS_UNIQUE, DELTA_SMALL, DELTAS_BIG, ENSEMBLE_MEAN_SUBSET_B_VALUES_S_MM2,
                     ENSEMBLE_MEAN_SUBSET_DELTA_PAIRS_MS, SimConfig)
from . import signal as sig

MADI_LIBRARY_SCHEMA_V5 = "madi-library-v5"
MADI_LIBRARY_SCHEMA_V4 = "madi-library-v4"
MADI_LIBRARY_ENTRY_SCHEMA_V5 = "madi-library-entry-v5"
ENSEMBLE_MEAN_SUBSET_N_COLUMNS = len(ENSEMBLE_MEAN_SUBSET_DELTA_PAIRS_MS) * len(ENSEMBLE_MEAN_SUBSET_B_VALUES_S_MM2)


@dataclass
class LibraryEntry:
    kio: float
    rho: float
    V: float
    vector: np.ndarray
    signal_imag: Optional[np.ndarray] = None
    signal_variance: Optional[np.ndarray] = None
    ensemble_means_subset: Optional[np.ndarray] = None
    vi: Optional[float] = None
    weight: Optional[float] = None
    kio_nominal: Optional[float] = None
    rho_nominal: Optional[float] = None
    V_nominal: Optional[float] = None
    pp: Optional[float] = None
    kio_analytic_eq5: Optional[float] = None
    is_free_water: bool = False
    metadata: dict = field(default_factory=dict)

    @property
    def realised_vi(self) -> float:
        if self.vi is not None and np.isfinite(self.vi):
            return float(self.vi)
        return float(self.rho) * float(self.V) * 1e-6


DEFAULT_KIOS = [2, 5, 8, 12, 18, 25, 35, 50, 75, 100]
DEFAULT_RHOS = [100_000, 200_000, 400_000, 600_000, 800_000]
DEFAULT_VS = [0.5, 1.0, 2.0, 3.0, 4.0, 5.0]


def _cell_widths(values, lower_bound=None, upper_bound=None) -> np.ndarray:
    """Midpoint quadrature widths of a strictly increasing 1-D grid."""
    a = np.asarray(values, dtype=float)
    if a.ndim != 1 or len(a) < 2 or np.any(np.diff(a) <= 0.0):
        raise ValueError("grid axis must be strictly increasing with at least two values")
    mids = 0.5 * (a[:-1] + a[1:])
    lo = float(lower_bound) if lower_bound is not None else a[0] - 0.5 * (a[1] - a[0])
    hi = float(upper_bound) if upper_bound is not None else a[-1] + 0.5 * (a[-1] - a[-2])
    if lo > a[0] or hi < a[-1]:
        raise ValueError("quadrature bounds must enclose every grid node")
    return np.diff(np.concatenate([[lo], mids, [hi]]))


@dataclass(frozen=True)
class LogGridDefinition:
    """Masked log-coordinate (rho, V) x linear k_io grid plus one free-water atom."""

    kios: np.ndarray
    rhos: np.ndarray
    Vs: np.ndarray
    vi_min: float = 0.40
    vi_max: float = 0.99
    free_water_weight: float = 1.0

    def triplets_and_weights(self):
        if np.any(self.rhos <= 0.0) or np.any(self.Vs <= 0.0):
            raise ValueError("log-coordinate rho and V grid values must be positive")
        if np.any(self.kios < 0.0):
            raise ValueError("k_io grid values must be non-negative")
        lr, lv = np.log(self.rhos), np.log(self.Vs)
        wr = _cell_widths(lr, lr[0], lr[-1])
        wv = _cell_widths(lv, lv[0], lv[-1])
        wk = _cell_widths(self.kios, 0.0, float(self.kios[-1]))
        trip = [(0.0, 0.0, 0.0)]
        weights = {_entry_key(0.0, 0.0, 0.0): float(self.free_water_weight)}
        for ik, k in enumerate(self.kios):
            for ir, r in enumerate(self.rhos):
                for iv, v in enumerate(self.Vs):
                    vi = float(r * v * 1e-6)
                    if self.vi_min <= vi <= self.vi_max:
                        t = (float(k), float(r), float(v))
                        trip.append(t)
                        weights[_entry_key(*t)] = float(r * v * wr[ir] * wv[iv] * wk[ik])
        return trip, weights

    def metadata(self) -> dict:
        return {"coordinate_transform": {"rho": "uniform_log", "V": "uniform_log", "kio": "piecewise_uniform_linear"},
                "vi_min": float(self.vi_min), "vi_max": float(self.vi_max), "rho_values": self.rhos.tolist(),
                "V_values": self.Vs.tolist(), "kio_values": self.kios.tolist(),
                "free_water_weight": float(self.free_water_weight),
                "weight_expression": "rho * V * dlogrho * dlogV * dkio"}


def make_remediation_log_grid(*, n_rho=64, n_V=64, kios=None, rho_min=1.0e4, rho_max=1.0e7, V_min=0.01,
                              V_max=200.0, vi_min=0.40, vi_max=0.99) -> LogGridDefinition:
    if not (0.0 < rho_min < rho_max):
        raise ValueError("remediation rho bounds must satisfy 0 < min < max")
    if not (0.0 < V_min < V_max):
        raise ValueError("remediation V bounds must satisfy 0 < min < max")
    if kios is None:
        kios = np.concatenate([[0.0], np.arange(1.0, 31.0), np.arange(35.0, 131.0, 5.0)])
    return LogGridDefinition(np.asarray(kios, float), np.geomspace(rho_min, rho_max, int(n_rho)),
                             np.geomspace(V_min, V_max, int(n_V)), float(vi_min), float(vi_max))


def _entry_key(kio, rho, V):
    if not np.isfinite(kio) or (rho == 0.0 and V == 0.0):
        return ("free_water", 0.0, 0.0)
    return (round(float(kio), 4), round(float(rho), 1), round(float(V), 6))


def _existing_keys(library):
    return {_entry_key(e.kio if e.kio_nominal is None else e.kio_nominal,
                       e.rho if e.rho_nominal is None else e.rho_nominal,
                       e.V if e.V_nominal is None else e.V_nominal) for e in library}


VI_HARD_MAX = 0.99


def _filter_valid(triplets, vi_min=0.0, vi_max=VI_HARD_MAX):
    top = min(vi_max, VI_HARD_MAX)
    out = []
    for k, r, v in triplets:
        if r == 0.0 and v == 0.0:
            out.append((k, r, v))
        elif vi_min <= (r * 1e-9) * (v * 1e3) <= top:
            out.append((k, r, v))
    return out


def _summarise_realised_geometry(per_ensemble: list, cfg: SimConfig) -> dict:
    """Aggregate of the realised ensembles (labels only; never fed back into Eq. 5)."""
    if not per_ensemble:
        return {"vi": 0.0, "rho_per_uL": 0.0, "mean_volume_pL": 0.0, "governing_mean_A_over_V_um_inv": 0.0,
                "n_seeds_sim": 0}
    cells = np.array([int(x["n_seeds_sim"]) for x in per_ensemble], float)
    vis = np.array([float(x["realised_vi"]) for x in per_ensemble], float)
    vols = np.array([float(x["sim_side_um"]) ** 3 for x in per_ensemble])
    n_cells, vol, vol_in = float(cells.sum()), float(vols.sum()), float(np.sum(vis * vols))
    rho = n_cells / vol * 1e9 if vol else 0.0
    V = vol_in / n_cells / 1e3 if n_cells else 0.0
    w = vols / max(vol, 1.0)

    def vw(name):
        return float(np.sum(w * np.array([float(x[name]) for x in per_ensemble])))
    return {
        "vi": vol_in / vol if vol else 0.0,
        "vi_between_ensemble_sd": float(np.std(vis, ddof=1)) if len(vis) > 1 else 0.0,
        "rho_per_uL": float(rho), "mean_volume_pL": float(V), "mean_volume_um3": float(V * 1e3),
        "governing_mean_A_over_V_um_inv": vw("governing_mean_A_over_V_um_inv"),
        "annulus_mean_um": vw("annulus_mean_um"), "annulus_std_um": vw("annulus_std_um"),
        "annulus_min_um": float(min(float(x["annulus_min_um"]) for x in per_ensemble)),
        "annulus_max_um": float(max(float(x["annulus_max_um"]) for x in per_ensemble)),
        "annulus_q05_um": vw("annulus_q05_um"), "annulus_q50_um": vw("annulus_q50_um"),
        "annulus_q95_um": vw("annulus_q95_um"), "n_seeds_sim": int(n_cells),
        "sim_side_um": [float(x["sim_side_um"]) for x in per_ensemble],
        "source_side_um": [float(x["source_side_um"]) for x in per_ensemble],
    }


def ensemble_mean_subset_column_indices(columns) -> np.ndarray:
    """Full-vector indices of the declared v5 subset (8 pairs x the 25-value b grid)."""
    if not np.array_equal(np.asarray(columns.b_values, float), np.asarray(ENSEMBLE_MEAN_SUBSET_B_VALUES_S_MM2, float)):
        raise ValueError("madi-library-v5 requires the declared 25-point b grid for the per-ensemble "
                         "covariance diagnostic subset")
    where = {(float(a), float(b)): i for i, (a, b) in enumerate(columns.delta_pairs)}
    if len(where) != len(columns.delta_pairs):
        raise ValueError("main storage grid contains duplicate (delta, Delta) pairs")
    missing = [p for p in ENSEMBLE_MEAN_SUBSET_DELTA_PAIRS_MS if p not in where]
    if missing:
        raise ValueError(f"madi-library-v5 main storage grid omits declared ensemble-mean diagnostic pairs: {missing!r}")
    return np.array([where[p] * columns.n_b + b for p in ENSEMBLE_MEAN_SUBSET_DELTA_PAIRS_MS
                     for b in range(columns.n_b)], dtype=np.int64)


def _v5_diagnostics_from_result(result: dict, columns, cfg: SimConfig):
    """(signal_imag, between-ensemble sample variance, ensemble subset, imaginary check)."""
    er, ei = result.get("ensemble_S"), result.get("ensemble_S_imag")
    if er is None or ei is None:
        raise RuntimeError("v5 library build requires per-ensemble reduced signals")
    er, ei = np.asarray(er, np.float64), np.asarray(ei, np.float64)
    shape = (int(cfg.n_ensembles), columns.n_pairs, columns.n_b)
    if er.shape != shape or ei.shape != shape:
        raise RuntimeError(f"per-ensemble reduced signal shape does not match the configured ensemble/grid "
                           f"contract: got real={er.shape}, imag={ei.shape}, expected={shape}")
    if not (np.all(np.isfinite(er)) and np.all(np.isfinite(ei))):
        raise RuntimeError("per-ensemble reduced signals contain non-finite values")
    if int(cfg.n_ensembles) < 2:
        raise ValueError("madi-library-v5 requires at least two ensembles for sample variance")
    imag = np.asarray(result["S_imag"], np.float64).reshape(columns.n_pairs, columns.n_b)
    var = np.var(er, axis=0, ddof=1)
    subset = er.reshape(int(cfg.n_ensembles), -1)[:, ensemble_mean_subset_column_indices(columns)]
    im_mean = np.mean(ei, axis=0)
    im_se = np.std(ei, axis=0, ddof=1) / np.sqrt(cfg.n_ensembles)
    z = np.zeros_like(im_mean)
    pos = im_se > 0.0
    z[pos] = np.abs(im_mean[pos] / im_se[pos])
    zero_nonzero = (~pos) & (np.abs(im_mean) > 0.0)
    z[zero_nonzero] = np.inf
    k = int(np.argmax(z))
    pi, bi = np.unravel_index(k, z.shape)
    check = {
        "method": "absolute Student statistic of the mean of independent per-ensemble imaginary signals (ddof=1)",
        "n_ensembles": int(cfg.n_ensembles), "degrees_of_freedom": int(cfg.n_ensembles - 1),
        "max_abs_standardized_deviation": float(z.flat[k]),
        "max_column": {"delta_ms": float(columns.delta_pairs[pi][0]), "Delta_ms": float(columns.delta_pairs[pi][1]),
                       "b_s_mm2": float(columns.b_values[bi])},
        "mean_imaginary_signal": float(im_mean.flat[k]), "standard_error": float(im_se.flat[k]),
        "zero_standard_error_nonzero_count": int(np.count_nonzero(zero_nonzero)),
    }
    return (imag.astype(np.float32).ravel(), var.astype(np.float32).ravel(), subset.astype(np.float32), check)


# ---------------------------------------------------------------------------
# Builder
# ---------------------------------------------------------------------------

def build_library_from_triplets(triplets, cfg: Optional[SimConfig] = None, save_path: Optional[str] = None,
                                existing_library=None, seed: int = 0, vi_min: float = 0.0,
                                vi_max: float = VI_HARD_MAX, entry_weights: Optional[Mapping] = None,
                                grid_metadata: Optional[dict] = None, verbose: bool = True, *,
                                v5_diagnostics: bool = True, max_jobs_per_launch: int = 4096,
                                ensemble_threads: int = 8, launch=None) -> list:
    """Build or extend a library from (kio, rho, V) triplets (madi/library.py:445-642).

    Entries already present (by nominal key) are skipped.  Geometry seeds come
    from (seed, ensemble index) only, so neighbouring (rho, V) entries share
    common random numbers.  All (group, ensemble, k_io) walks of a chunk run in
    one persistent launch; the npz is written after every chunk.
    ``v5_diagnostics=False`` (GB300 addition) stores a v4 artifact, for column
    grids without the declared 25-value b grid.
    """
    from .walker_gpu import (WalkJob, _build_ensembles_for_entry, _merge_results, _pp_for, _walk_seed,
                             results_to_reduced, simulate_jobs)
    if cfg is None:
        cfg = SimConfig()
    if v5_diagnostics and int(cfg.n_ensembles) < 2:
        raise ValueError("madi-library-v5 requires at least two independently constructed ensembles so that "
                         "per-column sample variance is defined")
    library = list(existing_library) if existing_library is not None else []
    done = _existing_keys(library)
    if library and v5_diagnostics and not all(
            e.signal_imag is not None and e.signal_variance is not None and e.ensemble_means_subset is not None
            for e in library):
        raise ValueError("cannot append v5 entries to a pre-v5 library: the existing artifact lacks required "
                         "Monte-Carlo diagnostic arrays")
    valid = _filter_valid(triplets, vi_min=vi_min, vi_max=vi_max)
    new = [t for t in valid if _entry_key(*t) not in done]
    if verbose:
        print(f"  Requested: {len(triplets)} triplets; skipped {len(triplets) - len(valid)} (v_i) + "
              f"{len(valid) - len(new)} (existing); new {len(new)}")
    if not new:
        if save_path:
            _save_library(library, save_path, cfg=cfg, grid_metadata=grid_metadata, build_seed=seed)
        return library
    columns = sig.build_columns(cfg)
    if v5_diagnostics:
        ensemble_mean_subset_column_indices(columns)
    groups = defaultdict(list)
    for k, r, v in new:
        groups[(r, v)].append(k)
    order = sorted(groups.items(), key=lambda kv: kv[0][0] * kv[0][1])
    t0 = time.time()
    # ensembles of every group (host construction in parallel threads)
    with ThreadPoolExecutor(max_workers=max(1, ensemble_threads)) as ex:
        ens_by_group = list(ex.map(lambda g: _build_ensembles_for_entry(g[0][0], g[0][1], cfg, seed, False), order))
    cols = (columns.j_delta, columns.j_Delta, columns.j_sum, columns.phase_coef)
    jobs, keys = [], []
    for gi, ((rho, V), kios) in enumerate(order):
        for e, ens in enumerate(ens_by_group[gi]):
            for k in sorted(kios):
                jobs.append(WalkJob(ens, _pp_for(ens, k, cfg), _walk_seed(seed, e), int(cfg.n_walkers)))
                keys.append((gi, e, k))
    per_entry = defaultdict(list)
    for a in range(0, len(jobs), max_jobs_per_launch):
        chunk = jobs[a:a + max_jobs_per_launch]
        res = simulate_jobs(chunk, cfg, cols, launch=launch)
        for (gi, e, k), job, r in zip(keys[a:a + max_jobs_per_launch], chunk, res):
            per_entry[(gi, k)].append((e, results_to_reduced(job.ensemble, job.pp, cfg, r, job.n_walkers)))
        if verbose:
            print(f"    walked {min(a + max_jobs_per_launch, len(jobs))}/{len(jobs)} jobs ({time.time() - t0:.1f}s)")
    for gi, ((rho, V), kios) in enumerate(order):
        for k in sorted(kios):
            parts = [r for _, r in sorted(per_entry[(gi, k)], key=lambda t: t[0])]
            result = sig._assemble(_merge_results(parts), columns)
            library.append(_entry_from_result(result, columns, cfg, k, rho, V, entry_weights, v5_diagnostics))
    if save_path:
        _save_library(library, save_path, cfg=cfg, columns=columns, grid_metadata=grid_metadata, build_seed=seed)
    if verbose:
        print(f"Library: {len(library)} entries ({len(new)} new in {time.time() - t0:.1f}s)")
    return library


def _entry_from_result(result, columns, cfg, kio, rho, V, entry_weights, v5) -> LibraryEntry:
    vec = sig.signals_to_flat(result)
    imag = var = subset = None
    check = None
    if v5:
        imag, var, subset, check = _v5_diagnostics_from_result(result, columns, cfg)
    summary = _summarise_realised_geometry(result["geometry_stats"], cfg)
    free = rho == 0.0 and V == 0.0
    key = _entry_key(kio, rho, V)
    weight = None if entry_weights is None else entry_weights.get(key)
    meta = {
        "schema": MADI_LIBRARY_ENTRY_SCHEMA_V5,
        "nominal": {"kio": float(kio), "rho": float(rho), "V": float(V)},
        "realised_geometry": summary,
        "per_ensemble_geometry": result["geometry_stats"],
        "exchange": {"kio_analytic_eq5_s_inv": float(result["kio_analytic_eq5"]), "p_p_mean": float(result["pp"]),
                     "definition": "MADI I Eq. 5 using SI §S.IV untrimmed governing-process arithmetic <A/V>; "
                                   "no residence-time proxy is used."},
        "boundary": {"mode": cfg.boundary_mode, "n_escaped": int(result["n_escaped"]),
                     "n_walkers_total": int(result["n_eff"] // (len(cfg.direction_array()))),
                     "fatal_on_escape": cfg.boundary_mode == "si_fatal_escape",
                     "occupancy_fraction": np.asarray(result["occupancy_fraction"]).tolist()},
        "weight": None if weight is None else float(weight),
        "imaginary_signal_check": check,
    }
    return LibraryEntry(kio=float("nan") if free else float(kio), rho=0.0 if free else summary["rho_per_uL"],
                        V=0.0 if free else summary["mean_volume_pL"], vector=vec, signal_imag=imag,
                        signal_variance=var, ensemble_means_subset=subset, vi=0.0 if free else summary["vi"],
                        weight=None if weight is None else float(weight), kio_nominal=float(kio),
                        rho_nominal=float(rho), V_nominal=float(V), pp=float(result["pp"]),
                        kio_analytic_eq5=float(result["kio_analytic_eq5"]), is_free_water=free, metadata=meta)


def build_library(kios=None, rhos=None, Vs=None, cfg=None, save_path=None, existing_library=None, seed=0,
                  vi_min=0.0, vi_max=VI_HARD_MAX, entry_weights=None, grid_metadata=None, verbose=True, **kw):
    """Cross product kios x rhos x Vs through build_library_from_triplets."""
    kios = DEFAULT_KIOS if kios is None else kios
    rhos = DEFAULT_RHOS if rhos is None else rhos
    Vs = DEFAULT_VS if Vs is None else Vs
    trip = [(k, r, v) for k in kios for r in rhos for v in Vs]
    return build_library_from_triplets(trip, cfg=cfg, save_path=save_path, existing_library=existing_library,
                                       seed=seed, vi_min=vi_min, vi_max=vi_max, entry_weights=entry_weights,
                                       grid_metadata=grid_metadata, verbose=verbose, **kw)


# ---------------------------------------------------------------------------
# npz schema
# ---------------------------------------------------------------------------

def _json_default(value):
    if isinstance(value, np.generic):
        return value.item()
    if isinstance(value, np.ndarray):
        return value.tolist()
    raise TypeError(f"cannot JSON-serialise {type(value)!r}")


def _cfg_metadata(cfg: SimConfig, *, schema: str = MADI_LIBRARY_SCHEMA_V5, build_seed=None) -> dict:
    """Physics / build configuration embedded in the artifact (key set of madi/library.py:685-801)."""
    m = {
        "schema": schema, "D0_um2_ms": cfg.D0, "ts_ms": cfg.ts, "T_max_ms": cfg.T_max_ms,
        "domain_sizing": "MADI I SI Eq. S8; per-entry W unless diagnostic L override",
        "diagnostic_domain_L_override_um": cfg.L, "source_fraction": cfg.source_fraction,
        "boundary_mode": cfg.boundary_mode, "kappa": cfg.kappa,
        "population_certification": {"equations": ["S10", "S11", "S12"],
                                     "initial_margin_cell_spacings": cfg.population_initial_margin_cell_spacings,
                                     "certification_spacing_um": cfg.population_certification_spacing_um,
                                     "max_expansions": cfg.population_max_expansions},
        "geometry_reference": {"path": cfg.geometry_reference_path,
                               "required_single_cells": cfg.geometry_reference_required_cells,
                               "required_alpha_values": cfg.geometry_reference_required_alpha_values,
                               "allow_uncertified": cfg.allow_uncertified_geometry_reference,
                               "mean_estimator": "untrimmed_arithmetic_mean_A_over_V"},
        "geometry_validation_points": cfg.geometry_validation_points,
        "geometry_vi_tolerance": cfg.geometry_vi_tolerance,
        "walkers_per_ensemble": cfg.n_walkers, "ensembles_per_entry": cfg.n_ensembles,
        "axis_walks_per_entry": 3 * int(cfg.n_walkers) * int(cfg.n_ensembles),
        "build_seed": None if build_seed is None else int(build_seed), "phase_model": cfg.phase_model,
        "checkpoint_h_ms": cfg.h_ms,
        "common_random_numbers": "base_seed + ensemble_index; shared across rho,V,kio",
        "classifier": ("exact full-facet shifted-Voronoi contraction at every endpoint; SI Eq. S2, with the "
                       "provable d1+2*alpha1 adaptive KD radius bound" if cfg.classifier_mode == "exact" else
                       "exact full-facet shifted-Voronoi contraction with conservative two-tier proof cache; "
                       "SI Eq. S2 fallback uses the provable d1+2*alpha1 adaptive KD radius bound"),
        "classifier_cache": {
            "mode": cfg.classifier_mode,
            "equivalence_contract": ("cache hits are used only after a conservative proof; all other endpoints "
                                     "invoke the unchanged exact SI Eq. S2 classifier"),
            "tier1": "cumulative displacement from a fixed reference is strictly below a shifted-facet safety radius",
            "tier2": ("finite candidate superset radius d1_ref + 2*max(alpha) + 2*delta_max; overflow disables "
                      "the cache and falls back exact"),
            "delta_max_um": float(cfg.classifier_cache_delta_max_um),
            "min_safe_radius_um": float(cfg.classifier_cache_min_safe_radius_um),
            "candidate_capacity": int(cfg.classifier_cache_candidate_capacity)},
        "kio_label": "MADI I Eq. 5 with governing-process untrimmed arithmetic <A/V>",
        "residence_time_measurement": "intentionally absent: SI §S.IV states k_io != 1/<tau_i>",
    }
    if schema == MADI_LIBRARY_SCHEMA_V5:
        m["uncertainty"] = {
            "signal_imag": {"array": "signal_imag", "dtype": "float32", "shape": ["entry", "column"],
                            "definition": "collapsed mean(sin(phase)) over all axis-walks"},
            "between_ensemble_variance": {
                "array": "signal_variance", "dtype": "float32", "shape": ["entry", "column"],
                "definition": ("sample variance (ddof=1) of per-ensemble mean real signals; consumer SE is "
                               "sqrt(signal_variance / n_ensembles)"),
                "n_ensembles": int(cfg.n_ensembles)},
            "ensemble_means_subset": {
                "array": "ensemble_means_subset", "dtype": "float32",
                "shape": ["entry", "ensemble_index", "declared_column"],
                "declared_delta_Delta_pairs_ms": [[float(a), float(b)] for a, b in ENSEMBLE_MEAN_SUBSET_DELTA_PAIRS_MS],
                "declared_b_values_s_mm2": np.asarray(ENSEMBLE_MEAN_SUBSET_B_VALUES_S_MM2, float).tolist(),
                "column_order": "pair-major, then b-major within each pair"},
            "ensemble_index_ordering_contract": {
                "axis_position_in_ensemble_means_subset": 1, "index_values": "0..n_ensembles-1",
                "same_order_across_entries": True, "independent_of": ["rho", "V", "k_io"],
                "walk_seed_formula": "(build_seed + 104729 * ensemble_index) mod 2^31",
                "geometry_seed_formula": "(build_seed + 97003 * ensemble_index) mod 2^31",
                "purpose": "ensemble index e is the common-random-number partner across entries"},
        }
    return m


def _v5_entry_arrays(lib: list, n_columns: int):
    have = [e.signal_imag is not None and e.signal_variance is not None and e.ensemble_means_subset is not None
            for e in lib]
    if not any(have):
        return None
    if not all(have):
        raise ValueError("library mixes entries with and without v5 Monte-Carlo diagnostics")
    im, va, su = [], [], []
    n_ens = None
    for i, e in enumerate(lib):
        a, b, c = np.asarray(e.signal_imag), np.asarray(e.signal_variance), np.asarray(e.ensemble_means_subset)
        if a.shape != (n_columns,):
            raise ValueError(f"entry {i} signal_imag shape {a.shape} != ({n_columns},)")
        if b.shape != (n_columns,):
            raise ValueError(f"entry {i} signal_variance shape {b.shape} != ({n_columns},)")
        if c.ndim != 2 or c.shape[1] != ENSEMBLE_MEAN_SUBSET_N_COLUMNS:
            raise ValueError(f"entry {i} ensemble_means_subset shape {c.shape} != (n_ensembles, "
                             f"{ENSEMBLE_MEAN_SUBSET_N_COLUMNS})")
        if n_ens is None:
            n_ens = c.shape[0]
        elif c.shape[0] != n_ens:
            raise ValueError("v5 entries disagree on the number of ensembles")
        if n_ens < 2:
            raise ValueError("v5 diagnostic arrays require at least two ensembles")
        if not (np.all(np.isfinite(a)) and np.all(np.isfinite(b)) and np.all(np.isfinite(c))):
            raise ValueError(f"entry {i} has non-finite v5 diagnostic values")
        if np.any(b < 0.0):
            raise ValueError(f"entry {i} has negative between-ensemble variance")
        im.append(a.astype(np.float32)); va.append(b.astype(np.float32)); su.append(c.astype(np.float32))
    out = np.stack(im), np.stack(va), np.stack(su)
    if not all(np.all(np.isfinite(x)) for x in out):
        raise ValueError("float32 conversion made v5 diagnostic values non-finite")
    if np.any(out[1] < 0.0):
        raise ValueError("float32 conversion made between-ensemble variance negative")
    return out


def _save_library(lib: list, path: str, cfg: Optional[SimConfig] = None, columns=None,
                  grid_metadata: Optional[dict] = None, build_metadata: Optional[dict] = None, build_seed=None):
    """Write the npz artifact (key set and dtypes of madi/library.py:940-971)."""
    cfg = cfg or SimConfig()
    columns = columns or sig.build_columns(cfg)
    n_cols = int(columns.n_pairs * columns.n_b)
    v5 = _v5_entry_arrays(lib, n_cols)
    schema = MADI_LIBRARY_SCHEMA_V5 if v5 is not None else MADI_LIBRARY_SCHEMA_V4

    def col(f, default=np.nan):
        return np.array([default if f(e) is None else f(e) for e in lib], dtype=float)
    meta = dict(build_metadata) if build_metadata is not None else {
        **_cfg_metadata(cfg, schema=schema, build_seed=build_seed), "grid": grid_metadata or {}}
    if meta.get("schema") != schema:
        raise ValueError(f"library-schema mismatch between entries and build metadata: entries imply {schema!r}, "
                         f"metadata has {meta.get('schema')!r}")
    if grid_metadata is not None:
        meta["grid"] = grid_metadata
    weights = col(lambda e: e.weight)
    payload = dict(
        library_schema=np.array(schema),
        kios=col(lambda e: e.kio), rhos=col(lambda e: e.rho), Vs=col(lambda e: e.V),
        vis=np.array([e.realised_vi for e in lib], float), vectors=np.array([e.vector for e in lib]),
        nominal_kios=np.array([e.kio if e.kio_nominal is None else e.kio_nominal for e in lib], float),
        nominal_rhos=np.array([e.rho if e.rho_nominal is None else e.rho_nominal for e in lib], float),
        nominal_Vs=np.array([e.V if e.V_nominal is None else e.V_nominal for e in lib], float),
        weights=weights, has_weights=np.array(bool(np.all(np.isfinite(weights)))),
        pps=col(lambda e: e.pp), kio_analytic_eq5=col(lambda e: e.kio_analytic_eq5),
        is_free_water=np.array([e.is_free_water for e in lib], dtype=np.bool_),
        entry_metadata_json=np.array([json.dumps(e.metadata, sort_keys=True, default=_json_default) for e in lib]),
        build_metadata_json=np.array(json.dumps(meta, sort_keys=True, default=_json_default)),
        pair_deltas=np.array([a for a, _ in columns.delta_pairs], float),
        pair_Deltas=np.array([b for _, b in columns.delta_pairs], float),
        b_values=np.asarray(columns.b_values, float), n_b=np.array(columns.n_b), h_ms=np.array(float(cfg.h_ms)),
    )
    if v5 is not None:
        payload.update(signal_imag=v5[0], signal_variance=v5[1], ensemble_means_subset=v5[2],
                       ensemble_subset_pair_deltas=np.array([a for a, _ in ENSEMBLE_MEAN_SUBSET_DELTA_PAIRS_MS], float),
                       ensemble_subset_pair_Deltas=np.array([b for _, b in ENSEMBLE_MEAN_SUBSET_DELTA_PAIRS_MS], float),
                       ensemble_subset_b_values=np.asarray(ENSEMBLE_MEAN_SUBSET_B_VALUES_S_MM2, float),
                       ensemble_subset_n_b=np.array(len(ENSEMBLE_MEAN_SUBSET_B_VALUES_S_MM2)))
    np.savez(path, **payload)


def load_library(path: str) -> list:
    """Entries of an npz artifact (v5, v4 or legacy); every array is read once."""
    with np.load(path) as z:
        data = {k: z[k] for k in z.files}
    n = len(data["kios"])

    def opt(name, default):
        return data[name] if name in data else default
    vis = opt("vis", np.asarray([None] * n, dtype=object))
    weights = opt("weights", np.full(n, np.nan))
    nk, nr, nv = opt("nominal_kios", data["kios"]), opt("nominal_rhos", data["rhos"]), opt("nominal_Vs", data["Vs"])
    pps = opt("pps", np.full(n, np.nan))
    eq5 = opt("kio_analytic_eq5", np.full(n, np.nan))
    free = opt("is_free_water", np.zeros(n, bool))
    ej = opt("entry_metadata_json", np.asarray(["{}"] * n))
    diag = [opt(k, None) for k in ("signal_imag", "signal_variance", "ensemble_means_subset")]
    if any(x is not None for x in diag) and not all(x is not None for x in diag):
        raise ValueError(f"{path}: incomplete v5 Monte-Carlo diagnostic arrays")
    if diag[0] is not None and any(x.shape[0] != n for x in diag):
        raise ValueError(f"{path}: v5 Monte-Carlo diagnostic entry axis has wrong length")
    out = []
    for i in range(n):
        try:
            meta = json.loads(str(ej[i]))
        except (TypeError, ValueError):
            meta = {}
        out.append(LibraryEntry(
            kio=float(data["kios"][i]), rho=float(data["rhos"][i]), V=float(data["Vs"][i]), vector=data["vectors"][i],
            signal_imag=None if diag[0] is None else diag[0][i], signal_variance=None if diag[1] is None else diag[1][i],
            ensemble_means_subset=None if diag[2] is None else diag[2][i],
            vi=None if vis.dtype == object or not np.isfinite(vis[i]) else float(vis[i]),
            weight=None if not np.isfinite(weights[i]) else float(weights[i]),
            kio_nominal=float(nk[i]), rho_nominal=float(nr[i]), V_nominal=float(nv[i]),
            pp=None if not np.isfinite(pps[i]) else float(pps[i]),
            kio_analytic_eq5=None if not np.isfinite(eq5[i]) else float(eq5[i]),
            is_free_water=bool(free[i]), metadata=meta))
    return out


def load_library_meta(path: str) -> dict:
    """Column-grid metadata of an artifact, legacy fixed-delta files normalised to delta_pairs."""
    with np.load(path) as z:
        files = set(z.files)
        get = {k: z[k] for k in files}
    meta = {}
    if "library_schema" in files:
        meta["library_schema"] = str(get["library_schema"])
    meta["has_weights"] = bool(get["has_weights"]) if "has_weights" in files else False
    if "build_metadata_json" in files:
        try:
            meta["build_metadata"] = json.loads(str(get["build_metadata_json"]))
        except (TypeError, ValueError):
            meta["build_metadata"] = None
    if "pair_deltas" in files and "pair_Deltas" in files:
        meta["format"] = "v2"
        meta["delta_pairs"] = list(zip(np.asarray(get["pair_deltas"], float).tolist(),
                                       np.asarray(get["pair_Deltas"], float).tolist()))
        meta["n_b"] = int(get["n_b"]) if "n_b" in files else None
        meta["b_values"] = list(np.asarray(get["b_values"], float)) if "b_values" in files else None
        meta["h_ms"] = float(get["h_ms"]) if "h_ms" in files else None
        meta["has_free_water"] = bool(np.any(get["is_free_water"])) if "is_free_water" in files else False
        names = {"signal_imag", "signal_variance", "ensemble_means_subset", "ensemble_subset_pair_deltas",
                 "ensemble_subset_pair_Deltas", "ensemble_subset_b_values", "ensemble_subset_n_b"}
        meta["has_v5_diagnostics"] = names <= files
        if meta["has_v5_diagnostics"]:
            meta["signal_imag_shape"] = tuple(get["signal_imag"].shape)
            meta["signal_variance_shape"] = tuple(get["signal_variance"].shape)
            meta["ensemble_means_subset_shape"] = tuple(get["ensemble_means_subset"].shape)
            meta["ensemble_subset_delta_pairs"] = list(zip(
                np.asarray(get["ensemble_subset_pair_deltas"], float).tolist(),
                np.asarray(get["ensemble_subset_pair_Deltas"], float).tolist()))
            meta["ensemble_subset_b_values"] = list(np.asarray(get["ensemble_subset_b_values"], float))
            meta["ensemble_subset_n_b"] = int(get["ensemble_subset_n_b"])
        return meta
    meta["format"] = "legacy"
    deltas = list(get["deltas"]) if "deltas" in files else list(DELTAS_BIG)
    n_b = int(get["n_b"]) if "n_b" in files else len(BVALS_UNIQUE)
    small = float(get["small_delta"]) if "small_delta" in files else DELTA_SMALL
    meta["delta_pairs"] = [(small, D) for D in deltas]
    meta["n_b"] = n_b
    meta["b_values"] = (list(np.asarray(get["b_values"], float)) if "b_values" in files
                        else (list(BVALS_UNIQUE.astype(float)) if n_b == len(BVALS_UNIQUE) else None))
    meta["small_delta"] = small
    meta["h_ms"] = None
    meta["has_v5_diagnostics"] = False
    return meta


def library_summary(lib: list, meta: Optional[dict] = None):
    if not lib:
        print("  (empty library)")
        return
    cell = [e for e in lib if not e.is_free_water]
    print(f"  Entries: {len(lib)}  cellular: {len(cell)}  free-water atom: {any(e.is_free_water for e in lib)}")
    if cell:
        print(f"  kio {min(e.kio for e in cell):g}-{max(e.kio for e in cell):g}, "
              f"rho {min(e.rho for e in cell):g}-{max(e.rho for e in cell):g}, "
              f"V {min(e.V for e in cell):g}-{max(e.V for e in cell):g}, "
              f"vi {min(e.realised_vi for e in cell):.3f}-{max(e.realised_vi for e in cell):.3f}")
    print(f"  Vector length: {lib[0].vector.size}")
    if meta is not None:
        print(f"  Format: {meta.get('format', '?')}  pairs: {len(meta['delta_pairs'])}  n_b: {meta['n_b']}")


# ---------------------------------------------------------------------------
# Column resolution, candidate matrix, matching
# ---------------------------------------------------------------------------

B_SNAP_TOL_S_MM2 = 30.0
TIMING_SNAP_TOL_MS = 1.5


def _nearest_pair_index(delta: float, Delta: float, lib_pairs: np.ndarray) -> int:
    return int(np.argmin((lib_pairs[:, 0] - delta) ** 2 + (lib_pairs[:, 1] - Delta) ** 2))


def resolve_grid_columns(fit_triples, lib_delta_pairs, lib_b_values, n_b, b_tol=B_SNAP_TOL_S_MM2,
                         timing_tol=TIMING_SNAP_TOL_MS):
    """Nearest stored column of every (delta, Delta, b) request within the snap tolerances."""
    if lib_b_values is None:
        raise ValueError("Library has no stored b-values. Rebuild the library with the current _save_library, "
                         "or pass lib_b_values explicitly.")
    pairs = np.asarray(lib_delta_pairs, float)
    bvals = np.asarray(lib_b_values, float)
    cols = np.empty(len(fit_triples), dtype=int)
    events, seen_t, seen_b = [], set(), set()
    for i, (delta, Delta, b) in enumerate(fit_triples):
        p = _nearest_pair_index(delta, Delta, pairs)
        nd, nD = pairs[p]
        od, oD = abs(float(nd - delta)), abs(float(nD - Delta))
        if od > timing_tol or oD > timing_tol:
            raise ValueError(f"(δ={delta:g}, Δ={Delta:g}) ms is outside the {timing_tol:g} ms timing snap tolerance; "
                             f"nearest stored pair is (δ={nd:g}, Δ={nD:g}) ms. No interpolation is implemented.")
        key = (float(delta), float(Delta), float(nd), float(nD))
        if (od > 1e-12 or oD > 1e-12) and key not in seen_t:
            seen_t.add(key)
            events.append({"axis": "timing", "requested": {"delta_ms": float(delta), "Delta_ms": float(Delta)},
                           "used": {"delta_ms": float(nd), "Delta_ms": float(nD)},
                           "abs_offset": {"delta_ms": od, "Delta_ms": oD},
                           "rel_offset": {"delta": od / max(abs(float(delta)), 1e-12),
                                          "Delta": oD / max(abs(float(Delta)), 1e-12)}})
        bi = int(np.argmin(np.abs(bvals - b)))
        bu = float(bvals[bi])
        ob = abs(bu - float(b))
        if ob > b_tol:
            raise ValueError(f"b = {b} s/mm² not within {b_tol:g} of any library b-value {sorted(lib_b_values)}.")
        if ob > 1e-12 and (float(b), bu) not in seen_b:
            seen_b.add((float(b), bu))
            events.append({"axis": "b", "requested": float(b), "used": bu, "abs_offset": ob,
                           "rel_offset": ob / max(abs(float(b)), 1e-12)})
        cols[i] = p * n_b + bi
    return cols, events


def _grid_columns(fit_triples, lib_delta_pairs, lib_b_values, n_b, b_tol=B_SNAP_TOL_S_MM2,
                  pair_warn_tol=TIMING_SNAP_TOL_MS):
    return resolve_grid_columns(fit_triples, lib_delta_pairs, lib_b_values, n_b, b_tol=b_tol,
                                timing_tol=pair_warn_tol)[0]


def _candidate_mask(library, vi_min, vi_max, rho_max, include_free_water):
    vis = np.array([e.realised_vi for e in library])
    rhos = np.array([e.rho for e in library])
    free = np.array([e.is_free_water for e in library], bool)
    mask = (vis >= vi_min) & (vis <= vi_max)
    mask = (mask | free) if include_free_water else (mask & ~free)
    if rho_max is not None:
        mask &= rhos <= rho_max
    return mask


def _build_candidate_lib_matrix(library, lib_delta_pairs, lib_b_values, n_b, vi_min, vi_max, rho_max, fit_triples,
                                *, include_free_water=False, return_weights=False, require_weights=False):
    """(lib_mat [n_candidates, n_features], kios, rhos, Vs[, weights]) of the filtered library."""
    mask = _candidate_mask(library, vi_min, vi_max, rho_max, include_free_water)
    n = int(mask.sum())
    if n == 0:
        raise ValueError(f"No library entries survive vi in [{vi_min}, {vi_max}] and rho <= {rho_max}.")
    if n < 50:
        import warnings
        warnings.warn(f"Only {n} library entries pass the filter.")
    ents = [e for e, m in zip(library, mask) if m]
    mat = np.array([e.vector for e in ents])[:, _grid_columns(fit_triples, lib_delta_pairs, lib_b_values, n_b)]
    out = (mat, np.array([e.kio for e in ents]), np.array([e.rho for e in ents]), np.array([e.V for e in ents]))
    if not return_weights:
        return out
    w = np.array([np.nan if e.weight is None else float(e.weight) for e in ents], float)
    if require_weights and not np.all(np.isfinite(w) & (w > 0.0)):
        raise ValueError("Bayesian fitting requires positive per-entry quadrature weights. This library is "
                         "legacy/unweighted; rebuild it with the remediation grid.")
    return (*out, w)


def edge_railing_diagnostics(kio_values, rho_values, V_values, library, *, vi_min, vi_max, rho_max=None,
                             include_free_water=False) -> dict:
    """Fraction of fits at the realised candidate-library edges (free water reported apart)."""
    vis = np.asarray([e.realised_vi for e in library], float)
    rhos = np.asarray([e.rho for e in library], float)
    free = np.asarray([e.is_free_water for e in library], bool)
    cand = (vis >= float(vi_min)) & (vis <= float(vi_max)) & ~free
    if include_free_water:
        cand |= free
    if rho_max is not None:
        cand &= rhos <= float(rho_max)
    cell = [e for e, k in zip(library, cand) if k and not e.is_free_water]
    if not cell:
        raise ValueError("edge diagnostic has no cellular candidate entries")
    kio, rho, vol = (np.asarray(x, float) for x in (kio_values, rho_values, V_values))
    if not (kio.shape == rho.shape == vol.shape):
        raise ValueError("kio, rho and V diagnostic arrays must have the same shape")
    n = int(kio.size)
    fw = (~np.isfinite(kio)) & (rho == 0.0) & (vol == 0.0)

    def one(vals, grid):
        fin = np.isfinite(vals) & ~fw
        lo, hi = float(np.min(grid)), float(np.max(grid))
        a = fin & np.isclose(vals, lo, rtol=1e-10, atol=1e-12)
        b = fin & np.isclose(vals, hi, rtol=1e-10, atol=1e-12)
        d = max(n, 1)
        return {"lower_value": lo, "upper_value": hi, "at_lower_count": int(a.sum()), "at_upper_count": int(b.sum()),
                "at_lower_fraction": float(a.sum() / d), "at_upper_fraction": float(b.sum() / d)}
    return {"n_voxels": n, "free_water_count": int(fw.sum()), "free_water_fraction": float(fw.sum() / max(n, 1)),
            "rho": one(rho, np.array([e.rho for e in cell])), "V": one(vol, np.array([e.V for e in cell])),
            "kio": one(kio, np.array([e.kio for e in cell]))}


def _check_gpu(use_gpu):
    from . import fitters_gpu
    if use_gpu is False:
        raise RuntimeError("custom_madi_gb300 matches on the GPU only (use_gpu=False)")
    if not fitters_gpu.HAS_CUDA:
        raise RuntimeError("use_gpu=True but CUDA is not available.")
    return fitters_gpu


def match_voxels_batch(measured_batch, library, lib_delta_pairs, lib_b_values, n_b, fit_triples, log_space=False,
                       s_floor=1e-3, vi_min=0.5, vi_max=0.95, rho_max=None, include_free_water=False, use_gpu=None,
                       *, precision: str = "fp32"):
    """Fixed-S0 nearest library entry per voxel: (kio, rho, V, residual)."""
    fg = _check_gpu(use_gpu)
    mat, k, r, v = _build_candidate_lib_matrix(library, lib_delta_pairs, lib_b_values, n_b, vi_min, vi_max, rho_max,
                                               fit_triples, include_free_water=include_free_water)
    if log_space:
        meas = np.log(np.clip(measured_batch, s_floor, 1.0))
        mat = np.log(np.clip(mat, s_floor, 1.0))
    else:
        meas = measured_batch
    return fg.map_match_gpu(meas, mat, k, r, v, precision=precision)


def match_voxels_batch_fits0(raw_signal, library, lib_delta_pairs, lib_b_values, n_b, fit_triples, vi_min=0.5,
                             vi_max=0.95, rho_max=None, include_free_water=False, use_gpu=None, *,
                             precision: str = "fp32"):
    """Free-S0 nearest library entry per voxel: (kio, rho, V, residual, S0)."""
    fg = _check_gpu(use_gpu)
    mat, k, r, v = _build_candidate_lib_matrix(library, lib_delta_pairs, lib_b_values, n_b, vi_min, vi_max, rho_max,
                                               fit_triples, include_free_water=include_free_water)
    return fg.map_match_fits0_gpu(raw_signal, mat, k, r, v, precision=precision)
