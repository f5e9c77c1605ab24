"""Bayesian posterior-mean fitting over the library (madi/fitters.py:1-335 interface).

``bayes_fit`` weights every candidate entry by its quadrature weight times a
Gaussian likelihood of its residual, exp(-r / (2 sigma_m^2)), and reports the
posterior mean and standard deviation of (kio, rho, V), the weighted residual
and n_eff = 1 / sum(w^2) (weights normalised); ``fit_s0=True`` fits S0 per
candidate (negative S0 weighs 0) and reports the weighted S0.  It runs on the
GPU (``madi_bayes``); ``use_gpu=False`` raises.  ``calibrate_sigma_m`` bisects
sigma_m on a voxel subsample so the median n_eff hits a target
(madi/fitters.py:246-333).  The AMICO regression of the reference is not part
of this package.
"""

from __future__ import annotations

from typing import Optional

import numpy as np

from .library import _build_candidate_lib_matrix
from . import fitters_gpu

DEFAULT_SIGMA_M = 0.02


def _weighted_mean_std(w, kios, rhos, Vs) -> dict:
    """Posterior mean / std of each parameter from row-normalised weights [n_vox, n_lib]."""
    out = {}
    for name, vals in (("kio", kios), ("rho", rhos), ("V", Vs)):
        mean = w @ vals
        var = np.maximum(w @ (np.asarray(vals) ** 2) - mean ** 2, 0.0)
        out[f"{name}_mean"] = mean
        out[f"{name}_std"] = np.sqrt(var)
    return out


def estimate_sigma_m(sigma_rician, s0_median, mean_n_dir) -> Optional[float]:
    """sigma_m ~ sigma_rician / (S0_median sqrt(mean_n_dir)) on the normalised signal."""
    if sigma_rician is None or s0_median is None or s0_median <= 0:
        return None
    return float(sigma_rician) / (float(s0_median) * np.sqrt(max(float(mean_n_dir), 1.0)))


def bayes_fit(measured_batch, library, *, sigma_m, lib_delta_pairs, lib_b_values, n_b, fit_triples, vi_min=0.5,
              vi_max=0.95, rho_max=None, include_free_water=False, log_space=False, s_floor=1e-3, fit_s0=False,
              raw_signal=None, use_gpu=None) -> dict:
    """Posterior means / stds of (kio, rho, V) per voxel (madi/fitters.py:110-243)."""
    lib_mat, kios, rhos, Vs, q = _build_candidate_lib_matrix(
        library, lib_delta_pairs, lib_b_values, n_b, vi_min, vi_max, rho_max, fit_triples,
        include_free_water=include_free_water, return_weights=True, require_weights=True)
    if sigma_m <= 0:
        raise ValueError(f"sigma_m must be > 0, got {sigma_m}")
    if use_gpu is False:
        raise RuntimeError("custom_madi_gb300 fits on the GPU only (use_gpu=False)")
    if not fitters_gpu.HAS_CUDA:
        raise RuntimeError("use_gpu=True but CUDA is not available.")
    if fit_s0:
        if raw_signal is None:
            raise ValueError("fit_s0=True requires raw_signal.")
        return fitters_gpu.bayes_fit_gpu(np.asarray(raw_signal, np.float64), lib_mat, kios, rhos, Vs, sigma_m,
                                         fit_s0=True, quadrature_weights=q)
    if log_space:
        meas = np.log(np.clip(measured_batch, s_floor, 1.0))
        lib_m = np.log(np.clip(lib_mat, s_floor, 1.0))
    else:
        meas, lib_m = np.asarray(measured_batch, np.float64), np.asarray(lib_mat, np.float64)
    return fitters_gpu.bayes_fit_gpu(meas, lib_m, kios, rhos, Vs, sigma_m, fit_s0=False, quadrature_weights=q)


def calibrate_sigma_m(measured_batch, library, *, lib_delta_pairs, lib_b_values, n_b, fit_triples, target_n_eff,
                      fit_s0=False, raw_signal=None, vi_min=0.5, vi_max=0.95, rho_max=None, sigma_lo=1e-5,
                      sigma_hi=1.0, n_iter=25, sample_size=1500, rng_seed=0, use_gpu=None, verbose=True) -> float:
    """Bisect log sigma_m so that the median n_eff of a voxel subsample hits target_n_eff
    (n_eff grows monotonically with sigma_m)."""
    if target_n_eff <= 0:
        raise ValueError(f"target_n_eff must be > 0, got {target_n_eff}")
    if fit_s0 and raw_signal is None:
        raise ValueError("fit_s0=True requires raw_signal.")
    n_vox = measured_batch.shape[0]
    n_sample = min(sample_size, n_vox)
    idx = np.random.default_rng(rng_seed).choice(n_vox, size=n_sample, replace=False)
    meas = measured_batch[idx]
    raw = raw_signal[idx] if fit_s0 else None

    def median_n_eff(sigma):
        n_eff = bayes_fit(meas, library, sigma_m=sigma, lib_delta_pairs=lib_delta_pairs, lib_b_values=lib_b_values,
                          n_b=n_b, fit_triples=fit_triples, vi_min=vi_min, vi_max=vi_max, rho_max=rho_max,
                          fit_s0=fit_s0, raw_signal=raw, use_gpu=use_gpu)["n_eff"]
        valid = n_eff[n_eff > 0]
        return float(np.median(valid)) if valid.size else 0.0

    lo_n, hi_n = median_n_eff(sigma_lo), median_n_eff(sigma_hi)
    if not (lo_n <= target_n_eff <= hi_n):
        raise ValueError(f"target_n_eff={target_n_eff:g} is outside the achievable range [{lo_n:g}, {hi_n:g}] for "
                         f"sigma_m in [{sigma_lo:g}, {sigma_hi:g}] on this {n_sample}-voxel sample; widen "
                         f"sigma_lo/sigma_hi.")
    a, b = np.log(sigma_lo), np.log(sigma_hi)
    for i in range(n_iter):
        mid = 0.5 * (a + b)
        n_mid = median_n_eff(float(np.exp(mid)))
        if verbose:
            print(f"    calibrate_sigma_m [{i + 1}/{n_iter}]: sigma_m={np.exp(mid):.4g} -> median n_eff={n_mid:.1f} "
                  f"(target {target_n_eff:g})")
        if n_mid < target_n_eff:
            a = mid
        else:
            b = mid
    return float(np.exp(0.5 * (a + b)))
