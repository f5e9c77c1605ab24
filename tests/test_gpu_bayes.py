"""Bayesian posterior-mean fit (madi_bayes) against the reference's bayes_fit
(fixture made by the reference's CPU path, madi/fitters.py:110-243) and
against the oracle's fp64 restatement on larger libraries.

Tolerance: the kernel's log-weights carry an fp32 error of ~1e-5-1e-4 at
these sigma_m, so posterior means and standard deviations are compared to
1e-3 of the posterior standard deviation (plus 1e-6 of the mean), n_eff and
the weighted residual to a relative 1e-3.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(got: dict, want: dict, tag: str):
    for name in ("kio", "rho", "V"):
        sd = np.asarray(want[f"{name}_std"])
        mean = np.asarray(want[f"{name}_mean"])
        tol = 1e-3 * sd + 1e-6 * np.abs(mean) + 1e-12
        for key in (f"{name}_mean", f"{name}_std"):
            d = np.abs(np.asarray(got[key]) - np.asarray(want[key]))
            assert np.all(d <= tol), (tag, key, float((d / tol).max()))
    np.testing.assert_allclose(got["n_eff"], want["n_eff"], rtol=1e-3, err_msg=tag)
    np.testing.assert_allclose(got["residual"], want["residual"], rtol=1e-3, atol=1e-9, err_msg=tag)
    if "s0_fit" in want:
        np.testing.assert_allclose(got["s0_fit"], want["s0_fit"], rtol=1e-4, err_msg=tag)


def test_bayes_fit_matches_reference_fixture():
    """Through the drop-in API: LibraryEntry list, candidate filter, quadrature weights."""
    import pathlib
    from custom_madi_gb300.fitters import bayes_fit
    from custom_madi_gb300.library import LibraryEntry
    b = dict(np.load(pathlib.Path(__file__).parent / "golden" / "bayes.npz"))
    ents = [LibraryEntry(float(k), float(r), float(v), b["lib"][i], vi=float(vi), weight=float(w))
            for i, (k, r, v, vi, w) in enumerate(zip(b["kio"], b["rho"], b["V"], b["vi"], b["weight"]))]
    bv = list(b["bvals"])
    kw = dict(lib_delta_pairs=[(10.0, 20.0)], lib_b_values=bv, n_b=len(bv), fit_triples=[(10.0, 20.0, x) for x in bv],
              vi_min=0.5, vi_max=0.95)
    sig = float(b["sigma_m"])
    fixed = bayes_fit(b["measured"], ents, sigma_m=sig, **kw)
    _close(fixed, {k[len("bayes_fixed_"):]: v for k, v in b.items() if k.startswith("bayes_fixed_")}, "fixed")
    free = bayes_fit(b["measured"], ents, sigma_m=sig, fit_s0=True, raw_signal=b["raw"], **kw)
    _close(free, {k[len("bayes_free_"):]: v for k, v in b.items() if k.startswith("bayes_free_")}, "free")
    with pytest.raises(ValueError):
        bayes_fit(b["measured"], [LibraryEntry(1.0, 1e6, 0.7, b["lib"][0], vi=0.7)], sigma_m=sig, **kw)


@pytest.mark.parametrize("sigma_m", [0.01, 0.03])
def test_bayes_gpu_matches_oracle_on_a_20k_library(sigma_m):
    """20,000-entry, 20-column library (smooth decays), 2e4 Rician voxels at
    SNR 30, random quadrature weights: fixed S0 and free S0 (raw signal with S0
    in [100, 2000]) against the fp64 oracle."""
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.fitters_gpu import bayes_fit_gpu
    from oracle import oracle as O
    lib, params = WL.match_library(n_lib=20_000)
    vox, _ = WL.rician_voxels(lib, n_vox=20_000, seed=21)
    rng = np.random.default_rng(5)
    q = rng.uniform(0.2, 5.0, len(lib))
    k, r, v = params.T
    vox32 = vox.astype(np.float32).astype(np.float64)       # the fp32 inputs the GPU sees
    lib32 = lib.astype(np.float32).astype(np.float64)
    got = bayes_fit_gpu(vox, lib, k, r, v, sigma_m, quadrature_weights=q)
    want = O.bayes(vox32, lib32, k, r, v, q, sigma_m)
    _close(got, want, f"fixed sigma {sigma_m}")
    assert np.median(want["n_eff"]) > 1.5            # the posterior spreads over several entries
    s0 = rng.uniform(100.0, 2000.0, (len(vox), 1))
    raw = (vox * s0).astype(np.float32).astype(np.float64)
    got = bayes_fit_gpu(raw, lib, k, r, v, sigma_m, fit_s0=True, quadrature_weights=q)
    want = O.bayes(raw, lib32, k, r, v, q, sigma_m, fit_s0=True)
    _close(got, want, f"free sigma {sigma_m}")


def test_bayes_free_s0_voxel_without_support_gives_zeros():
    from custom_madi_gb300.fitters_gpu import bayes_fit_gpu
    lib = np.abs(np.random.default_rng(1).uniform(0.1, 1.0, (300, 8)))
    meas = np.vstack([-lib[:2], lib[5:7]])                  # first two rows project negatively on every entry
    out = bayes_fit_gpu(meas, lib, np.arange(300.0), np.full(300, 1e6), np.full(300, 0.7), 0.05, fit_s0=True,
                        quadrature_weights=np.ones(300))
    for key in ("kio_mean", "kio_std", "n_eff", "residual", "s0_fit"):
        assert np.all(out[key][:2] == 0.0)
    assert np.all(out["n_eff"][2:] >= 1.0)


def test_calibrate_sigma_m_hits_the_target_n_eff():
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.fitters import bayes_fit, calibrate_sigma_m
    from custom_madi_gb300.library import LibraryEntry
    lib, params = WL.match_library(n_lib=3000)
    vox, _ = WL.rician_voxels(lib, n_vox=3000, seed=4)
    ents = [LibraryEntry(float(k), float(r), float(v), lib[i], vi=0.7, weight=1.0) for i, (k, r, v) in enumerate(params)]
    from custom_madi_gb300.workloads import PGSE
    pairs = [(6.0, D) for D in PGSE["big_deltas"]]
    bv = PGSE["b_values"]
    kw = dict(lib_delta_pairs=pairs, lib_b_values=bv, n_b=len(bv),
              fit_triples=[(6.0, D, b) for D in PGSE["big_deltas"] for b in bv])
    sig = calibrate_sigma_m(vox, ents, target_n_eff=20.0, sample_size=1000, n_iter=18, verbose=False, **kw)
    n_eff = bayes_fit(vox[np.random.default_rng(0).choice(3000, 1000, replace=False)], ents, sigma_m=sig,
                      **kw)["n_eff"]
    assert abs(np.median(n_eff) / 20.0 - 1.0) < 0.05
