"""Host-API vectors produced by the reference (tests/golden/api.npz, written by
tests/golden/make_golden.py --only api): the golden-replay random stream's draw
order and the ordered merge of per-ensemble results."""

from __future__ import annotations

import numpy as np

from custom_madi_gb300.config import SimConfig


def test_make_walk_random_stream_matches_reference_draws(golden):
    """make_walk_random_stream (madi/walker_gpu.py:115-127): init, increments and
    uniforms drawn from default_rng(seed) in the reference's order, bit-exact."""
    from custom_madi_gb300.walker_gpu import make_walk_random_stream
    g = golden("api.npz")
    cfg = SimConfig(L=float(g["stream_L"]), n_walkers=int(g["stream_n_walkers"]), n_ensembles=1, ts=0.01,
                    T_max_ms=0.04, h_ms=0.01, small_deltas=[0.01], big_deltas=[0.01], b_values=[0.0])
    assert cfg.n_steps == int(g["stream_n_steps"])
    st = make_walk_random_stream(cfg, int(g["stream_seed"]))
    assert np.array_equal(st.initial_positions, g["stream_init"])
    assert np.array_equal(st.increments, g["stream_incr"])
    assert np.array_equal(st.acceptance_uniforms, g["stream_unif"])
    assert np.all(st.initial_positions >= g["stream_source_lo"]) and np.all(st.initial_positions < g["stream_source_hi"])


def test_merge_results_keeps_ensemble_order(golden):
    """_merge_results (madi/walker_gpu.py:1066-1090): sums in ensemble order and
    per-ensemble lists concatenated unsorted (the CRN partner identity)."""
    from custom_madi_gb300.walker_gpu import ReducedResult, _merge_results
    g = golden("api.npz")
    parts = []
    for e in range(3):
        parts.append(ReducedResult(
            cos_sum=g["merge_in_cos"][e].copy(), sin_sum=g["merge_in_sin"][e].copy(), n_walkers=10 + e,
            n_escaped=0, occupancy_counts=g["merge_in_occ"][e].copy(), pp_values=[0.01 * (e + 1)],
            analytic_kio_eq5_values=[1.5 * (e + 1)], geometry_stats=[{"e": e}],
            ensemble_cos_means=[g["merge_in_ens_cos"][e]], ensemble_sin_means=[g["merge_in_ens_sin"][e]],
            classifier_cache_stats=[{"full": e}]))
    m = _merge_results(parts)
    assert np.array_equal(m.cos_sum, g["merge_cos"]) and np.array_equal(m.sin_sum, g["merge_sin"])
    assert m.n_walkers == int(g["merge_n_walkers"])
    assert np.array_equal(m.occupancy_counts, g["merge_occ"])
    assert np.array_equal(np.asarray(m.pp_values), g["merge_pp"])
    assert np.array_equal(np.asarray(m.analytic_kio_eq5_values), g["merge_kio"])
    assert np.array_equal(np.asarray(m.ensemble_cos_means), g["merge_ens_cos"])
    assert np.array_equal(np.asarray(m.ensemble_sin_means), g["merge_ens_sin"])
    assert [s["e"] for s in m.geometry_stats] == [0, 1, 2]
    # merging leaves the inputs untouched
    assert np.array_equal(parts[0].cos_sum, g["merge_in_cos"][0])
