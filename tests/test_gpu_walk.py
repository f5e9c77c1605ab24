"""GPU walker parity: fixed-stream replays against the reference golden walk, and
Philox walks against the oracle (same key: near-identical; independent key:
within 3 Monte Carlo standard errors)."""

import numpy as np
import pytest

from custom_madi_gb300.config import SimConfig

pytestmark = pytest.mark.gpu

C0 = dict(ts=0.01, T_max_ms=46.0, small_deltas=[6.0], big_deltas=[15.0, 25.0, 30.0, 40.0],
          b_values=[0.0, 1000.0, 2500.0, 4000.0, 6000.0])


def _golden_case(golden):
    from custom_madi_gb300.ensemble import ensemble_from_arrays
    from custom_madi_gb300.walker_gpu import WalkRandomStream
    w = golden("golden_walk.npz")
    ens = ensemble_from_arrays(w["seeds"], w["annulus"], float(w["L"]), source_lo=float(w["source_lo"]),
                               source_hi=float(w["source_hi"]), rho_per_uL=1.0e6)
    cfg = SimConfig(L=float(w["L"]), n_walkers=len(w["init"]), n_ensembles=1, ts=float(w["ts"]),
                    T_max_ms=float(w["T_max_ms"]), h_ms=float(w["h_ms"]), small_deltas=[1.0, 2.0],
                    big_deltas=[2.0, 3.0, 5.0], b_values=[0.0, 500.0, 1000.0, 2000.0])
    stream = WalkRandomStream(w["init"], w["incr"], w["unif"])
    return w, ens, cfg, stream


def test_fp64_replay_matches_reference_golden(golden):
    """Reference tolerance (scripts/run_gpu_golden_check.py:27-28): rtol 5e-11, atol 5e-12."""
    from custom_madi_gb300.walker_gpu import run_walk_Y
    w, ens, cfg, stream = _golden_case(golden)
    Y, n_esc, tel = run_walk_Y(ens, 0.0, cfg, pp=float(w["pp"]), random_stream=stream, return_telemetry=True,
                               verbose=False)
    np.testing.assert_allclose(Y, w["Y"], rtol=5e-11, atol=5e-12)
    assert np.array_equal(tel["inside_trace"], w["inside_trace"])
    assert np.array_equal(tel["occupancy_fraction"], w["occupancy_fraction"])
    assert n_esc == 0
    print("fp64 replay max |dY| =", float(np.abs(Y - w["Y"]).max()))


def test_fp32_replay_tracks_reference_golden(golden):
    """Production fp32 walker on the same stream.

    fp32 positions differ from the fp64 ones by rounding (~1e-6 um), so a walker
    standing within that distance of a shifted facet can take the other
    accept/reject branch; such a walker then carries an offset of one step.
    Labels at the storage points must agree, and at least 95 % of the walkers
    must follow the reference trajectory to fp32 precision.
    """
    from custom_madi_gb300.walker_gpu import run_walk_Y
    w, ens, cfg, stream = _golden_case(golden)
    Y, _, tel = run_walk_Y(ens, 0.0, cfg, pp=float(w["pp"]), random_stream=stream, return_telemetry=True,
                           precision=32, verbose=False)
    assert np.mean(np.all(tel["inside_trace"] == w["inside_trace"], axis=1)) >= 0.95
    close = np.all(np.abs(Y - w["Y"]) <= 2e-3 + 1e-6 * np.abs(w["Y"]), axis=(1, 2))
    assert np.mean(close) >= 0.95, np.flatnonzero(~close)


def _periodic_c0(n_walkers, seed=0, n_cells=64):
    from custom_madi_gb300.ensemble import create_ensemble
    cfg = SimConfig(boundary_mode="periodic", n_cells=n_cells, n_walkers=n_walkers, n_ensembles=1,
                    geometry_validation_points=50_000, geometry_vi_tolerance=0.05, **C0)
    ens = create_ensemble(2.0e5, 4.0, cfg, seed=seed)
    return cfg, ens


def _oracle_sums(ens, cfg, cols, pp, key, n, dirs=None):
    from oracle import oracle as O
    from custom_madi_gb300.walker_gpu import pair_layout
    lay = pair_layout(cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    out = O.walk(O.geom_arrays(ens), n_walkers=n, n_steps=cfg.n_steps, steps_per_h=cfg.steps_per_h,
                 n_grid=cfg.n_grid, sigma=cfg.sigma, ts=cfg.ts, pp=pp, key=key, want_Y=False,
                 columns=(lay.jd, lay.jD, lay.js, lay.coef), dirs=dirs)
    cs = out["cos_sum"].reshape(lay.n_pairs * lay.n_b, -1)
    return cs, out


def test_philox_walk_same_key_tracks_oracle():
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300.walker_gpu import WalkJob, simulate_jobs, kio_to_pp, PHILOX_KEY1
    cfg, ens = _periodic_c0(2000)
    cols = S.build_columns(cfg)
    pp = kio_to_pp(20.0, ens.mean_AV, cfg)
    res = simulate_jobs([WalkJob(ens, pp, 1234, 2000)], cfg, (cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef))
    g = res[0]["cos"] / 2000.0
    cs, out = _oracle_sums(ens, cfg, cols, pp, (1234, PHILOX_KEY1), 2000)
    o = cs / 2000.0
    assert np.max(np.abs(g - o)) < 5e-3
    assert np.abs(res[0]["occupancy"] - out["occupancy"]).max() <= 0.02 * 2000
    print("same-key max |dS| =", float(np.max(np.abs(g - o))), res[0]["counters"])


def test_philox_walk_within_3_se_of_independent_oracle():
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300.walker_gpu import WalkJob, simulate_jobs, kio_to_pp
    cfg, ens = _periodic_c0(20000, seed=3)
    cols = S.build_columns(cfg)
    pp = kio_to_pp(20.0, ens.mean_AV, cfg)
    ng, no = 20000, 3000
    res = simulate_jobs([WalkJob(ens, pp, 99, ng)], cfg, (cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef))
    Sg = res[0]["cos"].sum(axis=1) / (3.0 * ng)
    cs, _ = _oracle_sums(ens, cfg, cols, pp, (777, 5), no)
    So = cs.sum(axis=1) / (3.0 * no)
    se = np.sqrt(np.maximum(1.0 - So ** 2, 1e-4) * (1.0 / ng + 1.0 / no))
    assert np.all(np.abs(Sg - So) <= 3.0 * se + 1e-9), (Sg - So) / se


def test_free_water_finite_lobe_matches_stejskal_tanner():
    """tests/physics_audit/test_finite_delta_reference.py:35-61 criterion on the GPU walker."""
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300.ensemble import create_dummy_ensemble
    from custom_madi_gb300.walker_gpu import WalkJob, simulate_jobs
    cfg = SimConfig(n_walkers=20000, n_ensembles=1, **C0)
    ens = create_dummy_ensemble(cfg)
    cols = S.build_columns(cfg)
    r = simulate_jobs([WalkJob(ens, 0.0, 5, 20000)], cfg, (cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef))[0]
    Sv = r["cos"].sum(axis=1) / (3 * 20000.0)
    b = np.tile(np.asarray(cfg.b_values), 4)
    expect = np.exp(-b * cfg.D0 * 1e-3)
    se = np.sqrt(np.maximum(1 - Sv ** 2, 1e-6) / 20000.0)
    assert np.all(np.abs(Sv - expect) <= 5 * se + 0.012)


def test_fatal_escape_raises():
    from custom_madi_gb300.ensemble import create_dummy_ensemble
    from custom_madi_gb300.walker_gpu import WalkRandomStream, run_walk_Y
    cfg = SimConfig(L=2.0, n_walkers=1, n_ensembles=1, T_max_ms=2.0, small_deltas=[1.0], big_deltas=[1.0],
                    b_values=[0.0])
    inc = np.zeros((cfg.n_steps, 1, 3))
    inc[0, 0, 0] = 2.0
    st = WalkRandomStream(np.array([[1.0, 1.0, 1.0]]), inc, np.zeros((cfg.n_steps, 1)))
    for prec in (64, 32):
        with pytest.raises(RuntimeError, match="fatal boundary condition"):
            run_walk_Y(create_dummy_ensemble(cfg), 0.0, cfg, pp=0.0, random_stream=st, precision=prec, verbose=False)


def test_trapezoid_known_answer(golden):
    from custom_madi_gb300.ensemble import create_dummy_ensemble
    from custom_madi_gb300.walker_gpu import WalkRandomStream, run_walk_Y
    t = golden("trapezoid.npz")
    cfg = SimConfig(L=200.0, n_walkers=1, n_ensembles=1, T_max_ms=2.0, h_ms=1.0, small_deltas=[1.0],
                    big_deltas=[1.0, 2.0], b_values=[0.0, 1000.0])
    st = WalkRandomStream(t["init"], t["incr"], t["unif"])
    Y, _ = run_walk_Y(create_dummy_ensemble(cfg), 0.0, cfg, pp=0.0, random_stream=st, verbose=False)
    assert np.array_equal(Y, t["Y"])


def test_job_result_is_identical_alone_and_in_a_mixed_batch():
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300.walker_gpu import WalkJob, simulate_jobs
    cfg, ens = _periodic_c0(3000)
    _, ens2 = _periodic_c0(3000, seed=9, n_cells=40)
    cols = S.build_columns(cfg)
    c = (cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    a = WalkJob(ens, 0.01, 42, 3000)
    alone = simulate_jobs([a], cfg, c)[0]
    again = simulate_jobs([a], cfg, c)[0]
    mixed = simulate_jobs([WalkJob(ens2, 0.02, 7, 5000), a, WalkJob(ens, 0.0, 1, 700)], cfg, c)[1]
    assert np.array_equal(alone["cos_fixed"], again["cos_fixed"])
    assert np.array_equal(alone["cos_fixed"], mixed["cos_fixed"])
    assert np.array_equal(alone["sin_fixed"], mixed["sin_fixed"])
    assert np.array_equal(alone["occupancy"], mixed["occupancy"])


def test_per_step_labels_match_oracle_on_fixed_stream(golden):
    """Every step's intracellular label of the fp32 walker (label cache + cooperative
    classifier) equals the fp64 oracle's along the same stream, for every walker whose
    trajectory has not been displaced by an fp32-rounding decision."""
    from custom_madi_gb300.ensemble import ensemble_from_arrays
    from custom_madi_gb300.walker_gpu import WalkRandomStream, run_walk_Y
    from oracle import oracle as O
    d = golden("classify_si.npz")
    ens = ensemble_from_arrays(d["seeds"], d["annulus"], float(d["L"]), source_lo=float(d["source_lo"]),
                               source_hi=float(d["source_hi"]), rho_per_uL=float(d["rho"]))
    n, steps = 256, 400
    cfg = SimConfig(L=float(d["L"]), n_walkers=n, n_ensembles=1, ts=0.01, T_max_ms=4.0, h_ms=0.01,
                    small_deltas=[0.01], big_deltas=[0.01], b_values=[0.0])
    rng = np.random.default_rng(11)
    st = WalkRandomStream(rng.uniform(ens.source_lo, ens.source_hi, (n, 3)),
                          rng.normal(0.0, cfg.sigma, (steps, n, 3)), rng.uniform(0, 1, (steps, n)))
    Y, _, tel = run_walk_Y(ens, 0.0, cfg, pp=0.05, random_stream=st, return_telemetry=True, precision=32,
                           verbose=False)
    o = O.walk(O.geom_arrays(ens), n_walkers=n, n_steps=steps, steps_per_h=1, n_grid=steps + 1, sigma=cfg.sigma,
               ts=cfg.ts, pp=0.05, stream=(st.initial_positions, st.increments, st.acceptance_uniforms))
    same_path = np.all(np.abs(Y - o["Y"]) <= 1e-3 + 1e-6 * np.abs(o["Y"]), axis=(1, 2))
    assert np.mean(same_path) >= 0.95
    # A label may differ only where the oracle's fp64 point lies within fp32
    # rounding distance (1e-4 um) of a shifted facet: positions are recovered
    # from the oracle's Y by inverting the step trapezoid.
    seeds, ann = ens.classifier_seeds, ens.classifier_annulus
    for w, j in np.argwhere(tel["inside_trace"] != o["inside_trace"]):
        if not same_path[w]:
            continue
        x = st.initial_positions[w] - ens.L / 2.0
        for k in range(1, j + 1):
            x = 2.0 * (o["Y"][w, k] - o["Y"][w, k - 1]) / cfg.ts - x
        p = x + ens.L / 2.0
        dist = np.linalg.norm(seeds - p, axis=1)
        s1 = int(np.argmin(dist))
        sep = np.linalg.norm(seeds - seeds[s1], axis=1)
        sep[s1] = 1.0
        m = (dist ** 2 - dist[s1] ** 2) / (2.0 * sep)
        m[s1] = np.inf
        assert np.min(np.abs(m - ann[s1])) < 1e-4, (w, j, float(np.min(np.abs(m - ann[s1]))))
    assert 0.2 < float(np.mean(tel["inside_trace"])) < 0.95


def test_cuda_graph_replay_matches_eager_launch():
    """The captured batched launch gives the same sums as an eager launch, every replay."""
    import torch
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300.walker_gpu import WalkBatch, WalkGraph, WalkJob, pair_layout
    cfg, ens = _periodic_c0(3000)
    _, ens2 = _periodic_c0(3000, seed=9, n_cells=40)
    cols = S.build_columns(cfg)
    lay = pair_layout(cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    jobs = [WalkJob(ens, 0.01, 42, 3000), WalkJob(ens2, 0.02, 7, 1000)]
    b = WalkBatch(jobs, cfg, layout=lay, dirs=cfg.direction_array())
    b.launch()
    eager = [r["cos_fixed"].copy() for r in b.results()]
    g = WalkGraph(b)
    for _ in range(2):
        g.replay()
        torch.cuda.synchronize()
        got = [r["cos_fixed"] for r in b.results()]
        for a, c in zip(eager, got):
            assert np.array_equal(a, c)


@pytest.mark.parametrize("n_cells", [27, 64])
def test_per_step_labels_match_oracle_on_periodic_box(n_cells):
    """Periodic box: every step's label of the fp32 walker (facet table with
    nearest-image offsets, per-walker label cache, cooperative facet passes)
    equals the fp64 oracle's along the same stream, for every walker whose path
    no fp32-rounding decision has displaced; small boxes put many steps across
    the box faces."""
    from custom_madi_gb300.ensemble import create_ensemble
    from custom_madi_gb300.walker_gpu import WalkRandomStream, run_walk_Y
    from oracle import oracle as O
    n, steps = 256, 400
    cfg = SimConfig(boundary_mode="periodic", n_cells=n_cells, n_walkers=n, n_ensembles=1, ts=0.01, T_max_ms=4.0,
                    h_ms=0.01, small_deltas=[0.01], big_deltas=[0.01], b_values=[0.0],
                    geometry_validation_points=20_000, geometry_vi_tolerance=0.1)
    ens = create_ensemble(4.0e6, 0.15, cfg, seed=5, verify_vi=False)
    L = ens.L
    rng = np.random.default_rng(21)
    st = WalkRandomStream(rng.uniform(0.0, L, (n, 3)), rng.normal(0.0, cfg.sigma, (steps, n, 3)),
                          rng.uniform(0, 1, (steps, n)))
    Y, _, tel = run_walk_Y(ens, 0.0, cfg, pp=0.05, random_stream=st, return_telemetry=True, precision=32,
                           verbose=False)
    o = O.walk(O.geom_arrays(ens), n_walkers=n, n_steps=steps, steps_per_h=1, n_grid=steps + 1, sigma=cfg.sigma,
               ts=cfg.ts, pp=0.05, stream=(st.initial_positions, st.increments, st.acceptance_uniforms))
    same_path = np.all(np.abs(Y - o["Y"]) <= 1e-3 + 1e-6 * np.abs(o["Y"]), axis=(1, 2))
    assert np.mean(same_path) >= 0.95
    seeds, ann = ens.classifier_seeds, ens.classifier_annulus
    for w, j in np.argwhere(tel["inside_trace"] != o["inside_trace"]):
        if not same_path[w]:
            continue
        x = st.initial_positions[w] - L / 2.0
        for k in range(1, j + 1):
            x = 2.0 * (o["Y"][w, k] - o["Y"][w, k - 1]) / cfg.ts - x
        p = np.mod(x + L / 2.0, L)
        dist = np.linalg.norm(seeds - p, axis=1)
        s1 = int(np.argmin(dist))
        sep = np.linalg.norm(seeds - seeds[s1], axis=1)
        sep[s1] = 1.0
        m = (dist ** 2 - dist[s1] ** 2) / (2.0 * sep)
        m[s1] = np.inf
        assert np.min(np.abs(m - ann[s1])) < 1e-4, (w, j, float(np.min(np.abs(m - ann[s1]))))
    assert 0.2 < float(np.mean(tel["inside_trace"])) < 0.98
    # the facet table decided nearly every step; the voxel-grid rule is the rare fallback
    c = tel["classifier_cache"]
    assert c["tier1"] >= 0.99 * n * steps and c["facet_pass"] > 0


def test_walk_and_reduce_one_ensemble_helper():
    """The reference's private helper (used by its benchmark scripts) walks one
    ensemble at one p_p and returns the reduced result of the batched walk."""
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300.walker_gpu import (WalkJob, _walk_and_reduce_one_ensemble, kio_to_pp, results_to_reduced,
                                              simulate_jobs)
    cfg, ens = _periodic_c0(2000)
    cols = S.build_columns(cfg)
    pp = kio_to_pp(20.0, ens.mean_AV, cfg)
    cfg2 = cfg                      # n_walkers = 2000
    got = _walk_and_reduce_one_ensemble(ens, pp, cfg2, cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef, 77)
    r = simulate_jobs([WalkJob(ens, pp, 77, 2000)], cfg2, (cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef))[0]
    want = results_to_reduced(ens, pp, cfg2, r, 2000)
    assert got.n_walkers == 2000 and got.n_escaped == 0
    np.testing.assert_array_equal(got.cos_sum, want.cos_sum)
    np.testing.assert_array_equal(got.occupancy_counts, want.occupancy_counts)
    with pytest.raises(ValueError):
        _walk_and_reduce_one_ensemble(ens, pp, cfg2, cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef, 77,
                                      narrow_snapshot_steps=np.zeros(1))


def test_philox_si_walk_tracks_oracle_same_key(golden):
    """Finite SI box (fatal escape, unclosed outer cells in the facet table): the
    fp32 Philox walker and the fp64 oracle on the same key follow the same path
    and labels for nearly every walker (fp32 rounding can flip a decision only
    within ~1e-6 um of a shifted facet)."""
    from custom_madi_gb300.ensemble import ensemble_from_arrays
    from custom_madi_gb300.walker_gpu import PHILOX_KEY1, run_walk_Y
    from oracle import oracle as O
    d = golden("classify_si.npz")
    ens = ensemble_from_arrays(d["seeds"], d["annulus"], float(d["L"]), source_lo=float(d["source_lo"]),
                               source_hi=float(d["source_hi"]), rho_per_uL=float(d["rho"]))
    n, steps = 512, 400
    cfg = SimConfig(L=float(d["L"]), n_walkers=n, n_ensembles=1, ts=0.01, T_max_ms=4.0, h_ms=0.01,
                    small_deltas=[0.01], big_deltas=[0.01], b_values=[0.0])
    Y, _, tel = run_walk_Y(ens, 0.0, cfg, seed=4321, pp=0.05, return_telemetry=True, precision=32, verbose=False)
    o = O.walk(O.geom_arrays(ens), n_walkers=n, n_steps=steps, steps_per_h=1, n_grid=steps + 1, sigma=cfg.sigma,
               ts=cfg.ts, pp=0.05, key=(4321, PHILOX_KEY1))
    same = np.all(np.abs(Y - o["Y"]) <= 1e-3 + 1e-6 * np.abs(o["Y"]), axis=(1, 2))
    assert np.mean(same) >= 0.95, np.mean(same)
    assert np.mean(tel["inside_trace"][same] == o["inside_trace"][same]) >= 0.999
    assert 0.2 < float(np.mean(tel["inside_trace"])) < 0.95


def test_fp64_philox_walk_matches_oracle_same_key(golden):
    """The fp64 walker on Philox numbers (the reference's walker design:
    one thread per walker, exact KD rule every step, Y stored) against the
    fp64 oracle on the same key, finite SI box with fatal escape.  Both evaluate
    the same separately rounded fp64 arithmetic; log / sin / cos may differ by
    an ulp between CUDA and the C library, so Y agrees to 1e-9 um ms and the
    labels exactly for (nearly) every walker."""
    from custom_madi_gb300.ensemble import ensemble_from_arrays
    from custom_madi_gb300.walker_gpu import PHILOX_KEY1, run_walk_Y
    from oracle import oracle as O
    d = golden("classify_si.npz")
    ens = ensemble_from_arrays(d["seeds"], d["annulus"], float(d["L"]), source_lo=float(d["source_lo"]),
                               source_hi=float(d["source_hi"]), rho_per_uL=float(d["rho"]))
    n, steps = 512, 400
    cfg = SimConfig(L=float(d["L"]), n_walkers=n, n_ensembles=1, ts=0.01, T_max_ms=4.0, h_ms=0.01,
                    small_deltas=[0.01], big_deltas=[0.01], b_values=[0.0])
    Y, _, tel = run_walk_Y(ens, 0.0, cfg, seed=4321, pp=0.05, return_telemetry=True, precision=64, verbose=False)
    o = O.walk(O.geom_arrays(ens), n_walkers=n, n_steps=steps, steps_per_h=1, n_grid=steps + 1, sigma=cfg.sigma,
               ts=cfg.ts, pp=0.05, key=(4321, PHILOX_KEY1))
    same = np.all(np.abs(Y - o["Y"]) <= 1e-9, axis=(1, 2))
    assert np.mean(same) >= 0.998, np.mean(same)
    assert np.array_equal(tel["inside_trace"][same], o["inside_trace"][same])
    assert 0.2 < float(np.mean(tel["inside_trace"])) < 0.95
    print("fp64 Philox max |dY| over matching walkers =", float(np.abs(Y - o["Y"])[same].max()))


def test_reference_design_path_matches_oracle_signal():
    """simulate_jobs(precision=64): per-entry fp64 walk storing Y, then the tiled
    column reduction, on a periodic 64-cell box; the signal sums agree with the
    oracle's fp64 walk on the same key to 1e-9 of the walker count."""
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300.walker_gpu import PHILOX_KEY1, WalkJob, kio_to_pp, pair_layout, simulate_jobs
    cfg, ens = _periodic_c0(1000)
    cols = S.build_columns(cfg)
    pp = kio_to_pp(20.0, ens.mean_AV, cfg)
    r = simulate_jobs([WalkJob(ens, pp, 555, 1000)], cfg, (cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef),
                      dirs=np.eye(3), precision=64)[0]
    cs, out = _oracle_sums(ens, cfg, cols, pp, (555, PHILOX_KEY1), 1000, dirs=np.eye(3))
    lay = pair_layout(cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    want = np.full(len(cols.phase_coef), np.nan)
    for p in range(lay.n_pairs):                 # oracle sums are per (pair, b) of the layout
        for b in range(lay.n_b):
            if lay.col_of[p, b] >= 0:
                want[lay.col_of[p, b]] = cs[p * lay.n_b + b].sum()
    got = r["cos"][:, 0]
    assert not np.isnan(want).any()
    assert np.max(np.abs(got - want)) <= 1e-9 * 1000, np.max(np.abs(got - want))
    assert np.array_equal(r["occupancy"], out["occupancy"])
