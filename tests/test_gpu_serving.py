"""Serving loop on the GPU: every result is the same alone and in the mix."""

from dataclasses import replace

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup():
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300.config import SimConfig, fibonacci_directions
    from custom_madi_gb300.ensemble import create_ensemble
    from custom_madi_gb300.walker_gpu import pair_layout
    cfg = SimConfig(boundary_mode="periodic", n_cells=40, n_walkers=1000, n_ensembles=1,
                    geometry_validation_points=20_000, geometry_vi_tolerance=0.1, ts=0.01, T_max_ms=12.0,
                    h_ms=1.0, small_deltas=[2.0], big_deltas=[5.0, 8.0], b_values=[0.0, 1000.0, 3000.0],
                    directions=fibonacci_directions(6).tolist())
    cols = S.build_columns(cfg)
    lay = pair_layout(cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    e1 = create_ensemble(2.0e5, 4.0, cfg, seed=0)
    e2 = create_ensemble(3.0e5, 2.5, replace(cfg, n_cells=30), seed=5)
    return cfg, cols, lay, e1, e2


def _requests(cfg, e1, e2, lib):
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.serving import FitRequest, SimRequest
    from custom_madi_gb300.walker_gpu import kio_to_pp
    vox, _ = WL.rician_voxels(lib, n_vox=3000, seed=4)
    return [SimRequest(e1, kio_to_pp(20.0, e1.mean_AV, cfg), 42, 5000, arrival=0.0),
            SimRequest(e2, kio_to_pp(5.0, e2.mean_AV, cfg), 7, 3000, arrival=0.001),
            FitRequest(vox.astype(np.float32), precision="bf16", topk=32, arrival=0.0015),
            SimRequest(e1, kio_to_pp(60.0, e1.mean_AV, cfg), 9, 12000, arrival=0.002)]


def _server(cfg, lay, lib, **kw):
    from custom_madi_gb300.serving import Server
    return Server(cfg, lay, cfg.direction_array(), library=lib, **kw)


def _same(a, b):
    if "cos_fixed" in a:
        assert np.array_equal(a["cos_fixed"], b["cos_fixed"])
        assert np.array_equal(a["sin_fixed"], b["sin_fixed"])
        assert np.array_equal(a["occupancy"], b["occupancy"])
        assert a["counters"] == b["counters"]
    else:
        assert np.array_equal(a["best_idx"], b["best_idx"])
        assert np.array_equal(a["best_resid"], b["best_resid"])


def test_results_identical_alone_and_in_the_mix():
    """All four requests queued at once: round-robin chunks force launches that mix
    requests; each result equals the request served alone and the one-launch path."""
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.walker_gpu import WalkJob, simulate_jobs
    cfg, cols, lay, e1, e2 = _setup()
    lib, _ = WL.match_library(n_lib=2000)
    reqs = [replace(r, arrival=0.0) for r in _requests(cfg, e1, e2, lib)]
    srv = _server(cfg, lay, lib, chunk_walkers=2048, launch_walkers=4096)
    mix = srv.run(reqs, realtime=False)
    assert any(len(l) >= 2 for l in srv.launch_log), "no launch mixed two requests"
    assert mix["launches"] >= 5
    for i, r in enumerate(reqs):
        alone = _server(cfg, lay, lib).run([r], realtime=False)
        _same(mix["records"][i].result, alone["records"][0].result)
    one = simulate_jobs([WalkJob(reqs[3].ensemble, reqs[3].pp, reqs[3].seed, reqs[3].n_walkers)], cfg,
                        (cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef), dirs=cfg.direction_array())[0]
    assert np.array_equal(one["cos_fixed"], mix["records"][3].result["cos_fixed"])
    assert mix["records"][3].result["counters"]["walkers"] == 12000


def test_staggered_arrivals_in_real_time():
    """Requests arriving while others run (wall clock) give the same results and
    finite p50/p99 latencies."""
    from custom_madi_gb300 import workloads as WL
    cfg, cols, lay, e1, e2 = _setup()
    lib, _ = WL.match_library(n_lib=2000)
    reqs = _requests(cfg, e1, e2, lib)
    ref = _server(cfg, lay, lib, chunk_walkers=2048, launch_walkers=4096).run(
        [replace(r, arrival=0.0) for r in reqs], realtime=False)
    out = _server(cfg, lay, lib, chunk_walkers=2048, launch_walkers=4096).run(reqs, realtime=True)
    for a, b in zip(ref["records"], out["records"]):
        _same(a.result, b.result)
    for r in out["records"]:
        assert r.admit >= r.arrival and r.finish >= r.admit
    assert np.isfinite(out["p50_s"]) and out["p99_s"] >= out["p50_s"]
    assert out["walker_steps"] == sum(r.n_walkers for r in reqs if hasattr(r, "n_walkers")) * cfg.n_steps


def test_budget_admits_one_geometry_at_a_time():
    """With room for one geometry, queued simulations are admitted one after the other
    (wall clock) and still give the same results."""
    from custom_madi_gb300 import workloads as WL
    cfg, cols, lay, e1, e2 = _setup()
    lib, _ = WL.match_library(n_lib=2000)
    reqs = [replace(r, arrival=0.0) for r in _requests(cfg, e1, e2, lib) if hasattr(r, "ensemble")]
    free = _server(cfg, lay, lib).run(reqs, realtime=True)
    assert all(r.admit < free["records"][0].finish for r in free["records"])   # all admitted at once
    probe = _server(cfg, lay, lib, n_slots=4)
    geo = max(e.device(str(probe.dev)).nbytes for e in (e1, e2))
    tight = _server(cfg, lay, lib, n_slots=4, budget_bytes=probe.pool_bytes + geo + 1)
    out = tight.run(reqs, realtime=True)
    recs = out["records"]
    for a, b in zip(recs[:-1], recs[1:]):
        assert b.admit >= a.finish          # one admitted at a time
    for a, b in zip(free["records"], recs):
        _same(a.result, b.result)


def test_native_server_matches_python_server():
    """The C++ serving loop (madi_serve_*) gives the same sums as the Python loop
    and as one launch per request."""
    from custom_madi_gb300 import _native as N
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.serving import NativeSimServer
    cfg, cols, lay, e1, e2 = _setup()
    lib, _ = WL.match_library(n_lib=2000)
    reqs = [replace(r, arrival=0.0) for r in _requests(cfg, e1, e2, lib) if hasattr(r, "ensemble")]
    py = _server(cfg, lay, lib).run(reqs, realtime=False)
    nat = NativeSimServer(cfg, lay, cfg.direction_array(), boundary=N.MADI_BOUNDARY_PERIODIC,
                          chunk_walkers=2048, launch_walkers=4096, n_slots=8)
    out = nat.run(reqs, realtime=True)
    nat.close()
    for a, b in zip(py["records"], out["records"]):
        _same(a.result, b.result)
    assert out["walker_steps"] == sum(r.n_walkers for r in reqs) * cfg.n_steps
