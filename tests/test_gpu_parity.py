"""Parity of the benchmarked configurations against the oracle.

The batched library build (periodic boxes of 27-512 cells over the full
(kio, rho, V) ranges, 24 Fibonacci directions, 4 Delta x 5 b) and the plain
64-cell box are checked the way the reference accepts a walker
(madi/walker_gpu.py:954-968 with tests/physics_audit/test_finite_delta_reference.py:35-61):
signals agree with an independent CPU walk within 3 Monte Carlo standard
errors.  The standard error of a mean of cos(phase) over N walkers is taken
from the rigorous bound Var(cos) <= 1 - S^2 (|cos| <= 1, mean S), so the
test's 3 SE are at least 3 true SE.

Also: the same Philox key gives the same walk per (column, direction); the
large-grid column reduction madi_reduce_Y against the oracle's reduction; a
library entry of build_library_from_triplets against the oracle signal; the
public simulate entry points against the oracle.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import replace

import numpy as np
import pytest

from custom_madi_gb300.config import SimConfig

pytestmark = pytest.mark.gpu


def _se(S, n):
    """Upper bound of the standard error of a mean of cos over n walkers."""
    return np.sqrt(np.maximum(1.0 - np.asarray(S, np.float64) ** 2, 0.0) / float(n))


def _within_3se(Sg, ng, So, no):
    """|Sg - So| <= 3 combined SE, the pooled mean giving the bound; returns the z-scores too."""
    pooled = (Sg * ng + So * no) / float(ng + no)
    se = np.sqrt(_se(pooled, ng) ** 2 + _se(pooled, no) ** 2)
    z = np.abs(Sg - So) / np.maximum(se, 1e-300)
    ok = np.abs(Sg - So) <= 3.0 * se + 1e-12
    return ok, z


def _columns(cfg):
    from custom_madi_gb300 import signal as S
    cols = S.build_columns(cfg)
    return cols, (cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)


def _oracle_dir_sums(ens, cfg, pp, key, n, dirs):
    """Oracle walk of one ensemble: cos / sin sums [n_cols, n_dirs] and the run record."""
    from oracle import oracle as O
    from custom_madi_gb300.walker_gpu import pair_layout
    cols, c = _columns(cfg)
    lay = pair_layout(*c)
    out = O.walk(O.geom_arrays(ens), n_walkers=n, n_steps=cfg.n_steps, steps_per_h=cfg.steps_per_h,
                 n_grid=cfg.n_grid, sigma=cfg.sigma, ts=cfg.ts, pp=pp, key=key, want_Y=False,
                 columns=(lay.jd, lay.jD, lay.js, lay.coef), dirs=dirs)
    D = len(dirs)
    return out["cos_sum"].reshape(-1, D), out["sin_sum"].reshape(-1, D), out


def _plain_box(n_walkers):
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.ensemble import create_ensemble
    cfg = WL.plain_config(n_walkers=n_walkers)
    return cfg, create_ensemble(2.0e5, 4.0, cfg, seed=0)


# ---------------------------------------------------------------------------
# Plain 64-cell box, 24 Fibonacci directions
# ---------------------------------------------------------------------------

def test_plain_box_24_directions_within_3_se_of_independent_oracle():
    """1e5 fp32 GPU walkers vs 2e4 fp64 oracle walkers on an independent key:
    every (column, direction) of S[4 Delta x 5 b, 24 dir] within 3 SE, the
    imaginary part too; the direction average as well."""
    from custom_madi_gb300.walker_gpu import WalkJob, kio_to_pp, simulate_jobs
    ng, no = 100_000, 20_000
    cfg, ens = _plain_box(ng)
    u = cfg.direction_array()
    assert u.shape == (24, 3)
    _, c = _columns(cfg)
    pp = kio_to_pp(20.0, ens.mean_AV, cfg)
    r = simulate_jobs([WalkJob(ens, pp, 11, ng)], cfg, c, dirs=u)[0]
    cos_o, sin_o, _ = _oracle_dir_sums(ens, cfg, pp, (90210, 17), no, u)
    for g, o in ((r["cos"], cos_o), (r["sin"], sin_o)):
        ok, z = _within_3se(g / ng, ng, o / no, no)
        assert ok.all(), (np.argwhere(~ok), z.max())
    ok, z = _within_3se(r["cos"].mean(axis=1) / ng, ng, cos_o.mean(axis=1) / no, no)
    assert ok.all(), z.max()
    # the signal decays with b and is 1 at b = 0
    S = r["cos"].mean(axis=1).reshape(4, 5) / ng
    assert np.all(S[:, 0] == 1.0) and np.all(np.diff(S, axis=1) < 0)
    print("24-dir plain box: max z =", float(z.max()))


def test_plain_box_24_directions_same_key_tracks_oracle():
    """Same Philox key, same walkers: per (column, direction) the fp32 walk and
    the fp64 oracle differ only by walkers an fp32 rounding decision displaced."""
    from custom_madi_gb300.walker_gpu import PHILOX_KEY1, WalkJob, kio_to_pp, simulate_jobs
    n = 20_000
    cfg, ens = _plain_box(n)
    u = cfg.direction_array()
    _, c = _columns(cfg)
    pp = kio_to_pp(20.0, ens.mean_AV, cfg)
    r = simulate_jobs([WalkJob(ens, pp, 2024, n)], cfg, c, dirs=u)[0]
    cos_o, sin_o, out = _oracle_dir_sums(ens, cfg, pp, (2024, PHILOX_KEY1), n, u)
    d_cos = np.abs(r["cos"] - cos_o) / n
    d_sin = np.abs(r["sin"] - sin_o) / n
    assert d_cos.max() < 5e-3 and d_sin.max() < 5e-3, (d_cos.max(), d_sin.max())
    assert np.abs(r["occupancy"] - out["occupancy"]).max() <= 0.01 * n
    print("24-dir same key: max |dS| =", float(d_cos.max()), float(d_sin.max()))


# ---------------------------------------------------------------------------
# Entries of the batched library build, walked together in one persistent launch
# ---------------------------------------------------------------------------

# Indices into batch_triplets(256, seed=1): 131 has the fewest cells (31), 161
# the lowest rho (and largest V), 10 the highest rho, 135 the smallest V, 160
# the lowest kio, 81 the highest kio, 0 and 1 the first draws.
BATCH_PICKS = (131, 161, 10, 135, 160, 81, 0, 1)


def test_batched_entries_within_3_se_of_independent_oracle():
    """Eight entries of the 256-entry batch plus a 27-cell box, all in one
    WalkBatch launch (1e5 walkers each, 24 directions), each against an
    independent oracle walk of 2e4 walkers: every (column, direction) within 3 SE."""
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.walker_gpu import (LaunchConfig, WalkBatch, WalkJob, kio_to_pp, pair_layout,
                                              _walk_seed)
    ng, no = 100_000, 20_000
    cfg = WL.batch_config(n_walkers=ng)
    trip = WL.batch_triplets(256, seed=1)
    picks = [trip[i] for i in BATCH_PICKS]
    k0, r0, v0, _ = trip[0]
    picks.append((k0, r0, v0, 27))
    ens = WL.build_ensembles(picks, cfg, seed=500, threads=8)
    assert len(ens[-1].seeds) == 27
    u = cfg.direction_array()
    _, c = _columns(cfg)
    lay = pair_layout(*c)
    jobs = [WalkJob(e, kio_to_pp(t[0], e.mean_AV, cfg), _walk_seed(0, 0), ng) for e, t in zip(ens, picks)]
    batch = WalkBatch(jobs, cfg, layout=lay, dirs=u, launch=LaunchConfig())
    batch.launch()
    res = batch.results()
    worst = 0.0
    for i, (e, j, r) in enumerate(zip(ens, jobs, res)):
        assert r["counters"]["escaped"] == 0 and r["counters"]["classifier_error"] == 0
        cos_o, sin_o, _ = _oracle_dir_sums(e, cfg, j.pp, (31337 + i, 99), no, u)
        for g, o in ((r["cos"], cos_o), (r["sin"], sin_o)):
            ok, z = _within_3se(g / ng, ng, o / no, no)
            assert ok.all(), (i, picks[i], np.argwhere(~ok), float(z.max()))
            worst = max(worst, float(z.max()))
    print("batched entries: max z over", len(jobs), "entries =", worst)


# ---------------------------------------------------------------------------
# Column reduction of stored Y (grids beyond the fused epilogue)
# ---------------------------------------------------------------------------

def test_reduce_Y_matches_oracle_reduction_on_a_large_column_grid():
    """madi_reduce_Y over a 12-pair x 6-b grid (72 columns, beyond the fused
    epilogue) equals the oracle's fp64 reduction of the same Y to 1e-9."""
    import torch
    from custom_madi_gb300 import _native as N
    from custom_madi_gb300.ensemble import create_ensemble
    from custom_madi_gb300.walker_gpu import WalkBatch, WalkJob, fused_supported, pair_layout, simulate_jobs
    from oracle import oracle as O
    n = 4096
    cfg = SimConfig(boundary_mode="periodic", n_cells=64, n_walkers=n, n_ensembles=1, ts=0.01, T_max_ms=30.0,
                    h_ms=1.0, small_deltas=[2.0, 4.0, 6.0], big_deltas=[8.0, 12.0, 16.0, 20.0],
                    b_values=[0.0, 500.0, 1000.0, 2000.0, 4000.0, 6000.0],
                    geometry_validation_points=20_000, geometry_vi_tolerance=0.1)
    cols, c = _columns(cfg)
    assert cols.n_pairs == 12 and not fused_supported(pair_layout(*c), 3)
    ens = create_ensemble(2.0e5, 4.0, cfg, seed=3)
    b = WalkBatch([WalkJob(ens, 0.01, 5, n)], cfg, out_mode=N.MADI_OUT_Y)
    b.launch()
    dev = b.dev
    jd, jD, js = (torch.from_numpy(np.asarray(x, np.int32)).to(dev) for x in c[:3])
    pc = torch.from_numpy(np.asarray(c[3], np.float64)).to(dev)
    cs = torch.empty(len(pc), dtype=torch.float64, device=dev)
    ss = torch.empty_like(cs)
    N.reduce_Y(b.Y, n, cfg.n_grid, jd, jD, js, pc, cs, ss, torch.cuda.current_stream(dev))
    Y = b.Y.cpu().numpy()
    oc, os_ = O.reduce(Y, *c)
    np.testing.assert_allclose(cs.cpu().numpy(), oc, rtol=1e-9, atol=1e-9 * 3 * n)
    np.testing.assert_allclose(ss.cpu().numpy(), os_, rtol=1e-9, atol=1e-9 * 3 * n)
    # the public path (simulate_jobs falls back to Y + reduce here) gives the same sums
    r = simulate_jobs([WalkJob(ens, 0.01, 5, n)], cfg, c, dirs=np.eye(3))[0]
    np.testing.assert_allclose(r["cos"][:, 0], oc, rtol=1e-9, atol=1e-9 * 3 * n)


# ---------------------------------------------------------------------------
# Public entry points against the oracle
# ---------------------------------------------------------------------------

def _periodic_cfg(n_walkers, n_ens=2, n_cells=48, directions=None):
    from custom_madi_gb300 import workloads as WL
    return replace(WL.plain_config(n_walkers=n_walkers, directions=directions or 0), n_cells=n_cells,
                   n_ensembles=n_ens, geometry_validation_points=20_000, geometry_vi_tolerance=0.1)


def _oracle_entry(rho, V, kio, cfg, seed, no):
    """Oracle signal S [n_cols] of one (rho, V, kio) entry over the entry's ensembles
    (rebuilt from the same seeds), each walked on an independent key."""
    from custom_madi_gb300.walker_gpu import _build_ensembles_for_entry, _pp_for
    u = cfg.direction_array()
    tot = 0.0
    for e, ens in enumerate(_build_ensembles_for_entry(rho, V, cfg, seed, False)):
        cs, _, _ = _oracle_dir_sums(ens, cfg, _pp_for(ens, kio, cfg), (777 + e, 3), no, u)
        tot = tot + cs.sum(axis=1)
    return tot / (len(u) * no * int(cfg.n_ensembles))


def test_run_simulation_reduced_and_multi_kio_within_3_se_of_oracle():
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300.walker_gpu import run_simulation_multi_kio_reduced, run_simulation_reduced
    ng, no = 40_000, 10_000
    cfg = _periodic_cfg(ng)
    cols, c = _columns(cfg)
    one = run_simulation_reduced(3.0e5, 2.5, 15.0, *c, cfg=cfg, seed=4, verbose=False)
    assert one.n_walkers == 2 * ng and one.n_escaped == 0 and len(one.ensemble_cos_means) == 2
    Sg = one.cos_sum / one.n_eff
    So = _oracle_entry(3.0e5, 2.5, 15.0, cfg, 4, no)
    ok, z = _within_3se(Sg, 2 * ng, So, 2 * no)
    assert ok.all(), z.max()
    multi = S.compute_signals_multi_kio(3.0e5, 2.5, [15.0, 60.0], cfg, seed=4, verbose=False)
    # the same (ensemble, kio) job gives the same exact sums whether walked alone or in the sweep
    np.testing.assert_array_equal(multi[15.0]["S"].ravel(), Sg)
    So60 = _oracle_entry(3.0e5, 2.5, 60.0, cfg, 4, no)
    ok, z = _within_3se(multi[60.0]["S"].ravel(), 2 * ng, So60, 2 * no)
    assert ok.all(), z.max()
    # faster exchange, lower signal at the longest Delta and highest b
    assert multi[60.0]["S"][-1, -1] < multi[15.0]["S"][-1, -1]
    raw = run_simulation_multi_kio_reduced(3.0e5, 2.5, [15.0], *c, cfg=cfg, seed=4, verbose=False)[15.0]
    assert [float(x[0]) for x in raw.ensemble_cos_means] == [float(x[0]) for x in one.ensemble_cos_means]


def test_library_entry_vector_within_3_se_of_oracle_signal():
    """One entry of build_library_from_triplets (two ensembles, 24 directions,
    v4 artifact) against the oracle signal of the same ensembles."""
    from custom_madi_gb300.library import build_library_from_triplets
    ng, no = 40_000, 10_000
    cfg = _periodic_cfg(ng, directions=24)
    lib = build_library_from_triplets([(25.0, 1.5e6, 0.5), (8.0, 1.5e6, 0.5)], cfg=cfg, seed=9, verbose=False,
                                      v5_diagnostics=False)
    assert len(lib) == 2
    e = [x for x in lib if x.kio_nominal == 25.0][0]
    So = _oracle_entry(1.5e6, 0.5, 25.0, cfg, 9, no)
    ok, z = _within_3se(e.vector, 2 * ng, So, 2 * no)
    assert ok.all(), z.max()


def test_build_library_sub_grid_mode_equals_its_triplets():
    """build_library (cross product, madi/library.py:649-670) builds exactly the
    triplet-mode entries of its kios x rhos x Vs grid, bit-identical, and skips
    existing keys on append."""
    from custom_madi_gb300.library import _entry_key, build_library, build_library_from_triplets
    cfg = _periodic_cfg(4000, n_cells=32)
    kios, rhos, Vs = [5.0, 40.0], [4.0e5], [1.5, 2.0]
    grid = build_library(kios, rhos, Vs, cfg=cfg, seed=2, verbose=False, v5_diagnostics=False)
    trip = build_library_from_triplets([(k, r, v) for k in kios for r in rhos for v in Vs], cfg=cfg, seed=2,
                                       verbose=False, v5_diagnostics=False)
    key = lambda e: _entry_key(e.kio_nominal, e.rho_nominal, e.V_nominal)  # noqa: E731
    assert sorted(map(key, grid)) == sorted(_entry_key(k, r, v) for k in kios for r in rhos for v in Vs)
    tb = {key(e): e for e in trip}
    for e in grid:
        np.testing.assert_array_equal(e.vector, tb[key(e)].vector)
    again = build_library(kios, rhos, Vs + [1.0], cfg=cfg, seed=2, verbose=False, v5_diagnostics=False,
                          existing_library=grid)
    assert len(again) == len(grid) + 2
    assert all(a is b for a, b in zip(again[:len(grid)], grid))


# ---------------------------------------------------------------------------
# C ABI: the persistent batched entry point
# ---------------------------------------------------------------------------

def test_walk_batched_abi_equals_walk():
    """madi_walk_batched (grid sized by the library) gives the exact sums of madi_walk."""
    import torch
    from custom_madi_gb300 import _native as N
    from custom_madi_gb300.walker_gpu import WalkBatch, WalkJob, pair_layout
    cfg, ens = _plain_box(3000)
    _, c = _columns(cfg)
    lay = pair_layout(*c)
    _, ens2 = _plain_box(3000)
    jobs = [WalkJob(ens, 0.01, 42, 3000), WalkJob(ens2, 0.02, 7, 1500)]
    b = WalkBatch(jobs, cfg, layout=lay, dirs=cfg.direction_array())
    b.launch()
    want = [r["cos_fixed"].copy() for r in b.results()]
    d = N.MadiWalkDesc.from_buffer_copy(bytes(b.desc))
    d.grid_blocks = 0
    s = torch.cuda.current_stream(b.dev)
    b.work_counter.zero_()
    b.accum.zero_()
    b.occupancy.zero_()
    b.counters.zero_()
    N.check(N.lib().madi_walk_batched(C.byref(d), s.cuda_stream), "madi_walk_batched")
    got = [r["cos_fixed"] for r in b.results()]
    for a, g in zip(want, got):
        np.testing.assert_array_equal(a, g)


def test_reduce_Y_at_the_production_column_grid():
    """The reference's default (delta, Delta, b) grid: 1,245 pairs x 25 b =
    31,125 columns at T = 128 ms.  A walked Y of 1,024 walkers reduced on the GPU
    equals the oracle's fp64 reduction to 1e-9, bit-identically run to run."""
    import torch
    from custom_madi_gb300 import _native as N
    from custom_madi_gb300.ensemble import create_ensemble
    from custom_madi_gb300.walker_gpu import WalkBatch, WalkJob
    from oracle import oracle as O
    n = 1024
    cfg = SimConfig(boundary_mode="periodic", n_cells=64, n_walkers=n, n_ensembles=1, ts=0.01,
                    geometry_validation_points=20_000, geometry_vi_tolerance=0.1)
    cols, c = _columns(cfg)
    assert len(c[3]) == 31_125 and cfg.n_grid == 129
    ens = create_ensemble(2.0e5, 4.0, cfg, seed=8)
    b = WalkBatch([WalkJob(ens, 0.02, 17, n)], cfg, out_mode=N.MADI_OUT_Y)
    b.launch()
    dev = b.dev
    jd, jD, js = (torch.from_numpy(np.asarray(x, np.int32)).to(dev) for x in c[:3])
    pc = torch.from_numpy(np.asarray(c[3], np.float64)).to(dev)
    outs = []
    for _ in range(2):
        cs = torch.empty(len(pc), dtype=torch.float64, device=dev)
        ss = torch.empty_like(cs)
        N.reduce_Y(b.Y, n, cfg.n_grid, jd, jD, js, pc, cs, ss, torch.cuda.current_stream(dev))
        outs.append((cs.cpu().numpy(), ss.cpu().numpy()))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    oc, os_ = O.reduce(b.Y.cpu().numpy(), *c)
    np.testing.assert_allclose(outs[0][0], oc, rtol=1e-9, atol=1e-9 * 3 * n)
    np.testing.assert_allclose(outs[0][1], os_, rtol=1e-9, atol=1e-9 * 3 * n)
