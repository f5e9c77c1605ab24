"""Generate the golden fixtures under tests/golden/ from the reference itself.

The reference checkout is named on the command line (or by the
MADI_REFERENCE_ROOT environment variable); it is only read.  The reference
package imports matplotlib unconditionally; a two-file stub is placed on
sys.path for the import.  The fixtures are small .npz / .json files that the
tests read; nothing at test time imports the reference.

    python tests/golden/make_golden.py --reference PATH [--only base|api]

``base`` writes the classifier, walk, matcher, analytic, population and
library fixtures; ``api`` the host-API fixtures (random stream, result merge,
Bayes fit, shard merge: api.npz, bayes.npz, shards/).  Without ``--only`` both
are written.
"""

from __future__ import annotations

import json
import os
import sys
import tempfile
from dataclasses import asdict, replace
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REFERENCE_ROOT: Path = None  # set by main() from --reference / MADI_REFERENCE_ROOT


def _import_reference():
    stub = Path(tempfile.mkdtemp(prefix="mpl_stub_")) / "matplotlib"
    stub.mkdir()
    (stub / "__init__.py").write_text("")
    (stub / "pyplot.py").write_text("def __getattr__(name):\n    raise ImportError('stub')\n")
    sys.path[:0] = [str(stub.parent), str(REFERENCE_ROOT)]
    import madi  # noqa: F401
    from madi import config, ensemble, walker_gpu, signal, library
    return config, ensemble, walker_gpu, signal, library


def _test_reference_table(path: Path, ens_mod) -> Path:
    """The schema-valid 26-row uncertified table the reference tests use."""
    vi = np.linspace(0.40, 1.00, 26)
    ax = np.asarray([0.0 if v >= 1.0 else ens_mod.alpha_star_from_vi(v, 1.0e9) for v in vi])
    meta = {"schema": "madi-si-geometry-test-fixture-v1", "source": "unit-test fixture",
            "rho_reference": 1.0, "kappa": 0.90, "n_single_cells": 16, "n_alpha": 26,
            "alpha_spacing": "linear", "mean_estimator": "untrimmed_arithmetic_mean_A_over_V",
            "contraction_rule": "all_shifted_voronoi_facets_S2"}
    np.savez(path, vi=vi, alpha_x=ax, mean_A_over_V_norm=4.0 - 2.0 * vi,
             metadata_json=np.array(json.dumps(meta, sort_keys=True)))
    return path


def main(argv=None) -> int:
    import argparse
    global REFERENCE_ROOT
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reference", default=os.environ.get("MADI_REFERENCE_ROOT"),
                    help="path of the reference checkout (the directory holding the madi package)")
    ap.add_argument("--only", choices=("base", "api"), default=None)
    args = ap.parse_args(argv)
    if not args.reference or not (Path(args.reference) / "madi" / "__init__.py").exists():
        ap.error("--reference (or MADI_REFERENCE_ROOT) must name a checkout of the reference holding madi/")
    REFERENCE_ROOT = Path(args.reference)
    if args.only in (None, "base"):
        base_fixtures()
    if args.only in (None, "api"):
        api_fixtures()
    print("golden fixtures written to", HERE)
    return 0


def base_fixtures() -> None:
    config, E, W, S, Lb = _import_reference()
    tmp = Path(tempfile.mkdtemp(prefix="madi_golden_"))
    table = _test_reference_table(tmp / "table.npz", E)

    # ---- 1. SI-mode classifier: classify_cpu vs brute force on 2,000 points -------
    cfg = config.SimConfig(L=80.0, geometry_reference_path=str(table), allow_uncertified_geometry_reference=True,
                           geometry_validation_points=8000, geometry_vi_tolerance=0.04, n_walkers=96,
                           n_ensembles=1, T_max_ms=4.0, small_deltas=[1.0], big_deltas=[2.0, 3.0],
                           b_values=[0.0, 500.0, 1000.0])
    ens = E.create_ensemble(5.0e5, 1.4, cfg, seed=20_260_901, verify_vi=False)
    pts = np.random.default_rng(20_260_902).uniform(0.0, ens.L, size=(2000, 3))
    ids, inside = ens.classify_cpu(pts)
    pts32 = pts.astype(np.float32).astype(np.float64)
    ids32, inside32 = ens.classify_cpu(pts32)
    # Points concentrated near facets: random points pulled towards seed bisectors.
    rng = np.random.default_rng(20_260_903)
    s1 = ens.seeds[rng.integers(0, len(ens.seeds), 3000)]
    s2 = s1 + rng.normal(0.0, 6.0, size=s1.shape)
    near = 0.5 * (s1 + s2) + rng.normal(0.0, 0.3, size=s1.shape)
    near = near[np.all((near >= 0) & (near < ens.L), axis=1)][:2000]
    near32 = near.astype(np.float32).astype(np.float64)
    ids_n, in_n = ens.classify_cpu(near32)
    np.savez_compressed(
        HERE / "classify_si.npz", seeds=ens.seeds, annulus=ens.annulus, L=ens.L, source_lo=ens.source_lo,
        source_hi=ens.source_hi, kd_node_seed=ens.kd_node_seed, kd_node_axis=ens.kd_node_axis,
        kd_node_left=ens.kd_node_left, kd_node_right=ens.kd_node_right, kd_node_parent=ens.kd_node_parent,
        points=pts, cell=ids, inside=inside, points32=pts32, cell32=ids32, inside32=inside32,
        near32=near32, cell_near32=ids_n, inside_near32=in_n, alpha_star=ens.alpha_star, mean_AV=ens.mean_AV,
        rho=5.0e5, V=1.4, seed=20_260_901)

    # ---- 2. periodic 64-cell box (rho=2e5, v_i=0.8): 27-image tiling -> classify_cpu -
    rho, vi = 2.0e5, 0.8
    L = (64 / (rho * 1e-9)) ** (1.0 / 3.0)
    base = np.random.default_rng(0).uniform(0.0, L, size=(64, 3))
    from scipy.spatial import cKDTree
    nn = cKDTree(base, boxsize=L).query(base, k=2)[0][:, 1]
    a_star = E.alpha_star_from_vi(vi, rho)
    ann = np.minimum(a_star, 0.9 * nn / 2.0)
    shifts = np.array([[i, j, k] for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)], np.float64) * L
    tiled = (base[None, :, :] + shifts[:, None, :]).reshape(-1, 3)
    tiled_ann = np.tile(ann, 27)
    ens_p = replace(ens, seeds=tiled, annulus=tiled_ann, tree=None, L=L)
    ppts = np.random.default_rng(7).uniform(0.0, L, size=(4000, 3)).astype(np.float32).astype(np.float64)
    pid, pin = ens_p.classify_cpu(ppts)
    np.savez_compressed(HERE / "classify_periodic.npz", base_seeds=base, annulus=ann, L=L, rho=rho, vi=vi,
                        alpha_star=a_star, points=ppts, cell=(pid % 64).astype(np.int32), inside=pin)

    # ---- 3. KD tree layout of the reference builder ---------------------------------
    kd = E._build_gpu_kdtree(ens.seeds[:3000])
    np.savez_compressed(HERE / "kdtree.npz", seeds=ens.seeds[:3000], node_seed=kd[0], node_axis=kd[1],
                        node_left=kd[2], node_right=kd[3], node_parent=kd[4])

    # ---- 4. fixed-stream walk (create_gpu_golden semantics, smaller) ----------------
    gcfg = config.SimConfig(L=160.0, geometry_reference_path=str(table), allow_uncertified_geometry_reference=True,
                            geometry_validation_points=10_000, geometry_vi_tolerance=0.03, n_walkers=48,
                            n_ensembles=1, ts=0.01, T_max_ms=10.0, small_deltas=[1.0, 2.0],
                            big_deltas=[2.0, 3.0, 5.0], b_values=[0.0, 500.0, 1000.0, 2000.0])
    gens = E.create_ensemble(1.0e6, 0.9, gcfg, seed=20_260_811, verify_vi=False)
    stream = W.make_walk_random_stream(gcfg, 20_260_812, gens)
    pp = 0.02
    Y, n_esc, tel = W.run_walk_Y(gens, 0.0, gcfg, pp=pp, seed=0, verbose=False, return_telemetry=True,
                                 classifier="exact", random_stream=stream, use_gpu=False)
    _, _, inside_tr, _, _ = W._walk_cpu(gens, pp, gcfg, random_stream=stream)
    cols = S.build_columns(gcfg)
    cs, ss = W._reduce_cpu(Y, cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    np.savez_compressed(
        HERE / "golden_walk.npz", seeds=gens.seeds, annulus=gens.annulus, L=gens.L, source_lo=gens.source_lo,
        source_hi=gens.source_hi, kd_node_seed=gens.kd_node_seed, kd_node_axis=gens.kd_node_axis,
        kd_node_left=gens.kd_node_left, kd_node_right=gens.kd_node_right, kd_node_parent=gens.kd_node_parent,
        init=stream.initial_positions, incr=stream.increments, unif=stream.acceptance_uniforms, pp=pp,
        ts=gcfg.ts, T_max_ms=gcfg.T_max_ms, h_ms=gcfg.h_ms, sigma=gcfg.sigma, Y=Y, inside_trace=inside_tr,
        occupancy_fraction=tel["occupancy_fraction"], n_escaped=n_esc, j_delta=cols.j_delta,
        j_Delta=cols.j_Delta, j_sum=cols.j_sum, phase_coef=cols.phase_coef, cos_sum=cs, sin_sum=ss,
        n_pairs=cols.n_pairs, n_b=cols.n_b)

    # ---- 5. Y trapezoid known answer (tests/physics_audit/test_finite_delta_reference.py:64-99)
    tcfg = config.SimConfig(L=200.0, n_walkers=1, n_ensembles=1, T_max_ms=2.0, h_ms=1.0,
                            small_deltas=[1.0], big_deltas=[1.0, 2.0], b_values=[0.0, 1000.0])
    steps = tcfg.n_steps
    t = np.arange(steps) * tcfg.ts
    inc = np.zeros((steps, 1, 3))
    inc[:, 0, 0] = 4.0e-3 + 2.0e-3 * np.sin(2.0 * np.pi * t / 0.37)
    inc[:, 0, 1] = -1.0e-3 + 1.0e-3 * np.cos(2.0 * np.pi * t / 0.23)
    tstream = W.WalkRandomStream(np.array([[100.0, 100.0, 100.0]]), inc, np.zeros((steps, 1)))
    Yt, _ = W.run_walk_Y(E.create_dummy_ensemble(tcfg), 0.0, tcfg, pp=0.0, seed=0, verbose=False,
                         random_stream=tstream, use_gpu=False)
    np.savez_compressed(HERE / "trapezoid.npz", init=tstream.initial_positions, incr=inc,
                        unif=np.zeros((steps, 1)), L=200.0, ts=tcfg.ts, T_max_ms=2.0, h_ms=1.0, Y=Yt)

    # ---- 6. matcher (fixed and free S0) ---------------------------------------------
    r = np.random.default_rng(3)
    n_lib, n_feat = 400, 12
    Dv = r.uniform(0.2, 3.0, n_lib)[:, None]
    bgrid = np.linspace(0.0, 3.0, n_feat)[None, :]
    lib_mat = np.exp(-bgrid * Dv) * r.uniform(0.8, 1.0, (n_lib, 1)) + 0.02 * r.normal(size=(n_lib, n_feat))
    entries = [Lb.LibraryEntry(float(k), 1.0e6, float(v), lib_mat[i]) for i, (k, v) in
               enumerate(zip(r.uniform(1, 100, n_lib), r.uniform(0.55, 0.9, n_lib)))]
    pairs = [(10.0, 20.0)]
    bvals = list(np.arange(n_feat) * 500.0)
    triples = [(10.0, 20.0, b) for b in bvals]
    meas = lib_mat[r.integers(0, n_lib, 1500)] + 0.01 * r.normal(size=(1500, n_feat))
    kio, rh, vv, res = Lb.match_voxels_batch(meas, entries, pairs, bvals, n_feat, triples, use_gpu=False)
    raw = meas * r.uniform(0.5, 2.0, (1500, 1))
    k2, r2, v2, res2, s02 = Lb.match_voxels_batch_fits0(raw, entries, pairs, bvals, n_feat, triples, use_gpu=False)
    np.savez_compressed(HERE / "match.npz", lib=lib_mat, kio=np.array([e.kio for e in entries]),
                        rho=np.array([e.rho for e in entries]), V=np.array([e.V for e in entries]),
                        measured=meas, best_kio=kio, best_V=vv, best_resid=res, raw=raw, free_kio=k2, free_V=v2,
                        free_resid=res2, free_s0=s02, bvals=np.array(bvals))

    # ---- 7. analytic known answers --------------------------------------------------
    c0 = config.SimConfig(ts=0.01, T_max_ms=46.0, small_deltas=[6.0], big_deltas=[15.0, 25.0, 30.0, 40.0],
                          b_values=[0.0, 1000.0, 2500.0, 4000.0, 6000.0])
    cols0 = S.build_columns(c0)
    an = {
        "alpha_star": [[v, rr, E.alpha_star_from_vi(v, rr)] for v in (0.4, 0.5, 0.6, 0.784, 0.8, 0.9, 0.95, 0.99)
                       for rr in (4.4e3, 1e5, 2e5, 5e5, 1e6, 5.8e7)],
        "mean_AV": [[v, rr, E.governing_mean_A_over_V(v, rr, c0)[0]] for v in (0.5, 0.6, 0.8, 0.9, 0.99)
                    for rr in (4.4e3, 2e5, 1e6)],
        "si_domain_side": [[rr, tm, E.si_domain_side_um(rr, config.SimConfig(T_max_ms=tm, small_deltas=[1.0],
                                                                               big_deltas=[1.0]))]
                           for rr in (0.0, 1e4, 5e5, 1e7) for tm in (46.0, 128.0)],
        "kio_to_pp": [[k, av, W.kio_to_pp(k, av, c0)] for k in (1.0, 20.0, 130.0) for av in (0.5, 1.3, 2.5)],
        "G_from_b": [[b, d, D, S.G_from_b(b, d, D)] for b in (0.0, 1000.0, 6000.0) for d, D in ((6.0, 15.0), (6.0, 40.0),
                                                                                             (20.0, 50.0))],
        "c0_columns": {"j_delta": cols0.j_delta.tolist(), "j_Delta": cols0.j_Delta.tolist(),
                       "j_sum": cols0.j_sum.tolist(), "phase_coef": cols0.phase_coef.tolist(),
                       "n_pairs": cols0.n_pairs, "n_b": cols0.n_b},
        "default_pairs_count": len(config.valid_delta_pairs()),
        "default_n_cols": len(config.valid_delta_pairs()) * len(config.evenly_spaced_bvalues()),
        "walk_seed": [[s, e, W._walk_seed(s, e), W._ensemble_seed(s, e)] for s in (0, 1, 12345) for e in range(4)],
        "entry_key": [[k, rr, v, list(Lb._entry_key(k, rr, v))] for k, rr, v in ((20.0, 2e5, 4.0), (1.23456789, 12345.678, 0.0123456789))],
        "grid_cols": Lb._grid_columns([(20.0, 50.0, 0.0), (20.0, 50.0, 1000.0)], [(1.0, 1.0), (20.0, 50.0)],
                                      [0.0, 500.0, 1000.0], 3).tolist(),
    }
    (HERE / "analytic.json").write_text(json.dumps(an, indent=1))

    # ---- 8. population draw order (seeds + annulus of create_ensemble) --------------
    pcfg = config.SimConfig(L=None, geometry_reference_path=str(table), allow_uncertified_geometry_reference=True,
                            T_max_ms=8.0, small_deltas=[1.0], big_deltas=[1.0], geometry_validation_points=4000)
    pens = E.create_ensemble(5.0e5, 1.6, pcfg, seed=4242, verify_vi=False)
    np.savez_compressed(HERE / "population.npz", seeds=pens.seeds, annulus=pens.annulus, L=pens.L,
                        rho=5.0e5, V=1.6, seed=4242, T_max_ms=8.0,
                        certificate=json.dumps(pens.geometry.population.to_dict()))

    # ---- 9. v5 library artifact written by the reference ----------------------------
    lcfg = config.SimConfig(n_walkers=2, n_ensembles=2, small_deltas=[5.0, 7.0, 10.0, 12.0, 15.0, 20.0, 25.0, 30.0],
                            big_deltas=[15.0, 25.0, 30.0, 36.0, 40.0, 50.0, 60.0, 80.0])
    lcols = S.build_columns(lcfg)
    nc = lcols.n_pairs * lcols.n_b
    sub = Lb.ensemble_mean_subset_column_indices(lcols)
    entries5 = []
    for i in range(3):
        vec = np.linspace(1.0, 0.1 * (i + 1), nc)
        em = np.stack([vec - 0.01, vec + 0.01]).astype(np.float32)
        entries5.append(Lb.LibraryEntry(kio=10.0 * (i + 1), rho=1e5 * (i + 1), V=4.0 / (i + 1), vector=vec,
                                        signal_imag=np.zeros(nc, np.float32),
                                        signal_variance=np.full(nc, 0.02, np.float32),
                                        ensemble_means_subset=em[:, sub], vi=0.4, weight=1.5,
                                        kio_nominal=10.0 * (i + 1), rho_nominal=1e5 * (i + 1),
                                        V_nominal=4.0 / (i + 1), pp=0.01, kio_analytic_eq5=10.0 * (i + 1),
                                        metadata={"i": i}))
    Lb._save_library(entries5, str(HERE / "library_v5.npz"), cfg=lcfg, columns=lcols, build_seed=7,
                     grid_metadata={"kind": "fixture"})


def api_fixtures() -> None:
    """Host-API vectors: make_walk_random_stream's draws, _merge_results order, bayes_fit."""
    config, E, W, S, Lb = _import_reference()
    # ---- 10. make_walk_random_stream (madi/walker_gpu.py:115-127) -------------------
    scfg = config.SimConfig(L=30.0, n_walkers=5, n_ensembles=1, ts=0.01, T_max_ms=0.04, h_ms=0.01,
                            small_deltas=[0.01], big_deltas=[0.01], b_values=[0.0])
    st = W.make_walk_random_stream(scfg, 424242)
    dummy = E.create_dummy_ensemble(scfg)
    # ---- 11. _merge_results (madi/walker_gpu.py:1066-1090) --------------------------
    rng = np.random.default_rng(5)
    parts = []
    for e in range(3):
        parts.append(W.ReducedResult(
            cos_sum=rng.normal(size=4), sin_sum=rng.normal(size=4), n_walkers=10 + e, n_escaped=0,
            occupancy_counts=rng.integers(0, 9, 3).astype(np.int64), pp_values=[0.01 * (e + 1)],
            analytic_kio_eq5_values=[1.5 * (e + 1)], geometry_stats=[{"e": e}],
            ensemble_cos_means=[rng.normal(size=4)], ensemble_sin_means=[rng.normal(size=4)],
            classifier_cache_stats=[{"full": e}]))
    m = W._merge_results(parts)
    # ---- 12. bayes_fit, CPU path of the reference (madi/fitters.py:110-243) ---------
    from madi import fitters as Fi
    r12 = np.random.default_rng(12)
    n_lib, n_feat = 300, 10
    Dv = r12.uniform(0.2, 3.0, n_lib)[:, None]
    bgrid = np.linspace(0.0, 3.0, n_feat)[None, :]
    bmat = np.exp(-bgrid * Dv) * r12.uniform(0.85, 1.0, (n_lib, 1))
    bkio, brho, bV = r12.uniform(1, 100, n_lib), r12.uniform(1e5, 1e6, n_lib), r12.uniform(0.6, 0.9, n_lib)
    bq = r12.uniform(0.5, 2.0, n_lib)
    bents = [Lb.LibraryEntry(float(bkio[i]), float(brho[i]), float(bV[i] * 1e6 / brho[i]), bmat[i],
                             vi=float(bV[i]), weight=float(bq[i])) for i in range(n_lib)]
    bpairs, bbv = [(10.0, 20.0)], list(np.arange(n_feat) * 500.0)
    btrip = [(10.0, 20.0, b) for b in bbv]
    bmeas = bmat[r12.integers(0, n_lib, 400)] + 0.02 * r12.normal(size=(400, n_feat))
    braw = bmeas * r12.uniform(50.0, 2000.0, (400, 1))
    kw = dict(lib_delta_pairs=bpairs, lib_b_values=bbv, n_b=n_feat, fit_triples=btrip, vi_min=0.5, vi_max=0.95,
              use_gpu=False)
    bfix = Fi.bayes_fit(bmeas, bents, sigma_m=0.03, **kw)
    bfree = Fi.bayes_fit(bmeas, bents, sigma_m=0.03, fit_s0=True, raw_signal=braw, **kw)
    # ---- 13. shard merge by the reference's own script (scripts/merge_shards.py) ------
    import subprocess
    sdir = HERE / "shards"
    sdir.mkdir(exist_ok=True)
    for old in sdir.glob("*.npz"):
        old.unlink()
    mcfg = config.SimConfig(n_walkers=2, n_ensembles=2, small_deltas=[5.0, 7.0, 10.0, 12.0, 15.0, 20.0, 25.0, 30.0],
                            big_deltas=[15.0, 25.0, 30.0, 36.0, 40.0, 50.0, 60.0, 80.0])
    mcols = S.build_columns(mcfg)
    mnc = mcols.n_pairs * mcols.n_b
    msub = Lb.ensemble_mean_subset_column_indices(mcols)
    r13 = np.random.default_rng(13)

    def entry(k, rho, V, free=False):
        vec = np.linspace(1.0, 0.05 + 0.001 * k, mnc)
        em = (vec[None, :] + r13.normal(0.0, 0.01, (2, mnc))).astype(np.float32)
        return Lb.LibraryEntry(kio=float("nan") if free else k, rho=0.0 if free else rho, V=0.0 if free else V,
                               vector=vec, signal_imag=r13.normal(0, 1e-3, mnc).astype(np.float32),
                               signal_variance=np.full(mnc, 1e-4, np.float32), ensemble_means_subset=em[:, msub],
                               vi=0.0 if free else rho * V * 1e-6, weight=1.0 + k / 100.0, kio_nominal=k,
                               rho_nominal=rho, V_nominal=V, pp=0.01, kio_analytic_eq5=k, is_free_water=free,
                               metadata={"k": k})
    shard_sets = [[entry(5.0, 2e5, 4.0), entry(10.0, 2e5, 4.0), entry(0.0, 0.0, 0.0, free=True)],
                  [entry(10.0, 2e5, 4.0), entry(15.0, 3e5, 2.0), entry(0.0, 0.0, 0.0, free=True)],
                  [entry(20.0, 3e5, 2.0), entry(5.0, 2e5, 4.0), entry(25.0, 1e5, 5.5)]]
    for i, ents in enumerate(shard_sets):
        Lb._save_library(ents, str(sdir / f"lib.shard{i}.npz"), cfg=mcfg, columns=mcols, build_seed=3,
                         grid_metadata={"kind": "shard fixture"})
    env = dict(os.environ, PYTHONPATH=os.pathsep.join(sys.path))
    subprocess.run([sys.executable, str(REFERENCE_ROOT / "scripts" / "merge_shards.py"),
                    *[str(sdir / f"lib.shard{i}.npz") for i in range(3)], "-o", str(sdir / "merged_by_reference.npz"),
                    "--require-shards", "3"], check=True, env=env, stdout=subprocess.DEVNULL)
    bayes = {f"bayes_fixed_{k}": v for k, v in bfix.items()}
    bayes.update({f"bayes_free_{k}": v for k, v in bfree.items()})
    np.savez_compressed(
        HERE / "bayes.npz", lib=bmat, kio=bkio, rho=brho, V=np.array([e.V for e in bents]), vi=bV, weight=bq,
        measured=bmeas, raw=braw, bvals=np.array(bbv), sigma_m=0.03, **bayes)
    np.savez_compressed(
        HERE / "api.npz", stream_seed=424242, stream_n_walkers=5, stream_n_steps=scfg.n_steps,
        stream_L=30.0, stream_source_lo=dummy.source_lo, stream_source_hi=dummy.source_hi,
        stream_init=st.initial_positions, stream_incr=st.increments, stream_unif=st.acceptance_uniforms,
        merge_in_cos=np.stack([p.cos_sum for p in parts]), merge_in_sin=np.stack([p.sin_sum for p in parts]),
        merge_in_occ=np.stack([p.occupancy_counts for p in parts]),
        merge_in_ens_cos=np.stack([p.ensemble_cos_means[0] for p in parts]),
        merge_in_ens_sin=np.stack([p.ensemble_sin_means[0] for p in parts]),
        merge_cos=m.cos_sum, merge_sin=m.sin_sum, merge_n_walkers=m.n_walkers, merge_occ=m.occupancy_counts,
        merge_pp=np.asarray(m.pp_values), merge_kio=np.asarray(m.analytic_kio_eq5_values),
        merge_ens_cos=np.asarray(m.ensemble_cos_means), merge_ens_sin=np.asarray(m.ensemble_sin_means))


if __name__ == "__main__":
    raise SystemExit(main())
