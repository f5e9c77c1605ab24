"""Library builder (batched walker) and the reference-facing match API on the GPU."""

import numpy as np
import pytest

from custom_madi_gb300 import library as Lb
from custom_madi_gb300.config import SimConfig, evenly_spaced_bvalues

pytestmark = pytest.mark.gpu


def test_match_voxels_batch_api_vs_reference(golden):
    m = golden("match.npz")
    lib = [Lb.LibraryEntry(float(k), float(r), float(v), m["lib"][i]) for i, (k, r, v) in
           enumerate(zip(m["kio"], m["rho"], m["V"]))]
    triples = [(10.0, 20.0, float(b)) for b in m["bvals"]]
    kw = dict(lib_delta_pairs=[(10.0, 20.0)], lib_b_values=list(m["bvals"]), n_b=len(m["bvals"]), fit_triples=triples)
    kio, rho, V, res = Lb.match_voxels_batch(m["measured"], lib, **kw)
    assert np.mean(kio == m["best_kio"]) >= 0.995
    k2, _, _, _, s0 = Lb.match_voxels_batch_fits0(m["raw"], lib, **kw)
    assert np.mean(k2 == m["free_kio"]) >= 0.995
    with pytest.raises(RuntimeError, match="GPU only"):
        Lb.match_voxels_batch(m["measured"], lib, use_gpu=False, **kw)


def test_batched_v5_build_save_load_append(tmp_path):
    cfg = SimConfig(boundary_mode="periodic", n_cells=40, n_walkers=512, n_ensembles=2, ts=0.01, T_max_ms=110.0,
                    small_deltas=[5.0, 7.0, 10.0, 12.0, 15.0, 20.0, 25.0, 30.0],
                    big_deltas=[15.0, 25.0, 30.0, 36.0, 40.0, 50.0, 60.0, 80.0],
                    b_values=list(evenly_spaced_bvalues()), geometry_validation_points=20_000,
                    geometry_vi_tolerance=0.1)
    path = tmp_path / "lib.npz"
    lib = Lb.build_library_from_triplets([(10.0, 4.0e5, 1.75), (30.0, 4.0e5, 1.75), (0.0, 0.0, 0.0)], cfg,
                                         save_path=str(path), seed=3, verbose=False)
    assert len(lib) == 3
    cols = Lb.sig.build_columns(cfg)
    for e in lib:
        S = e.vector.reshape(cols.n_pairs, cols.n_b)
        assert np.all(S[:, 0] == 1.0)                       # b = 0: cos(0) summed exactly
        assert np.all(S > -0.05) and np.all(S <= 1.0)
        assert np.all(e.signal_variance >= 0.0) and e.ensemble_means_subset.shape == (2, 200)
    free = [e for e in lib if e.is_free_water][0]
    cell = [e for e in lib if not e.is_free_water]
    assert np.isnan(free.kio) and cell[0].kio_nominal == 10.0
    assert np.mean(cell[1].vector) > np.mean(free.vector)   # restriction slows the decay
    back = Lb.load_library(str(path))
    assert [e.kio_nominal for e in back] == [e.kio_nominal for e in lib]
    assert np.array_equal(back[0].vector, lib[0].vector)
    again = Lb.build_library_from_triplets([(10.0, 4.0e5, 1.75), (50.0, 4.0e5, 1.75)], cfg, existing_library=back,
                                           seed=3, verbose=False)
    assert len(again) == 4 and again[-1].kio_nominal == 50.0


def test_v5_entry_on_the_si_production_grid():
    """One v5 entry in the reference's production configuration: SI finite
    domain (fatal escape, the certified <A/V> table), dt = 1 us, T = 128 ms
    (128,000 steps), the 31,125-column grid (stored Y + column reduction), two
    ensembles.  The v5 arrays have the reference's shapes; S(b = 0) = 1; the
    200-column ensemble subset of each ensemble lies within 3 Monte Carlo
    standard errors of the oracle's walk of the same ensemble."""
    from custom_madi_gb300.walker_gpu import _build_ensembles_for_entry, _pp_for, pair_layout
    from oracle import oracle as O
    ng, no = 4096, 1024
    cfg = SimConfig(n_walkers=ng, n_ensembles=2)
    cols = Lb.sig.build_columns(cfg)
    assert cols.n_pairs * cols.n_b == 31_125 and cfg.n_steps == 128_000
    lib = Lb.build_library_from_triplets([(20.0, 2.0e5, 4.0)], cfg, seed=5, verbose=False)
    e = lib[0]
    assert e.vector.shape == (31_125,) and e.signal_variance.shape == (31_125,)
    assert e.signal_imag.shape == (31_125,) and e.ensemble_means_subset.shape == (2, 200)
    S = e.vector.reshape(cols.n_pairs, cols.n_b)
    assert np.all(S[:, 0] == 1.0)
    assert e.metadata["boundary"]["n_escaped"] == 0
    sub = Lb.ensemble_mean_subset_column_indices(cols)
    jd, jD, js, pc = (np.asarray(x)[sub] for x in (cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef))
    lay = pair_layout(jd, jD, js, pc)
    for k, ens in enumerate(_build_ensembles_for_entry(2.0e5, 4.0, cfg, 5, False)):
        out = O.walk(O.geom_arrays(ens), n_walkers=no, n_steps=cfg.n_steps, steps_per_h=cfg.steps_per_h,
                     n_grid=cfg.n_grid, sigma=cfg.sigma, ts=cfg.ts, pp=_pp_for(ens, 20.0, cfg), key=(900 + k, 1),
                     want_Y=False, columns=(lay.jd, lay.jD, lay.js, lay.coef))
        So = np.zeros(len(sub))
        cs = out["cos_sum"].sum(axis=2) / (3.0 * no)             # [pairs, b] of the layout
        for p in range(lay.n_pairs):
            for b in range(lay.n_b):
                if lay.col_of[p, b] >= 0:
                    So[lay.col_of[p, b]] = cs[p, b]
        Sg = e.ensemble_means_subset[k].astype(np.float64)
        se = np.sqrt(np.maximum(1.0 - So ** 2, 0.0) * (1.0 / ng + 1.0 / no)) + 1e-6   # fp32 storage of the subset
        assert np.all(np.abs(Sg - So) <= 3.0 * se), float(np.max(np.abs(Sg - So) / se))
