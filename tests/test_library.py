"""Library schema, column resolution and grid helpers against the reference's outputs."""

import json
from pathlib import Path

import numpy as np
import pytest

from custom_madi_gb300 import library as Lb
from custom_madi_gb300 import signal as S
from custom_madi_gb300.config import SimConfig

ROOT = Path(__file__).resolve().parents[1]


def _v5_cfg():
    return SimConfig(n_walkers=2, n_ensembles=2, small_deltas=[5.0, 7.0, 10.0, 12.0, 15.0, 20.0, 25.0, 30.0],
                     big_deltas=[15.0, 25.0, 30.0, 36.0, 40.0, 50.0, 60.0, 80.0])


def test_reference_artifact_round_trips_identically(tmp_path):
    """load_library(reference npz) -> _save_library -> every array and the metadata JSON are equal."""
    ref = ROOT / "tests" / "golden" / "library_v5.npz"
    lib = Lb.load_library(str(ref))
    assert len(lib) == 3 and lib[1].weight == 1.5 and lib[2].metadata == {"i": 2}
    cfg = _v5_cfg()
    out = tmp_path / "again.npz"
    Lb._save_library(lib, str(out), cfg=cfg, columns=S.build_columns(cfg), build_seed=7,
                     grid_metadata={"kind": "fixture"})
    a, b = np.load(ref), np.load(out)
    assert set(a.files) == set(b.files)
    for k in a.files:
        if k == "build_metadata_json":
            assert json.loads(str(a[k])) == json.loads(str(b[k]))
        else:
            assert np.array_equal(a[k], b[k]), k
            assert a[k].dtype == b[k].dtype, k
    meta = Lb.load_library_meta(str(out))
    assert meta["format"] == "v2" and meta["has_v5_diagnostics"] and meta["ensemble_means_subset_shape"] == (3, 2, 200)


def test_v5_diagnostics_sample_variance_and_subset():
    cfg = SimConfig(n_walkers=2, n_ensembles=3, small_deltas=[5.0, 7.0, 10.0, 12.0, 15.0, 20.0, 25.0, 30.0],
                    big_deltas=[15.0, 25.0, 30.0, 36.0, 40.0, 50.0, 60.0, 80.0])
    cols = S.build_columns(cfg)
    er = np.stack([np.full((cols.n_pairs, cols.n_b), v) for v in (0.2, 0.4, 0.8)])
    res = {"ensemble_S": er, "ensemble_S_imag": np.zeros_like(er), "S_imag": np.zeros((cols.n_pairs, cols.n_b))}
    im, var, sub, chk = Lb._v5_diagnostics_from_result(res, cols, cfg)
    assert im.dtype == var.dtype == sub.dtype == np.float32
    assert np.allclose(var, np.var([0.2, 0.4, 0.8], ddof=1))
    assert sub.shape == (3, Lb.ENSEMBLE_MEAN_SUBSET_N_COLUMNS)
    assert np.allclose(sub, er.reshape(3, -1)[:, Lb.ensemble_mean_subset_column_indices(cols)])
    assert chk["max_abs_standardized_deviation"] == 0.0


def test_column_resolution_and_keys_vs_reference():
    an = json.loads((ROOT / "tests" / "golden" / "analytic.json").read_text())
    assert Lb._grid_columns([(20.0, 50.0, 0.0), (20.0, 50.0, 1000.0)], [(1.0, 1.0), (20.0, 50.0)],
                            [0.0, 500.0, 1000.0], 3).tolist() == an["grid_cols"]
    for k, r, v, key in an["entry_key"]:
        assert list(Lb._entry_key(k, r, v)) == key
    cols, ev = Lb.resolve_grid_columns([(20.5, 50.0, 1010.0)], [(20.0, 50.0)], [0.0, 1000.0], 2)
    assert cols.tolist() == [1] and {e["axis"] for e in ev} == {"timing", "b"}
    with pytest.raises(ValueError, match="snap tolerance"):
        Lb.resolve_grid_columns([(25.0, 50.0, 0.0)], [(20.0, 50.0)], [0.0], 1)
    with pytest.raises(ValueError, match="not within"):
        Lb.resolve_grid_columns([(20.0, 50.0, 100.0)], [(20.0, 50.0)], [0.0], 1)
    assert Lb._filter_valid([(1, 1e6, 0.5), (1, 1e6, 0.995), (5, 0.0, 0.0)]) == [(1, 1e6, 0.5), (5, 0.0, 0.0)]


def test_remediation_grid_known_answers():
    """tests/physics_audit/test_p0_remediation.py:449-476 pilot grid numbers."""
    g = Lb.make_remediation_log_grid(n_rho=8, n_V=12, kios=np.asarray([0.0, 20.0, 130.0]))
    trip, w = g.triplets_and_weights()
    pairs = sorted({(r, v) for _, r, v in trip if r > 0.0})
    vis = np.array([r * v * 1e-6 for r, v in pairs])
    assert len(pairs) == 8 and len(trip) == 25
    assert np.min(vis) == pytest.approx(0.4282828134809622)
    assert np.max(vis) == pytest.approx(0.9664172475849011)
    assert np.allclose(Lb._cell_widths(np.asarray([0.0, 1.0, 5.0]), 0.0, 5.0), [0.5, 2.5, 2.0])
    assert w[("free_water", 0.0, 0.0)] > 0.0
