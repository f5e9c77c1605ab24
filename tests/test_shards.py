"""Streamed shard merge against the reference's own merge script
(scripts/merge_shards.py, run by tests/golden/make_golden.py on shards the
reference wrote): same entries in the same order, same arrays."""

from __future__ import annotations

import shutil
from pathlib import Path

import numpy as np
import pytest

from custom_madi_gb300.shards import check_coverage, main, merge_shards, npz_member

SHARDS = Path(__file__).resolve().parent / "golden" / "shards"


def _paths():
    return [str(SHARDS / f"lib.shard{i}.npz") for i in range(3)]


@pytest.mark.parametrize("chunk_rows", [4096, 1])
def test_merge_equals_reference_merge(tmp_path, chunk_rows):
    out = tmp_path / "merged.npz"
    rep = merge_shards(_paths(), str(out), require_shards=3, chunk_rows=chunk_rows, verbose=False)
    assert [s["new"] for s in rep["shards"]] == [3, 1, 2]            # duplicates: first occurrence wins
    ref = np.load(SHARDS / "merged_by_reference.npz")
    got = np.load(out)
    assert set(got.files) == set(ref.files)
    for k in ref.files:
        a, b = got[k], ref[k]
        assert a.shape == b.shape, k
        if a.dtype.kind in "US":
            assert a.tolist() == b.tolist(), k
        else:
            assert a.dtype == b.dtype, k
            assert np.array_equal(a, b, equal_nan=a.dtype.kind == "f"), k


def test_merged_artifact_loads_and_the_signal_matrix_is_memory_mapped(tmp_path):
    from custom_madi_gb300.library import load_library, load_library_meta
    out = tmp_path / "merged.npz"
    merge_shards(_paths(), str(out), verbose=False)
    lib = load_library(str(out))
    assert len(lib) == 6 and sum(e.is_free_water for e in lib) == 1
    assert load_library_meta(str(out))["has_v5_diagnostics"]
    v = npz_member(str(out), "vectors")
    assert isinstance(v, np.memmap) and v.shape == (6, len(lib[0].vector))
    assert np.array_equal(np.asarray(v), np.stack([e.vector for e in lib]))


def test_merge_refuses_mismatched_or_incomplete_shards(tmp_path):
    with pytest.raises(ValueError, match="coverage"):
        check_coverage(_paths()[:2], 3)
    from custom_madi_gb300.library import load_library, _save_library, load_library_meta
    from custom_madi_gb300.config import SimConfig
    from custom_madi_gb300.signal import build_columns
    odd = tmp_path / "lib.shard3.npz"
    meta = load_library_meta(_paths()[0])["build_metadata"]
    meta = dict(meta, build_seed=99)
    cfg = SimConfig(n_walkers=2, n_ensembles=2, small_deltas=[5.0, 7.0, 10.0, 12.0, 15.0, 20.0, 25.0, 30.0],
                    big_deltas=[15.0, 25.0, 30.0, 36.0, 40.0, 50.0, 60.0, 80.0])
    _save_library(load_library(_paths()[0]), str(odd), cfg=cfg, columns=build_columns(cfg), build_metadata=meta)
    with pytest.raises(ValueError, match="mismatch"):
        merge_shards(_paths() + [str(odd)], str(tmp_path / "x.npz"), verbose=False)
    shutil.copy(_paths()[0], tmp_path / "lib.shard0.npz")
    assert main([str(tmp_path / "lib.shard0.npz"), "-o", str(tmp_path / "y.npz"), "--require-shards", "1"]) == 0
