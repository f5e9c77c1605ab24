"""The package as a drop-in for the reference's ``madi``: the alias resolves every
submodule, and the contracts the reference's API-level tests hold
(tests/physics_audit/test_reference_path.py:19-100,
tests/physics_audit/test_p0_remediation.py:38-110) hold here, called through
``import madi``.  The calls that run a walk or a match need the GPU (this
package has no CPU path) and are marked accordingly."""

from __future__ import annotations

import inspect
import math
import sys
from dataclasses import fields

import numpy as np
import pytest


@pytest.fixture(scope="module")
def madi():
    import custom_madi_gb300 as pkg
    saved = {k: v for k, v in sys.modules.items() if k == "madi" or k.startswith("madi.")}
    for k in saved:
        del sys.modules[k]
    pkg.install_madi_alias()
    import madi as m
    yield m
    for k in [k for k in sys.modules if k == "madi" or k.startswith("madi.")]:
        del sys.modules[k]
    sys.modules.update(saved)


def test_alias_resolves_every_submodule(madi):
    import custom_madi_gb300 as pkg
    from madi.walker_gpu import run_simulation_multi_kio_reduced, run_walk_Y  # noqa: F401
    from madi.library import LibraryEntry, match_voxels_batch  # noqa: F401
    from madi import signal as sig, config, ensemble, fitters_gpu  # noqa: F401
    assert madi is pkg and sig is pkg.signal and madi.walker_gpu is pkg.walker_gpu
    with pytest.raises(RuntimeError):
        pkg.install_madi_alias("json")          # a different module already owns that name


def test_constants_step_and_einstein_increment(madi):
    from madi.config import D0_UM2_MS, GAMMA_RAD, SimConfig
    cfg = SimConfig()
    assert D0_UM2_MS == 3.0 and cfg.ts == 1e-3
    assert math.isclose(cfg.sigma, math.sqrt(6.0e-3))
    assert math.isclose(cfg.ls_rms ** 2, 6.0 * cfg.D0 * cfg.ts)
    assert math.isclose(GAMMA_RAD, 2.675222e8)


def test_eq5_round_trip_and_rejection(madi):
    from madi.config import SimConfig
    from madi.walker_gpu import kio_to_pp, pp_to_kio, pp_to_kio_eq5
    cfg = SimConfig()
    pp = kio_to_pp(12.0, 0.5, cfg)
    assert math.isclose(pp, (12.0 / 1000.0) / (math.sqrt(3.0 / 0.006) * 0.5))
    assert math.isclose(pp_to_kio(pp, 0.5, cfg), 12.0)
    assert math.isclose(pp_to_kio_eq5(0.005, 0.5, cfg), 0.005 * math.sqrt(3.0 / 0.006) * 0.5 * 1000.0)
    with pytest.raises(ValueError, match=r"\[0, 1\]"):
        kio_to_pp(1.0e7, 0.5, cfg)


def test_gradient_of_b_round_trips(madi):
    from madi.config import GAMMA_RAD
    from madi.signal import G_from_b
    g = G_from_b(4000.0, 20.0, 50.0)
    b = (GAMMA_RAD * g * 20.0e-3) ** 2 * ((50.0 - 20.0 / 3.0) * 1e-3) / 1e6
    assert math.isclose(b, 4000.0)


def test_column_order_is_pair_major(madi):
    from madi.library import _grid_columns
    cols = _grid_columns([(20.0, 50.0, 0.0), (20.0, 50.0, 1000.0)], [(1.0, 1.0), (20.0, 50.0)],
                         [0.0, 500.0, 1000.0], n_b=3)
    assert cols.tolist() == [3, 5]


def test_withdrawn_calibration_api_is_absent(madi, tmp_path):
    from madi import signal as sig
    from madi.config import SimConfig
    from madi.library import LibraryEntry, _save_library
    from madi.walker_gpu import run_simulation_multi_kio_reduced, run_simulation_reduced
    assert "calibrate_exchange" not in inspect.signature(run_simulation_reduced).parameters
    assert "calibrate_exchange" not in inspect.signature(run_simulation_multi_kio_reduced).parameters
    assert "kio_measured_se" not in {f.name for f in fields(LibraryEntry)}
    cfg = SimConfig(n_walkers=8, n_ensembles=2, T_max_ms=4.0, small_deltas=[1.0], big_deltas=[2.0],
                    b_values=[0.0, 500.0])
    out = tmp_path / "lib.npz"
    _save_library([LibraryEntry(10.0, 5.0e5, 1.4, np.asarray([1.0, 0.7]), vi=0.7)], str(out), cfg=cfg,
                  columns=sig.build_columns(cfg))
    with np.load(out, allow_pickle=False) as d:
        assert "kio_measured_se" not in d.files


def test_signal_payload_has_no_survivor_bookkeeping(madi):
    from madi import signal as sig
    from madi.config import SimConfig
    from madi.walker_gpu import ReducedResult
    cfg = SimConfig(T_max_ms=4.0, small_deltas=[1.0], big_deltas=[2.0], b_values=[0.0, 500.0])
    cols = sig.build_columns(cfg)
    r = ReducedResult(cos_sum=np.ones(cols.n_pairs * cols.n_b), sin_sum=np.zeros(cols.n_pairs * cols.n_b),
                      n_walkers=8, n_escaped=0, occupancy_counts=np.zeros(cfg.n_grid, np.int64))
    payload = sig._assemble(r, cols)
    assert payload["n_escaped"] == 0 and "surviving_walkers_by_checkpoint" not in payload
    assert np.allclose(payload["S"], 1.0 / 24.0)      # n_eff = 3 axes x 8 walkers = 24


def test_cpu_paths_raise_instead_of_falling_back(madi):
    from madi.config import SimConfig
    from madi.ensemble import create_dummy_ensemble
    from madi.library import LibraryEntry, match_voxels_batch
    from madi.walker_gpu import run_walk_Y
    cfg = SimConfig(L=2.0, n_walkers=1, n_ensembles=1, T_max_ms=2.0, small_deltas=[1.0], big_deltas=[1.0],
                    b_values=[0.0])
    with pytest.raises(RuntimeError, match="GPU only"):
        run_walk_Y(create_dummy_ensemble(cfg), 0.0, cfg, pp=0.0, verbose=False, use_gpu=False)
    lib = [LibraryEntry(11.0, 1e6, 0.8, np.array([0.8, 0.5, 0.3]))]
    with pytest.raises(RuntimeError, match="GPU only"):
        match_voxels_batch(np.ones((1, 3)), lib, [(20.0, 50.0)], [500.0, 1000.0, 1500.0], 3,
                           [(20.0, 50.0, b) for b in (500.0, 1000.0, 1500.0)], use_gpu=False)


@pytest.mark.gpu
def test_matcher_is_exhaustive_deterministic_lowest_index_on_ties(madi):
    from madi.library import LibraryEntry, match_voxels_batch
    lib = [LibraryEntry(11.0, 1_000_000.0, 0.80, np.array([0.8, 0.5, 0.3])),
           LibraryEntry(22.0, 1_000_000.0, 0.81, np.array([0.8, 0.5, 0.3])),
           LibraryEntry(33.0, 1_000_000.0, 0.82, np.array([0.7, 0.4, 0.2]))]
    kw = dict(lib_delta_pairs=[(20.0, 50.0)], lib_b_values=[500.0, 1000.0, 1500.0], n_b=3,
              fit_triples=[(20.0, 50.0, b) for b in (500.0, 1000.0, 1500.0)])
    meas = np.array([[0.8, 0.5, 0.3], [0.71, 0.39, 0.19]])
    for precision in ("fp32", "bf16"):
        first = match_voxels_batch(meas, lib, precision=precision, **kw)
        second = match_voxels_batch(meas, lib, precision=precision, **kw)
        for a, b in zip(first, second):
            assert np.array_equal(a, b)
        kio, rho, V, resid = first
        assert kio.tolist() == [11.0, 33.0] and V.tolist() == [0.80, 0.82]
        assert np.all(resid >= -1e-6)


@pytest.mark.gpu
def test_escape_is_a_hard_error_through_the_alias(madi):
    from madi.config import SimConfig
    from madi.ensemble import create_dummy_ensemble
    from madi.walker_gpu import WalkRandomStream, run_walk_Y
    cfg = SimConfig(L=2.0, n_walkers=1, n_ensembles=1, T_max_ms=2.0, small_deltas=[1.0], big_deltas=[1.0],
                    b_values=[0.0])
    inc = np.zeros((cfg.n_steps, 1, 3))
    inc[0, 0, 0] = 2.0
    st = WalkRandomStream(np.asarray([[1.0, 1.0, 1.0]]), inc, np.zeros((cfg.n_steps, 1)))
    with pytest.raises(RuntimeError, match="fatal boundary condition"):
        run_walk_Y(create_dummy_ensemble(cfg), 0.0, cfg, pp=0.0, verbose=False, random_stream=st)
