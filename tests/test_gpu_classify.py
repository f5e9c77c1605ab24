"""madi_classify (through the C ABI) against the reference's labels: bit-exact."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _classify(ens, pts, method, f32):
    import torch
    from custom_madi_gb300 import _native as N
    dev = ens.device()
    p = torch.from_numpy(np.ascontiguousarray(pts, np.float32 if f32 else np.float64)).cuda()
    n = len(pts)
    cell = torch.empty(n, dtype=torch.int32, device="cuda")
    inside = torch.empty(n, dtype=torch.uint8, device="cuda")
    path = torch.empty(n, dtype=torch.uint8, device="cuda")
    st = N.lib().madi_classify(C.byref(dev.struct), N.ptr(p), 1 if f32 else 0, n, method, N.ptr(cell),
                               N.ptr(inside), N.ptr(path), torch.cuda.current_stream().cuda_stream)
    N.check(st, "madi_classify")
    torch.cuda.synchronize()
    return cell.cpu().numpy(), inside.cpu().numpy().astype(bool), path.cpu().numpy()


def _si_ensemble(d):
    from custom_madi_gb300.ensemble import ensemble_from_arrays
    return ensemble_from_arrays(d["seeds"], d["annulus"], float(d["L"]), source_lo=float(d["source_lo"]),
                                source_hi=float(d["source_hi"]), rho_per_uL=float(d["rho"]))


def test_kd_fp64_bit_exact_vs_reference(golden):
    d = golden("classify_si.npz")
    ens = _si_ensemble(d)
    assert np.array_equal(ens.kd_node_seed, d["kd_node_seed"])
    c, i, path = _classify(ens, d["points"], 0, False)
    assert np.array_equal(c, d["cell"]) and np.array_equal(i, d["inside"])
    assert np.all(path == 2)


@pytest.mark.parametrize("pts,cell,inside", [("points32", "cell32", "inside32"), ("near32", "cell_near32", "inside_near32")])
def test_grid_fp32_bit_exact_vs_reference(golden, pts, cell, inside):
    d = golden("classify_si.npz")
    ens = _si_ensemble(d)
    c, i, path = _classify(ens, d[pts], 1, True)
    assert np.array_equal(c, d[cell]) and np.array_equal(i, d[inside])
    assert np.mean(path == 1) < 0.05       # fp64 fallbacks are rare
    assert np.all(path != 255)
    c64, i64, _ = _classify(ens, d[pts], 1, False)
    assert np.array_equal(c64, d[cell]) and np.array_equal(i64, d[inside])


def test_grid_periodic_bit_exact_vs_27_image_reference(golden):
    from custom_madi_gb300.ensemble import ensemble_from_arrays
    d = golden("classify_periodic.npz")
    ens = ensemble_from_arrays(d["base_seeds"], d["annulus"], float(d["L"]), source_lo=0.0, source_hi=float(d["L"]),
                               rho_per_uL=float(d["rho"]), boundary_mode="periodic")
    for method, f32 in ((1, True), (0, False), (1, False)):
        c, i, _ = _classify(ens, d["points"], method, f32)
        assert np.array_equal(i, d["inside"]), (method, f32)
        assert np.array_equal(c, d["cell"]), (method, f32)


def test_classify_random_stream_vs_oracle_large():
    """2e5 random fp32 points of a fresh periodic ensemble: device == oracle brute force."""
    from custom_madi_gb300.config import SimConfig
    from custom_madi_gb300.ensemble import create_ensemble
    from oracle import oracle as O
    cfg = SimConfig(boundary_mode="periodic", n_cells=100, ts=0.01, T_max_ms=46.0, small_deltas=[6.0],
                    big_deltas=[15.0, 25.0, 30.0, 40.0], geometry_validation_points=20000, geometry_vi_tolerance=0.05)
    ens = create_ensemble(3.0e5, 0.9 * 1e6 / 3.0e5, cfg, seed=11)
    pts = np.random.default_rng(5).uniform(0, ens.L, size=(200_000, 3)).astype(np.float32).astype(np.float64)
    c, i, path = _classify(ens, pts, 1, True)
    oc, oi = O.classify_kd(O.geom_arrays(ens), pts)
    assert np.array_equal(i, oi) and np.array_equal(c, oc)
    assert np.mean(path == 1) < 0.01
