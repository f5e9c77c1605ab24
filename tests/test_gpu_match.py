"""madi_match against the reference fp64 matcher (fixtures) and the oracle."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_fp32_fixed_s0_vs_reference(golden):
    from custom_madi_gb300.fitters_gpu import map_match_gpu
    m = golden("match.npz")
    kio, rho, V, res = map_match_gpu(m["measured"], m["lib"], m["kio"], m["rho"], m["V"])
    agree = np.mean(kio == m["best_kio"])
    assert agree >= 0.995
    ok = kio == m["best_kio"]
    np.testing.assert_allclose(res[ok], m["best_resid"][ok], rtol=2e-3, atol=2e-6)


def test_fp32_free_s0_vs_reference(golden):
    from custom_madi_gb300.fitters_gpu import map_match_fits0_gpu
    m = golden("match.npz")
    kio, rho, V, res, s0 = map_match_fits0_gpu(m["raw"], m["lib"], m["kio"], m["rho"], m["V"])
    ok = kio == m["free_kio"]
    assert np.mean(ok) >= 0.995
    np.testing.assert_allclose(s0[ok], m["free_s0"][ok], rtol=1e-4)


def test_noise_free_voxels_recover_their_entry():
    from custom_madi_gb300.fitters_gpu import match_device
    rng = np.random.default_rng(0)
    lib = rng.uniform(0.0, 1.0, size=(3000, 20)).astype(np.float32)
    pick = rng.integers(0, 3000, 5000)
    idx, res, _ = match_device(lib[pick], lib)
    assert np.array_equal(idx.cpu().numpy(), pick)
    assert float(res.max()) == 0.0


def test_ties_pick_lowest_index():
    from custom_madi_gb300.fitters_gpu import match_device
    lib = np.array([[0.8, 0.5, 0.3], [0.8, 0.5, 0.3], [0.7, 0.4, 0.2]], np.float32)
    idx, _, _ = match_device(np.array([[0.8, 0.5, 0.3], [0.71, 0.39, 0.19]], np.float32), lib)
    assert idx.cpu().numpy().tolist() == [0, 2]
