"""The oracle (C restatement) against vectors produced by the reference itself.

The fixtures come from tests/golden/make_golden.py, which runs the reference's
own classify_cpu, _walk_cpu, _reduce_cpu, match_voxels_batch(_fits0) here.
"""

import numpy as np
import pytest

from oracle import oracle as O


def _si_geom(d):
    kd = (d["kd_node_seed"], d["kd_node_axis"], d["kd_node_left"], d["kd_node_right"], d["kd_node_parent"])
    return O.Geometry(d["seeds"], d["annulus"], kd, float(d["L"]), float(d["source_lo"]), float(d["source_hi"]))


@pytest.mark.parametrize("pts,cell,inside", [("points", "cell", "inside"), ("points32", "cell32", "inside32"),
                                             ("near32", "cell_near32", "inside_near32")])
def test_oracle_classifier_bit_exact_vs_reference(golden, pts, cell, inside):
    d = golden("classify_si.npz")
    g = _si_geom(d)
    c, i = O.classify_kd(g, d[pts])
    assert np.array_equal(c, d[cell]) and np.array_equal(i, d[inside])
    cb, ib = O.classify_brute(g, d[pts])
    assert np.array_equal(cb, d[cell]) and np.array_equal(ib, d[inside])


def test_oracle_periodic_classifier_on_27_images(golden):
    """classify_cpu over the 27-image tiling (cell = tiled index mod 64) == oracle brute force."""
    d = golden("classify_periodic.npz")
    L = float(d["L"])
    base = d["base_seeds"]
    shifts = np.array([[i, j, k] for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)], float) * L
    tiled = (base[None] + shifts[:, None]).reshape(-1, 3)
    ann = np.tile(d["annulus"], 27)
    cell = np.tile(np.arange(64, dtype=np.int32), 27)
    from oracle.geometry import kd_build        # the oracle's own KD build
    kd = kd_build(tiled)
    g = O.Geometry(tiled, ann, kd, L, cell=cell, periodic=True)
    c, i = O.classify_brute(g, d["points"])
    assert np.array_equal(i, d["inside"]) and np.array_equal(c, d["cell"])
    c2, i2 = O.classify_kd(g, d["points"])
    assert np.array_equal(i2, d["inside"]) and np.array_equal(c2, d["cell"])
    assert abs(float(np.mean(d["inside"])) - 0.8) < 0.03


def test_oracle_golden_walk_bit_exact(golden):
    """Fixed-stream walk: Y and inside trace identical to the reference _walk_cpu."""
    w = golden("golden_walk.npz")
    g = _si_geom(w)
    ts = float(w["ts"])
    n_steps = int(round(float(w["T_max_ms"]) / ts))
    sph = int(round(float(w["h_ms"]) / ts))
    ng = int(round(float(w["T_max_ms"]) / float(w["h_ms"]))) + 1
    out = O.walk(g, n_walkers=len(w["init"]), n_steps=n_steps, steps_per_h=sph, n_grid=ng, sigma=float(w["sigma"]),
                 ts=ts, pp=float(w["pp"]), stream=(w["init"], w["incr"], w["unif"]), n_threads=4)
    assert np.array_equal(out["Y"], w["Y"])
    assert np.array_equal(out["inside_trace"], w["inside_trace"])
    assert np.array_equal(out["occupancy"] / len(w["init"]), w["occupancy_fraction"])
    assert out["counters"]["escaped"] == int(w["n_escaped"]) == 0
    assert out["counters"]["cross_accept"] > 0 and out["counters"]["cross_reject"] > 0
    cs, ss = O.reduce(out["Y"], w["j_delta"], w["j_Delta"], w["j_sum"], w["phase_coef"])
    np.testing.assert_allclose(cs, w["cos_sum"], rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(ss, w["sin_sum"], rtol=1e-12, atol=1e-10)


def test_oracle_trapezoid_known_answer(golden):
    t = golden("trapezoid.npz")
    ts = float(t["ts"])
    n_steps = int(round(float(t["T_max_ms"]) / ts))
    sph = int(round(float(t["h_ms"]) / ts))
    free = O.Geometry(np.zeros((2, 3)), np.zeros(2), (np.array([0, 1]), np.array([0, 0]), np.array([-1, -1]),
                                                         np.array([1, -1]), np.array([-1, 0])),
                      float(t["L"]), 0.0, float(t["L"]), has_cells=False)
    out = O.walk(free, n_walkers=1, n_steps=n_steps, steps_per_h=sph, n_grid=3, sigma=0.0, ts=ts, pp=0.0,
                 stream=(t["init"], t["incr"], t["unif"]), n_threads=1)
    assert np.array_equal(out["Y"], t["Y"])


def test_philox_known_answers():
    """Random123 Philox4x32-10 known-answer vectors."""
    assert [hex(x) for x in O.philox([0, 0, 0, 0], 0, 0)] == ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(x) for x in O.philox([0xFFFFFFFF] * 4, 0xFFFFFFFF, 0xFFFFFFFF)] == \
        ["0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(x) for x in O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], 0xA4093822, 0x299F31D0)] == \
        ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_oracle_matcher_vs_reference(golden):
    m = golden("match.npz")
    idx, res = O.match_fixed(m["measured"], m["lib"], chunk=500)
    assert np.array_equal(m["kio"][idx], m["best_kio"]) and np.array_equal(m["V"][idx], m["best_V"])
    np.testing.assert_allclose(res, m["best_resid"], rtol=1e-9, atol=1e-12)
    idx2, res2, s02 = O.match_free(m["raw"], m["lib"], chunk=700)
    assert np.array_equal(m["kio"][idx2], m["free_kio"])
    np.testing.assert_allclose(res2, m["free_resid"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(s02, m["free_s0"], rtol=1e-12)


def test_oracle_matcher_tie_picks_lowest_index():
    lib = np.array([[0.8, 0.5, 0.3], [0.8, 0.5, 0.3], [0.7, 0.4, 0.2]])
    idx, _ = O.match_fixed(np.array([[0.8, 0.5, 0.3], [0.71, 0.39, 0.19]]), lib)
    assert idx.tolist() == [0, 2]


def test_oracle_bayes_matches_reference_bayes_fit(golden):
    """The oracle's fp64 Bayesian fit equals the reference bayes_fit
    (madi/fitters.py:110-243, CPU path) on its fixture, fixed and free S0."""
    from oracle import oracle as O
    b = golden("bayes.npz")
    for mode, meas, free in (("fixed", b["measured"], False), ("free", b["raw"], True)):
        got = O.bayes(meas, b["lib"], b["kio"], b["rho"], b["V"], b["weight"], float(b["sigma_m"]), fit_s0=free)
        for key, val in got.items():
            np.testing.assert_allclose(val, b[f"bayes_{mode}_{key}"], rtol=1e-9, atol=1e-12, err_msg=f"{mode} {key}")
