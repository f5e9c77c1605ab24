"""Host-side logic and the C ABI boundary (no GPU work)."""

import ctypes as C
import json
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from custom_madi_gb300 import _native as N
from custom_madi_gb300 import config as cfgmod
from custom_madi_gb300 import ensemble as E
from custom_madi_gb300.config import SimConfig
from oracle import oracle as O

ROOT = Path(__file__).resolve().parents[1]


# ------------------------------------------------------------------ C ABI
def test_library_exports_every_declared_symbol():
    header = (ROOT / "include" / "madi_gb300.h").read_text()
    declared = set(re.findall(r"^\s*(?:madi_status|int64_t|int32_t|const char\*)\s+(madi_\w+)\s*\(", header, re.M))
    assert declared >= set(N.EXPORTED) - {"madi_last_error_string"}
    lib = N.lib()
    for name in sorted(declared | set(N.EXPORTED)):
        assert hasattr(lib, name), name
    assert lib.madi_abi_version() == 1


def test_struct_layout_matches_header(tmp_path):
    """ctypes mirrors == the C compiler's layout of the header structs."""
    structs = {"madi_geometry": N.MadiGeometry, "madi_walk_job": N.MadiWalkJob,
               "madi_walk_desc": N.MadiWalkDesc, "madi_match_desc": N.MadiMatchDesc,
               "madi_launch_shape": N.MadiLaunchShape, "madi_serve_config": N.MadiServeConfig,
               "madi_serve_request": N.MadiServeRequest, "madi_serve_done": N.MadiServeDone}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{ROOT}/include/madi_gb300.h"', "int main(void){"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n") if l)
    for cname, py in structs.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(py, fname).offset, (cname, fname)


def test_header_constants_match_the_python_mirror():
    """Every numeric #define of the header that _native mirrors has the same value."""
    header = (ROOT / "include" / "madi_gb300.h").read_text()
    defines = {m.group(1): int(m.group(2)) for m in re.finditer(r"^#define\s+(MADI_\w+)\s+(\d+)\b", header, re.M)}
    mirrored = {k: v for k, v in defines.items() if hasattr(N, k)}
    assert {"MADI_MATCH_FLAG_TEST_STALL", "MADI_MATCH_FLAG_FULL_SCAN"} <= set(mirrored)
    for k, v in mirrored.items():
        assert getattr(N, k) == v, k


def test_bf16_match_scratch_holds_the_candidate_lists():
    """The BF16 scratch grows by two k-entry candidate lists (int32) per voxel."""
    lib = N.lib()
    b8 = lib.madi_match_scratch_bytes(100_000, 20_000, 20, N.MADI_MATCH_BF16, 8)
    b32 = lib.madi_match_scratch_bytes(100_000, 20_000, 20, N.MADI_MATCH_BF16, 32)
    assert b8 > 0 and b32 - b8 >= 100_000 * 2 * (32 - 8) * 4
    assert lib.madi_match_scratch_bytes(200_000, 20_000, 20, N.MADI_MATCH_BF16, 32) > b32


def test_error_string_and_invalid_arguments():
    lib = N.lib()
    st = lib.madi_kdtree_build(None, 0, None, None, None, None, None)
    assert st == N.MADI_ERR_INVALID
    assert b"kdtree_build" in lib.madi_last_error_string()
    with pytest.raises(ValueError, match="kdtree_build"):
        N.check(st, "madi_kdtree_build")


# ------------------------------------------------------------------ config
def test_config_accepts_periodic_and_validates():
    SimConfig(boundary_mode="periodic", small_deltas=[6.0], big_deltas=[15.0], T_max_ms=21.0).assert_grid_alignment()
    with pytest.raises(ValueError, match="boundary_mode"):
        SimConfig(boundary_mode="reflect", small_deltas=[1.0], big_deltas=[1.0], T_max_ms=2.0).assert_grid_alignment()
    with pytest.raises(ValueError, match="integer multiple"):
        cfgmod.grid_time_index(1.5, 1.0)
    with pytest.raises(ValueError, match="T_max_ms"):
        SimConfig(small_deltas=[30.0], big_deltas=[80.0], T_max_ms=100.0).assert_grid_alignment()
    with pytest.raises(RuntimeError):
        SimConfig().grid_size
    c = SimConfig()
    assert np.isclose(c.sigma, np.sqrt(2 * 3.0 * 1e-3)) and c.n_grid == 129 and c.steps_per_h == 1000
    u = cfgmod.fibonacci_directions(24)
    assert u.shape == (24, 3) and np.allclose(np.linalg.norm(u, axis=1), 1.0)
    assert abs(np.mean(u, axis=0)).max() < 0.05


def test_analytic_values_vs_reference(golden):
    an = json.loads((ROOT / "tests" / "golden" / "analytic.json").read_text())
    for vi, rho, a in an["alpha_star"]:
        assert E.alpha_star_from_vi(vi, rho) == a          # the reference's arithmetic, bit for bit
    c0 = SimConfig(ts=0.01, T_max_ms=46.0, small_deltas=[6.0], big_deltas=[15.0, 25.0, 30.0, 40.0],
                   b_values=[0.0, 1000.0, 2500.0, 4000.0, 6000.0])
    for vi, rho, av in an["mean_AV"]:
        assert E.governing_mean_A_over_V(vi, rho, c0)[0] == av
    for rho, tm, side in an["si_domain_side"]:
        assert E.si_domain_side_um(rho, SimConfig(T_max_ms=tm, small_deltas=[1.0], big_deltas=[1.0])) == side
    from custom_madi_gb300 import walker_gpu as W
    from custom_madi_gb300 import signal as S
    for k, av, pp in an["kio_to_pp"]:
        assert W.kio_to_pp(k, av, c0) == pytest.approx(pp, rel=1e-15)
    for b, d, D, G in an["G_from_b"]:
        assert S.G_from_b(b, d, D) == pytest.approx(G, rel=1e-15)
    cols = S.build_columns(c0)
    ref = an["c0_columns"]
    for key in ("j_delta", "j_Delta", "j_sum"):
        assert getattr(cols, key).tolist() == ref[key]
    np.testing.assert_allclose(cols.phase_coef, ref["phase_coef"], rtol=1e-15)
    assert len(cfgmod.valid_delta_pairs()) == an["default_pairs_count"]
    for s, e, ws, es in an["walk_seed"]:
        assert W._walk_seed(s, e) == ws and W._ensemble_seed(s, e) == es
    with pytest.raises(ValueError, match=r"\[0, 1\]"):
        W.kio_to_pp(1.0e7, 0.5, c0)


def test_kdtree_builder_matches_reference_layout(golden):
    k = golden("kdtree.npz")
    seed, axis, left, right, parent = E._build_gpu_kdtree(k["seeds"])
    assert np.array_equal(seed, k["node_seed"]) and np.array_equal(axis, k["node_axis"])
    assert np.array_equal(left, k["node_left"]) and np.array_equal(right, k["node_right"])
    assert np.array_equal(parent, k["node_parent"])


def test_population_draw_order_matches_reference(golden):
    p = golden("population.npz")
    cfg = SimConfig(L=None, T_max_ms=float(p["T_max_ms"]), small_deltas=[1.0], big_deltas=[1.0])
    side = E.si_domain_side_um(float(p["rho"]), cfg)
    assert side == pytest.approx(float(p["L"]))
    rng = np.random.default_rng(int(p["seed"]))
    seeds, _, nn, cert = E._make_population(float(p["rho"]) * 1e-9, side, cfg, rng)
    vi = float(p["rho"]) * float(p["V"]) * 1e-6
    ann = np.minimum(E.alpha_star_from_vi(vi, float(p["rho"])), 0.9 * nn / 2.0)
    assert np.array_equal(seeds, p["seeds"])
    np.testing.assert_allclose(ann, p["annulus"], rtol=1e-14)
    assert json.loads(str(p["certificate"]))["s10_pass"] == cert.s10_pass


def _grid_superset_check(seeds, ann, L, G, h, cap, n_pts, rng):
    xyza = np.column_stack([seeds, ann])
    eps = 1e-4 * h + 1e-6 * L
    off, ids, _ = E.build_voxel_grid(xyza, G, h, eps, cap)
    pts = rng.uniform(0.0, L, size=(n_pts, 3))
    amax = float(np.max(ann))
    for p in pts:
        v = np.minimum((p / h).astype(int), G - 1)
        vox = (v[2] * G + v[1]) * G + v[0]
        lst = set(ids[off[vox]:off[vox + 1]].tolist())
        d = np.linalg.norm(seeds - p, axis=1)
        need = set(np.flatnonzero(d <= d.min() + 2 * amax + 2 * cap).tolist())
        assert need <= lst
    return off, ids


def test_voxel_grid_lists_are_proven_supersets(golden):
    d = golden("classify_si.npz")
    L = float(d["L"])
    G, h, cap = E.default_grid_params(5.0e5, float(np.max(d["annulus"])), L)
    off, ids = _grid_superset_check(d["seeds"], d["annulus"], L, G, h, cap, 3000, np.random.default_rng(1))
    assert len(off) == G ** 3 + 1 and off[-1] == len(ids)


def test_periodic_tiling_is_classification_equivalent(golden):
    """The margin-limited image set labels points exactly like the full 27-image tiling."""
    d = golden("classify_periodic.npz")
    ens = E.ensemble_from_arrays(d["base_seeds"], d["annulus"], float(d["L"]), source_lo=0.0,
                                 source_hi=float(d["L"]), rho_per_uL=float(d["rho"]), boundary_mode="periodic")
    g = O.geom_arrays(ens)
    c, i = O.classify_brute(g, d["points"])
    assert np.array_equal(i, d["inside"]) and np.array_equal(c, d["cell"])
    assert len(ens.classifier_seeds) < 27 * 64


def test_pair_layout_and_thresholds():
    from custom_madi_gb300 import walker_gpu as W
    from custom_madi_gb300 import signal as S
    c0 = SimConfig(ts=0.01, T_max_ms=46.0, small_deltas=[6.0], big_deltas=[15.0, 25.0, 30.0, 40.0],
                   b_values=[0.0, 1000.0, 2500.0, 4000.0, 6000.0])
    cols = S.build_columns(c0)
    lay = W.pair_layout(cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    assert lay.n_pairs == 4 and lay.n_b == 5
    assert lay.col_of.ravel().tolist() == list(range(20))
    assert W.fused_supported(lay, 24) and not W.fused_supported(lay, 33)
    t1, t2 = W._thresholds(0.25)
    assert t1 == 1 << 62 and t2 == 1 << 60
    assert W._thresholds(1.0)[0] == (1 << 64) - 1
    m = W._membrane_transition_counts([1, 1, 1, 1, 1], [True, False, True, True, False], [1, 1, 2, 1, 1],
                                      [False, True, True, True, False])
    assert m.tolist() == [1, 1, 2, 0, 0]


def test_autotune_cache_store_load_roundtrip(tmp_path):
    """Native launch-shape cache: absent -> empty, store / replace / reload, bad keys rejected."""
    import ctypes as C
    from custom_madi_gb300 import _native as N
    path = str(tmp_path / "sub" / "tune.tsv").encode()
    sh = N.MadiLaunchShape()
    assert N.lib().madi_autotune_load(path, b"sm152/seeds512", C.byref(sh)) == 0 and sh.tile_walkers == 0
    for key, tw in ((b"sm152/seeds512", 128), (b"sm152/seeds1024", 256), (b"sm152/seeds512", 64)):
        st = N.lib().madi_autotune_store(path, key, C.byref(N.MadiLaunchShape(tw, 0, 2, 49152, 6.4e9)))
        assert st == 0, N.lib().madi_last_error_string()
    assert N.lib().madi_autotune_load(path, b"sm152/seeds512", C.byref(sh)) == 0
    assert (sh.tile_walkers, sh.blocks_per_sm, sh.min_blocks, sh.stage_budget) == (64, 0, 2, 49152)
    assert sh.walker_steps_per_s == 6.4e9
    assert N.lib().madi_autotune_load(path, b"sm152/seeds1024", C.byref(sh)) == 0 and sh.tile_walkers == 256
    lines = (tmp_path / "sub" / "tune.tsv").read_text().splitlines()
    assert len(lines) == 2
    assert N.lib().madi_autotune_store(path, b"bad\tkey", C.byref(N.MadiLaunchShape(1, 0, 1, 0, 1.0))) == N.MADI_ERR_INVALID


def test_autotune_python_cache_uses_native_store(tmp_path, monkeypatch):
    from custom_madi_gb300 import autotune
    monkeypatch.setenv("MADI_AUTOTUNE_CACHE", str(tmp_path / "t.tsv"))
    assert autotune.load("k1") is None
    assert autotune.store("k1", 256, 0, 1, 0, 5.0e9)
    e = autotune.load("k1")
    assert (e.tile_walkers, e.min_blocks) == (256, 1)


def test_walk_smem_bytes_bounds_the_fused_layout():
    """madi_walk_smem_bytes is an upper bound of the walker's fused shared-memory
    layout (the same sum walker_gpu.WalkBatch sizes its launches with)."""
    from custom_madi_gb300 import _native as N
    from custom_madi_gb300.walker_gpu import FC_BYTES_PER_WALKER
    for stage, tw, n_grid, n_out, np_ in ((0, 128, 47, 4 * 5 * 24, 4), (4096, 256, 401, 8 * 32 * 32, 8)):
        need = stage + 16 * n_out + 12 * ((n_grid + 3) // 4 * 4) + (24 + FC_BYTES_PER_WALKER + 4 * (3 + 3 * np_) + 12) * tw
        assert N.lib().madi_walk_smem_bytes(stage, tw, n_grid) >= need


def test_stage_block_refuses_offsets_past_32_bits():
    """The walker reads stage offsets as uint32: a block of 4 GiB or more (here
    a voxel grid of 2^32 ids' bytes, given as sizes only) is refused, never
    stored wrapped."""
    from custom_madi_gb300 import _native as N
    from custom_madi_gb300.ensemble import stage_offsets
    offs = stage_offsets([16 * 5, 4 * 5, 4 * 9, 2 * 17, 16 * 5, 0, 0])
    assert offs.tolist() == [0, 80, 112, 160, 208, 288, 288, 288]
    with pytest.raises(N.MadiError, match="4 GiB") as ei:
        stage_offsets([16 * 1000, 4 * 1000, 4 * 513, 2 ** 32, 0, 0, 0])
    assert ei.value.status == N.MADI_ERR_CAPACITY
    assert int(stage_offsets([16, 16, 16, 2 ** 32 - 16 * 4, 0, 0, 0])[-1]) == 2 ** 32 - 16
    with pytest.raises(N.MadiError):
        stage_offsets([16, 16, 16, 2 ** 32 - 16 * 3, 0, 0, 0])      # each part under the limit, the sum at it


@pytest.mark.parametrize("rho,V,n_cells,seed", [(2.0e5, 4.0, 64, 0), (5.39597446e7, 0.0152563555, 486, 10),
                                               (4484.29, 177.71676748, 31, 161)])
def test_oracle_geometry_restatement_equals_product_builder(rho, V, n_cells, seed):
    """The oracle's host-only periodic ensemble (the reference arm's geometry)
    draws the package's seeds and annuli bit for bit, with the same alpha*,
    <A/V> and Eq. 5 p_p; its KD build equals the native builder on the same
    distinct-coordinate seeds (a tiled set has exact coordinate ties, where
    the median element is the selection algorithm's choice: both trees are
    exact); and its 27-image classifier set labels points exactly as the
    package's proven-margin set and as the all-seed rule do."""
    from dataclasses import replace
    from custom_madi_gb300 import workloads as WL
    from custom_madi_gb300.walker_gpu import kio_to_pp
    from oracle import geometry as OG
    cfg = replace(WL.batch_config(n_walkers=1000), n_cells=n_cells)
    ens = E.create_ensemble(rho, V, cfg, seed=seed, verify_vi=False, measure_vi=False)
    og = OG.periodic_ensemble(rho, V, n_cells, seed)
    assert np.array_equal(og["seeds"], ens.seeds) and np.array_equal(og["annulus"], ens.annulus)
    assert og["L"] == ens.L and og["alpha_star"] == pytest.approx(ens.alpha_star, rel=1e-12)
    assert og["mean_AV"] == pytest.approx(ens.mean_AV, rel=1e-14)
    assert OG.kio_to_pp(20.0, og["mean_AV"], cfg.D0, cfg.ts) == pytest.approx(kio_to_pp(20.0, ens.mean_AV, cfg),
                                                                              rel=1e-13)
    for a, b in zip(OG.kd_build(og["seeds"]), E._build_gpu_kdtree(og["seeds"])):
        assert np.array_equal(a, b)
    pts = np.random.default_rng(seed + 1).uniform(0.0, ens.L, (3000, 3))
    geo = OG.oracle_geometry(og)
    c_o, i_o = O.classify_kd(geo, pts)
    c_p, i_p = O.classify_kd(O.geom_arrays(ens), pts)
    c_b, i_b = O.classify_brute(geo, pts)
    assert np.array_equal(c_o, c_p) and np.array_equal(i_o, i_p)
    assert np.array_equal(c_o, c_b) and np.array_equal(i_o, i_b)
    assert 0.0 < i_o.mean() < 1.0
