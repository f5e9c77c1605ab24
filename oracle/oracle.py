"""Oracle: TEST INFRASTRUCTURE, NOT PRODUCT CODE.

CPU restatement of the reference MADI hot path (jadenfigger/Custom_MADI).  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
checker; custom_madi_gb300 never imports it.

* classify_kd / classify_brute / walk / reduce: ctypes wrappers of
  oracle/madi_oracle.c (see its header for the reference lines it restates);
* match_fixed / match_free: the reference's fp64 numpy matcher
  (madi/library.py:1444-1450 and :1495-1522), chunked over voxels;
* geom_arrays: the classifier inputs of an ensemble-like object.

Pinned against vectors generated from the reference itself
(tests/golden/make_golden.py -> tests/golden/*.npz).
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libmadi_oracle.so"


class _Geom(C.Structure):
    _fields_ = [
        ("n_seeds", C.c_int), ("seeds", C.c_void_p), ("annulus", C.c_void_p), ("cell", C.c_void_p),
        ("kd_seed", C.c_void_p), ("kd_left", C.c_void_p), ("kd_right", C.c_void_p),
        ("kd_parent", C.c_void_p), ("kd_axis", C.c_void_p),
        ("L", C.c_double), ("source_lo", C.c_double), ("source_hi", C.c_double),
        ("periodic", C.c_int), ("has_cells", C.c_int),
    ]


class _Walk(C.Structure):
    _fields_ = [
        ("n_walkers", C.c_int), ("n_steps", C.c_int), ("steps_per_h", C.c_int), ("n_grid", C.c_int),
        ("sigma", C.c_double), ("ts", C.c_double), ("pp", C.c_double),
        ("rng", C.c_int), ("key0", C.c_uint32), ("key1", C.c_uint32), ("walker_base", C.c_uint32),
        ("init", C.c_void_p), ("incr", C.c_void_p), ("unif", C.c_void_p),
        ("Y", C.c_void_p), ("inside_trace", C.c_void_p),
        ("n_pairs", C.c_int), ("n_b", C.c_int), ("n_dirs", C.c_int),
        ("jd", C.c_void_p), ("jD", C.c_void_p), ("js", C.c_void_p),
        ("coef", C.c_void_p), ("dirs", C.c_void_p),
        ("cos_sum", C.c_void_p), ("sin_sum", C.c_void_p), ("occupancy", C.c_void_p),
        ("counters", C.c_int64 * 8), ("n_threads", C.c_int),
    ]


_lib = None


def build() -> Path:
    """Compile the C restatement with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
        _lib.oracle_walk.argtypes = [C.POINTER(_Geom), C.POINTER(_Walk)]
        _lib.oracle_walk.restype = C.c_int
        for name in ("oracle_classify_kd", "oracle_classify_brute"):
            getattr(_lib, name).argtypes = [C.POINTER(_Geom), C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
            getattr(_lib, name).restype = None
        _lib.oracle_reduce.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        _lib.oracle_philox.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]
    return _lib


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class Geometry:
    """Classifier inputs: seeds (N,3), annulus, base cell ids, KD arrays, box."""

    def __init__(self, seeds, annulus, kd, L, source_lo=0.0, source_hi=None, cell=None,
                 periodic=False, has_cells=True):
        self.seeds = _c(seeds, np.float64)
        self.annulus = _c(annulus, np.float64)
        self.cell = None if cell is None else _c(cell, np.int32)
        self.kd = [_c(kd[0], np.int32), _c(kd[1], np.int8), _c(kd[2], np.int32), _c(kd[3], np.int32),
                   _c(kd[4], np.int32)]
        self.s = _Geom(len(self.seeds), self.seeds.ctypes.data, self.annulus.ctypes.data,
                       0 if self.cell is None else self.cell.ctypes.data,
                       self.kd[0].ctypes.data, self.kd[2].ctypes.data, self.kd[3].ctypes.data,
                       self.kd[4].ctypes.data, self.kd[1].ctypes.data, float(L), float(source_lo),
                       float(L if source_hi is None else source_hi), int(bool(periodic)), int(bool(has_cells)))


def geom_arrays(ens) -> Geometry:
    """Oracle geometry of a custom_madi_gb300 Ensemble (the tiled set when periodic)."""
    seeds = ens.classifier_seeds if ens.classifier_seeds is not None else ens.seeds
    ann = ens.classifier_annulus if ens.classifier_annulus is not None else ens.annulus
    cell = ens.classifier_cell
    kd = (ens.kd_node_seed, ens.kd_node_axis, ens.kd_node_left, ens.kd_node_right, ens.kd_node_parent)
    return Geometry(seeds, ann, kd, ens.L, ens.source_lo, ens.source_hi, cell,
                    periodic=ens.boundary_mode == "periodic", has_cells=not ens.is_free_water)


def classify_kd(geom: Geometry, pts) -> tuple[np.ndarray, np.ndarray]:
    p = _c(pts, np.float64)
    cell = np.empty(len(p), np.int32)
    inside = np.empty(len(p), np.uint8)
    lib().oracle_classify_kd(C.byref(geom.s), len(p), p.ctypes.data, cell.ctypes.data, inside.ctypes.data)
    return cell, inside.astype(bool)


def classify_brute(geom: Geometry, pts) -> tuple[np.ndarray, np.ndarray]:
    p = _c(pts, np.float64)
    cell = np.empty(len(p), np.int32)
    inside = np.empty(len(p), np.uint8)
    lib().oracle_classify_brute(C.byref(geom.s), len(p), p.ctypes.data, cell.ctypes.data, inside.ctypes.data)
    return cell, inside.astype(bool)


def philox(ctr, key0, key1) -> np.ndarray:
    c = _c(ctr, np.uint32)
    out = np.empty(4, np.uint32)
    lib().oracle_philox(c.ctypes.data, int(key0), int(key1), out.ctypes.data)
    return out


def walk(geom: Geometry, *, n_walkers, n_steps, steps_per_h, n_grid, sigma, ts, pp,
         stream=None, key=(0, 0), walker_base=0, want_Y=True, columns=None, dirs=None,
         n_threads=None) -> dict:
    """One ensemble walk in fp64.  stream=(init, incr, unif) replays a fixed stream.

    columns=(jd, jD, js, coef[n_pairs, n_b]) with dirs (D,3) asks for the
    per-(pair, b, dir) cos / sin sums of the walkers' phases.
    """
    a = _Walk()
    a.n_walkers, a.n_steps, a.steps_per_h, a.n_grid = int(n_walkers), int(n_steps), int(steps_per_h), int(n_grid)
    a.sigma, a.ts, a.pp = float(sigma), float(ts), float(pp)
    keep = []
    if stream is not None:
        init, incr, unif = (_c(x, np.float64) for x in stream)
        keep += [init, incr, unif]
        a.rng, a.init, a.incr, a.unif = 1, init.ctypes.data, incr.ctypes.data, unif.ctypes.data
    else:
        a.rng = 0
    a.key0, a.key1, a.walker_base = int(key[0]) & 0xFFFFFFFF, int(key[1]) & 0xFFFFFFFF, int(walker_base)
    out = {}
    if want_Y:
        Y = np.zeros((n_walkers, n_grid, 3), np.float64)
        it = np.zeros((n_walkers, n_grid), np.int8)
        a.Y, a.inside_trace = Y.ctypes.data, it.ctypes.data
        out["Y"], out["inside_trace"] = Y, it
    occ = np.zeros(n_grid, np.int64)
    a.occupancy = occ.ctypes.data
    if columns is not None:
        jd, jD, js = (_c(x, np.int32) for x in columns[:3])
        coef = _c(columns[3], np.float64)
        u = _c(np.eye(3) if dirs is None else dirs, np.float64)
        keep += [jd, jD, js, coef, u]
        a.n_pairs, a.n_b, a.n_dirs = len(jd), coef.shape[1], len(u)
        a.jd, a.jD, a.js, a.coef, a.dirs = jd.ctypes.data, jD.ctypes.data, js.ctypes.data, coef.ctypes.data, u.ctypes.data
        cs = np.zeros(len(jd) * coef.shape[1] * len(u))
        ss = np.zeros_like(cs)
        a.cos_sum, a.sin_sum = cs.ctypes.data, ss.ctypes.data
        out["cos_sum"], out["sin_sum"] = cs.reshape(len(jd), coef.shape[1], len(u)), ss.reshape(len(jd), coef.shape[1], len(u))
    a.n_threads = int(n_threads or min(os.cpu_count() or 1, 64))
    lib().oracle_walk(C.byref(geom.s), C.byref(a))
    out["occupancy"] = occ
    cnt = list(a.counters)
    out["counters"] = dict(walkers=cnt[0], escaped=cnt[1], classifier_error=cnt[2], full=cnt[3],
                           cross_accept=cnt[6], cross_reject=cnt[7])
    return out


def reduce(Y, jd, jD, js, coef) -> tuple[np.ndarray, np.ndarray]:
    """Sum over walkers and the 3 axes of cos / sin(coef * dM) (madi/walker_gpu.py:954-968)."""
    Yc = _c(Y, np.float64)
    jd, jD, js = (_c(x, np.int32) for x in (jd, jD, js))
    coef = _c(coef, np.float64)
    cs = np.zeros(len(coef))
    ss = np.zeros(len(coef))
    lib().oracle_reduce(Yc.ctypes.data, Yc.shape[0], Yc.shape[1], jd.ctypes.data, jD.ctypes.data,
                        js.ctypes.data, coef.ctypes.data, len(coef), cs.ctypes.data, ss.ctypes.data)
    return cs, ss


def match_fixed(measured, lib_mat, chunk: int = 20_000) -> tuple[np.ndarray, np.ndarray]:
    """fp64 fixed-S0 MAP: argmin_j |m|^2 + |L_j|^2 - 2 m.L_j, lowest index on ties."""
    M = np.asarray(measured, np.float64)
    Lm = np.asarray(lib_mat, np.float64)
    l2 = np.sum(Lm ** 2, axis=1)[None, :]
    idx = np.empty(len(M), np.int64)
    res = np.empty(len(M), np.float64)
    for s in range(0, len(M), chunk):
        m = M[s:s + chunk]
        d = np.sum(m ** 2, axis=1, keepdims=True) + l2 - 2.0 * m @ Lm.T
        b = np.argmin(d, axis=1)
        idx[s:s + chunk] = b
        res[s:s + chunk] = d[np.arange(len(b)), b]
    return idx, res


def match_free(raw, lib_mat, chunk: int = 20_000) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """fp64 free-S0 MAP: argmin over S0 = m.r/r.r > 0 of |m|^2 - (m.r)^2 / r.r."""
    M = np.asarray(raw, np.float64)
    R = np.asarray(lib_mat, np.float64)
    rr = np.maximum(np.sum(R * R, axis=1), 1e-30)
    idx = np.empty(len(M), np.int64)
    res = np.empty(len(M), np.float64)
    s0 = np.empty(len(M), np.float64)
    for s in range(0, len(M), chunk):
        m = M[s:s + chunk]
        mr = m @ R.T
        cand = mr / rr[None, :]
        r = np.sum(m * m, axis=1)[:, None] - mr ** 2 / rr[None, :]
        r = np.where(cand > 0, r, np.inf)
        b = np.argmin(r, axis=1)
        rows = np.arange(len(b))
        idx[s:s + chunk], res[s:s + chunk], s0[s:s + chunk] = b, r[rows, b], cand[rows, b]
    return idx, res, s0


def bayes(measured, lib_mat, kios, rhos, Vs, weights, sigma_m, fit_s0=False, chunk: int = 4000) -> dict:
    """fp64 Bayesian posterior means (madi/fitters.py:159-243): log-weights
    log q - r / (2 sigma_m^2), shifted by their row maximum, normalised; free S0
    uses the raw residual |m|^2 - (m.r)^2/|r|^2 divided by S0^2 for the weight
    and masks S0 <= 0; rows with no admissible entry give zeros."""
    M = np.asarray(measured, np.float64)
    R = np.asarray(lib_mat, np.float64)
    lq = np.log(np.asarray(weights, np.float64))[None, :]
    k, r_, v = (np.asarray(a, np.float64) for a in (kios, rhos, Vs))
    keys = ("kio_mean", "rho_mean", "V_mean", "kio_std", "rho_std", "V_std", "residual", "n_eff") + \
        (("s0_fit",) if fit_s0 else ())
    out = {key: np.empty(len(M)) for key in keys}
    for s in range(0, len(M), chunk):
        m = M[s:s + chunk]
        if fit_s0:
            rr = np.maximum(np.sum(R * R, axis=1), 1e-30)
            mr = m @ R.T
            s0 = mr / rr[None, :]
            resid = np.sum(m * m, axis=1)[:, None] - mr ** 2 / rr[None, :]
            resid = np.where(s0 > 0, resid, np.inf)
            wres = resid / np.where(s0 > 0, s0, 1.0) ** 2
        else:
            resid = np.maximum(np.sum(m * m, axis=1)[:, None] + np.sum(R * R, axis=1)[None, :] - 2.0 * m @ R.T, 0.0)
            wres = resid
        lw = lq - wres / (2.0 * sigma_m ** 2)
        mx = np.max(lw, axis=1, keepdims=True)
        bad = ~np.isfinite(mx)
        w = np.where(bad, 0.0, np.exp(lw - np.where(bad, 0.0, mx)))
        w /= np.maximum(np.sum(w, axis=1, keepdims=True), 1e-300)
        sl = slice(s, s + len(m))
        for name, vals in (("kio", k), ("rho", r_), ("V", v)):
            mean = w @ vals
            out[f"{name}_mean"][sl] = mean
            out[f"{name}_std"][sl] = np.sqrt(np.maximum(w @ vals ** 2 - mean ** 2, 0.0))
        out["residual"][sl] = np.sum(w * np.where(np.isfinite(resid), resid, 0.0), axis=1)
        out["n_eff"][sl] = np.where(bad[:, 0], 0.0, 1.0 / np.maximum(np.sum(w ** 2, axis=1), 1e-300))
        if fit_s0:
            out["s0_fit"][sl] = np.sum(w * s0, axis=1)
    return out
