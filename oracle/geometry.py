"""Oracle geometry: TEST INFRASTRUCTURE, NOT PRODUCT CODE.

CPU restatement of the ensemble construction the oracle walk needs, so that
the CPU baseline and the reference arm of bench.py build their geometry
without the package's native library:

* alpha_star_from_vi: the physical root of SI Eq. S7a by the cubic's roots
  (madi/ensemble.py:426-457);
* mean_A_over_V: the certified single-cell <A/V> table, linearly
  interpolated at v_i and scaled by rho^(1/3) (madi/ensemble.py:512-522; the
  table is the data file the package ships);
* kd_build: the balanced KD tree, median of the widest-spread axis, preorder
  node numbering (madi/ensemble.py:525-563);
* periodic_ensemble: a periodic box of n uniform seeds drawn from
  default_rng(seed) in the package's order, annuli min(alpha*, kappa d_nn / 2)
  from periodic nearest neighbours (madi/ensemble.py:679), and the 27-image
  tiling that the reference's classify_cpu sees in periodic mode;
* kio_to_pp: MADI I Eq. 5 inverted (madi/walker_gpu.py:50-74).

Only tests/ and bench.py's CPU legs use it; custom_madi_gb300 never imports it.
"""

from __future__ import annotations

import math
from pathlib import Path

import numpy as np
from scipy.spatial import cKDTree

ROOT = Path(__file__).resolve().parents[1]
TABLE = ROOT / "custom_madi_gb300" / "data" / "geometry_reference_si_kappa_0p9.npz"
S7A = (-0.570444, 10.6047, -5.81457, 1.0)      # v_i(x) = a x^3 + b x^2 + c x + d, x = rho^(1/3) alpha
KAPPA = 0.90
_table = None


def _per_um3(rho_per_uL: float) -> float:
    return float(rho_per_uL) / 1.0e9                 # cells/uL -> cells/um^3 (madi/ensemble.py:43-45)


def alpha_star_from_vi(vi: float, rho_per_uL: float) -> float:
    a, b, c, d = S7A
    rho = _per_um3(rho_per_uL)
    roots = np.roots([a, b, c, d - float(vi)])
    x_turn = min(float(x.real) for x in np.roots([3 * a, 2 * b, c]) if abs(x.imag) < 1e-10 and x.real > 0)
    phys = [float(x.real) for x in roots if abs(x.imag) < 1e-10 and -1e-12 <= x.real <= x_turn + 1e-12]
    if len(phys) != 1:
        raise RuntimeError(f"no unique physical S7a root for v_i={vi}")
    return phys[0] / rho ** (1.0 / 3.0)


def mean_A_over_V(vi: float, rho_per_uL: float) -> float:
    global _table
    if _table is None:
        with np.load(TABLE, allow_pickle=False) as t:
            _table = (np.asarray(t["vi"], np.float64), np.asarray(t["mean_A_over_V_norm"], np.float64))
    v, av = _table
    if not (v[0] <= vi <= v[-1]):
        raise RuntimeError(f"v_i={vi} outside the certified table")
    return float(np.interp(float(vi), v, av)) * _per_um3(rho_per_uL) ** (1.0 / 3.0)


def kio_to_pp(kio: float, mean_av: float, D0: float, ts: float) -> float:
    pp = (float(kio) / 1000.0) / (math.sqrt(D0 / (6.0 * ts)) * float(mean_av))
    if not (0.0 <= pp <= 1.0):
        raise ValueError(f"p_p must be finite and in [0, 1], got {pp!r}")
    return pp


def kd_build(seeds):
    """(node_seed i32, node_axis i8, node_left, node_right, node_parent i32)."""
    pts = np.asarray(seeds, np.float64)
    n = len(pts)
    ns = np.empty(n, np.int32)
    na = np.empty(n, np.int8)
    nl = np.full(n, -1, np.int32)
    nr = np.full(n, -1, np.int32)
    npar = np.empty(n, np.int32)
    count = 0

    def build(idx, parent):
        nonlocal count
        if len(idx) == 0:
            return -1
        sub = pts[idx]
        axis = int(np.argmax(sub.max(axis=0) - sub.min(axis=0)))
        mid = len(idx) // 2
        arranged = idx[np.argpartition(sub[:, axis], mid)]
        node = count
        count += 1
        ns[node], na[node], npar[node] = arranged[mid], axis, parent
        nl[node] = build(arranged[:mid], node)
        nr[node] = build(arranged[mid + 1:], node)
        return node

    build(np.arange(n, dtype=np.int32), -1)
    return ns, na, nl, nr, npar


def periodic_ensemble(rho_per_uL: float, V_pL: float, n_cells: int, seed: int) -> dict:
    """Base seeds, annuli and the 27-image classifier set of one periodic box."""
    rho = _per_um3(rho_per_uL)
    vi = rho * (float(V_pL) * 1.0e3)                 # rho [um^-3] x V [um^3] (madi/ensemble.py:667-668)
    alpha = alpha_star_from_vi(vi, rho_per_uL)
    side = (int(n_cells) / rho) ** (1.0 / 3.0)
    rng = np.random.default_rng(seed)
    base = rng.uniform(0.0, side, size=(int(n_cells), 3)).astype(np.float64)
    base[base >= side] = 0.0
    nn = np.asarray(cKDTree(base, boxsize=side).query(base, k=2)[0][:, 1], np.float64)
    ann = np.minimum(alpha, KAPPA * nn / 2.0).astype(np.float64)
    shifts = side * np.array([[i, j, k] for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)
                              if (i, j, k) != (0, 0, 0)], np.float64)
    tiled = np.concatenate([base] + [base + s for s in shifts])
    return {"L": side, "vi": vi, "alpha_star": alpha, "mean_AV": mean_A_over_V(vi, rho_per_uL),
            "seeds": base, "annulus": ann, "tiled_seeds": tiled, "tiled_annulus": np.tile(ann, 27),
            "tiled_cell": np.tile(np.arange(int(n_cells), dtype=np.int32), 27)}


def oracle_geometry(ens: dict):
    """The oracle classifier/walker geometry of a periodic_ensemble()."""
    from . import oracle as O
    kd = kd_build(ens["tiled_seeds"])
    return O.Geometry(ens["tiled_seeds"], ens["tiled_annulus"], kd, ens["L"], 0.0, ens["L"], ens["tiled_cell"],
                      periodic=True, has_cells=True)
