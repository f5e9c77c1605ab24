"""Contracted Poisson-Voronoi ensembles: host-side construction, device packing.

Mirrors ``madi/ensemble.py`` of the reference: SI Eq. S7a inversion
(alpha_star_from_vi, :426-457), the certified single-cell <A/V> table
(governing_mean_A_over_V, :464-522), the SI Eq. S8 domain (si_domain_side_um,
:405-423), the certified Poisson population (_make_population, :566-638), the
per-seed annulus min(alpha*, kappa d_nn / 2) (:679) and create_ensemble /
create_dummy_ensemble (:649-792).  The random draws are made in the same order
from ``numpy.random.default_rng(seed)`` so the same seed yields the same seeds.

GB300 additions:
* ``boundary_mode="periodic"``: ``n_cells`` uniform seeds in [0, L)^3 with
  periodic nearest-neighbour annuli; the classifier sees every periodic image
  within a proven margin of the box (tiled seeds carry their base cell id).
* every ensemble carries a voxel candidate grid (native builder) and packs into
  the device layout of ``madi_geometry`` (include/madi_gb300.h).
* classification (``classify`` / ``classify_cpu``) and the v_i measurement run
  on the GPU through ``madi_classify``; there is no CPU classifier here.
"""

from __future__ import annotations

import ctypes as C
import json
from dataclasses import asdict, dataclass, field
from pathlib import Path
from typing import Any, Optional, Tuple

import numpy as np
from scipy.spatial import cKDTree

from .config import SimConfig
from . import _native as N

_S7A = (-0.570444, 10.6047, -5.81457, 1.0)   # SI Eq. S7a: v_i(x), x = rho^(1/3) alpha


def _rho_um3(rho_per_uL: float) -> float:
    return float(rho_per_uL) / 1.0e9        # the reference's arithmetic (bit-identical v_i, L, alpha*)


def _V_um3(V_pL: float) -> float:
    return float(V_pL) * 1e3


def _rho_per_uL(rho_um3: float) -> float:
    return float(rho_um3) * 1e9


def _s7a(x: float) -> float:
    a, b, c, d = _S7A
    return ((a * x + b) * x + c) * x + d


@dataclass(frozen=True)
class GeometryReference:
    vi: np.ndarray
    alpha_x: np.ndarray
    mean_A_over_V_norm: np.ndarray
    metadata: dict
    path: str


@dataclass(frozen=True)
class PopulationCertificate:
    pop_margin_um: float
    s10_distance_upper_um: float
    s10_pass: bool
    n_relevant_seeds: int
    s11_min_clearance_margin_um: float
    s11_pass: bool
    certification_spacing_um: float
    expansion_index: int

    def to_dict(self) -> dict:
        return asdict(self)


@dataclass(frozen=True)
class GeometryStats:
    target_vi: float
    realised_vi: float
    realised_vi_se: float
    realised_rho_per_uL: float
    realised_mean_volume_pL: float
    alpha_star_um: float
    governing_mean_A_over_V_um_inv: float
    annulus_mean_um: float
    annulus_std_um: float
    annulus_min_um: float
    annulus_max_um: float
    annulus_q05_um: float
    annulus_q50_um: float
    annulus_q95_um: float
    n_seeds_pop: int
    n_seeds_sim: int
    n_validation_points: int
    sim_side_um: float
    source_side_um: float
    population: PopulationCertificate
    reference_path: str
    reference_metadata: dict

    def to_dict(self) -> dict:
        out = asdict(self)
        out["population"] = self.population.to_dict()
        return out


# ---------------------------------------------------------------------------
# Analytic pieces
# ---------------------------------------------------------------------------

def alpha_star_from_vi(vi: float, rho_per_uL: float) -> float:
    """alpha* [um] from SI Eq. S7a on its decreasing physical branch.

    v_i(x) is a cubic in x = rho^(1/3) alpha with v_i(0) = 1 and v_i'(0) < 0;
    the physical root is the unique real root in [0, x_turn], x_turn the first
    positive stationary point (a root of v_i').  Both come from numpy's
    companion-matrix roots, the reference's own arithmetic, so alpha* (and every
    annulus min(alpha*, kappa d_nn / 2)) is the reference's value bit for bit.
    """
    vi = float(vi)
    rho = _rho_um3(rho_per_uL)
    if not (0.0 < vi < 1.0):
        raise ValueError(f"target v_i must lie in (0, 1), got {vi}")
    if rho <= 0.0:
        raise ValueError("rho must be positive for a cellular geometry")
    a, b, c, d = _S7A
    x_turn = min(float(t.real) for t in np.roots([3.0 * a, 2.0 * b, c]) if abs(t.imag) < 1e-10 and t.real > 0.0)
    branch = [float(x.real) for x in np.roots([a, b, c, d - vi])
              if abs(x.imag) < 1e-10 and -1e-12 <= x.real <= x_turn + 1e-12]
    if len(branch) != 1:
        raise RuntimeError(f"SI Eq. S7a has no unique physical root for v_i={vi}")
    return float(branch[0] / rho ** (1.0 / 3.0))


def _reference_default_path() -> Path:
    return Path(__file__).resolve().parent / "data" / "geometry_reference_si_kappa_0p9.npz"


def _load_reference(cfg: SimConfig) -> GeometryReference:
    """Certified single-cell <A/V> table with the reference's checks (madi/ensemble.py:464-509)."""
    path = Path(cfg.geometry_reference_path) if cfg.geometry_reference_path else _reference_default_path()
    if not path.is_file():
        raise RuntimeError(
            f"No SI-certified geometry reference table was found at {path}. Refusing to "
            "substitute a finite Ω_sim A/V.")
    with np.load(path, allow_pickle=False) as data:
        missing = {"vi", "alpha_x", "mean_A_over_V_norm", "metadata_json"} - set(data.files)
        if missing:
            raise RuntimeError(f"geometry reference {path} is missing {sorted(missing)}")
        try:
            meta = json.loads(str(data["metadata_json"]))
        except (TypeError, ValueError) as exc:
            raise RuntimeError(f"geometry reference {path} has invalid metadata_json") from exc
        vi = np.asarray(data["vi"], dtype=np.float64)
        ax = np.asarray(data["alpha_x"], dtype=np.float64)
        av = np.asarray(data["mean_A_over_V_norm"], dtype=np.float64)
    if vi.ndim != 1 or len(vi) < 2 or len(ax) != len(vi) or len(av) != len(vi):
        raise RuntimeError("geometry reference axes must be matching 1-D arrays")
    if not (np.all(np.diff(vi) > 0) and np.all(np.diff(ax) < 0)):
        raise RuntimeError("geometry reference v_i must increase while alpha_x decreases")
    if not np.all(np.isfinite(av)) or np.any(av <= 0):
        raise RuntimeError("geometry reference contains invalid <A/V> values")
    if abs(float(meta.get("kappa", np.nan)) - 0.90) > 1e-12:
        raise RuntimeError("geometry reference must use SI κ=0.9")
    if meta.get("mean_estimator") != "untrimmed_arithmetic_mean_A_over_V":
        raise RuntimeError("geometry reference must store the untrimmed arithmetic <A/V> mean")
    if meta.get("contraction_rule") != "all_shifted_voronoi_facets_S2":
        raise RuntimeError("geometry reference must use the full SI Eq. S2 shifted-facet contraction")
    if not cfg.allow_uncertified_geometry_reference:
        if int(meta.get("n_single_cells", 0)) < cfg.geometry_reference_required_cells:
            raise RuntimeError(
                "geometry reference is not SI-certified: it must contain at least "
                f"{cfg.geometry_reference_required_cells:,} independent single cells")
        if int(meta.get("n_alpha", 0)) != cfg.geometry_reference_required_alpha_values:
            raise RuntimeError(
                "geometry reference is not SI-certified: it must contain exactly "
                f"{cfg.geometry_reference_required_alpha_values} alpha values")
    return GeometryReference(vi, ax, av, meta, str(path.resolve()))


def governing_mean_A_over_V(vi: float, rho_per_uL: float, cfg: SimConfig) -> Tuple[float, GeometryReference]:
    """<A/V> [1/um]: table value at v_i (linear interpolation) times rho^(1/3)."""
    ref = _load_reference(cfg)
    if vi < ref.vi[0] or vi > ref.vi[-1]:
        raise RuntimeError(
            f"requested v_i={vi:.6f} is outside certified reference range "
            f"[{ref.vi[0]:.6f}, {ref.vi[-1]:.6f}]; no clamping is allowed")
    av = float(np.interp(float(vi), ref.vi, ref.mean_A_over_V_norm))
    return float(av * _rho_um3(rho_per_uL) ** (1.0 / 3.0)), ref


def si_domain_side_um(rho_per_uL: float, cfg: SimConfig) -> float:
    """SI Eq. S8 domain edge W [um] (cfg.L overrides)."""
    if cfg.L is not None:
        if cfg.L <= 0.0:
            raise ValueError("diagnostic L override must be positive")
        return float(cfg.L)
    rw = float(np.sqrt(2.0 * cfg.D0 * cfg.tRW_max))
    rho = _rho_um3(rho_per_uL)
    if rho <= 0.0:
        return float(20.0 * rw)
    return float(max(10.0 * rw, min(20.0 * rw, (8.0e5 / rho) ** (1.0 / 3.0))))


def periodic_box_side_um(rho_per_uL: float, cfg: SimConfig) -> float:
    """Edge of a periodic box holding cfg.n_cells seeds at density rho (cfg.L overrides)."""
    if cfg.L is not None:
        return float(cfg.L)
    return float((int(cfg.n_cells) / _rho_um3(rho_per_uL)) ** (1.0 / 3.0))


# ---------------------------------------------------------------------------
# Native builders
# ---------------------------------------------------------------------------

def _build_gpu_kdtree(seeds: np.ndarray):
    """Balanced KD tree over seeds (madi/ensemble.py:525-563) via the native builder."""
    s = np.ascontiguousarray(seeds, dtype=np.float64)
    n = len(s)
    out = [np.empty(n, np.int32), np.empty(n, np.int8), np.empty(n, np.int32),
           np.empty(n, np.int32), np.empty(n, np.int32)]
    st = N.lib().madi_kdtree_build(s.ctypes.data, n, out[0].ctypes.data, out[1].ctypes.data,
                                   out[2].ctypes.data, out[3].ctypes.data, out[4].ctypes.data)
    N.check(st, "madi_kdtree_build")
    return tuple(out)


def build_voxel_grid(seeds_xyza: np.ndarray, G: int, h: float, eps: float, cap: float):
    """(offsets uint32 [G^3+1], ids uint16/uint32) of the proven candidate grid."""
    s = np.ascontiguousarray(seeds_xyza, dtype=np.float64)
    n = len(s)
    u32 = 1 if n > 65535 else 0
    total = C.c_int64(0)
    offsets = np.zeros(G ** 3 + 1, dtype=np.uint32)
    cap_ids = 40 * G ** 3                       # a guess; one retry with the exact size if short
    for _ in range(2):
        ids = np.zeros(max(cap_ids, 1), dtype=np.uint32 if u32 else np.uint16)
        st = N.lib().madi_grid_build(s.ctypes.data, n, G, h, eps, cap, offsets.ctypes.data, ids.ctypes.data,
                                     u32, len(ids), C.byref(total))
        if st == N.MADI_ERR_CAPACITY and total.value > cap_ids:
            cap_ids = int(total.value)
            continue
        N.check(st, "madi_grid_build")
        # a copy, so the oversized guess is freed before the stage block is packed
        return offsets, ids[: int(total.value)].copy(), bool(u32)
    raise RuntimeError("madi_grid_build: candidate count changed between calls")


def build_facets(seeds_xyza: np.ndarray, periodic: bool, L: float):
    """Voronoi facet table of every base cell (madi_facets_build):
    (begin uint32 [n+1], planes float32 [T, 4], nbr int32 [T], h_max, reach)."""
    s = np.ascontiguousarray(seeds_xyza, dtype=np.float64)
    n = len(s)
    begin = np.zeros(n + 1, dtype=np.uint32)
    cap = 48 * n
    for _ in range(2):
        planes = np.zeros((cap, 4), dtype=np.float32)
        nbr = np.zeros(cap, dtype=np.int32)
        total = C.c_int64(0)
        stats = np.zeros(2, dtype=np.float64)
        st = N.lib().madi_facets_build(s.ctypes.data, n, 1 if periodic else 0, float(L), begin.ctypes.data,
                                       planes.ctypes.data, nbr.ctypes.data, cap, C.byref(total), stats.ctypes.data)
        if st == N.MADI_ERR_CAPACITY and total.value > cap:
            cap = int(total.value)
            continue
        N.check(st, "madi_facets_build")
        t = int(total.value)
        return begin, planes[:t], nbr[:t], float(stats[0]), float(stats[1])
    raise RuntimeError("madi_facets_build: facet count changed between calls")


def pack_facets(fbeg: np.ndarray, planes: np.ndarray, nbr: np.ndarray):
    """(stride, planes [n, stride, 4], nbr [n, stride]) of a facet table at a
    fixed stride per cell, so the walker loads a cell's slots without first
    reading where they start.  stride = max count rounded up to 32; unused slots
    hold (0, 0, 0, 3e38) / -1.  Stride 0 (and empty arrays) when a cell has more
    than 64 slots: the walker's margin keys carry the slot in 6 bits, and such a
    geometry (never met with Poisson seeds) stays on the voxel-grid classifier."""
    cnt = np.diff(np.asarray(fbeg, np.int64))
    n = len(cnt)
    stride = int(max(32, -(-int(cnt.max(initial=0)) // 32) * 32))
    if stride > 64:
        return 0, np.zeros((0, 32, 4), np.float32), np.zeros((0, 32), np.int32)
    fpl = np.zeros((n, stride, 4), np.float32)
    fpl[:, :, 3] = 3.0e38
    fnb = np.full((n, stride), -1, np.int32)
    slot = np.arange(int(cnt.sum())) - np.repeat(np.asarray(fbeg[:-1], np.int64), cnt)
    row = np.repeat(np.arange(n), cnt)
    fpl[row, slot] = planes
    fnb[row, slot] = nbr
    return stride, fpl, fnb


# ---------------------------------------------------------------------------
# Ensemble
# ---------------------------------------------------------------------------

@dataclass
class Ensemble:
    """One contracted Poisson-Voronoi realisation (madi/ensemble.py:183-206)."""

    seeds: np.ndarray
    annulus: np.ndarray
    rho: float
    V: float
    vi: float
    alpha_star: float
    L: float
    source_lo: float
    source_hi: float
    mean_AV: float
    geometry: GeometryStats
    rho_requested: float
    V_requested: float
    kd_node_seed: np.ndarray
    kd_node_axis: np.ndarray
    kd_node_left: np.ndarray
    kd_node_right: np.ndarray
    kd_node_parent: np.ndarray
    tree: Optional[Any] = None
    is_free_water: bool = False
    # --- GB300 additions ---------------------------------------------------
    boundary_mode: str = "si_fatal_escape"
    # Seeds the classifier sees (periodic: images within a proven margin) and
    # the base cell id of each.  Equal to seeds / arange for the SI mode.
    classifier_seeds: Optional[np.ndarray] = None
    classifier_annulus: Optional[np.ndarray] = None
    classifier_cell: Optional[np.ndarray] = None
    grid_h: float = 0.0
    grid_n: int = 1
    safe_cap: float = 0.0
    _device: dict = field(default_factory=dict, repr=False)

    def _tree(self) -> cKDTree:
        if self.tree is None:
            self.tree = cKDTree(self.seeds)
        return self.tree

    # -- classification (device) --------------------------------------------
    def classify(self, positions: np.ndarray, method: str = "grid") -> Tuple[np.ndarray, np.ndarray]:
        """SI Eq. S2 labels (cell id, inside) of (N, 3) positions, on the GPU.

        ``method="kd"`` runs the reference's fp64 KD rule, ``"grid"`` the
        walker's voxel-grid rule (fp64 inputs are decided in fp64 on the same
        proven candidate lists).  Periodic positions are wrapped into [0, L).
        """
        import torch
        pts = np.asarray(positions, dtype=np.float64)
        if pts.ndim != 2 or pts.shape[1] != 3:
            raise ValueError("positions must have shape (N, 3)")
        if self.is_free_water:
            return np.zeros(len(pts), np.int32), np.zeros(len(pts), bool)
        if self.boundary_mode == "periodic":
            pts = np.mod(pts, self.L)
            pts[pts >= self.L] = 0.0
        dev = self.device()
        p = torch.from_numpy(np.ascontiguousarray(pts)).to(dev.device)
        cell = torch.empty(len(pts), dtype=torch.int32, device=dev.device)
        inside = torch.empty(len(pts), dtype=torch.uint8, device=dev.device)
        st = N.lib().madi_classify(C.byref(dev.struct), N.ptr(p), 0, len(pts),
                                   0 if method == "kd" else 1, N.ptr(cell), N.ptr(inside), None,
                                   torch.cuda.current_stream(dev.device).cuda_stream)
        N.check(st, "madi_classify")
        c = cell.cpu().numpy()
        if np.any(c < 0):
            raise RuntimeError("CUDA full-facet classification failed (coincident seeds or empty candidate list)")
        return c, inside.cpu().numpy().astype(bool)

    def classify_cpu(self, positions: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
        """Drop-in name of the reference classifier (madi/ensemble.py:213); runs on the GPU."""
        return self.classify(positions, method="grid")

    def classify_exact_cpu(self, positions: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
        return self.classify(positions, method="grid")

    def device(self, device: Optional[str] = None) -> "DeviceGeometry":
        """The ensemble packed in device memory (cached per device)."""
        import torch
        dev = torch.device(device or "cuda")
        if dev.type != "cuda":
            raise RuntimeError("custom_madi_gb300 geometry lives on a CUDA device")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        key = str(dev)
        if key not in self._device:
            self._device[key] = DeviceGeometry(self, dev)
        return self._device[key]


class DeviceGeometry:
    """Device buffers of one ensemble + its ``madi_geometry`` descriptor."""

    def __init__(self, ens: Ensemble, device):
        import torch
        self.device = device
        seeds = np.asarray(ens.classifier_seeds if ens.classifier_seeds is not None else ens.seeds, np.float64)
        ann = np.asarray(ens.classifier_annulus if ens.classifier_annulus is not None else ens.annulus, np.float64)
        cellid = (np.asarray(ens.classifier_cell, np.int32) if ens.classifier_cell is not None
                  else np.arange(len(seeds), dtype=np.int32))
        n = len(seeds)
        xyza = np.empty((n, 4), np.float64)
        xyza[:, :3] = seeds
        xyza[:, 3] = ann
        hi = xyza.astype(np.float32)
        # per-axis bound on |fp32 seed - fp64 seed| (2x the half-ulp at the largest coordinate)
        self.coord_err = float(np.max(np.abs(seeds - hi[:, :3].astype(np.float64)))) * 2.0 + \
            2.0 ** -24 * float(np.max(np.abs(seeds))) if n else 0.0
        if ens.is_free_water:
            G, h, offsets, ids, u32 = 1, max(ens.L, 1.0), np.zeros(2, np.uint32), np.zeros(0, np.uint16), False
        else:
            G, h = int(ens.grid_n), float(ens.grid_h)
            eps = 1e-4 * h + 1e-6 * ens.L
            offsets, ids, u32 = build_voxel_grid(xyza, G, h, eps, float(ens.safe_cap))
        self.grid_total = int(len(ids))
        self.candidates_mean = float(len(ids)) / float(G ** 3)
        # facet table of the base cells (periodic: the first n_cells seeds, images generated natively)
        periodic = ens.boundary_mode == "periodic"
        if ens.is_free_water:
            n_cells, centers, self.facet_stride = 0, np.zeros((0, 4), np.float32), 0
            self.facet_reach = 0.0
            fpl, fnbr, h_max = np.zeros((0, 4), np.float32), np.zeros(0, np.int32), 0.0
        else:
            n_cells = int(cellid.max()) + 1
            base = xyza[:n_cells]
            if not np.array_equal(cellid[:n_cells], np.arange(n_cells)):
                raise RuntimeError("classifier seeds must list the base cells first")
            fbeg, fpl_csr, fnbr_csr, h_max, self.facet_reach = build_facets(base, periodic, float(ens.L))
            centers = base.astype(np.float32)
            self.facet_stride, fpl, fnbr = pack_facets(fbeg, fpl_csr, fnbr_csr)
            # the stage block's byte offsets are uint32: a table that would not
            # fit leaves the walker on the voxel-grid classifier
            head = hi.nbytes + cellid.nbytes + offsets.nbytes + ids.nbytes + centers.nbytes + 64
            if self.facet_stride == 0 or head + fpl.nbytes + fnbr.nbytes >= 2 ** 32:
                n_cells, self.facet_stride = 0, 32
                fpl, fnbr = np.zeros((0, 32, 4), np.float32), np.zeros((0, 32), np.int32)
        self.n_cells = n_cells
        self.facets_mean = float(np.count_nonzero(fnbr >= 0)) / max(n_cells, 1)
        # |m - m_exact| <= 2 e + 2^-21 (h + |w|_1 + L) for fp32 facet margins, taken twice
        a_max = float(np.max(ann)) if n else 0.0
        self.facet_tol = 2.0 * (2.0 * self.coord_err + 2.0 ** -21 * (h_max + a_max + float(ens.L)))

        def pad16(b: bytes) -> bytes:
            return b + b"\0" * ((-len(b)) % 16)

        offs = stage_offsets([a.nbytes for a in (hi, cellid, offsets, ids, centers, fpl, fnbr)])
        parts = [hi.tobytes(), pad16(cellid.tobytes()), pad16(offsets.tobytes()), pad16(ids.tobytes()),
                 pad16(centers.tobytes()), pad16(fpl.tobytes()), pad16(fnbr.tobytes())]
        off_cell, off_go, off_gi = int(offs[1]), int(offs[2]), int(offs[3])
        blob = b"".join(parts)
        if len(blob) != int(offs[-1]):
            raise RuntimeError("stage block layout mismatch")
        self.stage = torch.frombuffer(bytearray(blob), dtype=torch.uint8).to(device)
        self.seed_f64 = torch.from_numpy(xyza).to(device)
        if ens.kd_node_seed is None or len(ens.kd_node_seed) != n:
            raise RuntimeError("ensemble KD tree does not match its classifier seeds")
        self.kd = [torch.from_numpy(np.ascontiguousarray(a)).to(device) for a in
                   (ens.kd_node_seed, ens.kd_node_left, ens.kd_node_right, ens.kd_node_parent, ens.kd_node_axis)]
        s = N.MadiGeometry()
        s.stage = N.ptr(self.stage)
        s.seed_f64 = N.ptr(self.seed_f64)
        s.kd_seed, s.kd_left, s.kd_right, s.kd_parent, s.kd_axis = [N.ptr(t) for t in self.kd]
        s.off_cell, s.off_grid_offset, s.off_grid_ids = off_cell, off_go, off_gi
        s.stage_bytes = len(blob)
        s.n_seeds = n
        s.grid_n = G
        s.ids_u32 = 1 if u32 else 0
        s.boundary = N.MADI_BOUNDARY_PERIODIC if ens.boundary_mode == "periodic" else N.MADI_BOUNDARY_FATAL
        s.has_cells = 0 if ens.is_free_water else 1
        s.L = float(ens.L)
        s.grid_h = h
        s.safe_cap = float(ens.safe_cap)
        s.source_lo = float(ens.source_lo)
        s.source_hi = float(ens.source_hi)
        s.coord_err = self.coord_err
        s.off_cell_center, s.off_facet_plane, s.off_facet_nbr = (int(o) for o in offs[4:7])
        s.facet_stride = self.facet_stride
        s.n_cells = n_cells
        s.facet_tol = self.facet_tol
        self.struct = s
        self.stage_bytes = len(blob)

    @property
    def nbytes(self) -> int:
        """Device bytes held by this geometry (stage blob, fp64 seeds, KD arrays)."""
        ts = [self.stage, self.seed_f64, *self.kd]
        return int(sum(t.numel() * t.element_size() for t in ts))


def stage_offsets(part_bytes) -> np.ndarray:
    """Byte offsets of the parts of a geometry's stage block, each part padded
    to 16 bytes (the first is already a multiple of 16); the last entry is the
    block's size.  The walker reads these offsets and the size as uint32, so a
    block of 4 GiB or more is refused here with MADI_ERR_CAPACITY rather than
    stored wrapped (a ctypes uint32 field keeps only the low 32 bits)."""
    sizes = [int(b) for b in part_bytes]
    if any(b < 0 for b in sizes):
        raise ValueError("stage part sizes must be non-negative")
    offs = np.cumsum([0] + [b + (-b) % 16 for b in sizes], dtype=np.int64)
    if int(offs[-1]) >= 2 ** 32:
        raise N.MadiError(N.MADI_ERR_CAPACITY,
                          f"geometry stage block of {int(offs[-1])} bytes exceeds the 4 GiB the walker addresses "
                          "with 32-bit offsets (seeds {}, voxel-grid ids {} B)".format(sizes[0] // 16, sizes[3]))
    return offs


# ---------------------------------------------------------------------------
# Construction
# ---------------------------------------------------------------------------

def _distance_to_cube(points: np.ndarray, lo: float, hi: float) -> np.ndarray:
    p = np.asarray(points, np.float64)
    excess = np.maximum(np.maximum(lo - p, 0.0), p - hi)
    return np.sqrt(np.sum(excess * excess, axis=-1))


def _nearest_distance_upper_bound(tree: cKDTree, side: float, spacing: float, boxsize=None):
    """Max nearest-seed distance over a cube: cell-centre grid + Lipschitz term."""
    n = max(1, int(np.ceil(side / spacing)))
    h = side / n
    c = (np.arange(n, dtype=np.float64) + 0.5) * h
    best = 0.0
    yy, zz = np.meshgrid(c, c, indexing="ij")
    yz = np.column_stack((yy.ravel(), zz.ravel()))
    for x in c:
        d, _ = tree.query(np.column_stack((np.full(len(yz), x), yz)), k=1)
        best = max(best, float(np.max(d)))
    return best + 0.5 * np.sqrt(3.0) * h, h


def _make_population(rho_um3: float, side: float, cfg: SimConfig, rng: np.random.Generator):
    """Poisson seeds in Omega_pop certified against SI Eqs. S10-S12 (madi/ensemble.py:585-638)."""
    spacing = rho_um3 ** (-1.0 / 3.0)
    margin = max(cfg.population_initial_margin_cell_spacings * spacing,
                 2.0 * cfg.population_certification_spacing_um)
    for expansion in range(int(cfg.population_max_expansions)):
        lo, hi = -margin, side + margin
        n_seeds = int(rng.poisson(rho_um3 * (hi - lo) ** 3))
        if n_seeds < 2:
            margin *= 1.75
            continue
        seeds = rng.uniform(lo, hi, size=(n_seeds, 3)).astype(np.float64)
        tree = cKDTree(seeds)
        nn = np.asarray(tree.query(seeds, k=2)[0][:, 1], np.float64)
        s10, h = _nearest_distance_upper_bound(tree, side, cfg.population_certification_spacing_um)
        s10_pass = bool(s10 < margin)
        relevant = _distance_to_cube(seeds, 0.0, side) <= s10
        clearance = np.min(np.minimum(seeds - lo, hi - seeds), axis=1)
        s11 = clearance[relevant] - nn[relevant]
        cert = PopulationCertificate(
            pop_margin_um=float(margin), s10_distance_upper_um=float(s10), s10_pass=s10_pass,
            n_relevant_seeds=int(np.count_nonzero(relevant)),
            s11_min_clearance_margin_um=float(np.min(s11)) if np.any(relevant) else float("inf"),
            s11_pass=bool(np.all(s11 > 0.0)), certification_spacing_um=float(h),
            expansion_index=expansion)
        if cert.s10_pass and cert.s11_pass:
            return seeds, tree, nn, cert
        margin *= 1.75
    raise RuntimeError("Could not certify Ω_pop against SI Eqs. S10--S12 after "
                       f"{cfg.population_max_expansions} expansions.")


def default_grid_params(rho_per_uL: float, alpha_max: float, L: float,
                        voxel_per_spacing: float = 0.5, cap_per_spacing: float = 0.0,
                        max_voxels_per_axis: int = 96) -> Tuple[int, float, float]:
    """(G, h, cap): voxel edge and the extra candidate-list radius as fractions of
    the seed spacing (the lists always hold every seed that can be nearest or
    bind; cap > 0 widens them by that distance)."""
    spacing = _rho_um3(rho_per_uL) ** (-1.0 / 3.0)
    G = int(min(max_voxels_per_axis, max(1, int(np.ceil(L / (voxel_per_spacing * spacing))))))
    h = L / G
    cap = max(cap_per_spacing * spacing, 0.0)
    return G, float(h), float(cap)


def _stats_block(target_vi, realised, se, rho_real, vol, alpha_star, mean_av, ann_sim, n_pop, n_sim,
                 n_val, side, source_side, cert, ref) -> GeometryStats:
    return GeometryStats(
        target_vi=float(target_vi), realised_vi=float(realised), realised_vi_se=float(se),
        realised_rho_per_uL=float(rho_real), realised_mean_volume_pL=float(vol),
        alpha_star_um=float(alpha_star), governing_mean_A_over_V_um_inv=float(mean_av),
        annulus_mean_um=float(np.mean(ann_sim)),
        annulus_std_um=float(np.std(ann_sim, ddof=1)) if len(ann_sim) > 1 else 0.0,
        annulus_min_um=float(np.min(ann_sim)), annulus_max_um=float(np.max(ann_sim)),
        annulus_q05_um=float(np.quantile(ann_sim, 0.05)), annulus_q50_um=float(np.quantile(ann_sim, 0.5)),
        annulus_q95_um=float(np.quantile(ann_sim, 0.95)), n_seeds_pop=int(n_pop), n_seeds_sim=int(n_sim),
        n_validation_points=int(n_val), sim_side_um=float(side), source_side_um=float(source_side),
        population=cert, reference_path=ref.path, reference_metadata=ref.metadata)


def _tile_periodic(seeds: np.ndarray, annulus: np.ndarray, L: float, margin: float):
    """Every periodic image within `margin` of [0, L)^3: (seeds, annulus, base id)."""
    K = int(np.ceil(margin / L))
    base = np.arange(len(seeds), dtype=np.int32)
    out_s, out_a, out_c = [seeds], [annulus], [base]
    for i in range(-K, K + 1):
        for j in range(-K, K + 1):
            for k in range(-K, K + 1):
                if i == 0 and j == 0 and k == 0:
                    continue
                s = seeds + L * np.array([i, j, k], dtype=np.float64)
                keep = np.all((s >= -margin) & (s < L + margin), axis=1)
                out_s.append(s[keep]); out_a.append(annulus[keep]); out_c.append(base[keep])
    return np.concatenate(out_s), np.concatenate(out_a), np.concatenate(out_c)


def create_ensemble(rho: float, V: float, cfg: Optional[SimConfig] = None, seed: Optional[int] = None,
                    verbose: bool = False, verify_vi: bool = True, *,
                    voxel_per_spacing: float = 0.5, cap_per_spacing: float = 0.0,
                    measure_vi: bool = True) -> Ensemble:
    """Build one ensemble for the requested (rho [cells/uL], V [pL]) (madi/ensemble.py:649-757).

    cfg.boundary_mode selects the SI finite domain (fatal escape) or a periodic
    box of cfg.n_cells seeds.  v_i is target rho V 1e-6; the realised v_i is
    measured on the GPU with cfg.geometry_validation_points uniform points and
    accepted within max(cfg.geometry_vi_tolerance, 4 SE).
    """
    if cfg is None:
        cfg = SimConfig()
    cfg.assert_grid_alignment()
    rho_um3 = _rho_um3(rho)
    target_vi = rho_um3 * _V_um3(V)
    if not (0.0 < target_vi < 1.0):
        raise ValueError(f"rho={rho:g}, V={V:g} give invalid v_i={target_vi:g}")
    if rho_um3 <= 0.0:
        raise ValueError("rho must be positive for a cellular ensemble")
    alpha_star = alpha_star_from_vi(target_vi, rho)
    mean_av, ref = governing_mean_A_over_V(target_vi, rho, cfg)
    rng = np.random.default_rng(seed)
    periodic = cfg.boundary_mode == "periodic"
    spacing = rho_um3 ** (-1.0 / 3.0)
    if periodic:
        side = periodic_box_side_um(rho, cfg)
        n_cells = int(cfg.n_cells)
        seeds = rng.uniform(0.0, side, size=(n_cells, 3)).astype(np.float64)
        seeds[seeds >= side] = 0.0
        tree = cKDTree(seeds, boxsize=side)
        nn = np.asarray(tree.query(seeds, k=2)[0][:, 1], np.float64)
        if np.any(nn <= 0.0):
            raise RuntimeError("Poisson seed realization contains coincident seeds")
        annulus = np.minimum(alpha_star, cfg.kappa * nn / 2.0).astype(np.float64)
        G, h, cap = default_grid_params(rho, float(np.max(annulus)), side, voxel_per_spacing, cap_per_spacing)
        dmax, _ = _nearest_distance_upper_bound(tree, side, max(h / 2.0, 1e-3))
        # A seed farther than dmax + 2 alpha_max + 2 cap from every box point can be
        # neither nearest nor binding, nor within the extra list radius cap.
        margin = dmax + 2.0 * float(np.max(annulus)) + 2.0 * cap + np.sqrt(3.0) * h + 1e-6 * side
        cs, ca, cc = _tile_periodic(seeds, annulus, side, margin)
        cert = PopulationCertificate(
            pop_margin_um=float(margin), s10_distance_upper_um=float(dmax), s10_pass=True,
            n_relevant_seeds=int(len(cs)), s11_min_clearance_margin_um=float("inf"), s11_pass=True,
            certification_spacing_um=float(h), expansion_index=0)
        source_lo, source_hi = 0.0, side
        n_sim = n_cells
        ann_sim = annulus
        pop_count = n_cells
        kd_src = cs
    else:
        side = si_domain_side_um(rho, cfg)
        seeds, tree, nn, cert = _make_population(rho_um3, side, cfg, rng)
        annulus = np.minimum(alpha_star, cfg.kappa * nn / 2.0).astype(np.float64)
        source_side = cfg.source_fraction * side
        source_lo = 0.5 * (side - source_side)
        source_hi = source_lo + source_side
        in_sim = np.all((seeds >= 0.0) & (seeds < side), axis=1)
        n_sim = int(np.count_nonzero(in_sim))
        if n_sim < 2:
            raise RuntimeError("Ω_sim contains fewer than two seed points; increase W or density")
        ann_sim = annulus[in_sim]
        cs, ca, cc = seeds, annulus, np.arange(len(seeds), dtype=np.int32)
        G, h, cap = default_grid_params(rho, float(np.max(annulus)), side, voxel_per_spacing, cap_per_spacing)
        pop_count = len(seeds)
        kd_src = seeds
    kd = _build_gpu_kdtree(kd_src)
    rho_real = _rho_per_uL(n_sim / side ** 3)
    source_side = source_hi - source_lo
    stats = _stats_block(target_vi, float("nan"), float("nan"), rho_real, float("nan"), alpha_star, mean_av,
                         ann_sim, pop_count, n_sim, cfg.geometry_validation_points, side, source_side, cert, ref)
    ens = Ensemble(
        seeds=seeds, annulus=annulus, rho=rho_real, V=float("nan"), vi=float("nan"),
        alpha_star=alpha_star, L=side, source_lo=source_lo, source_hi=source_hi, mean_AV=mean_av,
        geometry=stats, rho_requested=float(rho), V_requested=float(V),
        kd_node_seed=kd[0], kd_node_axis=kd[1], kd_node_left=kd[2], kd_node_right=kd[3], kd_node_parent=kd[4],
        tree=None if periodic else tree, boundary_mode=cfg.boundary_mode,
        classifier_seeds=cs, classifier_annulus=ca, classifier_cell=cc,
        grid_h=h, grid_n=G, safe_cap=cap)
    if measure_vi or verify_vi:
        realised, se = _measure_vi(ens, cfg.geometry_validation_points, rng)
    else:       # host-only builds (CPU timing legs): v_i left at its target
        realised, se = float(target_vi), float("nan")
    allowed = max(float(cfg.geometry_vi_tolerance), 4.0 * se)
    if verify_vi and abs(realised - target_vi) > allowed:
        raise RuntimeError(
            "Finite Ω_sim packing failed SI geometry acceptance: "
            f"target={target_vi:.6f}, measured={realised:.6f}, allowed={allowed:.6f}.")
    vol = realised * side ** 3 / n_sim / 1.0e3
    ens.geometry = _stats_block(target_vi, realised, se, rho_real, vol, alpha_star, mean_av, ann_sim,
                                pop_count, n_sim, cfg.geometry_validation_points, side, source_side, cert, ref)
    ens.rho, ens.V, ens.vi = rho_real, vol, realised
    if verbose:
        print(f"    [geometry {cfg.boundary_mode}] W={side:.3f} um, seeds={n_sim}/{pop_count}, "
              f"target v_i={target_vi:.5f}, realised={realised:.5f}±{se:.5f}, alpha*={alpha_star:.5f} um, "
              f"<A/V>={mean_av:.5f} um^-1, grid {G}^3 h={h:.3f} cap={cap:.3f}")
    return ens


def _measure_vi(ens: Ensemble, n: int, rng: np.random.Generator) -> Tuple[float, float]:
    pts = rng.uniform(0.0, ens.L, size=(int(n), 3))
    _, inside = ens.classify(pts)
    vi = float(np.mean(inside))
    return vi, float(np.sqrt(max(vi * (1.0 - vi), 0.0) / max(len(pts), 1)))


def create_dummy_ensemble(cfg: SimConfig) -> Ensemble:
    """Acellular free-water control (madi/ensemble.py:760-792)."""
    periodic = cfg.boundary_mode == "periodic"
    side = float(cfg.L) if (periodic and cfg.L is not None) else si_domain_side_um(0.0, cfg)
    if periodic:
        lo, hi = 0.0, side
    else:
        src = cfg.source_fraction * side
        lo = 0.5 * (side - src)
        hi = lo + src
    cert = PopulationCertificate(0.0, 0.0, True, 0, float("inf"), True, 0.0, 0)
    stats = GeometryStats(0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0, 0, 0,
                          side, hi - lo, cert, "", {})
    return Ensemble(
        seeds=np.zeros((2, 3)), annulus=np.zeros(2), rho=0.0, V=0.0, vi=0.0, alpha_star=0.0, L=side,
        source_lo=lo, source_hi=hi, mean_AV=0.0, geometry=stats, rho_requested=0.0, V_requested=0.0,
        kd_node_seed=np.array([0, 1], np.int32), kd_node_axis=np.array([0, 0], np.int8),
        kd_node_left=np.array([-1, -1], np.int32), kd_node_right=np.array([1, -1], np.int32),
        kd_node_parent=np.array([-1, 0], np.int32), is_free_water=True, boundary_mode=cfg.boundary_mode,
        grid_h=max(side, 1.0), grid_n=1, safe_cap=0.0)


def ensemble_from_arrays(seeds: np.ndarray, annulus: np.ndarray, L: float, *, source_lo: float,
                         source_hi: float, mean_AV: float = 0.0, rho_per_uL: Optional[float] = None,
                         boundary_mode: str = "si_fatal_escape", n_cells: Optional[int] = None,
                         voxel_per_spacing: float = 0.5, cap_per_spacing: float = 0.0,
                         classifier: Optional[Tuple[np.ndarray, np.ndarray, np.ndarray]] = None) -> Ensemble:
    """Wrap externally supplied geometry (e.g. a stored golden case) as an Ensemble.

    For the periodic mode ``seeds`` are the base cells and the tiled classifier
    set is derived here unless ``classifier=(seeds, annulus, cell)`` is given.
    """
    seeds = np.asarray(seeds, np.float64)
    annulus = np.asarray(annulus, np.float64)
    n_base = len(seeds) if n_cells is None else int(n_cells)
    if rho_per_uL is None:
        vol = L ** 3
        rho_per_uL = _rho_per_uL(n_base / vol)
    G, h, cap = default_grid_params(rho_per_uL, float(np.max(annulus)), L, voxel_per_spacing, cap_per_spacing)
    if classifier is not None:
        cs, ca, cc = (np.asarray(classifier[0], np.float64), np.asarray(classifier[1], np.float64),
                      np.asarray(classifier[2], np.int32))
    elif boundary_mode == "periodic":
        tree = cKDTree(seeds, boxsize=L)
        dmax, _ = _nearest_distance_upper_bound(tree, L, max(h / 2.0, 1e-3))
        margin = dmax + 2.0 * float(np.max(annulus)) + 2.0 * cap + np.sqrt(3.0) * h + 1e-6 * L
        cs, ca, cc = _tile_periodic(seeds, annulus, L, margin)
    else:
        cs, ca, cc = seeds, annulus, np.arange(len(seeds), dtype=np.int32)
    kd = _build_gpu_kdtree(cs)
    cert = PopulationCertificate(0.0, 0.0, True, 0, float("inf"), True, 0.0, 0)
    stats = GeometryStats(0.0, float("nan"), float("nan"), float(rho_per_uL), float("nan"), 0.0, mean_AV,
                          float(np.mean(annulus)), 0.0, float(np.min(annulus)), float(np.max(annulus)),
                          0.0, 0.0, 0.0, len(seeds), n_base, 0, L, source_hi - source_lo, cert, "", {})
    return Ensemble(
        seeds=seeds, annulus=annulus, rho=float(rho_per_uL), V=float("nan"), vi=float("nan"), alpha_star=0.0,
        L=float(L), source_lo=float(source_lo), source_hi=float(source_hi), mean_AV=float(mean_AV),
        geometry=stats, rho_requested=float(rho_per_uL), V_requested=float("nan"),
        kd_node_seed=kd[0], kd_node_axis=kd[1], kd_node_left=kd[2], kd_node_right=kd[3], kd_node_parent=kd[4],
        boundary_mode=boundary_mode, classifier_seeds=cs, classifier_annulus=ca, classifier_cell=cc,
        grid_h=h, grid_n=G, safe_cap=cap)


def estimate_vi(ens: Ensemble, n: int = 200_000, seed: int = 42) -> float:
    if ens.is_free_water:
        return 0.0
    vi, _ = _measure_vi(ens, n, np.random.default_rng(seed))
    return vi


def governing_reference_summary(ens: Ensemble) -> dict:
    return {
        "mean_A_over_V_um_inv": ens.mean_AV,
        "source": "SI §S.IV 5e6 independent single-cell reference cloud",
        "reference_path": ens.geometry.reference_path,
        "reference_metadata": ens.geometry.reference_metadata,
    }
