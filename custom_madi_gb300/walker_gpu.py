"""Random walkers of the MADI finite / periodic geometry on the GB300.

Keeps the entry points of ``madi/walker_gpu.py``: kio_to_pp / pp_to_kio_eq5
(Eq. 5, :50-74), the CRN seed rules (:77-83), WalkRandomStream (:86-127),
ReducedResult (:130-165), run_walk_Y (:1093-1133), run_simulation_reduced
(:1145-1167) and run_simulation_multi_kio_reduced (:1170-1233).

Every walk runs through one native entry point, ``madi_walk``: a list of jobs
(one ensemble at one p_p each) is cut into walker tiles and consumed by one
persistent launch.  There is no CPU walker: ``use_gpu=False`` raises.
"""

from __future__ import annotations

import ctypes as C
import math
import sys
from dataclasses import dataclass, field, replace
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _native as N
from .config import PRODUCTION_AXIS_WALKS_PER_ENTRY, SimConfig
from .ensemble import Ensemble, create_dummy_ensemble, create_ensemble

try:
    import torch
    HAS_CUDA = bool(torch.cuda.is_available())
except Exception:  # pragma: no cover - torch is a hard dependency in practice
    torch = None
    HAS_CUDA = False

PAPER_WALKS_PER_ENTRY = PRODUCTION_AXIS_WALKS_PER_ENTRY
PHILOX_KEY1 = 0x4D414449  # "MADI": second Philox key word, fixed
FIXED_POINT_SCALE = 2.0 ** 32
# Per-walker label cache in the walker's shared memory (six float4); the
# kernel's layout uses the same figure.
FC_BYTES_PER_WALKER = 6 * 16


def pp_to_kio_eq5(pp: float, mean_AV: float, cfg: SimConfig) -> float:
    """MADI I Eq. 5 [1/s] with the governing-process <A/V>."""
    return float(pp) * math.sqrt(cfg.D0 / (6.0 * cfg.ts)) * float(mean_AV) * 1000.0


def kio_to_pp(kio: float, mean_AV: float, cfg: SimConfig) -> float:
    """Inverse of Eq. 5; raises rather than clamping p_p."""
    if kio < 0.0:
        raise ValueError(f"k_io must be non-negative, got {kio}")
    if mean_AV <= 0.0:
        raise ValueError("governing-process mean_A_over_V must be positive")
    return _checked_pp((float(kio) / 1000.0) / (math.sqrt(cfg.D0 / (6.0 * cfg.ts)) * mean_AV))


def pp_to_kio(pp: float, mean_AV: float, cfg: SimConfig) -> float:
    return pp_to_kio_eq5(pp, mean_AV, cfg)


def _checked_pp(pp: float) -> float:
    pp = float(pp)
    if not math.isfinite(pp) or pp < 0.0 or pp > 1.0:
        raise ValueError(f"p_p must be finite and in [0, 1], got {pp!r}")
    return pp


def _ensemble_seed(base_seed: int, ensemble_index: int) -> int:
    return (int(base_seed) + 97_003 * int(ensemble_index)) & 0x7FFFFFFF


def _walk_seed(base_seed: int, ensemble_index: int) -> int:
    """Common-random-number seed shared by every entry with this ensemble index."""
    return (int(base_seed) + 104_729 * int(ensemble_index)) & 0x7FFFFFFF


def _thresholds(pp: float) -> Tuple[int, int]:
    """floor(pp * 2^64), floor(pp^2 * 2^64): accept a crossing iff U64 < threshold."""
    if pp >= 1.0:
        return (1 << 64) - 1, (1 << 64) - 1
    return int(math.ldexp(pp, 64)), int(math.ldexp(pp * pp, 64))


@dataclass(frozen=True)
class WalkRandomStream:
    """Fixed random input (golden replay): init (N,3), increments (steps,N,3), uniforms (steps,N)."""

    initial_positions: np.ndarray
    increments: np.ndarray
    acceptance_uniforms: np.ndarray

    def validate(self, cfg: SimConfig, ensemble: Optional[Ensemble] = None) -> None:
        n, s = int(cfg.n_walkers), int(cfg.n_steps)
        if np.shape(self.initial_positions) != (n, 3):
            raise ValueError("golden initial_positions must have shape (n_walkers, 3)")
        if np.shape(self.increments) != (s, n, 3):
            raise ValueError("golden increments must have shape (n_steps, n_walkers, 3)")
        if np.shape(self.acceptance_uniforms) != (s, n):
            raise ValueError("golden acceptance_uniforms must have shape (n_steps, n_walkers)")
        if not (np.all(np.isfinite(self.initial_positions)) and np.all(np.isfinite(self.increments))
                and np.all(np.isfinite(self.acceptance_uniforms))):
            raise ValueError("golden stream contains non-finite values")
        u = np.asarray(self.acceptance_uniforms)
        if np.any(u < 0.0) or np.any(u >= 1.0):
            raise ValueError("golden acceptance uniforms lie outside [0,1)")
        if ensemble is not None and (np.any(np.asarray(self.initial_positions) < ensemble.source_lo)
                                     or np.any(np.asarray(self.initial_positions) >= ensemble.source_hi)):
            raise ValueError("golden initial positions must lie in Ω_src")


def make_walk_random_stream(cfg: SimConfig, seed: int, ensemble: Optional[Ensemble] = None) -> WalkRandomStream:
    """Deterministic stream from numpy's default_rng(seed), drawn in the reference's order."""
    if ensemble is None:
        ensemble = create_dummy_ensemble(cfg)
    rng = np.random.default_rng(int(seed))
    n = int(cfg.n_walkers)
    st = WalkRandomStream(
        rng.uniform(ensemble.source_lo, ensemble.source_hi, size=(n, 3)).astype(np.float64),
        rng.normal(0.0, cfg.sigma, size=(int(cfg.n_steps), n, 3)).astype(np.float64),
        rng.uniform(0.0, 1.0, size=(int(cfg.n_steps), n)).astype(np.float64))
    st.validate(cfg, ensemble)
    return st


@dataclass
class ReducedResult:
    cos_sum: np.ndarray
    sin_sum: np.ndarray
    n_walkers: int
    n_escaped: int
    occupancy_counts: np.ndarray
    pp_values: list = field(default_factory=list)
    analytic_kio_eq5_values: list = field(default_factory=list)
    geometry_stats: list = field(default_factory=list)
    ensemble_cos_means: list = field(default_factory=list)
    ensemble_sin_means: list = field(default_factory=list)
    classifier_cache_stats: list = field(default_factory=list)
    # GB300 addition: per-direction sums [n_cols, n_dirs] (None for 3-axis only use)
    cos_dir: Optional[np.ndarray] = None
    sin_dir: Optional[np.ndarray] = None
    n_dirs: int = 3

    @property
    def n_eff(self) -> int:
        """Independent phase samples: every walker is projected on n_dirs directions (3 axes)."""
        return int(self.n_dirs) * int(self.n_walkers)

    @property
    def analytic_kio_eq5(self) -> float:
        return float(np.mean(self.analytic_kio_eq5_values)) if self.analytic_kio_eq5_values else 0.0

    @property
    def mean_pp(self) -> float:
        return float(np.mean(self.pp_values)) if self.pp_values else 0.0

    @property
    def occupancy_fraction(self) -> np.ndarray:
        if self.n_walkers <= 0:
            return np.zeros_like(self.occupancy_counts, dtype=np.float64)
        return self.occupancy_counts.astype(np.float64) / self.n_walkers


def _membrane_transition_counts(old_cell, old_inside, new_cell, new_inside) -> np.ndarray:
    """Endpoint-only membrane count m in {0, 1, 2} (SI §S.IV.b.1)."""
    old_inside = np.asarray(old_inside, bool)
    new_inside = np.asarray(new_inside, bool)
    m = (old_inside != new_inside).astype(np.int8)
    m[old_inside & new_inside & (np.asarray(old_cell) != np.asarray(new_cell))] = 2
    return m


def _require_gpu(use_gpu: Optional[bool]) -> None:
    if use_gpu is False:
        raise RuntimeError("custom_madi_gb300 has no CPU walker: it runs on the GPU only (use_gpu=False)")
    if not HAS_CUDA:
        raise RuntimeError("CUDA is unavailable: custom_madi_gb300 walks run on a CUDA device only")


# ---------------------------------------------------------------------------
# Column layout for the fused epilogue
# ---------------------------------------------------------------------------

@dataclass
class PairLayout:
    """Columns grouped by (jd, jD, js): coef[pair, b] and the column of each (pair, b)."""
    jd: np.ndarray
    jD: np.ndarray
    js: np.ndarray
    coef: np.ndarray          # (n_pairs, n_b) float64
    col_of: np.ndarray        # (n_pairs, n_b) int, -1 = padding

    @property
    def n_pairs(self) -> int:
        return len(self.jd)

    @property
    def n_b(self) -> int:
        return self.coef.shape[1]


def pair_layout(j_delta, j_Delta, j_sum, phase_coef) -> PairLayout:
    jd, jD, js = (np.asarray(x, np.int64) for x in (j_delta, j_Delta, j_sum))
    pc = np.asarray(phase_coef, np.float64)
    order, groups = [], {}
    for c, key in enumerate(zip(jd.tolist(), jD.tolist(), js.tolist())):
        if key not in groups:
            groups[key] = []
            order.append(key)
        groups[key].append(c)
    nb = max(len(v) for v in groups.values()) if groups else 0
    coef = np.zeros((len(order), nb))
    col_of = -np.ones((len(order), nb), np.int64)
    for p, key in enumerate(order):
        for b, c in enumerate(groups[key]):
            coef[p, b] = pc[c]
            col_of[p, b] = c
    a = np.asarray(order, np.int64).reshape(-1, 3)
    return PairLayout(a[:, 0], a[:, 1], a[:, 2], coef, col_of)


def fused_supported(layout: PairLayout, n_dirs: int) -> bool:
    return (1 <= layout.n_pairs <= N.MADI_MAX_PAIRS and 1 <= layout.n_b <= N.MADI_MAX_B
            and 1 <= n_dirs <= N.MADI_MAX_DIRS and layout.n_pairs * layout.n_b * n_dirs <= 2048)


# ---------------------------------------------------------------------------
# Job launcher
# ---------------------------------------------------------------------------

@dataclass
class WalkJob:
    ensemble: Ensemble
    pp: float
    walk_seed: int
    n_walkers: int
    walker_base: int = 0


@dataclass
class LaunchConfig:
    tile_walkers: int = 128
    blocks_per_sm: int = 0          # 0 = occupancy-derived
    persistent: bool = True
    staged: Optional[bool] = None   # False = always read geometry in place
    stage_budget: int = 48 * 1024   # largest geometry staged into shared memory
    min_blocks: int = 2             # register budget: 2 -> 128 registers/thread, 1 -> 255


class WalkBatch:
    """Device-side plan of a batch of walk jobs: geometry table, job table, outputs.

    ``launch()`` enqueues the walk on the current stream (it can be captured in
    a CUDA graph: the work counter and the accumulators are zeroed by kernels
    of the same stream); ``results()`` reads the per-job sums back.
    """

    def __init__(self, jobs: Sequence[WalkJob], cfg: SimConfig, *, layout: Optional[PairLayout] = None,
                 dirs: Optional[np.ndarray] = None, out_mode: int = N.MADI_OUT_FUSED,
                 stream: Optional[WalkRandomStream] = None, precision: int = 32,
                 launch: Optional[LaunchConfig] = None, device=None,
                 outputs: Optional[Tuple] = None, slots: Optional[Sequence[int]] = None):
        """``outputs`` = (accum, occupancy, counters) pools owned by the caller and
        ``slots`` the pool row of each job: the walk then adds into those rows
        and never zeroes them (the sums are exact integers, so a job split over
        several launches adds up to the same values as one launch)."""
        if not jobs:
            raise ValueError("a walk batch needs at least one job")
        self.dev = torch.device(device or "cuda")
        if self.dev.index is None:
            self.dev = torch.device("cuda", torch.cuda.current_device())
        self.cfg = cfg
        self.jobs = list(jobs)
        self.launch_cfg = launch or LaunchConfig()
        self.out_mode = out_mode
        self.precision = precision
        lc = self.launch_cfg
        # geometries (dedup by identity)
        gidx, geoms = {}, []
        for j in self.jobs:
            if id(j.ensemble) not in gidx:
                gidx[id(j.ensemble)] = len(geoms)
                geoms.append(j.ensemble.device(str(self.dev)))
        modes = {g.struct.boundary for g in geoms}
        if len(modes) != 1:
            raise ValueError("a walk batch mixes periodic and fatal-escape geometries")
        self.geoms = geoms
        gbytes = b"".join(bytes(g.struct) for g in geoms)
        self.geom_table = torch.frombuffer(bytearray(gbytes), dtype=torch.uint8).to(self.dev)
        tw = lc.tile_walkers if precision == 32 else 128
        rows, tiles = 0, 0
        jbytes = []
        for s, j in enumerate(self.jobs):
            pp = _checked_pp(j.pp)
            t1, t2 = _thresholds(pp)
            nt = (int(j.n_walkers) + tw - 1) // tw
            slot = s if slots is None else int(slots[s])
            jb = N.MadiWalkJob(gidx[id(j.ensemble)], int(j.n_walkers), int(j.walker_base) & 0xFFFFFFFF,
                               int(j.walk_seed) & 0xFFFFFFFF, PHILOX_KEY1, slot, tiles, rows, pp, t1, t2)
            jbytes.append(bytes(jb))
            tiles += nt
            rows += int(j.n_walkers)
        self.n_tiles, self.n_rows = tiles, rows
        self.job_table = torch.frombuffer(bytearray(b"".join(jbytes)), dtype=torch.uint8).to(self.dev)
        n_slots = len(self.jobs)
        d = N.MadiWalkDesc()
        d.geoms, d.jobs = N.ptr(self.geom_table), N.ptr(self.job_table)
        d.n_geoms, d.n_jobs, d.n_tiles = len(geoms), len(self.jobs), tiles
        d.tile_walkers = tw
        d.boundary = modes.pop()
        d.precision = precision
        d.rng = N.MADI_RNG_STREAM if stream is not None else N.MADI_RNG_PHILOX
        d.out_mode = out_mode
        d.n_steps, d.steps_per_h, d.n_grid = cfg.n_steps, cfg.steps_per_h, cfg.n_grid
        d.sigma, d.ts = cfg.sigma, cfg.ts
        d.min_blocks = int(lc.min_blocks)
        u = np.eye(3) if dirs is None else np.asarray(dirs, np.float64)
        self.n_dirs = len(u)
        self.layout = layout
        if out_mode == N.MADI_OUT_FUSED:
            if layout is None or not fused_supported(layout, len(u)):
                raise ValueError("fused epilogue needs <= 8 pairs, <= 32 b values, <= 32 directions")
            d.n_pairs, d.n_b, d.n_dirs = layout.n_pairs, layout.n_b, len(u)
            for p in range(layout.n_pairs):
                d.pair_jd[p], d.pair_jD[p], d.pair_js[p] = int(layout.jd[p]), int(layout.jD[p]), int(layout.js[p])
                for b in range(layout.n_b):
                    d.coef[p * layout.n_b + b] = float(layout.coef[p, b])
            for k in range(len(u)):
                for a in range(3):
                    d.dirs[3 * k + a] = float(u[k, a])
            self.n_out = layout.n_pairs * layout.n_b * len(u)
            if outputs is None:
                self.accum = torch.zeros((n_slots, self.n_out * 2), dtype=torch.int64, device=self.dev)
        else:
            d.n_pairs, d.n_b, d.n_dirs = 0, 0, 0
            self.n_out = 0
            self.accum = torch.zeros((1, 2), dtype=torch.int64, device=self.dev)
            self.Y = torch.zeros((rows, cfg.n_grid, 3), dtype=torch.float64, device=self.dev)
            self.inside_trace = torch.zeros((rows, cfg.n_grid), dtype=torch.int8, device=self.dev)
            d.Y, d.inside_trace = N.ptr(self.Y), N.ptr(self.inside_trace)
        self.owns_outputs = outputs is None
        if outputs is None:
            self.occupancy = torch.zeros((n_slots, cfg.n_grid), dtype=torch.int64, device=self.dev)
            self.counters = torch.zeros((n_slots, N.MADI_CNT_N), dtype=torch.int64, device=self.dev)
        else:
            if out_mode != N.MADI_OUT_FUSED or slots is None or len(slots) != len(self.jobs):
                raise ValueError("external output pools need the fused epilogue and one slot per job")
            self.accum, self.occupancy, self.counters = outputs
            if self.accum.shape[1] != self.n_out * 2 or self.occupancy.shape[1] != cfg.n_grid:
                raise ValueError("output pool shapes do not match the layout / grid")
            if max(slots) >= self.accum.shape[0]:
                raise ValueError("slot outside the output pool")
        self.work_counter = torch.zeros(4, dtype=torch.int32, device=self.dev)
        d.accum, d.occupancy, d.counters = N.ptr(self.accum), N.ptr(self.occupancy), N.ptr(self.counters)
        d.work_counter = N.ptr(self.work_counter)
        if stream is not None:
            if len(self.jobs) != 1:
                raise ValueError("a replay stream drives exactly one job")
            self.s_init = torch.from_numpy(np.ascontiguousarray(stream.initial_positions, np.float64)).to(self.dev)
            self.s_incr = torch.from_numpy(np.ascontiguousarray(stream.increments, np.float64)).to(self.dev)
            self.s_unif = torch.from_numpy(np.ascontiguousarray(stream.acceptance_uniforms, np.float64)).to(self.dev)
            d.init, d.incr, d.unif = N.ptr(self.s_init), N.ptr(self.s_incr), N.ptr(self.s_unif)
        if precision == 64:
            d.n_tiles = (int(self.jobs[0].n_walkers) + 127) // 128
        # shared-memory staging (every geometry that fits the per-CTA budget) and persistent grid
        budget = lc.stage_budget if lc.staged is not False else 0
        np_ = 8 if (layout is not None and layout.n_pairs > 4) else 4
        fused_extra = 16 * self.n_out + 12 * ((cfg.n_grid + 3) // 4 * 4) + (24 + FC_BYTES_PER_WALKER + 4 * (3 + 3 * np_) + 12) * tw
        fits = [g.stage_bytes for g in geoms if g.stage_bytes + fused_extra <= min(budget, 227 * 1024)]
        d.stage_smem = ((max(fits) + 15) // 16 * 16) if (fits and precision == 32) else 0
        self.smem_bytes = d.stage_smem + fused_extra
        self.staged_fraction = float(np.mean([g.stage_bytes <= d.stage_smem for g in geoms])) if d.stage_smem else 0.0
        sms = torch.cuda.get_device_properties(self.dev).multi_processor_count
        if lc.persistent and precision == 32:
            bps = lc.blocks_per_sm or max(1, int(N.lib().madi_walk_blocks_per_sm(C.byref(d))))
            d.grid_blocks = int(min(tiles, sms * bps))
        else:
            d.grid_blocks = 0
        self.desc = d

    def launch(self, stream=None) -> None:
        s = stream if stream is not None else torch.cuda.current_stream(self.dev)
        with torch.cuda.stream(s):
            self.work_counter.zero_()
            if self.owns_outputs:
                self.accum.zero_()
                self.occupancy.zero_()
                self.counters.zero_()
        st = N.lib().madi_walk(C.byref(self.desc), s.cuda_stream)
        N.check(st, "madi_walk")

    def counters_np(self) -> np.ndarray:
        return self.counters.cpu().numpy()

    def _inputs(self) -> list:
        ins = [self.geom_table, self.job_table]
        for g in self.geoms:
            ins += [g.stage, g.seed_f64, *g.kd]
        return ins

    def host_mirror(self) -> dict:
        """Pinned host copies of every input buffer and pinned output buffers."""
        ins = [t.cpu().pin_memory() for t in self._inputs()]
        outs = [torch.empty(t.shape, dtype=t.dtype).pin_memory() for t in (self.accum, self.occupancy, self.counters)]
        return {"inputs": ins, "outputs": outs,
                "h2d_bytes": sum(t.numel() * t.element_size() for t in ins),
                "d2h_bytes": sum(t.numel() * t.element_size() for t in outs)}

    def run_from_host(self, host: dict) -> tuple:
        """End-to-end call: host inputs -> device, walk, device sums -> host (synchronous)."""
        s = torch.cuda.current_stream(self.dev)
        for dst, src in zip(self._inputs(), host["inputs"]):
            dst.copy_(src, non_blocking=True)
        self.launch(s)
        for src, dst in zip((self.accum, self.occupancy, self.counters), host["outputs"]):
            dst.copy_(src, non_blocking=True)
        s.synchronize()
        return tuple(host["outputs"])

    def results(self) -> list:
        """Per job: dict(cos [n_cols, n_dirs], sin, occupancy, counters)."""
        acc = self.accum.cpu().numpy()
        occ = self.occupancy.cpu().numpy()
        cnt = self.counters.cpu().numpy()
        out = []
        for s in range(len(self.jobs)):
            r = {"occupancy": occ[s], "counters": dict(zip(N.CNT_NAMES, cnt[s].tolist()))}
            if self.out_mode == N.MADI_OUT_FUSED:
                lay = self.layout
                a = acc[s].reshape(lay.n_pairs, lay.n_b, self.n_dirs, 2)
                n_cols = int(lay.col_of.max()) + 1
                cs = np.zeros((n_cols, self.n_dirs), np.int64)
                ss = np.zeros((n_cols, self.n_dirs), np.int64)
                for p in range(lay.n_pairs):
                    for b in range(lay.n_b):
                        c = lay.col_of[p, b]
                        if c >= 0:
                            cs[c] = a[p, b, :, 0]
                            ss[c] = a[p, b, :, 1]
                r["cos_fixed"], r["sin_fixed"] = cs, ss
                r["cos"] = cs.astype(np.float64) / FIXED_POINT_SCALE
                r["sin"] = ss.astype(np.float64) / FIXED_POINT_SCALE
            out.append(r)
        return out


def _raise_on_status(counters: dict, n: int) -> None:
    if counters.get("classifier_error", 0):
        raise RuntimeError("CUDA full-facet KD-tree classification failed")
    esc = counters.get("escaped", 0)
    if esc:
        raise RuntimeError(f"SI §S.III fatal boundary condition: {esc}/{n} walkers exited Ω_sim.")


def run_walk_Y(ens: Ensemble, kio: float, cfg: Optional[SimConfig] = None, seed: int = 0, verbose: bool = True,
               *, pp: Optional[float] = None, return_telemetry: bool = False, classifier: str = "exact",
               random_stream: Optional[WalkRandomStream] = None, use_gpu: Optional[bool] = None,
               precision: Optional[int] = None, launch: Optional[LaunchConfig] = None):
    """Walk one ensemble and return Y [N, n_grid, 3] (madi/walker_gpu.py:1093-1133).

    A replay stream runs the fp64 walker (reference arithmetic, exact KD rule)
    unless precision=32 asks for the production fp32 walker; without a stream
    the walker draws Philox4x32-10 numbers keyed by ``seed`` (fp32 walker by
    default; precision=64 walks the same numbers with the fp64 walker).
    """
    _require_gpu(use_gpu)
    if cfg is None:
        cfg = SimConfig()
    if classifier not in ("exact", "exact_cached"):
        raise ValueError("classifier must be 'exact' or 'exact_cached'")
    actual_pp = _checked_pp(pp if pp is not None else kio_to_pp(kio, ens.mean_AV, cfg))
    if random_stream is not None:
        random_stream.validate(cfg, ens)
    prec = precision or (64 if random_stream is not None else 32)
    batch = WalkBatch([WalkJob(ens, actual_pp, int(seed), int(cfg.n_walkers))], cfg, out_mode=N.MADI_OUT_Y,
                      stream=random_stream, precision=prec, launch=launch)
    batch.launch()
    torch.cuda.current_stream(batch.dev).synchronize()
    res = batch.results()[0]
    cnt = res["counters"]
    Y = batch.Y.cpu().numpy()
    inside = batch.inside_trace.cpu().numpy()
    if cnt["classifier_error"]:
        raise RuntimeError("CUDA full-facet KD-tree classification failed")
    n_escape = int(cnt["escaped"])
    if n_escape:
        raise RuntimeError(f"SI §S.III fatal boundary condition: {n_escape} walkers escaped Ω_sim")
    if return_telemetry:
        return Y, n_escape, {
            "occupancy_counts": np.sum(inside, axis=0),
            "occupancy_fraction": np.mean(inside, axis=0),
            "inside_trace": inside,
            "pp": actual_pp,
            "classifier_cache": cnt,
        }
    return Y, n_escape


def _build_ensembles_for_entry(rho: float, V: float, cfg: SimConfig, seed: int, verbose: bool) -> list:
    if rho <= 0.0 or V <= 0.0:
        return [create_dummy_ensemble(cfg) for _ in range(int(cfg.n_ensembles))]
    return [create_ensemble(rho, V, cfg, seed=_ensemble_seed(seed, i), verbose=verbose)
            for i in range(int(cfg.n_ensembles))]


def _pp_for(ens: Ensemble, kio: float, cfg: SimConfig) -> float:
    if ens.is_free_water or kio == 0.0:
        return 0.0
    return _checked_pp(kio_to_pp(kio, ens.mean_AV, cfg))


class WalkGraph:
    """A batch's whole launch (work-counter and accumulator zeroing + the
    persistent walk) captured once in a CUDA graph; ``replay()`` re-runs it on
    the same device buffers with one host call."""

    def __init__(self, batch: WalkBatch):
        self.batch = batch
        dev = batch.dev
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):                # warm-up outside the capture
            batch.launch(side)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            batch.launch()

    def replay(self) -> None:
        self.graph.replay()


def simulate_jobs(jobs: Sequence[WalkJob], cfg: SimConfig, columns: Tuple, *, dirs=None,
                  launch: Optional[LaunchConfig] = None, check: bool = True, precision: int = 32) -> list:
    """Walk every job in one persistent launch; per job cos / sin sums [n_cols, n_dirs].

    precision=64 runs the reference's GPU design instead (madi/walker_gpu.py:
    520-695, :989-1063): per job one fp64 walk launch that stores Y, then a
    column reduction over the 3 Cartesian axes (sums [n_cols, 1]).
    """
    _require_gpu(None)
    if precision not in (32, 64):
        raise ValueError("precision must be 32 or 64")
    layout = pair_layout(*columns)
    u = cfg.direction_array() if dirs is None else np.asarray(dirs, np.float64)
    if precision == 32 and fused_supported(layout, len(u)):
        batch = WalkBatch(jobs, cfg, layout=layout, dirs=u, launch=launch)
        batch.launch()
        torch.cuda.current_stream(batch.dev).synchronize()
        res = batch.results()
    else:
        if len(u) != 3 or not np.allclose(u, np.eye(3)):
            raise ValueError("column grids beyond the fused epilogue support the 3 Cartesian axes only")
        res = []
        jd, jD, js, pc = (torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (
            np.asarray(columns[0], np.int32), np.asarray(columns[1], np.int32), np.asarray(columns[2], np.int32),
            np.asarray(columns[3], np.float64)))
        for j in jobs:
            batch = WalkBatch([j], cfg, out_mode=N.MADI_OUT_Y, launch=launch, precision=precision)
            batch.launch()
            cs = torch.empty(len(pc), dtype=torch.float64, device=batch.dev)
            ss = torch.empty_like(cs)
            N.reduce_Y(batch.Y, batch.n_rows, cfg.n_grid, jd, jD, js, pc, cs, ss, torch.cuda.current_stream(batch.dev))
            r = batch.results()[0]
            r["cos"] = cs.cpu().numpy()[:, None]
            r["sin"] = ss.cpu().numpy()[:, None]
            res.append(r)
    if check:
        for j, r in zip(jobs, res):
            _raise_on_status(r["counters"], j.n_walkers)
    return res


def run_simulation_reduced(rho: float, V: float, kio: float, j_delta, j_Delta, j_sum, phase_coef,
                           cfg: Optional[SimConfig] = None, seed: int = 0, verbose: bool = True, *,
                           narrow_snapshot_steps=None, narrow_snapshot_index=None,
                           narrow_phase_coef=None) -> ReducedResult:
    out = run_simulation_multi_kio_reduced(rho, V, [kio], j_delta, j_Delta, j_sum, phase_coef, cfg=cfg, seed=seed,
                                           verbose=verbose, narrow_snapshot_steps=narrow_snapshot_steps,
                                           narrow_snapshot_index=narrow_snapshot_index,
                                           narrow_phase_coef=narrow_phase_coef)
    return out[float(kio)]


def _check_narrow(cfg: SimConfig, narrow_args) -> None:
    if any(x is None for x in narrow_args) and not all(x is None for x in narrow_args):
        raise ValueError("narrow-pulse reduction requires all endpoint arrays together")
    narrow = all(x is not None for x in narrow_args)
    if cfg.phase_model == "narrow_pulse" or narrow:
        raise ValueError("the narrow-pulse diagnostic is a CPU-only reference path and is not provided "
                         "by the GPU walker; use phase_model='finite_lobe'")


def results_to_reduced(ens: Ensemble, pp: float, cfg: SimConfig, r: dict, n_walkers: int) -> ReducedResult:
    cos_dir, sin_dir = r["cos"], r["sin"]
    n_dirs = cos_dir.shape[1]
    if "cos_fixed" in r:
        cos_sum = r["cos_fixed"].sum(axis=1).astype(np.float64) / FIXED_POINT_SCALE
        sin_sum = r["sin_fixed"].sum(axis=1).astype(np.float64) / FIXED_POINT_SCALE
    else:
        cos_sum, sin_sum = cos_dir.sum(axis=1), sin_dir.sum(axis=1)
        n_dirs = 3
    neff = float(n_dirs * n_walkers)
    cnt = r["counters"]
    return ReducedResult(
        cos_sum=cos_sum, sin_sum=sin_sum, n_walkers=int(n_walkers), n_escaped=int(cnt["escaped"]),
        occupancy_counts=np.asarray(r["occupancy"], np.int64), pp_values=[float(pp)],
        analytic_kio_eq5_values=[pp_to_kio_eq5(pp, ens.mean_AV, cfg)] if not ens.is_free_water else [0.0],
        geometry_stats=[ens.geometry.to_dict()], ensemble_cos_means=[cos_sum / neff],
        ensemble_sin_means=[sin_sum / neff], classifier_cache_stats=[cnt],
        cos_dir=cos_dir if cos_dir.shape[1] > 1 else None, sin_dir=sin_dir if sin_dir.shape[1] > 1 else None,
        n_dirs=n_dirs)


def _walk_and_reduce_one_ensemble(ens: Ensemble, pp: float, cfg: SimConfig, j_delta, j_Delta, j_sum, phase_coef,
                                  walk_seed: int, *, narrow_snapshot_steps=None, narrow_snapshot_index=None,
                                  narrow_phase_coef=None) -> ReducedResult:
    """One ensemble at one p_p, reduced over the columns (the reference helper of
    the same name, madi/walker_gpu.py:989-1063, called by its benchmark scripts).
    The reference walks in cfg.walker_chunk chunks seeded walk_seed + offset;
    here all cfg.n_walkers walkers are one job keyed by walk_seed in one launch.
    Escapes raise the same RuntimeError; narrow-pulse arrays raise ValueError."""
    _check_narrow(cfg, (narrow_snapshot_steps, narrow_snapshot_index, narrow_phase_coef))
    pp = _checked_pp(pp)
    n = int(cfg.n_walkers)
    r = simulate_jobs([WalkJob(ens, pp, int(walk_seed), n)], cfg, (j_delta, j_Delta, j_sum, phase_coef))[0]
    return results_to_reduced(ens, pp, cfg, r, n)


def _merge_results(results: Sequence[ReducedResult]) -> ReducedResult:
    """Sum in ensemble order; per-ensemble lists are concatenated unsorted (CRN partner order)."""
    if not results:
        raise ValueError("cannot merge no results")
    m = ReducedResult(cos_sum=np.zeros_like(results[0].cos_sum), sin_sum=np.zeros_like(results[0].sin_sum),
                      n_walkers=0, n_escaped=0, occupancy_counts=np.zeros_like(results[0].occupancy_counts),
                      n_dirs=results[0].n_dirs)
    for r in results:
        m.cos_sum = m.cos_sum + r.cos_sum
        m.sin_sum = m.sin_sum + r.sin_sum
        m.n_walkers += r.n_walkers
        m.n_escaped += r.n_escaped
        m.occupancy_counts = m.occupancy_counts + r.occupancy_counts
        m.pp_values.extend(r.pp_values)
        m.analytic_kio_eq5_values.extend(r.analytic_kio_eq5_values)
        m.geometry_stats.extend(r.geometry_stats)
        m.ensemble_cos_means.extend(r.ensemble_cos_means)
        m.ensemble_sin_means.extend(r.ensemble_sin_means)
        m.classifier_cache_stats.extend(r.classifier_cache_stats)
        if r.cos_dir is not None:
            m.cos_dir = r.cos_dir if m.cos_dir is None else m.cos_dir + r.cos_dir
            m.sin_dir = r.sin_dir if m.sin_dir is None else m.sin_dir + r.sin_dir
    return m


def run_simulation_multi_kio_reduced(rho: float, V: float, kios: Sequence[float], j_delta, j_Delta, j_sum,
                                     phase_coef, cfg: Optional[SimConfig] = None, seed: int = 0,
                                     verbose: bool = True, *, narrow_snapshot_steps=None,
                                     narrow_snapshot_index=None, narrow_phase_coef=None,
                                     ensembles: Optional[list] = None,
                                     launch: Optional[LaunchConfig] = None) -> dict:
    """All ensembles x k_io values of one (rho, V) entry in one persistent launch."""
    if cfg is None:
        cfg = SimConfig()
    cfg.assert_grid_alignment()
    _check_narrow(cfg, (narrow_snapshot_steps, narrow_snapshot_index, narrow_phase_coef))
    kios = [float(k) for k in kios]
    if any(k < 0.0 for k in kios):
        raise ValueError("k_io grid values must be non-negative")
    _require_gpu(None)
    u = cfg.direction_array()
    total = len(u) * int(cfg.n_ensembles) * int(cfg.n_walkers)
    if total < PAPER_WALKS_PER_ENTRY // 10 and verbose:
        sys.stderr.write(f"    WARNING: only {total:,} axis-walks per entry; production reference is "
                         f"~{PAPER_WALKS_PER_ENTRY:,}.\n")
    ens_list = ensembles if ensembles is not None else _build_ensembles_for_entry(rho, V, cfg, seed, verbose)
    jobs, keys = [], []
    for e, ens in enumerate(ens_list):
        ws = _walk_seed(seed, e)
        for k in kios:
            jobs.append(WalkJob(ens, _pp_for(ens, k, cfg), ws, int(cfg.n_walkers)))
            keys.append((e, k))
    res = simulate_jobs(jobs, cfg, (j_delta, j_Delta, j_sum, phase_coef), dirs=u, launch=launch)
    out = {k: [] for k in kios}
    for (e, k), job, r in zip(keys, jobs, res):
        rr = results_to_reduced(job.ensemble, job.pp, cfg, r, job.n_walkers)
        out[k].append(rr)
        if verbose:
            print(f"    ensemble {e + 1}/{len(ens_list)}, k_io={k:g}: p_p={job.pp:.7g}, "
                  f"Eq.5={rr.analytic_kio_eq5:.5g} s^-1")
    return {k: _merge_results(v) for k, v in out.items()}
