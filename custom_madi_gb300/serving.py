"""Continuous-batching request loop over the persistent walker and the library match.

Simulation requests (one ensemble, a membrane permeability, a seed and a walker
count) and fit requests (voxels matched against the server's library) arrive
over time.  A host admission controller admits them in arrival order while
the request's device memory fits the HBM budget (geometry arena + fit buffers;
walker output rows come from a fixed slot pool) and a slot is free.  Active
simulations are cut into walker chunks; every launch of the persistent walk
kernel takes the next chunk of each active simulation (round robin, up to a
walker budget per launch), so requests that arrive while others run join the
next launch and their work overlaps on the device.  Two launches are kept in
flight on two streams and fit requests run on a third.

A walker's trajectory depends only on (request seed, walker index) through
Philox, and the kernel adds each 128-walker tile's phase sums into the
request's slot as exact 64-bit integers; chunks start on tile boundaries, so a
tile holds the same walkers however the request was chunked, and a request's
result is bit-identical whatever it was batched with.

There is no counterpart in the reference (madi runs one ensemble per call,
madi/walker_gpu.py:1123-1203); the simulation entry used per chunk is the
same persistent walk as ``walker_gpu.simulate_jobs``.
"""

from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional, Sequence

import numpy as np

from . import _native as N
from .config import SimConfig
from .walker_gpu import FIXED_POINT_SCALE, LaunchConfig, PairLayout, WalkBatch, WalkJob

try:
    import torch
except Exception:  # pragma: no cover
    torch = None


@dataclass
class SimRequest:
    ensemble: Any
    pp: float
    seed: int
    n_walkers: int
    arrival: float = 0.0            # seconds after the start of the run


@dataclass
class FitRequest:
    voxels: Any                     # [n_vox, F] numpy or torch
    precision: str = "bf16"
    topk: int = 32
    free_s0: bool = False
    arrival: float = 0.0


@dataclass
class Record:
    rid: int
    kind: str
    arrival: float
    nbytes: int
    admit: Optional[float] = None
    finish: Optional[float] = None
    slot: int = -1
    result: Any = None
    walker_steps: int = 0

    @property
    def latency(self) -> float:
        return (self.finish - self.arrival) if self.finish is not None else float("nan")


# ---------------------------------------------------------------------------
# Admission and chunking (pure host logic)
# ---------------------------------------------------------------------------

@dataclass
class _Active:
    rid: int
    n_walkers: int
    issued: int = 0                 # walkers handed to launches
    done: int = 0                   # walkers whose launch completed


class Scheduler:
    """FIFO admission under a byte budget and a slot pool; round-robin chunks."""

    def __init__(self, budget_bytes: int, n_slots: int, chunk_walkers: int, launch_walkers: int, align: int = 1):
        """Chunks other than a request's last start and end on multiples of ``align``."""
        if budget_bytes <= 0 or n_slots <= 0 or chunk_walkers < align or launch_walkers < chunk_walkers:
            raise ValueError("scheduler needs a positive budget, slots and align <= chunk <= launch walker counts")
        self.align = int(align)
        chunk_walkers = chunk_walkers // align * align
        self.budget, self.used = int(budget_bytes), 0
        self.free_slots = list(range(n_slots))[::-1]
        self.chunk, self.launch_cap = int(chunk_walkers), int(launch_walkers)
        self.queue: deque = deque()            # (rid, nbytes, n_walkers or None)
        self.active: Dict[int, _Active] = {}
        self.bytes_of: Dict[int, int] = {}
        self.slot_of: Dict[int, int] = {}
        self._rr: deque = deque()              # round-robin order of active simulations

    def offer(self, rid: int, nbytes: int, n_walkers: Optional[int]) -> None:
        if nbytes > self.budget:
            raise ValueError(f"request {rid} needs {nbytes} bytes, more than the whole budget {self.budget}")
        self.queue.append((rid, int(nbytes), n_walkers))

    def admit(self) -> List[int]:
        """Admit from the head of the queue while memory and (for simulations) a slot are free."""
        out = []
        while self.queue:
            rid, nb, nw = self.queue[0]
            if self.used + nb > self.budget or (nw is not None and not self.free_slots):
                break
            self.queue.popleft()
            self.used += nb
            self.bytes_of[rid] = nb
            if nw is not None:
                self.slot_of[rid] = self.free_slots.pop()
                self.active[rid] = _Active(rid, int(nw))
                self._rr.append(rid)
            out.append(rid)
        return out

    def next_launch(self) -> List[tuple]:
        """(rid, slot, walker_base, n) chunks for one launch."""
        chunks, total = [], 0
        for _ in range(len(self._rr)):
            if total + 1 > self.launch_cap:
                break
            rid = self._rr[0]
            self._rr.rotate(-1)
            a = self.active[rid]
            rest = a.n_walkers - a.issued
            n = min(self.chunk, rest, self.launch_cap - total)
            if n < rest:
                n = n // self.align * self.align      # keep the next chunk tile-aligned
            if n <= 0:
                continue
            chunks.append((rid, self.slot_of[rid], a.issued, n))
            a.issued += n
            total += n
        return chunks

    def complete(self, chunks: Sequence[tuple]) -> List[int]:
        """Mark a launch's chunks done; returns simulations now finished."""
        fin = []
        for rid, _slot, _base, n in chunks:
            a = self.active[rid]
            a.done += n
            if a.done == a.n_walkers:
                fin.append(rid)
        return fin

    def release(self, rid: int) -> None:
        self.used -= self.bytes_of.pop(rid)
        if rid in self.active:
            del self.active[rid]
            self._rr.remove(rid)
            self.free_slots.append(self.slot_of.pop(rid))

    def has_work(self) -> bool:
        return any(a.issued < a.n_walkers for a in self.active.values())


# ---------------------------------------------------------------------------
# Device server
# ---------------------------------------------------------------------------

class Server:
    """Runs a request stream on one GPU; see the module docstring."""

    def __init__(self, cfg: SimConfig, layout: PairLayout, dirs: np.ndarray, *, library=None,
                 budget_bytes: int = 8 << 30, n_slots: int = 64, chunk_walkers: int = 65536,
                 launch_walkers: int = 155648, inflight: int = 2, launch: Optional[LaunchConfig] = None,
                 device=None):
        if torch is None or not torch.cuda.is_available():
            raise RuntimeError("the server runs on a CUDA device")
        self.dev = torch.device(device or "cuda")
        self.cfg, self.layout = cfg, layout
        self.dirs = np.asarray(dirs, np.float64)
        self.n_out = layout.n_pairs * layout.n_b * len(self.dirs)
        self.launch_cfg = launch or LaunchConfig()
        self.library = None if library is None else (library if torch.is_tensor(library) else
                                                     torch.from_numpy(np.ascontiguousarray(library, np.float32)))
        if self.library is not None:
            self.library = self.library.to(self.dev, torch.float32).contiguous()
        slot_bytes = (self.n_out * 2 + cfg.n_grid + N.MADI_CNT_N) * 8
        self.pool_bytes = n_slots * slot_bytes
        self.sched = Scheduler(budget_bytes - self.pool_bytes, n_slots, chunk_walkers, launch_walkers,
                               align=self.launch_cfg.tile_walkers)
        self.accum = torch.zeros((n_slots, self.n_out * 2), dtype=torch.int64, device=self.dev)
        self.occupancy = torch.zeros((n_slots, cfg.n_grid), dtype=torch.int64, device=self.dev)
        self.counters = torch.zeros((n_slots, N.MADI_CNT_N), dtype=torch.int64, device=self.dev)
        self.walk_streams = [torch.cuda.Stream(self.dev) for _ in range(max(1, inflight))]
        self.fit_stream = torch.cuda.Stream(self.dev)
        self.inflight = max(1, inflight)

    # -- request bookkeeping --------------------------------------------------
    def _nbytes(self, req) -> int:
        if isinstance(req, SimRequest):
            return req.ensemble.device(str(self.dev)).nbytes
        n, f = int(req.voxels.shape[0]), int(req.voxels.shape[1])
        prec = N.MADI_MATCH_BF16 if req.precision == "bf16" else N.MADI_MATCH_FP32
        scratch = int(N.lib().madi_match_scratch_bytes(n, int(self.library.shape[0]), f, prec, int(req.topk)))
        return n * f * 4 + n * 12 + scratch + 512

    def _slot_result(self, slot: int) -> dict:
        lay = self.layout
        a = self.accum[slot].cpu().numpy().reshape(lay.n_pairs, lay.n_b, len(self.dirs), 2)
        n_cols = int(lay.col_of.max()) + 1
        cs = np.zeros((n_cols, len(self.dirs)), np.int64)
        ss = np.zeros((n_cols, len(self.dirs)), np.int64)
        for p in range(lay.n_pairs):
            for b in range(lay.n_b):
                c = lay.col_of[p, b]
                if c >= 0:
                    cs[c], ss[c] = a[p, b, :, 0], a[p, b, :, 1]
        return {"cos_fixed": cs, "sin_fixed": ss, "cos": cs / FIXED_POINT_SCALE, "sin": ss / FIXED_POINT_SCALE,
                "occupancy": self.occupancy[slot].cpu().numpy(),
                "counters": dict(zip(N.CNT_NAMES, self.counters[slot].cpu().numpy().tolist()))}

    # -- the loop -------------------------------------------------------------
    def run(self, requests: Sequence, *, realtime: bool = True, poll_s: float = 2e-4) -> Dict[str, Any]:
        """Serve ``requests`` (arrival times relative to the start); returns per-request records
        and the run's latency and throughput statistics."""
        order = sorted(range(len(requests)), key=lambda i: requests[i].arrival)
        recs = {i: Record(i, "sim" if isinstance(requests[i], SimRequest) else "fit", float(requests[i].arrival),
                          self._nbytes(requests[i])) for i in order}
        pending = deque(order)
        launches: deque = deque()              # (event, batch, chunks)
        fits: deque = deque()                  # (event, rid, outputs)
        t0 = time.perf_counter()
        clock = (lambda: time.perf_counter() - t0) if realtime else None
        virtual = [0.0]

        def now() -> float:
            return clock() if realtime else virtual[0]

        n_launch, k = 0, 0
        self.launch_log: List[List[int]] = []
        while pending or launches or fits or self.sched.queue or self.sched.has_work():
            t = now()
            while pending and requests[pending[0]].arrival <= t:
                rid = pending.popleft()
                req = requests[rid]
                self.sched.offer(rid, recs[rid].nbytes, req.n_walkers if isinstance(req, SimRequest) else None)
            for rid in self.sched.admit():
                r = recs[rid]
                r.admit = now()
                req = requests[rid]
                if isinstance(req, SimRequest):
                    r.slot = self.sched.slot_of[rid]
                    with torch.cuda.stream(self.walk_streams[0]):
                        self.accum[r.slot].zero_()
                        self.occupancy[r.slot].zero_()
                        self.counters[r.slot].zero_()
                    for s in self.walk_streams[1:]:
                        s.wait_stream(self.walk_streams[0])
                    r.walker_steps = int(req.n_walkers) * self.cfg.n_steps
                else:
                    if self.library is None:
                        raise ValueError("a fit request needs a server library")
                    from .fitters_gpu import match_device
                    with torch.cuda.stream(self.fit_stream):
                        out = match_device(req.voxels, self.library, free_s0=req.free_s0, precision=req.precision,
                                           topk=req.topk, stream=self.fit_stream, check=False)
                        ev = torch.cuda.Event()
                        ev.record(self.fit_stream)
                    fits.append((ev, rid, out))
            # keep the walk streams fed
            while len(launches) < self.inflight and self.sched.has_work():
                chunks = self.sched.next_launch()
                if not chunks:
                    break
                s = self.walk_streams[k % len(self.walk_streams)]
                k += 1
                with torch.cuda.stream(s):
                    jobs = [WalkJob(requests[rid].ensemble, requests[rid].pp, requests[rid].seed, n, base)
                            for rid, _slot, base, n in chunks]
                    batch = WalkBatch(jobs, self.cfg, layout=self.layout, dirs=self.dirs, launch=self.launch_cfg,
                                      device=self.dev, outputs=(self.accum, self.occupancy, self.counters),
                                      slots=[slot for _rid, slot, _b, _n in chunks])
                    batch.launch(s)
                    ev = torch.cuda.Event()
                    ev.record(s)
                launches.append((ev, batch, chunks))
                self.launch_log.append(sorted({rid for rid, _s, _b, _n in chunks}))
                n_launch += 1
            progressed = False
            while launches and launches[0][0].query():
                _ev, _batch, chunks = launches.popleft()
                for rid in self.sched.complete(chunks):
                    r = recs[rid]
                    r.finish = now()
                    r.result = self._slot_result(r.slot)
                    self.sched.release(rid)
                progressed = True
            while fits and fits[0][0].query():
                _ev, rid, out = fits.popleft()
                out.check()               # the scan finished (raises if a bounded wait ran out)
                idx, res, s0 = out
                r = recs[rid]
                r.finish = now()
                r.result = {"best_idx": idx.cpu().numpy(), "best_resid": res.cpu().numpy(),
                            "best_s0": None if s0 is None else s0.cpu().numpy()}
                self.sched.release(rid)
                progressed = True
            if not progressed:
                if realtime:
                    time.sleep(poll_s)
                elif launches:
                    launches[0][0].synchronize()
                elif fits:
                    fits[0][0].synchronize()
                elif pending:
                    virtual[0] = max(virtual[0], requests[pending[0]].arrival)
        torch.cuda.synchronize(self.dev)
        done = [recs[i] for i in order]
        lat = np.array([r.latency for r in done])
        sims = [r for r in done if r.kind == "sim"]
        span = max(r.finish for r in done) - min(r.arrival for r in done) if done else 0.0
        steps = sum(r.walker_steps for r in sims)
        return {"records": done, "launches": n_launch,
                "p50_s": float(np.percentile(lat, 50)) if len(lat) else float("nan"),
                "p99_s": float(np.percentile(lat, 99)) if len(lat) else float("nan"),
                "walker_steps": steps, "span_s": span,
                "walker_steps_per_s": steps / span if span > 0 else float("nan")}


def _walk_template(cfg: SimConfig, layout: PairLayout, dirs: np.ndarray, boundary: int,
                   lc: LaunchConfig) -> "N.MadiWalkDesc":
    """The job-independent part of a fused fp32 Philox walk descriptor."""
    d = N.MadiWalkDesc()
    d.tile_walkers = int(lc.tile_walkers)
    d.boundary = int(boundary)
    d.precision = 32
    d.rng = N.MADI_RNG_PHILOX
    d.out_mode = N.MADI_OUT_FUSED
    d.n_steps, d.steps_per_h, d.n_grid = cfg.n_steps, cfg.steps_per_h, cfg.n_grid
    d.sigma, d.ts = cfg.sigma, cfg.ts
    d.min_blocks = int(lc.min_blocks)
    d.n_pairs, d.n_b, d.n_dirs = layout.n_pairs, layout.n_b, len(dirs)
    for p in range(layout.n_pairs):
        d.pair_jd[p], d.pair_jD[p], d.pair_js[p] = int(layout.jd[p]), int(layout.jD[p]), int(layout.js[p])
        for b in range(layout.n_b):
            d.coef[p * layout.n_b + b] = float(layout.coef[p, b])
    for k in range(len(dirs)):
        for a in range(3):
            d.dirs[3 * k + a] = float(dirs[k, a])
    d.stage_smem = 0                       # geometry read in place
    return d


class NativeSimServer:
    """Simulation requests served by the native loop (``madi_serve_*``): the same
    admission and chunking rules as ``Server``, run by the C++ runtime; results
    are read from the slot pools.  Periodic or fatal-escape geometries, one kind
    per server."""

    def __init__(self, cfg: SimConfig, layout: PairLayout, dirs: np.ndarray, *, boundary: int,
                 budget_bytes: int = 8 << 30, n_slots: int = 64, chunk_walkers: int = 65536,
                 launch_walkers: int = 155648, inflight: int = 2, launch: Optional[LaunchConfig] = None,
                 device=None):
        import ctypes as C
        if torch is None or not torch.cuda.is_available():
            raise RuntimeError("the server runs on a CUDA device")
        self.dev = torch.device(device or "cuda")
        self.cfg, self.layout = cfg, layout
        self.dirs = np.asarray(dirs, np.float64)
        self.n_out = layout.n_pairs * layout.n_b * len(self.dirs)
        lc = launch or LaunchConfig()
        self.accum = torch.zeros((n_slots, self.n_out * 2), dtype=torch.int64, device=self.dev)
        self.occupancy = torch.zeros((n_slots, cfg.n_grid), dtype=torch.int64, device=self.dev)
        self.counters = torch.zeros((n_slots, N.MADI_CNT_N), dtype=torch.int64, device=self.dev)
        sc = N.MadiServeConfig()
        sc.walk = _walk_template(cfg, layout, self.dirs, boundary, lc)
        sc.walk.accum, sc.walk.occupancy, sc.walk.counters = N.ptr(self.accum), N.ptr(self.occupancy), N.ptr(self.counters)
        sc.n_slots, sc.chunk_walkers, sc.launch_walkers, sc.inflight = n_slots, chunk_walkers, launch_walkers, inflight
        sc.budget_bytes = int(budget_bytes)
        need = int(N.lib().madi_serve_arena_bytes(C.byref(sc)))
        self.arena = torch.empty(need + 256, dtype=torch.uint8, device=self.dev)
        base = N.ptr(self.arena)
        sc.arena, sc.arena_bytes = base + ((-base) % 256), need
        self._cfg_struct = sc
        h = C.c_void_p()
        N.check(N.lib().madi_serve_create(C.byref(sc), C.byref(h)), "madi_serve_create")
        self._h = h
        self._C = C

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().madi_serve_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _result(self, slot: int) -> dict:
        lay = self.layout
        a = self.accum[slot].cpu().numpy().reshape(lay.n_pairs, lay.n_b, len(self.dirs), 2)
        n_cols = int(lay.col_of.max()) + 1
        cs = np.zeros((n_cols, len(self.dirs)), np.int64)
        ss = np.zeros((n_cols, len(self.dirs)), np.int64)
        for p in range(lay.n_pairs):
            for b in range(lay.n_b):
                c = lay.col_of[p, b]
                if c >= 0:
                    cs[c], ss[c] = a[p, b, :, 0], a[p, b, :, 1]
        return {"cos_fixed": cs, "sin_fixed": ss, "cos": cs / FIXED_POINT_SCALE, "sin": ss / FIXED_POINT_SCALE,
                "occupancy": self.occupancy[slot].cpu().numpy(),
                "counters": dict(zip(N.CNT_NAMES, self.counters[slot].cpu().numpy().tolist()))}

    def run(self, requests: Sequence[SimRequest], *, realtime: bool = True, poll_s: float = 2e-4) -> Dict[str, Any]:
        C = self._C
        torch.cuda.synchronize(self.dev)       # pools and geometry ready before the native streams start
        order = sorted(range(len(requests)), key=lambda i: requests[i].arrival)
        recs = {i: Record(i, "sim", float(requests[i].arrival),
                          requests[i].ensemble.device(str(self.dev)).nbytes) for i in order}
        for i in order:
            recs[i].walker_steps = int(requests[i].n_walkers) * self.cfg.n_steps
        pending, ids = list(order), {}
        done = (N.MadiServeDone * 64)()
        n_done, n_pend = C.c_int32(), C.c_int32()
        t0 = time.perf_counter()
        remaining = len(order)
        while remaining:
            t = time.perf_counter() - t0
            while pending and (not realtime or requests[pending[0]].arrival <= t):
                i = pending.pop(0)
                r = requests[i]
                q = N.MadiServeRequest()
                q.geometry = r.ensemble.device(str(self.dev)).struct
                q.pp, q.seed, q.n_walkers, q.nbytes = float(r.pp), int(r.seed) & 0xFFFFFFFF, int(r.n_walkers), recs[i].nbytes
                rid = C.c_int64()
                N.check(N.lib().madi_serve_submit(self._h, C.byref(q), C.byref(rid)), "madi_serve_submit")
                ids[rid.value] = i
                recs[i].admit = None
            N.check(N.lib().madi_serve_poll(self._h, 64, done, C.byref(n_done), C.byref(n_pend)), "madi_serve_poll")
            for k in range(n_done.value):
                d = done[k]
                i = ids[d.request_id]
                r = recs[i]
                r.slot = d.slot
                r.admit = r.arrival + (d.admit_s - d.submit_s)
                r.finish = time.perf_counter() - t0
                r.result = self._result(d.slot)
                N.check(N.lib().madi_serve_release(self._h, d.request_id), "madi_serve_release")
                remaining -= 1
            if remaining and n_done.value == 0:
                time.sleep(poll_s)
        recs_l = [recs[i] for i in order]
        lat = np.array([r.latency for r in recs_l])
        span = max(r.finish for r in recs_l) - min(r.arrival for r in recs_l)
        steps = sum(r.walker_steps for r in recs_l)
        return {"records": recs_l, "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                "walker_steps": steps, "span_s": span, "walker_steps_per_s": steps / span if span > 0 else float("nan")}


def to_reduced(rec: Record, req: SimRequest, cfg: SimConfig):
    """A finished simulation record as the reference's ReducedResult."""
    from .walker_gpu import results_to_reduced
    return results_to_reduced(req.ensemble, req.pp, cfg, rec.result, req.n_walkers)


def poisson_arrivals(n: int, rate_per_s: float, seed: int) -> np.ndarray:
    """Arrival times (s) of a Poisson process."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, n))
