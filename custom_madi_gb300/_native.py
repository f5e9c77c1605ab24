"""ctypes binding of the native library (C ABI in include/madi_gb300.h).

The library is built in-tree by ``custom_madi_gb300._build.build()``.  Nothing
here falls back to a CPU implementation: if the shared object is missing or a
CUDA device is absent, the call raises.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

from . import _build

MADI_OK = 0
MADI_ERR_INVALID = 1
MADI_ERR_CUDA = 2
MADI_ERR_CAPACITY = 3
MADI_ERR_TIMEOUT = 4
MADI_ERR_UNSUPPORTED = 5
MADI_ERR_GEOMETRY = 6
MADI_ERR_HOST_MEMORY = 7

MADI_BOUNDARY_FATAL = 0
MADI_BOUNDARY_PERIODIC = 1
MADI_RNG_PHILOX = 0
MADI_RNG_STREAM = 1
MADI_OUT_FUSED = 0
MADI_OUT_Y = 1
MADI_MAX_PAIRS = 8
MADI_MAX_B = 32
MADI_MAX_DIRS = 32
MADI_MAX_GRID = 512
MADI_MATCH_FIXED_S0 = 0
MADI_MATCH_FREE_S0 = 1
MADI_MATCH_FP32 = 0
MADI_MATCH_BF16 = 1
MADI_MATCH_FLAG_TEST_STALL = 1
MADI_MATCH_FLAG_FULL_SCAN = 2

CNT_NAMES = ("walkers", "escaped", "classifier_error", "full", "tier1", "fallback64",
             "cross_accept", "cross_reject", "facet_pass")
MADI_CNT_N = len(CNT_NAMES)

EXPORTED = (
    "madi_abi_version", "madi_last_error_string", "madi_classify", "madi_walk",
    "madi_walk_smem_bytes", "madi_reduce_Y", "madi_reduce_Y_scratch_bytes", "madi_match", "madi_match_wait", "madi_match_scratch_bytes",
    "madi_bayes", "madi_bayes_scratch_bytes",
    "madi_kdtree_build", "madi_grid_build", "madi_facets_build", "madi_walk_blocks_per_sm", "madi_walk_noalloc",
    "madi_walk_batched", "madi_autotune_load", "madi_autotune_store",
    "madi_serve_arena_bytes", "madi_serve_create", "madi_serve_submit", "madi_serve_poll",
    "madi_serve_release", "madi_serve_destroy",
)


class MadiLaunchShape(C.Structure):
    _fields_ = [("tile_walkers", C.c_int32), ("blocks_per_sm", C.c_int32), ("min_blocks", C.c_int32),
                ("stage_budget", C.c_int32), ("walker_steps_per_s", C.c_double)]


class MadiGeometry(C.Structure):
    _fields_ = [
        ("stage", C.c_void_p), ("seed_f64", C.c_void_p), ("kd_seed", C.c_void_p),
        ("kd_left", C.c_void_p), ("kd_right", C.c_void_p), ("kd_parent", C.c_void_p),
        ("kd_axis", C.c_void_p),
        ("off_cell", C.c_uint32), ("off_grid_offset", C.c_uint32),
        ("off_grid_ids", C.c_uint32), ("stage_bytes", C.c_uint32),
        ("n_seeds", C.c_int32), ("grid_n", C.c_int32), ("ids_u32", C.c_int32),
        ("boundary", C.c_int32), ("has_cells", C.c_int32), ("pad0", C.c_int32),
        ("L", C.c_double), ("grid_h", C.c_double), ("safe_cap", C.c_double),
        ("source_lo", C.c_double), ("source_hi", C.c_double), ("coord_err", C.c_double),
        ("off_cell_center", C.c_uint32), ("facet_stride", C.c_uint32),
        ("off_facet_plane", C.c_uint32), ("off_facet_nbr", C.c_uint32),
        ("n_cells", C.c_int32), ("pad1", C.c_int32), ("facet_tol", C.c_double),
    ]


class MadiWalkJob(C.Structure):
    _fields_ = [
        ("geom", C.c_int32), ("n_walkers", C.c_int32), ("walker_base", C.c_uint32),
        ("key0", C.c_uint32), ("key1", C.c_uint32), ("slot", C.c_int32),
        ("tile_begin", C.c_int32), ("y_row", C.c_int32), ("pp", C.c_double),
        ("thr1", C.c_uint64), ("thr2", C.c_uint64),
    ]


class MadiWalkDesc(C.Structure):
    _fields_ = [
        ("geoms", C.c_void_p), ("jobs", C.c_void_p),
        ("n_geoms", C.c_int32), ("n_jobs", C.c_int32), ("n_tiles", C.c_int32),
        ("tile_walkers", C.c_int32), ("grid_blocks", C.c_int32), ("stage_smem", C.c_int32),
        ("boundary", C.c_int32), ("precision", C.c_int32), ("rng", C.c_int32),
        ("out_mode", C.c_int32), ("n_steps", C.c_int32), ("steps_per_h", C.c_int32),
        ("n_grid", C.c_int32),
        ("sigma", C.c_double), ("ts", C.c_double),
        ("n_pairs", C.c_int32), ("n_b", C.c_int32), ("n_dirs", C.c_int32), ("min_blocks", C.c_int32),
        ("pair_jd", C.c_int32 * MADI_MAX_PAIRS), ("pair_jD", C.c_int32 * MADI_MAX_PAIRS),
        ("pair_js", C.c_int32 * MADI_MAX_PAIRS),
        ("coef", C.c_float * (MADI_MAX_PAIRS * MADI_MAX_B)),
        ("dirs", C.c_float * (MADI_MAX_DIRS * 3)),
        ("accum", C.c_void_p), ("occupancy", C.c_void_p), ("counters", C.c_void_p),
        ("Y", C.c_void_p), ("inside_trace", C.c_void_p),
        ("init", C.c_void_p), ("incr", C.c_void_p), ("unif", C.c_void_p),
        ("work_counter", C.c_void_p),
    ]


class MadiMatchDesc(C.Structure):
    _fields_ = [
        ("measured", C.c_void_p), ("lib", C.c_void_p), ("n_vox", C.c_int64),
        ("n_lib", C.c_int32), ("n_feat", C.c_int32), ("mode", C.c_int32),
        ("precision", C.c_int32), ("topk", C.c_int32), ("flags", C.c_int32),
        ("best_idx", C.c_void_p), ("best_resid", C.c_void_p), ("best_s0", C.c_void_p),
        ("scratch", C.c_void_p), ("scratch_bytes", C.c_int64),
    ]


class MadiBayesDesc(C.Structure):
    _fields_ = [
        ("measured", C.c_void_p), ("lib", C.c_void_p), ("log_weight", C.c_void_p), ("kio", C.c_void_p),
        ("rho", C.c_void_p), ("V", C.c_void_p), ("n_vox", C.c_int64), ("n_lib", C.c_int32),
        ("n_feat", C.c_int32), ("mode", C.c_int32), ("pad0", C.c_int32), ("sigma_m", C.c_double),
        ("out", C.c_void_p), ("scratch", C.c_void_p), ("scratch_bytes", C.c_int64),
    ]


MADI_BAYES_N_OUT = 9


class MadiServeConfig(C.Structure):
    _fields_ = [("walk", MadiWalkDesc), ("n_slots", C.c_int32), ("chunk_walkers", C.c_int32),
                ("launch_walkers", C.c_int32), ("inflight", C.c_int32), ("budget_bytes", C.c_int64),
                ("arena", C.c_void_p), ("arena_bytes", C.c_int64)]


class MadiServeRequest(C.Structure):
    _fields_ = [("geometry", MadiGeometry), ("pp", C.c_double), ("seed", C.c_uint32), ("pad0", C.c_uint32),
                ("n_walkers", C.c_int64), ("nbytes", C.c_int64)]


class MadiServeDone(C.Structure):
    _fields_ = [("request_id", C.c_int64), ("slot", C.c_int32), ("pad0", C.c_int32),
                ("submit_s", C.c_double), ("admit_s", C.c_double), ("finish_s", C.c_double)]


class MadiError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


_lib = None
_lock = threading.Lock()


def _declare(lib):
    P = C.c_void_p
    lib.madi_abi_version.restype = C.c_int32
    lib.madi_last_error_string.restype = C.c_char_p
    lib.madi_classify.argtypes = [C.POINTER(MadiGeometry), P, C.c_int, C.c_int64, C.c_int, P, P, P, P]
    lib.madi_walk.argtypes = [C.POINTER(MadiWalkDesc), P]
    lib.madi_walk_noalloc.argtypes = [C.POINTER(MadiWalkDesc), P]
    lib.madi_walk_batched.argtypes = [C.POINTER(MadiWalkDesc), P]
    lib.madi_autotune_load.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(MadiLaunchShape)]
    lib.madi_autotune_store.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(MadiLaunchShape)]
    lib.madi_serve_arena_bytes.argtypes = [C.POINTER(MadiServeConfig)]
    lib.madi_serve_arena_bytes.restype = C.c_int64
    lib.madi_serve_create.argtypes = [C.POINTER(MadiServeConfig), C.POINTER(C.c_void_p)]
    lib.madi_serve_submit.argtypes = [P, C.POINTER(MadiServeRequest), C.POINTER(C.c_int64)]
    lib.madi_serve_poll.argtypes = [P, C.c_int32, C.POINTER(MadiServeDone), C.POINTER(C.c_int32),
                                    C.POINTER(C.c_int32)]
    lib.madi_serve_release.argtypes = [P, C.c_int64]
    lib.madi_serve_destroy.argtypes = [P]
    lib.madi_walk_smem_bytes.argtypes = [C.c_int32, C.c_int32, C.c_int32]
    lib.madi_walk_smem_bytes.restype = C.c_int64
    lib.madi_walk_blocks_per_sm.argtypes = [C.POINTER(MadiWalkDesc)]
    lib.madi_walk_blocks_per_sm.restype = C.c_int32
    lib.madi_reduce_Y.argtypes = [P, C.c_int64, C.c_int32, P, P, P, P, C.c_int32, P, P, P, C.c_int64, P]
    lib.madi_reduce_Y_scratch_bytes.argtypes = [C.c_int32]
    lib.madi_reduce_Y_scratch_bytes.restype = C.c_int64
    lib.madi_match.argtypes = [C.POINTER(MadiMatchDesc), P]
    lib.madi_match_wait.argtypes = [C.POINTER(MadiMatchDesc), P]
    lib.madi_bayes.argtypes = [C.POINTER(MadiBayesDesc), P]
    lib.madi_bayes_scratch_bytes.argtypes = [C.c_int32, C.c_int32]
    lib.madi_bayes_scratch_bytes.restype = C.c_int64
    lib.madi_match_scratch_bytes.argtypes = [C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    lib.madi_match_scratch_bytes.restype = C.c_int64
    lib.madi_kdtree_build.argtypes = [P, C.c_int32, P, P, P, P, P]
    lib.madi_grid_build.argtypes = [P, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double,
                                    P, P, C.c_int32, C.c_int64, C.POINTER(C.c_int64)]
    lib.madi_facets_build.argtypes = [P, C.c_int32, C.c_int32, C.c_double, P, P, P, C.c_int64,
                                      C.POINTER(C.c_int64), P]
    for name in ("madi_classify", "madi_walk", "madi_walk_noalloc", "madi_walk_batched", "madi_reduce_Y",
                 "madi_match", "madi_match_wait", "madi_bayes", "madi_kdtree_build", "madi_grid_build", "madi_facets_build", "madi_autotune_load",
                 "madi_autotune_store", "madi_serve_create", "madi_serve_submit", "madi_serve_poll",
                 "madi_serve_release", "madi_serve_destroy"):
        getattr(lib, name).restype = C.c_int


def lib():
    """The loaded native library; builds it in-tree on first use if absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _build.library_path()
            if not path.exists():
                if os.environ.get("MADI_NO_AUTOBUILD"):
                    raise RuntimeError(f"native library missing: {path}")
                _build.build()
            handle = C.CDLL(str(path))
            _declare(handle)
            if handle.madi_abi_version() != 1:
                raise RuntimeError("custom_madi_gb300 native library ABI mismatch")
            _lib = handle
    return _lib


_lib_digest = None


def lib_digest() -> str:
    """Short hash of the loaded native library's file: tuned launch shapes are
    keyed on it, so a rebuilt kernel is tuned again."""
    global _lib_digest
    if _lib_digest is None:
        import hashlib
        lib()
        _lib_digest = hashlib.sha256(_build.library_path().read_bytes()).hexdigest()[:12]
    return _lib_digest


def check(status: int, what: str) -> None:
    if status == MADI_OK:
        return
    msg = (lib().madi_last_error_string() or b"").decode(errors="replace")
    text = f"{what}: {msg}" if msg else f"{what}: status {status}"
    if status in (MADI_ERR_INVALID,):
        raise ValueError(text)
    raise MadiError(status, text)


def ptr(t) -> int:
    """Device (or host) address of a torch tensor, 0 for None."""
    if t is None:
        return 0
    return int(t.data_ptr())


def reduce_Y(Y, n_walkers: int, n_grid: int, jd, jD, js, coef, cos_sum, sin_sum, stream) -> None:
    """madi_reduce_Y on device tensors (int32 jd / jD / js, fp64 coef and outputs),
    with a scratch buffer of the size the library asks for."""
    import torch
    n = int(coef.numel())
    scratch = torch.empty(max(int(lib().madi_reduce_Y_scratch_bytes(n)) // 8, 1), dtype=torch.int64, device=coef.device)
    st = lib().madi_reduce_Y(ptr(Y), int(n_walkers), int(n_grid), ptr(jd), ptr(jD), ptr(js), ptr(coef), n,
                             ptr(cos_sum), ptr(sin_sum), ptr(scratch), scratch.numel() * 8, stream.cuda_stream)
    check(st, "madi_reduce_Y")
