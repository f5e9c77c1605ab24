"""Library match on the GPU (madi/fitters_gpu.py:414-463 entry points).

``map_match_gpu`` / ``map_match_fits0_gpu`` keep the reference signatures and
return shapes; ``precision`` selects the exhaustive FP32 scan or the BF16
tensor-core scan with top-k FP32 rescoring.  Inputs are numpy (host) or torch
CUDA tensors; outputs are numpy.
"""

from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _native as N

try:
    import torch
    HAS_CUDA = bool(torch.cuda.is_available())
except Exception:  # pragma: no cover
    torch = None
    HAS_CUDA = False

DEFAULT_TOPK = 32


def _as_dev(x):
    if torch.is_tensor(x):
        return x.to(device="cuda", dtype=torch.float32).contiguous()
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).cuda()


class MatchOutput(tuple):
    """(best_idx, best_resid, best_s0) device tensors of one madi_match call.

    ``check()`` waits for the call and raises ``MadiError`` (a RuntimeError,
    status MADI_ERR_TIMEOUT) if a bounded wait of the tensor-core scan ran out;
    the rows it could not finish keep -1 in best_idx.  The inputs and scratch
    stay referenced until then.
    """

    def __new__(cls, idx, res, s0, desc, stream, keep):
        out = super().__new__(cls, (idx, res, s0))
        out._desc, out._stream, out._keep = desc, stream, keep
        return out

    def check(self) -> "MatchOutput":
        st = N.lib().madi_match_wait(C.byref(self._desc), self._stream.cuda_stream)
        N.check(st, "madi_match")
        return self


def match_device(measured, lib_mat, *, free_s0: bool = False, precision: str = "fp32", topk: int = DEFAULT_TOPK,
                 scratch=None, stream=None, check: bool = True, flags: int = 0) -> MatchOutput:
    """Run madi_match on device tensors; returns (best_idx, best_resid, best_s0) device tensors.

    ``check=True`` waits for the result and raises if the scan could not
    finish (see ``MatchOutput.check``); ``check=False`` returns as soon as the
    work is enqueued on ``stream`` and the caller calls ``.check()`` later.
    ``flags``: MADI_MATCH_FLAG_FULL_SCAN (BF16 fixed S0 without the
    principal-axis scan cut; same result up to BF16 score ties at the k-th
    place) or, for tests, MADI_MATCH_FLAG_TEST_STALL.
    """
    if not HAS_CUDA:
        raise RuntimeError("CUDA is unavailable: the library match runs on a CUDA device only")
    M = _as_dev(measured)
    Lm = _as_dev(lib_mat)
    if M.ndim != 2 or Lm.ndim != 2 or M.shape[1] != Lm.shape[1]:
        raise ValueError("measured (n_vox, F) and library (n_lib, F) must share F")
    n_vox, F = M.shape
    prec = {"fp32": N.MADI_MATCH_FP32, "bf16": N.MADI_MATCH_BF16}[precision]
    # BF16 CTAs that give up on a bounded wait leave their rows at -1
    idx = (torch.full((n_vox,), -1, dtype=torch.int32, device=M.device) if prec == N.MADI_MATCH_BF16
           else torch.empty(n_vox, dtype=torch.int32, device=M.device))
    res = torch.empty(n_vox, dtype=torch.float32, device=M.device)
    s0 = torch.empty(n_vox, dtype=torch.float32, device=M.device) if free_s0 else None
    need = int(N.lib().madi_match_scratch_bytes(n_vox, Lm.shape[0], F, prec, int(topk)))
    if need > 0 and (scratch is None or scratch.numel() < need + 256):
        scratch = torch.empty(need + 256, dtype=torch.uint8, device=M.device)
    d = N.MadiMatchDesc()
    d.measured, d.lib, d.n_vox, d.n_lib, d.n_feat = N.ptr(M), N.ptr(Lm), n_vox, Lm.shape[0], F
    d.mode = N.MADI_MATCH_FREE_S0 if free_s0 else N.MADI_MATCH_FIXED_S0
    d.precision, d.topk, d.flags = prec, int(topk), int(flags)
    d.best_idx, d.best_resid, d.best_s0 = N.ptr(idx), N.ptr(res), N.ptr(s0)
    if need > 0:
        base = N.ptr(scratch)
        pad = (-base) % 256
        d.scratch, d.scratch_bytes = base + pad, int(scratch.numel()) - pad
    else:
        d.scratch, d.scratch_bytes = 0, 0
    s = stream if stream is not None else torch.cuda.current_stream(M.device)
    st = N.lib().madi_match(C.byref(d), s.cuda_stream)
    N.check(st, "madi_match")
    out = MatchOutput(idx, res, s0, d, s, (M, Lm, scratch))
    return out.check() if check else out


def _indices(idx) -> np.ndarray:
    b = idx.cpu().numpy().astype(np.int64)
    if np.any(b < 0):
        raise RuntimeError("tensor-core library match gave up on a bounded wait; no result for some voxels")
    return b


def map_match_gpu(measured_batch, lib_mat, kios_arr, rhos_arr, Vs_arr, *, precision: str = "fp32",
                  topk: int = DEFAULT_TOPK):
    """Fixed-S0 MAP: (kio, rho, V, resid) of the best library entry per voxel."""
    idx, res, _ = match_device(measured_batch, lib_mat, precision=precision, topk=topk)
    b = _indices(idx)
    return (np.asarray(kios_arr)[b], np.asarray(rhos_arr)[b], np.asarray(Vs_arr)[b],
            res.cpu().numpy().astype(np.float64))


def map_match_fits0_gpu(raw_signal, lib_mat, kios_arr, rhos_arr, Vs_arr, *, precision: str = "fp32",
                        topk: int = DEFAULT_TOPK):
    """Free-S0 MAP: (kio, rho, V, resid, s0) of the best library entry per voxel."""
    idx, res, s0 = match_device(raw_signal, lib_mat, free_s0=True, precision=precision, topk=topk)
    b = _indices(idx)
    return (np.asarray(kios_arr)[b], np.asarray(rhos_arr)[b], np.asarray(Vs_arr)[b],
            res.cpu().numpy().astype(np.float64), s0.cpu().numpy().astype(np.float64))


def bayes_fit_gpu(measured_batch, lib_mat, kios_arr, rhos_arr, Vs_arr, sigma_m, fit_s0=False,
                  quadrature_weights=None, *, stream=None) -> dict:
    """GPU Bayesian posterior means (madi/fitters_gpu.py:466-528 signature).

    ``measured_batch`` is the normalised (and, if asked, log-transformed)
    signal for fixed S0 or the raw signal for ``fit_s0=True``.  Returns
    kio/rho/V means and stds, the weighted residual and n_eff (+ s0_fit) as
    fp64 numpy arrays; one ``madi_bayes`` launch.
    """
    if not HAS_CUDA:
        raise RuntimeError("CUDA is unavailable: the Bayesian fit runs on a CUDA device only")
    if quadrature_weights is None:
        raise ValueError("Bayesian GPU fitting requires positive quadrature weights.")
    q = np.ascontiguousarray(quadrature_weights, dtype=np.float64)
    kios_arr = np.asarray(kios_arr, np.float64)
    if q.shape != kios_arr.shape or not np.all(np.isfinite(q) & (q > 0.0)):
        raise ValueError("invalid Bayesian quadrature weights")
    if not (float(sigma_m) > 0.0):
        raise ValueError(f"sigma_m must be > 0, got {sigma_m}")
    M = _as_dev(measured_batch)
    Lm = _as_dev(lib_mat)
    if M.ndim != 2 or Lm.ndim != 2 or M.shape[1] != Lm.shape[1]:
        raise ValueError("measured (n_vox, F) and library (n_lib, F) must share F")
    dev = M.device
    n_vox, F = M.shape
    n_lib = Lm.shape[0]
    par = [torch.from_numpy(np.ascontiguousarray(a, np.float64)).to(dev)
           for a in (np.log(q), kios_arr, np.asarray(rhos_arr, np.float64), np.asarray(Vs_arr, np.float64))]
    out = torch.empty((N.MADI_BAYES_N_OUT, n_vox), dtype=torch.float64, device=dev)
    scratch = torch.empty(int(N.lib().madi_bayes_scratch_bytes(n_lib, F)) + 256, dtype=torch.uint8, device=dev)
    d = N.MadiBayesDesc()
    d.measured, d.lib = N.ptr(M), N.ptr(Lm)
    d.log_weight, d.kio, d.rho, d.V = (N.ptr(t) for t in par)
    d.n_vox, d.n_lib, d.n_feat = n_vox, n_lib, F
    d.mode = N.MADI_MATCH_FREE_S0 if fit_s0 else N.MADI_MATCH_FIXED_S0
    d.sigma_m = float(sigma_m)
    d.out = N.ptr(out)
    base = N.ptr(scratch)
    pad = (-base) % 256
    d.scratch, d.scratch_bytes = base + pad, int(scratch.numel()) - pad
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    N.check(N.lib().madi_bayes(C.byref(d), s.cuda_stream), "madi_bayes")
    o = out.cpu().numpy()
    res = dict(kio_mean=o[0], rho_mean=o[1], V_mean=o[2], kio_std=o[3], rho_std=o[4], V_std=o[5],
               residual=o[6], n_eff=o[7])
    if fit_s0:
        res["s0_fit"] = o[8]
    return res
