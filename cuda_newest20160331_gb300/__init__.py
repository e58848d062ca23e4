"""GB300-native voxel-network builder (BNAPlatform's correlation -> CSR ->
eigenvector-centrality path), Python host side over the C ABI of libbna.so.

Mapping to the reference (W/ = BNAPlatform-weighted-win64-cuda7.0-20160331/src):

  Builder.corr_csr     CorMat_gpu + post_block + FormFullGraph(_s) + FormCSRGraph
                       (W/CorMat/CUCorMat/CUCorMat/CorMat.cu:17, CorMat.cpp:683-918)
  Builder.ec           Lead_Vector_GPU (W/CUEC/weighted-net.cu:55-221)
  Builder.lead_vector  the same with host buffers and the reference's argument list
  Server               many subjects on one GPU: continuous admission by HBM budget,
                       each request CorMat -> CSR -> Lead_Vector (no reference counterpart)
  csr_write / csr_read the .csr format (CorMat.cpp:353-360, weighted-net.cu:275-287)

Device buffers are torch CUDA tensors (torch is plumbing for memory and
streams only); every computation runs in libbna.so's sm_103a kernels.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib as L
from ._lib import BnaError, lib

__all__ = ["Builder", "CsrResult", "Server", "Reply", "synth_bold", "csr_write", "csr_read",
           "ec_write", "request_bytes", "density_nnz", "nifti_mask", "nifti_bold", "BnaError",
           "lib"]


def _check(status: int, ctx=None, ok=(L.BNA_OK,)) -> int:
    if status not in ok:
        msg = lib().bna_ctx_last_error(ctx).decode() if ctx else ""
        raise BnaError(status, msg)
    return status


def synth_bold(N: int, T: int, K: int, seed: int, kind: str = "iid", phi: float = 0.7,
               load_sd: float = 0.3, jitter_sd: float = 0.0, block: int = 500,
               n_net: int = 60, threads: int = 0) -> np.ndarray:
    """Deterministic factor-model BOLD, float32 time-major [T][N]."""
    p = L.SynthParams(N=N, T=T, K=K, kind=L.SYNTH_KINDS[kind], seed=seed, phi=phi,
                      load_sd=load_sd, jitter_sd=jitter_sd, block=block, n_net=n_net)
    out = np.empty((T, N), dtype=np.float32)
    _check(lib().bna_synth_bold(C.byref(p), out.ctypes.data, threads))
    return out


@dataclass
class CsrResult:
    n: int
    nnz: int
    row_ptr: object   # torch.int32 [n+1] (device) or np.int32 (host)
    col_idx: object   # [nnz]
    val: object       # [nnz] float32 or None
    stats: dict

    def numpy(self) -> "CsrResult":
        def h(x):
            if x is None:
                return None
            return x.cpu().numpy() if hasattr(x, "cpu") else np.asarray(x)
        return CsrResult(self.n, self.nnz, h(self.row_ptr), h(self.col_idx), h(self.val),
                         self.stats)


class _DevArray:
    """Zero-copy __cuda_array_interface__ view of arena memory."""

    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr,
                                         "data": (ptr, False), "version": 3, "strides": None}


def _view(ptr, n, typestr, torch, device):
    if not ptr or n == 0:
        dt = {"<i4": torch.int32, "<f4": torch.float32, "<f8": torch.float64}[typestr]
        return torch.empty(0, dtype=dt, device=device)
    return torch.as_tensor(_DevArray(ptr, n, typestr), device=device)


def _opts(mode: str, value: float, precision: str, weighted: bool, delta: Optional[float]):
    if mode not in L.THR_MODES:
        raise ValueError(f"mode must be one of {sorted(L.THR_MODES)}")
    if precision not in L.PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(L.PRECISIONS)}")
    return L.CorrOpts(mode=L.THR_MODES[mode], precision=L.PRECISIONS[precision],
                      value=float(value), weighted=1 if weighted else 0,
                      delta=float(delta) if delta else 0.0)


class Builder:
    """One libbna context on one CUDA device (owns a reusable device arena)."""

    def __init__(self, device: int = 0):
        self.device = device
        h = C.c_void_p()
        _check(lib().bna_ctx_create(device, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().bna_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def arena_bytes(self) -> int:
        return int(lib().bna_ctx_arena_bytes(self._h))

    def trim(self):
        _check(lib().bna_ctx_trim(self._h), self._h)

    def autotune(self, N: int, T: int, mode: str = "r_gt", value: float = 0.5,
                 weighted: bool = True):
        """bna_autotune: -> (chosen precision name, {form: ms})."""
        o = _opts(mode, value, "auto", weighted, None)
        best = C.c_int32()
        ms = (C.c_float * 2)()
        _check(lib().bna_autotune(self._h, N, T, C.byref(o), C.byref(best), ms), self._h)
        names = {v: k for k, v in L.PRECISIONS.items()}
        return names[best.value], {"bf16x3": ms[0], "tf32": ms[1]}

    TUNE_BANDS = (16, 32, 64)

    def autotune_shape(self, N: int, T: int, mode: str = "r_gt", value: float = 0.5,
                       weighted: bool = True):
        """bna_autotune_shape: -> ((precision name, band), {(form, band): ms})."""
        o = _opts(mode, value, "auto", weighted, None)
        best = C.c_int32()
        band = C.c_int32()
        ms = (C.c_float * 6)()
        _check(lib().bna_autotune_shape(self._h, N, T, C.byref(o), C.byref(best),
                                        C.byref(band), ms), self._h)
        names = {v: k for k, v in L.PRECISIONS.items()}
        times = {(f, b): ms[i * 3 + j] for i, f in enumerate(("bf16x3", "tf32"))
                 for j, b in enumerate(self.TUNE_BANDS)}
        return (names[best.value], band.value), times

    def set_option(self, name: str, value: int):
        """bna_ctx_set_option: "tiles_per_launch", "max_nnz", "ec_iters_per_launch"
        or "tile_band" (0 = default)."""
        _check(lib().bna_ctx_set_option(self._h, L.OPTIONS[name], int(value)), self._h)

    GATE = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_int32, C.c_int64)

    def set_gate(self, fn=None):
        """bna_ctx_set_gate: fn(stream_handle, phase, done) is called between the
        launches of long passes (None removes it)."""
        self._gate = Builder.GATE(lambda user, stream, phase, done: fn(stream, phase, done)) \
            if fn else None
        _check(lib().bna_ctx_set_gate(self._h, C.cast(self._gate, C.c_void_p) if fn else None,
                                      None), self._h)

    @staticmethod
    def _stream(stream):
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        return C.c_void_p(s.cuda_stream)

    def zscore(self, bold, stream=None):
        """bold: torch CUDA float32 [T][N] -> z [N][ldz] (ldz = T rounded up to 32)."""
        import torch
        T, N = bold.shape
        ld = int(lib().bna_zscore_ld(T))
        z = torch.empty((N, ld), dtype=torch.float32, device=bold.device)
        _check(lib().bna_zscore(self._h, C.c_void_p(bold.data_ptr()), N, T,
                                C.c_void_p(z.data_ptr()), ld, self._stream(stream)), self._h)
        return z

    def corr_csr(self, bold, mode: str = "r_gt", value: float = 0.5, precision: str = "fp32",
                 weighted: bool = True, delta: Optional[float] = None, stream=None,
                 copy: bool = True) -> CsrResult:
        """Correlation -> thresholded CSR on the device.

        bold: torch CUDA float32, contiguous, time-major [T][N].  With copy=False
        the returned tensors alias the context's arena (valid until the next call).
        """
        import torch
        assert bold.is_cuda and bold.dtype == torch.float32 and bold.is_contiguous()
        T, N = bold.shape
        o = _opts(mode, value, precision, weighted, delta)
        out = L.Csr()
        st = L.CorrStats()
        _check(lib().bna_corr_csr(self._h, C.c_void_p(bold.data_ptr()), N, T, C.byref(o),
                                  C.byref(out), C.byref(st), self._stream(stream)), self._h)
        dev = bold.device
        rp = _view(out.row_ptr, N + 1, "<i4", torch, dev)
        ci = _view(out.col_idx, out.nnz, "<i4", torch, dev)
        va = _view(out.val, out.nnz, "<f4", torch, dev) if out.val else None
        if copy:
            rp, ci = rp.clone(), ci.clone()
            va = va.clone() if va is not None else None
        return CsrResult(N, int(out.nnz), rp, ci, va, st.as_dict())

    def corr_csr_batch(self, bolds, mode: str = "r_gt", value: float = 0.5,
                       precision: str = "bf16x3", weighted: bool = True,
                       delta: Optional[float] = None, stream=None, copy: bool = True):
        """A batch of subjects (bna_corr_csr_batch): one persistent count pass
        over all subjects' tiles.  bolds: torch CUDA float32 [T_k][N_k] tensors.
        -> list of CsrResult."""
        import torch
        n = len(bolds)
        ptrs = (C.c_void_p * n)(*[b.data_ptr() for b in bolds])
        Ns = (C.c_int32 * n)(*[b.shape[1] for b in bolds])
        Ts = (C.c_int32 * n)(*[b.shape[0] for b in bolds])
        o = _opts(mode, value, precision, weighted, delta)
        outs = (L.Csr * n)()
        sts = (L.CorrStats * n)()
        _check(lib().bna_corr_csr_batch(self._h, n, ptrs, Ns, Ts, C.byref(o), outs, sts,
                                        self._stream(stream)), self._h)
        res = []
        for k in range(n):
            dev = bolds[k].device
            N = bolds[k].shape[1]
            rp = _view(outs[k].row_ptr, N + 1, "<i4", torch, dev)
            ci = _view(outs[k].col_idx, outs[k].nnz, "<i4", torch, dev)
            va = _view(outs[k].val, outs[k].nnz, "<f4", torch, dev) if outs[k].val else None
            if copy:
                rp, ci = rp.clone(), ci.clone()
                va = va.clone() if va is not None else None
            res.append(CsrResult(N, int(outs[k].nnz), rp, ci, va, sts[k].as_dict()))
        return res

    def corr_csr_avg(self, bolds, mode: str = "r_gt", value: float = 0.5,
                     precision: str = "bf16x3", fisher: bool = False, weighted: bool = True,
                     delta: Optional[float] = None, stream=None, copy: bool = True) -> CsrResult:
        """Multi-subject average (to_average y/b, optional Fisher z) -> thresholded
        CSR.  bolds: torch CUDA float32 [T_k][N] tensors, same N."""
        import torch
        N = bolds[0].shape[1]
        assert all(b.is_cuda and b.dtype == torch.float32 and b.is_contiguous() and
                   b.shape[1] == N for b in bolds)
        ptrs = (C.c_void_p * len(bolds))(*[b.data_ptr() for b in bolds])
        Ts = (C.c_int32 * len(bolds))(*[b.shape[0] for b in bolds])
        o = _opts(mode, value, precision, weighted, delta)
        out = L.Csr()
        st = L.CorrStats()
        _check(lib().bna_corr_csr_avg(self._h, len(bolds), ptrs, N, Ts, 1 if fisher else 0,
                                      C.byref(o), C.byref(out), C.byref(st),
                                      self._stream(stream)), self._h)
        dev = bolds[0].device
        rp = _view(out.row_ptr, N + 1, "<i4", torch, dev)
        ci = _view(out.col_idx, out.nnz, "<i4", torch, dev)
        va = _view(out.val, out.nnz, "<f4", torch, dev) if out.val else None
        if copy:
            rp, ci = rp.clone(), ci.clone()
            va = va.clone() if va is not None else None
        return CsrResult(N, int(out.nnz), rp, ci, va, st.as_dict())

    def rethreshold(self, csr: CsrResult, mode: str, value: float, stream=None,
                    copy: bool = True) -> CsrResult:
        """CSR at a higher threshold of the same rule, derived from `csr` (the
        weighted device CSR of this context's last corr_csr) without another
        correlation pass (bna_csr_rethreshold)."""
        import torch
        c = L.Csr(n=csr.n, nnz=csr.nnz, row_ptr=csr.row_ptr.data_ptr(),
                  col_idx=csr.col_idx.data_ptr() if csr.nnz else None,
                  val=csr.val.data_ptr() if csr.val is not None and csr.nnz else None)
        out = L.Csr()
        band = C.c_int64()
        _check(lib().bna_csr_rethreshold(self._h, C.byref(c), L.THR_MODES[mode], float(value),
                                         C.byref(out), C.byref(band), self._stream(stream)),
               self._h)
        dev = csr.row_ptr.device
        rp = _view(out.row_ptr, csr.n + 1, "<i4", torch, dev)
        ci = _view(out.col_idx, out.nnz, "<i4", torch, dev)
        va = _view(out.val, out.nnz, "<f4", torch, dev)
        if copy:
            rp, ci, va = rp.clone(), ci.clone(), va.clone()
        return CsrResult(csr.n, int(out.nnz), rp, ci, va, {"band_1e6": band.value})

    def corr_csr_host(self, bold: np.ndarray, mode: str = "r_gt", value: float = 0.5,
                      precision: str = "fp32", weighted: bool = True,
                      delta: Optional[float] = None) -> CsrResult:
        """Host-buffer form: numpy float32 [T][N] in, numpy CSR out."""
        bold = np.ascontiguousarray(bold, dtype=np.float32)
        T, N = bold.shape
        o = _opts(mode, value, precision, weighted, delta)
        out = L.Csr()
        st = L.CorrStats()
        _check(lib().bna_corr_csr_host(self._h, bold.ctypes.data, N, T, C.byref(o), C.byref(out),
                                       C.byref(st)), self._h)
        try:
            rp = np.ctypeslib.as_array(C.cast(out.row_ptr, C.POINTER(C.c_int32)), (N + 1,)).copy()
            nnz = int(out.nnz)
            ci = (np.ctypeslib.as_array(C.cast(out.col_idx, C.POINTER(C.c_int32)), (nnz,)).copy()
                  if nnz else np.zeros(0, np.int32))
            va = None
            if out.val:
                va = (np.ctypeslib.as_array(C.cast(out.val, C.POINTER(C.c_float)), (nnz,)).copy()
                      if nnz else np.zeros(0, np.float32))
        finally:
            lib().bna_csr_free_host(C.byref(out))
        return CsrResult(N, nnz, rp, ci, va, st.as_dict())

    def corr_csr_host_into(self, bold: np.ndarray, row_ptr: np.ndarray, col_idx: np.ndarray,
                           val: Optional[np.ndarray], mode: str = "r_gt", value: float = 0.5,
                           precision: str = "fp32", delta: Optional[float] = None):
        """Host form into caller-owned buffers (pinned numpy views make it fast).

        Returns (nnz, stats); raises BnaError(13) when col_idx / val are too small."""
        assert bold.dtype == np.float32 and bold.flags.c_contiguous
        T, N = bold.shape
        assert row_ptr.dtype == np.int32 and len(row_ptr) >= N + 1
        o = _opts(mode, value, precision, val is not None, delta)
        nnz = C.c_int64()
        st = L.CorrStats()
        _check(lib().bna_corr_csr_host_into(
            self._h, bold.ctypes.data, N, T, C.byref(o), row_ptr.ctypes.data,
            col_idx.ctypes.data if len(col_idx) else None,
            val.ctypes.data if val is not None and len(val) else None, len(col_idx),
            C.byref(nnz), C.byref(st)), self._h)
        return int(nnz.value), st.as_dict()

    def tile_values(self, bold, I: int, J: int, precision: str = "fp32", stream=None):
        """Approximate r of the 128 x 128 tile (I, J) for a precision form."""
        import torch
        T, N = bold.shape
        out = torch.empty((128, 128), dtype=torch.float32, device=bold.device)
        _check(lib().bna_corr_tile_values(self._h, C.c_void_p(bold.data_ptr()), N, T,
                                          L.PRECISIONS[precision], I, J,
                                          C.c_void_p(out.data_ptr()), self._stream(stream)),
               self._h)
        return out

    def modularity(self, csr: CsrResult, lambda_min: float = 0.0, stream=None,
                   log: list | None = None):
        """Newman spectral modularity of a device CSR's binary graph ->
        (labels int32 [n] on the device, modules, Q).  With `log` (a list),
        one dict per round that held nodes is appended: round, nodes, iters
        (per Lead_Vector call), residual, lambda, divided."""
        import torch
        c = L.Csr(n=csr.n, nnz=csr.nnz, row_ptr=csr.row_ptr.data_ptr(),
                  col_idx=csr.col_idx.data_ptr() if csr.nnz else None, val=None)
        labels = torch.empty(csr.n, dtype=torch.int32, device=csr.row_ptr.device)
        m = C.c_int32()
        q = C.c_double()
        cap = 0 if log is None else 2 * csr.n + 2
        recs = (L.ModRound * max(cap, 1))()
        nrec = C.c_int32()
        _check(lib().bna_modularity(self._h, C.byref(c), float(lambda_min),
                                    C.c_void_p(labels.data_ptr()), C.byref(m), C.byref(q),
                                    recs, cap, C.byref(nrec), self._stream(stream)), self._h)
        if log is not None:
            for r in recs[:min(nrec.value, cap)]:
                log.append({"round": r.round, "nodes": r.nodes, "iters": list(r.iters),
                            "residual": list(r.residual), "lambda": r.lambda_,
                            "divided": bool(r.divided)})
        return labels, int(m.value), float(q.value)

    def ec(self, csr: CsrResult, max_iter: int = 10000, eps: float = 1e-6, stream=None):
        """Eigenvector centrality of a device CSR -> (ec float64 [n], lambda, iters, converged)."""
        import torch
        c = L.Csr(n=csr.n, nnz=csr.nnz, row_ptr=csr.row_ptr.data_ptr(),
                  col_idx=csr.col_idx.data_ptr() if csr.nnz else None,
                  val=csr.val.data_ptr() if csr.val is not None else None)
        ec = torch.empty(csr.n, dtype=torch.float64, device=csr.row_ptr.device)
        lam = C.c_double()
        it = C.c_int32()
        s = _check(lib().bna_ec(self._h, C.byref(c), max_iter, eps, C.c_void_p(ec.data_ptr()),
                                C.byref(lam), C.byref(it), self._stream(stream)), self._h,
                   ok=(L.BNA_OK, L.BNA_NOT_CONVERGED))
        return ec, lam.value, it.value, s == L.BNA_OK

    def degree(self, csr: CsrResult, stream=None):
        """Degree of every vertex of a device CSR (bna_degree): float32 [n]."""
        import torch
        c = L.Csr(n=csr.n, nnz=csr.nnz, row_ptr=csr.row_ptr.data_ptr(),
                  col_idx=csr.col_idx.data_ptr() if csr.nnz else None,
                  val=csr.val.data_ptr() if csr.val is not None and csr.nnz else None)
        deg = torch.empty(csr.n, dtype=torch.float32, device=csr.row_ptr.device)
        _check(lib().bna_degree(C.byref(c), C.c_void_p(deg.data_ptr()), self._stream(stream)))
        return deg

    def lead_vector(self, R: np.ndarray, Cc: np.ndarray, V: Optional[np.ndarray] = None):
        """Lead_Vector_GPU(R, C, V, N, ec) with host arrays -> (ec, lambda, iters, converged)."""
        R = np.ascontiguousarray(R, dtype=np.int32)
        Cc = np.ascontiguousarray(Cc, dtype=np.int32)
        Vd = None if V is None else np.ascontiguousarray(V, dtype=np.float64)
        N = len(R) - 1
        ec = np.empty(N, dtype=np.float64)
        lam = C.c_double()
        it = C.c_int32()
        s = _check(lib().bna_lead_vector(self._h, R.ctypes.data, Cc.ctypes.data if len(Cc) else None,
                                         Vd.ctypes.data if Vd is not None else None, N,
                                         ec.ctypes.data, C.byref(lam), C.byref(it)), self._h,
                   ok=(L.BNA_OK, L.BNA_NOT_CONVERGED))
        return ec, lam.value, it.value, s == L.BNA_OK


def density_nnz(N: int, percent: float) -> int:
    """Directed CSR entries of the density rule (the reference's Clength)."""
    return int(lib().bna_density_nnz(N, float(percent)))


def request_bytes(N: int, T: int, mode: str = "r_gt", value: float = 0.5,
                  precision: str = "bf16x3", weighted: bool = True, cap: int = 0,
                  ec: bool = True) -> int:
    """Device-memory estimate the server admits a request by (bna_request_bytes)."""
    o = _opts(mode, value, precision, weighted, None)
    return int(lib().bna_request_bytes(N, T, C.byref(o), cap, 1 if ec else 0))


@dataclass
class Reply:
    status: int
    tag: int
    slot: int
    nnz: int
    row_ptr: np.ndarray
    col_idx: np.ndarray
    val: Optional[np.ndarray]
    ec: Optional[np.ndarray]
    lam: float
    ec_iters: int
    ec_converged: bool
    t_submit: float
    t_start: float
    t_done: float
    t_corr: float
    stats: dict

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit


class Server:
    """bna_server: worker slots on one GPU admitting requests by HBM budget.

    submit() takes a host BOLD array [T][N] and returns a ticket; the CSR and
    centrality land in host buffers this object allocates (pinned when
    `pinned`), handed back by wait()."""

    def __init__(self, device: int = 0, slots: int = 4, hbm_budget: int = 64 << 30,
                 pinned: bool = True):
        h = C.c_void_p()
        _check(lib().bna_server_create(device, slots, int(hbm_budget), C.byref(h)))
        self._h = h
        self._pinned = pinned
        self._live = {}  # ticket -> (request struct, buffers) kept alive until wait()

    def _alloc(self, shape, dtype):
        if self._pinned:
            import torch
            tdt = {np.int32: torch.int32, np.float32: torch.float32, np.float64: torch.float64}
            t = torch.empty(shape, dtype=tdt[dtype]).pin_memory()
            return t.numpy()
        return np.empty(shape, dtype=dtype)

    def submit(self, bold: np.ndarray, mode: str = "r_gt", value: float = 0.5,
               precision: str = "bf16x3", weighted: bool = True, cap: Optional[int] = None,
               ec_max_iter: int = 10000, ec_eps: float = 1e-6, tag: int = 0,
               csr_out: bool = True, ec_out: Optional[np.ndarray] = None) -> int:
        """csr_out=False keeps the CSR on the device (only the centrality comes
        back); ec_out: caller's float64 [N] buffer for the centrality."""
        assert bold.dtype == np.float32 and bold.flags.c_contiguous
        T, N = bold.shape
        if cap is None:
            if mode == "density":
                cap = max(1, density_nnz(N, value))
            else:
                cap = max(1, N * (N - 1) // 20)  # 5 % density
        rp = self._alloc(N + 1, np.int32) if csr_out else None
        ci = self._alloc(max(cap, 1), np.int32) if csr_out else None
        va = self._alloc(max(cap, 1), np.float32) if weighted and csr_out else None
        ecv = ec_out if ec_out is not None else (
            self._alloc(N, np.float64) if ec_max_iter > 0 else None)
        r = L.Request(bold_host=bold.ctypes.data, N=N, T=T,
                      opts=_opts(mode, value, precision, weighted, None),
                      ec_max_iter=ec_max_iter, ec_eps=ec_eps,
                      row_ptr_host=rp.ctypes.data if rp is not None else None,
                      col_idx_host=ci.ctypes.data if ci is not None else None,
                      val_host=va.ctypes.data if va is not None else None,
                      cap=cap, ec_host=ecv.ctypes.data if ecv is not None else None, tag=tag)
        t = C.c_int64()
        _check(lib().bna_server_submit(self._h, C.byref(r), C.byref(t)))
        self._live[t.value] = (r, bold, rp, ci, va, ecv)
        return t.value

    def wait(self, ticket: int, timeout: float = -1.0) -> Reply:
        rep = L.Reply()
        _check(lib().bna_server_wait(self._h, ticket, float(timeout), C.byref(rep)))
        r, bold, rp, ci, va, ecv = self._live.pop(ticket)
        nnz = int(rep.nnz) if rep.status == L.BNA_OK else 0
        return Reply(status=rep.status, tag=rep.tag, slot=rep.slot, nnz=int(rep.nnz),
                     row_ptr=rp, col_idx=ci[:nnz] if ci is not None else None,
                     val=va[:nnz] if va is not None else None,
                     ec=ecv, lam=rep.lambda_, ec_iters=rep.ec_iters,
                     ec_converged=bool(rep.ec_converged), t_submit=rep.t_submit,
                     t_start=rep.t_start, t_done=rep.t_done, t_corr=rep.t_corr,
                     stats=rep.stats.as_dict())

    @property
    def device_bytes(self) -> int:
        return int(lib().bna_server_device_bytes(self._h))

    def close(self):
        if getattr(self, "_h", None):
            lib().bna_server_destroy(self._h)
            self._h = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def nifti_mask(path: str, cut: float):
    """-> (sel uint8 [total], N, dims) for the voxels with mask >= cut (bna_nifti_mask)."""
    dims = (C.c_int32 * 3)()
    total = C.c_int64()
    n = C.c_int32()
    _check(lib().bna_nifti_mask(os.fsencode(path), float(cut), dims, C.byref(total), C.byref(n),
                                None))
    sel = np.empty(total.value, np.uint8)
    _check(lib().bna_nifti_mask(os.fsencode(path), float(cut), dims, C.byref(total), C.byref(n),
                                sel.ctypes.data))
    return sel, n.value, tuple(dims)


def nifti_bold(path: str, sel: np.ndarray, N: int) -> np.ndarray:
    """Time-major float32 [T][N] series of the selected voxels (bna_nifti_bold)."""
    T = C.c_int32()
    _check(lib().bna_nifti_bold(os.fsencode(path), sel.ctypes.data, len(sel), N, None,
                                C.byref(T)))
    out = np.empty((T.value, N), np.float32)
    _check(lib().bna_nifti_bold(os.fsencode(path), sel.ctypes.data, len(sel), N,
                                out.ctypes.data, C.byref(T)))
    return out


def csr_write(path: str, row_ptr: np.ndarray, col_idx: np.ndarray,
              val: Optional[np.ndarray] = None) -> None:
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(col_idx, dtype=np.int32)
    va = None if val is None else np.ascontiguousarray(val, dtype=np.float32)
    c = L.Csr(n=len(rp) - 1, nnz=len(ci), row_ptr=rp.ctypes.data,
              col_idx=ci.ctypes.data if len(ci) else None,
              val=va.ctypes.data if va is not None else None)
    if va is not None and len(va) == 0:
        c.val = C.c_void_p(rp.ctypes.data)  # non-null marker: write an empty V section
    _check(lib().bna_csr_write(os.fsencode(path), C.byref(c)))


def csr_read(path: str):
    """-> (row_ptr, col_idx, val or None) as numpy arrays."""
    c = L.Csr()
    _check(lib().bna_csr_read(os.fsencode(path), C.byref(c)))
    try:
        n, nnz = c.n, int(c.nnz)
        rp = np.ctypeslib.as_array(C.cast(c.row_ptr, C.POINTER(C.c_int32)), (n + 1,)).copy()
        ci = (np.ctypeslib.as_array(C.cast(c.col_idx, C.POINTER(C.c_int32)), (nnz,)).copy()
              if nnz else np.zeros(0, np.int32))
        va = None
        if c.val:
            va = (np.ctypeslib.as_array(C.cast(c.val, C.POINTER(C.c_float)), (nnz,)).copy()
                  if nnz else np.zeros(0, np.float32))
    finally:
        lib().bna_csr_free_host(C.byref(c))
    return rp, ci, va


def ec_write(path: str, ec: np.ndarray) -> None:
    e = np.ascontiguousarray(ec, dtype=np.float64)
    _check(lib().bna_ec_write(os.fsencode(path), e.ctypes.data, len(e)))
