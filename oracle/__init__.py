"""ORACLE — test infrastructure only (the checker, never the product).

ctypes access to
  liboracle.so      the C restatement of the reference's CPU arithmetic (oracle.c)
  _ref/libref_w.so  the reference's own CorMat.cpp CPU functions (development host only)
  _ref/libref_u.so  the reference's own multi-threaded CPU correlation tool
  _ref/libref_m.so  the reference's own unweighted Newman modularity tool

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
MODES = {"r_gt": 0, "r_ge": 1, "abs_gt": 2, "abs_ge": 3, "r_eps": 5}

_o = None
_rw = None
_ru = None
_rm = None


def lib():
    global _o
    if _o is None:
        if not os.path.exists(_build.LIB):
            _build.build()
        o = C.CDLL(_build.LIB)
        P = C.c_void_p
        o.orc_zscore.argtypes = [P, C.c_int, C.c_int, P]
        o.orc_pair_r.argtypes = [P, C.c_int, C.c_int, C.c_int]
        o.orc_pair_r.restype = C.c_float
        o.orc_cormat_packed.argtypes = [P, C.c_int, C.c_int, P, C.c_int]
        o.orc_cormat_packed2.argtypes = [P, C.c_int, C.c_int, P, C.c_int, C.c_int]
        o.orc_pair_r_raw.argtypes = [P, C.c_int, C.c_int, C.c_int]
        o.orc_pair_r_raw.restype = C.c_float
        o.orc_threshold_csr.argtypes = [P, C.c_int, C.c_int, C.c_float, P, C.c_int64, P, P, P]
        o.orc_threshold_csr.restype = C.c_int64
        o.orc_density.argtypes = [P, C.c_int, C.c_double, C.POINTER(C.c_int64), P, C.c_int64,
                                  C.POINTER(C.c_int64)]
        o.orc_density.restype = C.c_float
        o.orc_density_k.argtypes = [C.c_int, C.c_double]
        o.orc_density_k.restype = C.c_int64
        o.orc_ec.argtypes = [P, P, P, C.c_int, C.c_int, C.c_double, P, C.POINTER(C.c_double),
                             C.POINTER(C.c_double), C.POINTER(C.c_double)]
        o.orc_ec.restype = C.c_int
        o.orc_cormat_mt_f32.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, P, C.c_int]
        o.orc_rows_csr.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, P,
                                   P, P, C.c_int]
        o.orc_rows_csr.restype = C.c_int64
        o.orc_rows_mt_f32_count.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                                            C.c_int]
        o.orc_rows_mt_f32_count.restype = C.c_int64
        o.orc_avg_accumulate.argtypes = [P, C.c_int64, C.c_int, P]
        o.orc_avg_finalize.argtypes = [P, C.c_int64, C.c_int, C.c_int]
        o.orc_modularity.argtypes = [P, P, C.c_int, C.c_double, P, C.POINTER(C.c_double),
                                     C.POINTER(C.c_int), P, C.POINTER(C.c_int)]
        o.orc_modularity.restype = C.c_int
        o.orc_synth_bold.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_double,
                                     C.c_double, C.c_double, C.c_int, C.c_int, P, C.c_int]
        o.orc_synth_bold.restype = C.c_int
        o.orc_mt_prepare.argtypes = [P, C.c_int, C.c_int, P, P]
        o.orc_mt_rows_csr.argtypes = [P, P, C.c_int, C.c_int, P, C.c_int, C.c_int, C.c_float,
                                      C.c_int, P, P, P, C.c_int64, P]
        o.orc_mt_rows_csr.restype = C.c_int64
        _o = o
    return _o


def ref_w():
    """The reference's CorMat.cpp CPU functions, or None when not built here."""
    global _rw
    if _rw is None and os.path.exists(_build.REF_W):
        r = C.CDLL(_build.REF_W)
        P = C.c_void_p
        r.ref_w_cormat_cpu.argtypes = [P, P, C.c_int, C.c_int]
        r.ref_w_form_full_graph.argtypes = [P, P, C.c_int, C.c_float]
        r.ref_w_form_full_graph.restype = C.c_longlong
        r.ref_w_form_full_graph_s.argtypes = [P, P, C.c_int, C.c_longlong]
        r.ref_w_form_full_graph_s.restype = C.c_float
        r.ref_w_form_csr_graph.argtypes = [P, P, P, P, C.c_int, P]
        r.ref_w_post_block.argtypes = [P, P, C.c_int, C.c_int, C.c_int]
        _rw = r
    return _rw


def ref_u():
    global _ru
    if _ru is None and os.path.exists(_build.REF_U):
        r = C.CDLL(_build.REF_U)
        P = C.c_void_p
        r.ref_u_cormat_cpu_mt.argtypes = [P, P, C.c_int, C.c_int, C.c_int]
        r.ref_u_cormat_cpu.argtypes = [P, P, C.c_int, C.c_int]
        r.ref_u_form_full_graph.argtypes = [P, P, C.c_int, C.c_float]
        r.ref_u_form_full_graph.restype = C.c_int
        r.ref_u_form_csr_graph.argtypes = [P, P, P, C.c_int]
        _ru = r
    return _ru


def ref_m():
    """The reference's unweighted Newman modularity tool, or None when not built here."""
    global _rm
    if _rm is None and os.path.exists(_build.REF_M):
        r = C.CDLL(_build.REF_M)
        P = C.c_void_p
        r.ref_m_partition.argtypes = [P, P, C.c_int, P]
        r.ref_m_partition.restype = C.c_int
        _rm = r
    return _rm


def modularity(R, Cc, lambda_min: float = 0.001, log: list | None = None):
    """-> (labels int32 [N], Q, modules, rounds): the restatement of the
    reference's spectral bisection (binary graph of R, C).  With `log` (a
    list), one dict per round that held nodes is appended: round, nodes,
    iters (per Lead_Vector call), lambda, divided."""
    R = np.ascontiguousarray(R, np.int32)
    Cc = np.ascontiguousarray(Cc, np.int32)
    N = len(R) - 1
    labels = np.empty(N, np.int32)
    q, rounds, nlog = C.c_double(), C.c_int(), C.c_int()
    buf = np.zeros((2 * N + 2, 6)) if log is not None else None
    m = lib().orc_modularity(_p(R), _p(Cc), N, lambda_min, _p(labels), C.byref(q),
                             C.byref(rounds), _p(buf), C.byref(nlog))
    if log is not None:
        for e in buf[:nlog.value]:
            log.append({"round": int(e[0]), "nodes": int(e[1]), "iters": [int(e[2]), int(e[3])],
                        "lambda": float(e[4]), "divided": bool(e[5])})
    return labels, q.value, m, rounds.value


def ref_modularity(R, Cc):
    """-> (labels int32 [N], modules) from the compiled reference tool."""
    R = np.ascontiguousarray(R, np.int32)
    Cc = np.ascontiguousarray(Cc, np.int32)
    labels = np.empty(len(R) - 1, np.int32)
    m = ref_m().ref_m_partition(_p(R), _p(Cc), len(R) - 1, _p(labels))
    return labels, m


def _p(a):
    return a.ctypes.data if a is not None else None


def zscore(bold: np.ndarray) -> np.ndarray:
    bold = np.ascontiguousarray(bold, np.float32)
    T, N = bold.shape
    z = np.empty((N, T), np.float32)
    lib().orc_zscore(_p(bold), N, T, _p(z))
    return z


def pair_r(z: np.ndarray, i: int, j: int) -> float:
    z = np.ascontiguousarray(z, np.float32)
    return float(lib().orc_pair_r(_p(z), z.shape[1], i, j))


def cormat_packed(z: np.ndarray, threads: int = 0, raw: bool = False) -> np.ndarray:
    """Packed upper triangle of the reference values (raw: without
    post_block's clamp, NaN for a zero-variance voxel)."""
    z = np.ascontiguousarray(z, np.float32)
    N, T = z.shape
    out = np.empty(N * (N - 1) // 2, np.float32)
    lib().orc_cormat_packed2(_p(z), N, T, _p(out), threads or (os.cpu_count() or 1),
                             1 if raw else 0)
    return out


def avg_packed(bolds, fisher: bool = False, threads: int = 0) -> np.ndarray:
    """Multi-subject average of the reference (packed, post_block accumulation
    in subject order, division, optional Fisher transforms)."""
    N = bolds[0].shape[1]
    m = N * (N - 1) // 2
    acc = np.zeros(m, np.float32)
    for b in bolds:
        P = cormat_packed(zscore(b), threads)
        lib().orc_avg_accumulate(_p(P), m, 1 if fisher else 0, _p(acc))
    lib().orc_avg_finalize(_p(acc), m, len(bolds), 1 if fisher else 0)
    return acc


def threshold_csr(packed: np.ndarray, N: int, mode: str, tau: float, drop=None,
                  weighted: bool = True):
    nd = 0 if drop is None else len(drop)
    dr = None if drop is None else np.ascontiguousarray(drop, np.uint64)
    R = np.empty(N + 1, np.int32)
    nnz = lib().orc_threshold_csr(_p(packed), N, MODES[mode], tau, _p(dr), nd, _p(R), None, None)
    Cc = np.empty(nnz, np.int32)
    V = np.empty(nnz, np.float32) if weighted else None
    lib().orc_threshold_csr(_p(packed), N, MODES[mode], tau, _p(dr), nd, _p(R), _p(Cc), _p(V))
    return R, Cc, V


def density(packed: np.ndarray, N: int, s_percent: float):
    """-> (tau, k, sorted dropped-tie keys)."""
    k = C.c_int64()
    nd = C.c_int64()
    cap = 1 << 16
    while True:
        drop = np.empty(cap, np.uint64)
        tau = lib().orc_density(_p(packed), N, s_percent, C.byref(k), _p(drop), cap, C.byref(nd))
        if nd.value >= 0:
            return float(tau), int(k.value), drop[: nd.value].copy()
        cap *= 16


def density_k(N: int, s_percent: float) -> int:
    """Undirected edge count of the density rule (CorMat.cpp:327-329 arithmetic)."""
    return int(lib().orc_density_k(N, s_percent))


def ec(R, Cc, V=None, max_iter: int = 10000, eps: float = 1e-6):
    R = np.ascontiguousarray(R, np.int32)
    Cc = np.ascontiguousarray(Cc, np.int32)
    Vd = None if V is None else np.ascontiguousarray(V, np.float64)
    N = len(R) - 1
    out = np.empty(N, np.float64)
    lam, e1, e2 = C.c_double(), C.c_double(), C.c_double()
    it = lib().orc_ec(_p(R), _p(Cc), _p(Vd), N, max_iter, eps, _p(out), C.byref(lam),
                      C.byref(e1), C.byref(e2))
    return out, lam.value, it, (e1.value <= eps or e2.value <= eps)


def rows_csr(z: np.ndarray, mode: str, tau: float, row0: int, row1: int, threads: int = 0):
    """Rows [row0, row1) of the thresholded CSR computed from z directly."""
    z = np.ascontiguousarray(z, np.float32)
    N, T = z.shape
    R = np.empty(row1 - row0 + 1, np.int32)
    th = threads or (os.cpu_count() or 1)
    nnz = lib().orc_rows_csr(_p(z), N, T, MODES[mode], tau, row0, row1, _p(R), None, None, th)
    Cc = np.empty(nnz, np.int32)
    V = np.empty(nnz, np.float32)
    lib().orc_rows_csr(_p(z), N, T, MODES[mode], tau, row0, row1, _p(R), _p(Cc), _p(V), th)
    return R, Cc, V


def cormat_mt_f32(bold: np.ndarray, row0: int, row1: int, threads: int) -> np.ndarray:
    bold = np.ascontiguousarray(bold, np.float32)
    T, N = bold.shape
    out = np.zeros(N * (N - 1) // 2, np.float32)
    lib().orc_cormat_mt_f32(_p(bold), N, T, row0, row1, _p(out), threads)
    return out


def rows_mt_f32_count(bold: np.ndarray, row0: int, row1: int, tau: float, threads: int) -> int:
    """Undirected |r| > tau edges among pairs (i in [row0,row1), j > i), reference MT arithmetic."""
    bold = np.ascontiguousarray(bold, np.float32)
    T, N = bold.shape
    return int(lib().orc_rows_mt_f32_count(_p(bold), N, T, row0, row1, tau, threads))


SYNTH_KINDS = {"iid": 0, "blocknet": 1}


def synth_bold(N: int, T: int, K: int, seed: int, kind: str = "iid", phi: float = 0.7,
               load_sd: float = 0.3, jitter_sd: float = 0.0, block: int = 500,
               n_net: int = 60, threads: int = 0) -> np.ndarray:
    """The workloads' seeded factor-model BOLD (float32 [T][N]), restated in
    C so that a CPU-only run needs nothing from the product library."""
    out = np.empty((T, N), np.float32)
    th = threads or (os.cpu_count() or 1)
    rc = lib().orc_synth_bold(N, T, K, SYNTH_KINDS[kind], seed, phi, load_sd, jitter_sd, block,
                              n_net, _p(out), th)
    if rc != 0:
        raise ValueError("bad synthetic-input parameters")
    return out


def mt_prepare(bold: np.ndarray):
    """-> (centred voxel-major rows [N][L], m2 [N]): CorMat_cpu_MT's one-time part."""
    bold = np.ascontiguousarray(bold, np.float32)
    L, N = bold.shape
    bt = np.empty((N, L), np.float32)
    m2 = np.empty(N, np.float32)
    lib().orc_mt_prepare(_p(bold), N, L, _p(bt), _p(m2))
    return bt, m2


def mt_rows_csr(bt: np.ndarray, m2: np.ndarray, rows, mode: str, tau: float, threads: int,
                weighted: bool = True):
    """The reference CPU tool's per-pair work on the pairs (i in rows, j > i):
    cross terms on `threads` threads, then its FormFullGraph / FormCSRGraph
    steps restricted to the sample.  -> (R [N+1], C, V or None, seconds of
    the three steps)."""
    N, L = bt.shape
    S = np.ascontiguousarray(np.unique(np.asarray(rows, np.int32)))
    R = np.empty(N + 1, np.int32)
    secs = np.zeros(3)
    cap = max(1 << 20, int(2 * sum(N - 1 - int(i) for i in S) * 0.02))
    while True:
        Cc = np.empty(cap, np.int32)
        V = np.empty(cap, np.float32) if weighted else None
        nnz = lib().orc_mt_rows_csr(_p(bt), _p(m2), N, L, _p(S), len(S), MODES[mode], tau,
                                    threads, _p(R), _p(Cc), _p(V), cap, _p(secs))
        if nnz >= 0:
            return R, Cc[:nnz], (V[:nnz] if weighted else None), secs
        cap = -nnz - 1


def csr_corr(bold: np.ndarray, mode: str, tau: float, weighted: bool = True, threads: int = 0):
    """Full restated path: z-score -> packed r -> CSR."""
    z = zscore(bold)
    packed = cormat_packed(z, threads, raw=(mode == "r_eps"))
    return threshold_csr(packed, bold.shape[1], mode, tau, weighted=weighted)


# ---- the reference's own functions (development host only) -----------------

def ref_csr(bold: np.ndarray, mode: str, tau: float):
    """CorMat_cpu + FormFullGraph + FormCSRGraph of the reference (W tree).

    FormFullGraph is the reference's r > tau rule; for r >= tau the value
    passed is the next float below tau (same edge set on float data)."""
    r = ref_w()
    assert r is not None, "reference CPU library not built"
    bold = np.ascontiguousarray(bold, np.float32)
    T, N = bold.shape
    M1 = N * (N - 1) // 2
    packed = np.empty(M1, np.float32)
    r.ref_w_cormat_cpu(_p(packed), _p(bold), N, T)
    adj = np.zeros(N * N, np.bool_)
    thr = np.float32(tau)
    if mode == "r_ge":
        thr = np.nextafter(thr, np.float32(-np.inf))
    elif mode != "r_gt":
        raise ValueError("the W tree implements the signed r rule only")
    clen = r.ref_w_form_full_graph(_p(adj), _p(packed), N, float(thr))
    R = np.empty(N + 1, np.int32)
    Cc = np.empty(clen, np.int32)
    V = np.empty(clen, np.float32)
    r.ref_w_form_csr_graph(_p(R), _p(Cc), _p(V), _p(adj), N, _p(packed))
    return R, Cc, V, packed


def ref_density_csr(bold: np.ndarray, s_percent: float):
    """CorMat_cpu + FormFullGraph_s + FormCSRGraph of the reference (W tree)."""
    r = ref_w()
    assert r is not None, "reference CPU library not built"
    bold = np.ascontiguousarray(bold, np.float32)
    T, N = bold.shape
    M1 = N * (N - 1) // 2
    packed = np.empty(M1, np.float32)
    r.ref_w_cormat_cpu(_p(packed), _p(bold), N, T)
    k = density_k(N, s_percent)
    clen = 2 * k
    adj = np.zeros(N * N, np.bool_)
    tau = r.ref_w_form_full_graph_s(_p(adj), _p(packed), N, k)
    R = np.empty(N + 1, np.int32)
    Cc = np.empty(clen, np.int32)
    V = np.empty(clen, np.float32)
    r.ref_w_form_csr_graph(_p(R), _p(Cc), _p(V), _p(adj), N, _p(packed))
    return float(tau), R, Cc, V, packed
