"""ctypes binding of libbna.so (the C ABI declared in include/bna.h).

The library is the product: there is no Python or CPU fallback.  If
libbna.so is missing, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libbna.so")

# enums (bna.h)
BNA_OK = 0
BNA_NOT_CONVERGED = 4
BNA_CAPACITY = 13
BNA_OVER_BUDGET = 14
OPTIONS = {"tiles_per_launch": 0, "max_nnz": 1, "ec_iters_per_launch": 2, "tile_band": 3}
THR_MODES = {"r_gt": 0, "r_ge": 1, "abs_gt": 2, "abs_ge": 3, "density": 4, "r_eps": 5}
PRECISIONS = {"fp32": 0, "bf16x3": 1, "tf32": 2, "auto": 3}
SYNTH_KINDS = {"iid": 0, "blocknet": 1}


class Csr(C.Structure):
    _fields_ = [("n", C.c_int32), ("nnz", C.c_int64), ("row_ptr", C.c_void_p),
                ("col_idx", C.c_void_p), ("val", C.c_void_p)]


class ModRound(C.Structure):
    _fields_ = [("round", C.c_int32), ("nodes", C.c_int32), ("iters", C.c_int32 * 2),
                ("residual", C.c_double * 2), ("lambda_", C.c_double), ("divided", C.c_int32),
                ("reserved", C.c_int32)]


class CorrOpts(C.Structure):
    _fields_ = [("mode", C.c_int32), ("precision", C.c_int32), ("value", C.c_double),
                ("weighted", C.c_int32), ("delta", C.c_double), ("reserved", C.c_int32 * 8)]


class CorrStats(C.Structure):
    _fields_ = [("tau", C.c_double), ("delta", C.c_double), ("nnz", C.c_int64),
                ("band_candidates", C.c_int64), ("band_edges", C.c_int64),
                ("band_1e6", C.c_int64), ("ties_dropped", C.c_int64),
                ("ms_zscore", C.c_float), ("ms_count", C.c_float), ("ms_recompute", C.c_float),
                ("ms_scan", C.c_float), ("ms_fill", C.c_float), ("ms_total", C.c_float),
                ("passes", C.c_int32), ("kernel_launches", C.c_int32),
                ("precision", C.c_int32), ("tile_band", C.c_int32),
                ("reserved", C.c_int32 * 4)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class Request(C.Structure):
    _fields_ = [("bold_host", C.c_void_p), ("N", C.c_int32), ("T", C.c_int32),
                ("opts", CorrOpts), ("ec_max_iter", C.c_int32), ("ec_eps", C.c_double),
                ("row_ptr_host", C.c_void_p), ("col_idx_host", C.c_void_p),
                ("val_host", C.c_void_p), ("cap", C.c_int64), ("ec_host", C.c_void_p),
                ("tag", C.c_int64)]


class Reply(C.Structure):
    _fields_ = [("status", C.c_int32), ("slot", C.c_int32), ("tag", C.c_int64),
                ("nnz", C.c_int64), ("lambda_", C.c_double), ("ec_iters", C.c_int32),
                ("ec_converged", C.c_int32), ("t_submit", C.c_double), ("t_start", C.c_double),
                ("t_done", C.c_double), ("t_corr", C.c_double), ("stats", CorrStats)]


class SynthParams(C.Structure):
    _fields_ = [("N", C.c_int32), ("T", C.c_int32), ("K", C.c_int32), ("kind", C.c_int32),
                ("seed", C.c_uint64), ("phi", C.c_double), ("load_sd", C.c_double),
                ("jitter_sd", C.c_double), ("block", C.c_int32), ("n_net", C.c_int32)]


# name -> (restype, argtypes); every symbol include/bna.h declares
SIGNATURES = {
    "bna_status_string": (C.c_char_p, [C.c_int32]),
    "bna_version": (C.c_char_p, []),
    "bna_ctx_create": (C.c_int32, [C.c_int32, C.POINTER(C.c_void_p)]),
    "bna_ctx_destroy": (C.c_int32, [C.c_void_p]),
    "bna_ctx_last_error": (C.c_char_p, [C.c_void_p]),
    "bna_ctx_trim": (C.c_int32, [C.c_void_p]),
    "bna_ctx_arena_bytes": (C.c_int64, [C.c_void_p]),
    "bna_zscore": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p,
                               C.c_int32, C.c_void_p]),
    "bna_zscore_ld": (C.c_int32, [C.c_int32]),
    "bna_corr_csr": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                 C.POINTER(CorrOpts), C.POINTER(Csr), C.POINTER(CorrStats),
                                 C.c_void_p]),
    "bna_corr_csr_host": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                      C.POINTER(CorrOpts), C.POINTER(Csr),
                                      C.POINTER(CorrStats)]),
    "bna_csr_free_host": (None, [C.POINTER(Csr)]),
    "bna_corr_csr_host_into": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                           C.POINTER(CorrOpts), C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_int64, C.POINTER(C.c_int64),
                                           C.POINTER(CorrStats)]),
    "bna_corr_tile_values": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                         C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "bna_ec": (C.c_int32, [C.c_void_p, C.POINTER(Csr), C.c_int32, C.c_double, C.c_void_p,
                           C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_void_p]),
    "bna_ec_noalloc": (C.c_int32, [C.POINTER(Csr), C.c_int32, C.c_double, C.c_void_p,
                                   C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_void_p]),
    "bna_lead_vector": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                    C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "bna_csr_write": (C.c_int32, [C.c_char_p, C.POINTER(Csr)]),
    "bna_csr_read": (C.c_int32, [C.c_char_p, C.POINTER(Csr)]),
    "bna_ec_write": (C.c_int32, [C.c_char_p, C.c_void_p, C.c_int32]),
    "bna_synth_bold": (C.c_int, [C.POINTER(SynthParams), C.c_void_p, C.c_int]),
    "bna_ctx_set_option": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int64]),
    "bna_ctx_set_gate": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "bna_modularity": (C.c_int32, [C.c_void_p, C.POINTER(Csr), C.c_double, C.c_void_p,
                                   C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                   C.POINTER(ModRound), C.c_int32, C.POINTER(C.c_int32),
                                   C.c_void_p]),
    "bna_modu_write": (C.c_int32, [C.c_char_p, C.c_void_p, C.c_int32]),
    "bna_server_create": (C.c_int32, [C.c_int32, C.c_int32, C.c_int64, C.POINTER(C.c_void_p)]),
    "bna_server_submit": (C.c_int32, [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_int64)]),
    "bna_server_wait": (C.c_int32, [C.c_void_p, C.c_int64, C.c_double, C.POINTER(Reply)]),
    "bna_server_device_bytes": (C.c_int64, [C.c_void_p]),
    "bna_server_destroy": (C.c_int32, [C.c_void_p]),
    "bna_density_nnz": (C.c_int64, [C.c_int32, C.c_double]),
    "bna_autotune": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(CorrOpts),
                                 C.POINTER(C.c_int32), C.c_void_p]),
    "bna_autotune_shape": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(CorrOpts),
                                       C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p]),
    "bna_corr_csr_batch": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.POINTER(CorrOpts), C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    "bna_corr_csr_avg": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                                     C.c_int32, C.POINTER(CorrOpts), C.POINTER(Csr),
                                     C.POINTER(CorrStats), C.c_void_p]),
    "bna_corr_packed": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                                    C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "bna_nifti_mask": (C.c_int32, [C.c_char_p, C.c_double, C.POINTER(C.c_int32),
                                   C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_void_p]),
    "bna_nifti_bold": (C.c_int32, [C.c_char_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p,
                                   C.POINTER(C.c_int32)]),
    "bna_degree": (C.c_int32, [C.POINTER(Csr), C.c_void_p, C.c_void_p]),
    "bna_csr_rethreshold": (C.c_int32, [C.c_void_p, C.POINTER(Csr), C.c_int32, C.c_double,
                                        C.POINTER(Csr), C.POINTER(C.c_int64), C.c_void_p]),
    "bna_request_bytes": (C.c_int64, [C.c_int32, C.c_int32, C.POINTER(CorrOpts), C.c_int64,
                                      C.c_int32]),
}

_lib = None


def lib() -> C.CDLL:
    """Load libbna.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        l = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


class BnaError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"bna status {status} ({lib().bna_status_string(status).decode()}): {msg}")
        self.status = status
