"""bna_ec_noalloc: centrality for callers that cannot allocate device memory
(host callbacks, allocator hooks, processes whose device memory belongs to
their own pool).  Its scratch is a fixed array inside libbna.so, so this test
calls it through the C ABI with only caller-owned buffers and checks it
against bna_ec, twice in a row (the second call must not be affected by the
first call's leftovers in the shared array).  Collected last on purpose."""
import ctypes as C
import os

import numpy as np
import pytest

import cuda_newest20160331_gb300 as bna
from cuda_newest20160331_gb300 import _lib as L

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _noalloc(csr, max_iter=10000, eps=1e-6):
    import torch
    c = L.Csr(n=csr.n, nnz=csr.nnz, row_ptr=csr.row_ptr.data_ptr(),
              col_idx=csr.col_idx.data_ptr() if csr.nnz else None,
              val=csr.val.data_ptr() if csr.val is not None else None)
    ec = torch.full((csr.n,), float("nan"), dtype=torch.float64, device="cuda")
    lam = C.c_double()
    it = C.c_int32()
    s = bna.lib().bna_ec_noalloc(C.byref(c), max_iter, eps, C.c_void_p(ec.data_ptr()),
                                 C.byref(lam), C.byref(it),
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return s, ec.cpu().numpy(), lam.value, it.value


def _csr(name):
    import torch
    g = np.load(os.path.join(GOLD, "ref_cases.npz"))
    R, Cc, V = g[name + "_R"], g[name + "_C"], g[name + "_V"]
    return bna.CsrResult(len(R) - 1, len(Cc), torch.from_numpy(R).cuda(),
                         torch.from_numpy(Cc).cuda(), torch.from_numpy(V).cuda(), {})


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    b = bna.Builder(0)
    try:
        for name in ["small_c1", "n1000_t64_gt"]:
            csr = _csr(name)
            ec_ref, lam_ref, it_ref, conv = b.ec(csr)
            ec_ref = ec_ref.cpu().numpy()
            for _ in range(2):
                s, ec, lam, it = _noalloc(csr)
                assert s == (L.BNA_OK if conv else L.BNA_NOT_CONVERGED)
                assert it == it_ref
                scale = np.max(np.abs(ec_ref))
                assert np.max(np.abs(ec - ec_ref)) <= 1e-5 * scale
                assert abs(lam - lam_ref) <= 1e-5 * abs(lam_ref)
    finally:
        b.close()


def test_noalloc_rejects_graphs_beyond_its_scratch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    n = (1 << 18) + 1
    rp = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    csr = bna.CsrResult(n, 0, rp, torch.zeros(1, dtype=torch.int32, device="cuda"), None, {})
    s, _, _, _ = _noalloc(csr)
    assert s == 12  # BNA_SCRATCH_LIMIT
