"""bna_ec_noalloc: centrality for callers that cannot allocate device memory
(a process whose device memory belongs to its own pool, an embedder that
fixes the library's memory at load).  Its scratch is a fixed array inside
libbna.so, so these tests call it through the C ABI with only caller-owned
buffers and check it against bna_ec and the oracle, twice in a row (the
second call must not be affected by the first call's leftovers in the shared
array), on graphs of both of its paths: one persistent launch (n <= 16,384)
and per-iteration launches (16,384 < n <= 262,144), converged and stopped at
max_iter.  Collected last on purpose."""
import ctypes as C
import os

import numpy as np
import pytest

import cuda_newest20160331_gb300 as bna
import oracle
from cuda_newest20160331_gb300 import _lib as L
from sparse_graphs import random_graph

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
            g = np.load(os.path.join(GOLD, "ref_cases.npz"))
            ec_o, lam_o, it_o, _ = oracle.ec(g[name + "_R"], g[name + "_C"],
                                             g[name + "_V"].astype(np.float64))
            for _ in range(2):
                s, ec, lam, it = _noalloc(csr)
                assert s == (L.BNA_OK if conv else L.BNA_NOT_CONVERGED)
                assert it == it_ref == it_o
                assert np.max(np.abs(ec - ec_o)) <= 1e-5 * np.max(np.abs(ec_o))
                scale = np.max(np.abs(ec_ref))
                assert np.max(np.abs(ec - ec_ref)) <= 1e-5 * scale
                assert abs(lam - lam_ref) <= 1e-5 * abs(lam_ref)
    finally:
        b.close()


def _dev_csr(R, Cc, V):
    import torch
    return bna.CsrResult(len(R) - 1, len(Cc), torch.from_numpy(R).cuda(),
                         torch.from_numpy(Cc).cuda(),
                         None if V is None else torch.from_numpy(V).cuda(), {})


@pytest.mark.parametrize("weighted", [True, False])
def test_noalloc_per_iteration_path_matches_oracle_and_bna_ec(weighted):
    """60,000 vertices: above the one-launch limit, so the per-iteration
    launches (32 per chunk, buffers chosen by launch index) run."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    R, Cc, V = random_graph(60000, 40, 91)
    Vw = V if weighted else None
    ec_o, lam_o, it_o, conv_o = oracle.ec(R, Cc, None if Vw is None else Vw.astype(np.float64))
    csr = _dev_csr(R, Cc, Vw)
    b = bna.Builder(0)
    try:
        ec_b, lam_b, it_b, conv_b = b.ec(csr)
        ec_b = ec_b.cpu().numpy()
    finally:
        b.close()
    scale = np.max(np.abs(ec_o))
    for _ in range(2):
        s, ec, lam, it = _noalloc(csr)
        assert s == (L.BNA_OK if conv_o else L.BNA_NOT_CONVERGED)
        assert it == it_o == it_b
        assert np.max(np.abs(ec - ec_o)) <= 1e-5 * scale
        # bna_ec may sum the rows in another order (its column-chunked form)
        assert np.max(np.abs(ec - ec_b)) <= 1e-12 * scale
        assert abs(lam - lam_o) <= 1e-5 * abs(lam_o) and abs(lam - lam_b) <= 1e-12 * abs(lam_b)


@pytest.mark.parametrize("n,deg,max_iter", [(60000, 6, 7), (60000, 6, 45), (3000, 4, 5)])
def test_noalloc_stops_at_max_iter_like_the_oracle(n, deg, max_iter):
    """A max_iter below convergence (these sparse graphs need 95 and 176
    iterations): BNA_NOT_CONVERGED, iters == max_iter and the output holds
    the last iterate (the oracle's, within 1e-5); 45 iterations cross the
    per-iteration path's chunks of 32 launches."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    R, Cc, V = random_graph(n, deg, 17)
    ec_o, lam_o, it_o, conv_o = oracle.ec(R, Cc, V.astype(np.float64), max_iter=max_iter)
    assert not conv_o and it_o == max_iter
    csr = _dev_csr(R, Cc, V)
    for _ in range(2):
        s, ec, lam, it = _noalloc(csr, max_iter=max_iter)
        assert s == L.BNA_NOT_CONVERGED and it == max_iter
        assert np.all(np.isfinite(ec))
        assert np.max(np.abs(ec - ec_o)) <= 1e-5 * np.max(np.abs(ec_o))
        assert abs(lam - lam_o) <= 1e-5 * abs(lam_o)


def test_noalloc_rejects_graphs_beyond_its_scratch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    n = (1 << 18) + 1
    rp = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    csr = bna.CsrResult(n, 0, rp, torch.zeros(1, dtype=torch.int32, device="cuda"), None, {})
    s, _, _, _ = _noalloc(csr)
    assert s == 12  # BNA_SCRATCH_LIMIT
