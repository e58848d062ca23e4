"""Serving engine (bna_server): continuous admission of several subjects on
one GPU.  Each request's CSR and centrality must be the same whether it runs
alone or in a mix of concurrent requests (bit-exact: every reduction has a
fixed order), and the same as the single-context path; the smallest request
is also checked against the oracle."""
import numpy as np
import pytest

import cuda_newest20160331_gb300 as bna
import oracle

pytestmark = pytest.mark.gpu

# (N, T, K, seed, mode, value)
SUBJECTS = [
    (2500, 120, 15, 501, "r_ge", 0.45),
    (5000, 240, 20, 502, "density", 1.0),
    (7000, 300, 25, 503, "r_gt", 0.4),
    (3000, 180, 10, 504, "density", 0.5),
    (9000, 200, 30, 505, "r_ge", 0.35),
    (4000, 150, 20, 506, "abs_ge", 0.4),
]


def _bold(N, T, K, seed):
    return bna.synth_bold(N, T, K, seed)


def _run(server, subjects, at_once):
    tickets, out = [], []
    bolds = [_bold(N, T, K, seed) for (N, T, K, seed, _, _) in subjects]  # before any submit
    for k, (N, T, K, seed, mode, value) in enumerate(subjects):
        t = server.submit(bolds[k], mode=mode, value=value, precision="bf16x3", tag=k)
        if at_once:
            tickets.append(t)
        else:
            out.append(server.wait(t))
    for t in tickets:
        out.append(server.wait(t))
    return sorted(out, key=lambda r: r.tag)


def _same(a, b):
    assert a.status == b.status == 0
    assert a.nnz == b.nnz
    assert np.array_equal(a.row_ptr, b.row_ptr)
    assert np.array_equal(a.col_idx, b.col_idx)
    assert np.array_equal(a.val, b.val)
    assert np.array_equal(a.ec, b.ec)
    assert a.lam == b.lam and a.ec_iters == b.ec_iters


def test_results_same_alone_and_in_the_mix():
    with bna.Server(0, slots=1) as s1:
        alone = _run(s1, SUBJECTS, at_once=False)
    with bna.Server(0, slots=3) as s3:
        mixed = _run(s3, SUBJECTS, at_once=True)
        assert len({r.slot for r in mixed}) > 1, "requests did not spread over the slots"
        # overlap: some request started before another one finished
        spans = sorted((r.t_start, r.t_done) for r in mixed)
        assert any(spans[i + 1][0] < spans[i][1] for i in range(len(spans) - 1))
    for a, m in zip(alone, mixed):
        _same(a, m)


def test_server_matches_single_context_and_oracle(builder):
    import torch
    N, T, K, seed, mode, value = SUBJECTS[0]
    b = _bold(N, T, K, seed)
    with bna.Server(0, slots=2) as s:
        r = s.wait(s.submit(b, mode=mode, value=value, precision="bf16x3"))
    ref = builder.corr_csr(torch.from_numpy(b).cuda(), mode=mode, value=value,
                           precision="bf16x3").numpy()
    assert np.array_equal(r.row_ptr, ref.row_ptr)
    assert np.array_equal(r.col_idx, ref.col_idx)
    assert np.array_equal(r.val, ref.val)
    R, Cc, V = oracle.csr_corr(b, mode, value)
    assert np.array_equal(r.row_ptr, R)
    assert np.array_equal(r.col_idx, Cc)
    e, lam, it, conv = oracle.ec(R, Cc, V)
    assert conv and r.ec_converged
    assert np.max(np.abs(r.ec - e)) <= 1e-5 * np.max(np.abs(e))
    assert abs(r.lam - lam) <= 1e-5 * lam


@pytest.mark.parametrize("N,T", [(3001, 151), (20011, 601)])
def test_page_locked_input_gives_the_same_result(N, T):
    """A page-locked series is uploaded by the SMs (csrc/hostcopy.cu), a pageable
    one by the copy engine: same CSR and centrality, bit for bit (N * T * 4 not a
    multiple of 16 exercises the tail bytes; 48 MB is several 16 KB chunks per
    warp of the copy)."""
    import torch
    K, seed, mode, value = (12, 507, "r_ge", 0.35)
    b = _bold(N, T, K, seed)
    pinned = torch.from_numpy(b.copy()).pin_memory().numpy()
    with bna.Server(0, slots=1) as s:
        r_pageable = s.wait(s.submit(b, mode=mode, value=value, precision="bf16x3"))
        r_pinned = s.wait(s.submit(pinned, mode=mode, value=value, precision="bf16x3"))
    _same(r_pageable, r_pinned)


def test_capacity_and_budget_refusals():
    N, T, K, seed, mode, value = SUBJECTS[0]
    b = _bold(N, T, K, seed)
    with bna.Server(0, slots=1) as s:
        r = s.wait(s.submit(b, mode=mode, value=value, cap=10, ec_max_iter=0))
        assert r.status == bna._lib.BNA_CAPACITY and r.nnz > 10
    with bna.Server(0, slots=1, hbm_budget=1 << 20) as s:
        with pytest.raises(bna.BnaError) as e:
            s.submit(b, mode=mode, value=value)
        assert e.value.status == bna._lib.BNA_OVER_BUDGET


def test_tiles_per_launch_gives_the_same_csr(builder):
    import torch
    b = torch.from_numpy(_bold(6000, 240, 20, 507)).cuda()
    for mode, value in [("r_gt", 0.4), ("density", 0.8)]:
        whole = builder.corr_csr(b, mode=mode, value=value, precision="bf16x3").numpy()
        builder.set_option("tiles_per_launch", 37)
        try:
            parts = builder.corr_csr(b, mode=mode, value=value, precision="bf16x3").numpy()
        finally:
            builder.set_option("tiles_per_launch", 0)
        assert np.array_equal(whole.row_ptr, parts.row_ptr)
        assert np.array_equal(whole.col_idx, parts.col_idx)
        assert np.array_equal(whole.val, parts.val)


@pytest.mark.parametrize("N", [6000, 17000])
def test_launch_gate_is_called_and_changes_nothing(builder, N):
    """A launch gate sees the launches of a chunked correlation pass, of the
    chunked fill and of the centrality segments (the persistent kernel below
    16,384 vertices, graph replays above); the CSR and the centrality equal
    the ungated ones."""
    import torch
    b = torch.from_numpy(_bold(N, 240, 20, 508)).cuda()
    whole = builder.corr_csr(b, mode="r_gt", value=0.4, precision="bf16x3")
    ec0, lam0, it0, _ = builder.ec(whole)
    calls = []
    builder.set_option("tiles_per_launch", 37)
    builder.set_option("ec_iters_per_launch", 3)
    builder.set_gate(lambda stream, phase, done: calls.append((phase, done)))
    try:
        gated = builder.corr_csr(b, mode="r_gt", value=0.4, precision="bf16x3")
        n_corr = len(calls)
        ec1, lam1, it1, _ = builder.ec(gated)
    finally:
        builder.set_gate(None)
        builder.set_option("tiles_per_launch", 0)
        builder.set_option("ec_iters_per_launch", 0)
    nb = (N + 127) // 128
    ntiles = sum((nb + 1) // 2 - I // 2 for I in range(nb))
    assert n_corr >= (ntiles + 36) // 37 - 1 + min(8, nb) - 1  # correlation + fill chunks
    per = 3 if N <= 16384 else 4  # replays hold an even number of iterations
    ec_calls = calls[n_corr:]
    assert len(ec_calls) >= (it0 - 1) // per
    assert all(p == 2 for p, _ in ec_calls) and [d for _, d in ec_calls] == sorted(
        d for _, d in ec_calls)
    assert {p for p, _ in calls[:n_corr]} == {0, 1}
    w, g = whole.numpy(), gated.numpy()
    assert np.array_equal(w.row_ptr, g.row_ptr) and np.array_equal(w.col_idx, g.col_idx)
    assert np.array_equal(w.val, g.val)
    assert it1 == it0 and lam1 == lam0
    assert torch.equal(ec0, ec1)
