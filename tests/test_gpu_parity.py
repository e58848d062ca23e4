"""Parity of the CUDA path (libbna.so through its C ABI) with the oracle and
with the reference's golden outputs.  Bar: z-scores, row_ptr and col_idx
bit-exact; val within the recompute band delta of the reference value (and
bit-exact for every pair the band recomputed); centrality within 1e-5
relative."""
import hashlib
import os

import numpy as np
import pytest

import cuda_newest20160331_gb300 as bna
import oracle
from sparse_graphs import SPARSE_CASES, random_graph as _random_graph, sparse_graphs
from sparse_graphs import sparse_hub_graph

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PRECISIONS = ["fp32", "bf16x3", "tf32"]


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def assert_csr_equal(res, R, C, V, delta, exact_vals=None):
    g = res.numpy()
    assert np.array_equal(g.row_ptr, R), "row_ptr differs"
    assert np.array_equal(g.col_idx, C), "col_idx differs"
    if V is not None:
        assert g.val is not None
        err = np.max(np.abs(g.val - V)) if len(V) else 0.0
        assert err <= delta, f"val error {err} > delta {delta}"


@pytest.mark.parametrize("precision", PRECISIONS)
def test_tile_values_within_error_bound(builder, precision):
    """max |r_form - r| over whole tiles, r = exact dot of the float z-scores;
    must sit well inside the recompute band delta."""
    N, T = 600, 240
    b = bna.synth_bold(N, T, 20, 77)
    z = oracle.zscore(b).astype(np.float64)
    res = builder.corr_csr(dev(b), mode="r_gt", value=0.5, precision=precision)
    delta = res.stats["delta"]
    worst = 0.0
    for I, J in [(0, 0), (0, 1), (1, 2), (2, 4), (3, 3), (4, 1)]:
        t = builder.tile_values(dev(b), I, J, precision=precision).cpu().numpy().astype(np.float64)
        zi = np.zeros((128, T))
        zj = np.zeros((128, T))
        ri = z[I * 128:(I + 1) * 128]
        rj = z[J * 128:(J + 1) * 128]
        zi[:len(ri)] = ri
        zj[:len(rj)] = rj
        ref = zi @ zj.T
        worst = max(worst, float(np.max(np.abs(t - ref))))
    print(f"{precision}: max |r - r_fp64| = {worst:.3e} (delta {delta:.3e})")
    assert worst <= 0.5 * delta


def test_zscore_bit_exact(builder):
    for N, T in [(1, 5), (127, 33), (300, 240), (1000, 7), (129, 1200)]:
        b = bna.synth_bold(N, T, 10, N + T)
        if N > 5:
            b[:, 3] = 1.25  # zero-variance voxel -> NaN row
        if N > 10:
            # wide dynamic range in one series (the exact integer mean sum does
            # not apply; the sequential double sum must), an offset series and
            # a series with zeros and subnormals
            rng = np.random.default_rng(T)
            b[:, 7] = (rng.standard_normal(T) * 10.0 ** rng.uniform(-8, 6, T)).astype(np.float32)
            b[:, 8] = b[:, 8] + np.float32(1000.0)
            b[::3, 9] = 0.0
            b[1::5, 9] = np.float32(1e-40)
        z = builder.zscore(dev(b)).cpu().numpy()
        ref = oracle.zscore(b)
        assert z.shape[1] >= T and not z[:, T:].any()
        assert np.array_equal(z[:, :T], ref, equal_nan=True), (N, T)


@pytest.mark.parametrize("kind", ["offset", "integer", "scaled"])
def test_zscore_bit_exact_scanner_like_series(builder, kind):
    """Scanner-like series: large baselines with small fluctuations (heavy
    cancellation in x - mean), integer-valued samples (structured values, many
    exact quotients), and per-voxel scales over many decades."""
    N, T = 4000, 300
    rng = np.random.default_rng({"offset": 11, "integer": 12, "scaled": 13}[kind])
    b = bna.synth_bold(N, T, 20, 99)
    if kind == "offset":
        b = (b * rng.uniform(0.5, 20.0, N) + rng.uniform(300.0, 3000.0, N)).astype(np.float32)
    elif kind == "integer":
        b = np.rint(b * 40.0 + rng.uniform(500.0, 1500.0, N)).astype(np.float32)
    else:
        b = (b * (10.0 ** rng.uniform(-20, 20, N))).astype(np.float32)
    z = builder.zscore(dev(b)).cpu().numpy()
    ref = oracle.zscore(b)
    assert np.array_equal(z[:, :T], ref, equal_nan=True)


def test_zscore_bit_exact_long_series(builder):
    """24 M elements of long (T = 1,200), offset series: z equals the
    reference's bit for bit."""
    N, T = 20000, 1200
    rng = np.random.default_rng(31)
    b = bna.synth_bold(N, T, 30, 31)
    b = (b * rng.uniform(1.0, 40.0, N) + rng.uniform(100.0, 5000.0, N)).astype(np.float32)
    z = builder.zscore(dev(b)).cpu().numpy()
    assert np.array_equal(z[:, :T], oracle.zscore(b), equal_nan=True)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("N,T,mode,tau", [
    (2, 10, "r_gt", -1.0), (127, 33, "r_gt", 0.3), (128, 240, "r_ge", 0.2),
    (129, 64, "abs_gt", 0.3), (300, 17, "abs_ge", 0.45), (1000, 240, "r_gt", 0.25),
    (700, 50, "r_ge", 0.0),
])
def test_corr_csr_matches_oracle(builder, precision, N, T, mode, tau):
    b = bna.synth_bold(N, T, 12, 7 * N + T)
    R, C, V = oracle.csr_corr(b, mode, tau)
    res = builder.corr_csr(dev(b), mode=mode, value=tau, precision=precision)
    assert_csr_equal(res, R, C, V, res.stats["delta"])
    assert res.nnz == len(C)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_binary_graph_and_zero_variance(builder, precision):
    b = bna.synth_bold(260, 40, 8, 99)
    b[:, 5] = 3.0
    b[:, 200] = -1.0
    R, C, V = oracle.csr_corr(b, "r_gt", 0.2, weighted=False)
    res = builder.corr_csr(dev(b), mode="r_gt", value=0.2, precision=precision, weighted=False)
    assert res.val is None
    assert_csr_equal(res, R, C, None, 0)
    # a negative threshold makes the clamped (NaN -> 0) pairs of a constant voxel edges
    R, C, V = oracle.csr_corr(b, "r_gt", -0.05)
    res = builder.corr_csr(dev(b), mode="r_gt", value=-0.05, precision=precision)
    assert_csr_equal(res, R, C, V, res.stats["delta"])


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name,N,T,K,seed,mode,value", [
    ("small_c1", 4096, 240, 20, 1, "r_ge", 0.5),
    ("n300_t33_gt", 300, 33, 20, 11, "r_gt", 0.3),
    ("n129_t240_ge", 129, 240, 20, 12, "r_ge", 0.25),
    ("n1000_t64_gt", 1000, 64, 10, 13, "r_gt", 0.45),
])
def test_corr_csr_matches_reference_golden(builder, precision, name, N, T, K, seed, mode, value):
    gold = np.load(os.path.join(GOLD, "ref_cases.npz"))
    b = bna.synth_bold(N, T, K, seed)
    assert hashlib.sha256(b.tobytes()).digest() == gold[name + "_sha"].tobytes()
    res = builder.corr_csr(dev(b), mode=mode, value=value, precision=precision)
    assert_csr_equal(res, gold[name + "_R"], gold[name + "_C"], gold[name + "_V"],
                     res.stats["delta"])


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name,N,T,K,seed,pct", [
    ("n1500_t240_dens1", 1500, 240, 20, 14, 1.0),
    ("n700_t50_dens5", 700, 50, 5, 15, 5.0),
])
def test_density_matches_reference_golden(builder, precision, name, N, T, K, seed, pct):
    """FormFullGraph_s: exactly k edges, tau* = the k-th largest r (CorMat.cpp:743-822)."""
    gold = np.load(os.path.join(GOLD, "ref_cases.npz"))
    b = bna.synth_bold(N, T, K, seed)
    res = builder.corr_csr(dev(b), mode="density", value=pct, precision=precision)
    assert np.float32(res.stats["tau"]) == gold[name + "_tau"]
    assert res.nnz == 2 * oracle.density_k(N, pct)
    assert_csr_equal(res, gold[name + "_R"], gold[name + "_C"], gold[name + "_V"],
                     res.stats["delta"])


@pytest.mark.parametrize("precision", PRECISIONS)
def test_density_drops_ties_like_reference(builder, precision):
    gold = np.load(os.path.join(GOLD, "ref_cases.npz"))
    N, T = 400, 48
    b = bna.synth_bold(N, T, 8, int(gold["dupties_seed"]))
    for k in range(6):
        b[:, N - 1 - k] = b[:, 3 * k + 1]
    res = builder.corr_csr(dev(b), mode="density", value=float(gold["dupties_percent"]),
                           precision=precision)
    assert res.stats["ties_dropped"] == int(gold["dupties_ndrop"]) >= 1
    assert np.float32(res.stats["tau"]) == gold["dupties_tau"]
    assert_csr_equal(res, gold["dupties_R"], gold["dupties_C"], gold["dupties_V"],
                     res.stats["delta"])


@pytest.mark.parametrize("precision", PRECISIONS)
def test_density_edge_cases(builder, precision):
    b = bna.synth_bold(300, 40, 8, 5)
    b[:, 11] = 2.0  # zero-variance voxel (its pairs are exact zeros)
    z = oracle.zscore(b)
    P = oracle.cormat_packed(z)
    for pct in (0.0, 0.01, 35.0, 60.0, 100.0):
        tau, k, drop = oracle.density(P, 300, pct)
        res = builder.corr_csr(dev(b), mode="density", value=pct, precision=precision)
        assert res.nnz == 2 * k, pct
        if k:
            R, C, V = oracle.threshold_csr(P, 300, "r_ge", tau, drop=drop)
            assert_csr_equal(res, R, C, V, res.stats["delta"])


def test_density_sampled_window_matches_oracle(builder):
    """Large enough for the sampled density histogram (>= 4 x 2048 tiles):
    the window comes from every s-th tile, the k-th value is selected on the
    device; the CSR must equal the oracle's for every form."""
    N, T, pct = 23100, 60, 0.8
    b = bna.synth_bold(N, T, 20, 31)
    z = oracle.zscore(b)
    P = oracle.cormat_packed(z)
    tau, k, drop = oracle.density(P, N, pct)
    R, C, V = oracle.threshold_csr(P, N, "r_ge", tau, drop=drop)
    del P
    for precision in PRECISIONS:
        res = builder.corr_csr(dev(b), mode="density", value=pct, precision=precision)
        assert res.nnz == 2 * k, precision
        assert np.float32(res.stats["tau"]) == np.float32(tau), precision
        assert_csr_equal(res, R, C, V, res.stats["delta"])


def test_density_sampled_window_miss_falls_back(builder):
    """A tight cluster of strongly correlated voxels holds more than k pairs:
    a tile sample that misses it puts the window far too low; the selection
    must detect that and rerun with the full histogram (same CSR as the plain
    FP32 form, exactly k edges)."""
    N, T, pct = 23100, 60, 0.05
    rng = np.random.default_rng(7)
    b = bna.synth_bold(N, T, 20, 32)
    base = rng.standard_normal(T).astype(np.float32)
    lo = 5000
    for i in range(lo, lo + 900):
        b[:, i] = base + np.float32(0.25) * rng.standard_normal(T).astype(np.float32)
    ref = builder.corr_csr(dev(b), mode="density", value=pct, precision="fp32").numpy()
    k = bna.density_nnz(N, pct) // 2
    assert ref.nnz == 2 * k
    for precision in ("bf16x3", "tf32"):
        res = builder.corr_csr(dev(b), mode="density", value=pct, precision=precision).numpy()
        print(precision, "passes", res.stats["passes"])
        assert res.nnz == 2 * k
        assert np.array_equal(res.row_ptr, ref.row_ptr)
        assert np.array_equal(res.col_idx, ref.col_idx)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_2mm_rule_matches_oracle(builder, precision):
    """BNA_THR_R_EPS, the 2mm / chunk GPU tools' rule (CorMat-2mm.cu:140,156,
    step2-dense2csr.cu:52): tau - 1e-6 < r <= 1 + 1e-6 in double on the raw
    value.  Thresholds at an actual r + 5e-7 (an edge here, not under r > tau),
    negative (a zero-variance voxel is never an edge, unlike post_block's 0),
    duplicated voxels (r = 1)."""
    N, T = 1100, 240
    b = bna.synth_bold(N, T, 20, 808)
    for k in range(6):
        b[:, 500 + k] = b[:, 3 * k] * np.float32(2.0) + np.float32(k)
    b[:, 33] = 1.5
    z = oracle.zscore(b)
    P = oracle.cormat_packed(z, raw=True)
    r0 = float(np.sort(P[np.isfinite(P)])[-4000])
    for tau in (np.float32(r0 + 5e-7), np.float32(0.4), np.float32(-0.2)):
        R, C, V = oracle.threshold_csr(P, N, "r_eps", float(tau))
        res = builder.corr_csr(dev(b), mode="r_eps", value=float(tau), precision=precision)
        g = res.numpy()
        assert np.array_equal(g.row_ptr, R) and np.array_equal(g.col_idx, C), tau
        assert np.max(np.abs(g.val - V)) <= res.stats["delta"]
    Rg, Cg, _ = oracle.threshold_csr(oracle.cormat_packed(z), N, "r_gt", float(np.float32(r0 + 5e-7)))
    R2, C2, _ = oracle.threshold_csr(P, N, "r_eps", float(np.float32(r0 + 5e-7)))
    assert len(C2) > len(Cg)  # the band below tau holds edges only under this rule


def test_2mm_rule_in_a_batch_and_refused_by_average(builder):
    shapes = [(1500, 100), (700, 300)]
    bolds = [dev(bna.synth_bold(N, T, 12, 900 + k)) for k, (N, T) in enumerate(shapes)]
    batch = builder.corr_csr_batch(bolds, mode="r_eps", value=0.35, precision="bf16x3")
    for k, bd in enumerate(bolds):
        R, C, V = oracle.csr_corr(bd.cpu().numpy(), "r_eps", 0.35)
        g = batch[k].numpy()
        assert np.array_equal(g.row_ptr, R) and np.array_equal(g.col_idx, C)
    with pytest.raises(bna.BnaError):
        builder.corr_csr_avg([bolds[0], bolds[0]], mode="r_eps", value=0.35)


@pytest.mark.parametrize("precision", ["bf16x3", "tf32"])
def test_tile_band_does_not_change_the_csr(precision):
    """The tensor-core tile order (bands of row blocks listed column by
    column, BNA_OPT_TILE_BAND) changes only which CTA computes which tile:
    the CSR is the same bit for bit, single builds and batches."""
    import torch
    b = dev(bna.synth_bold(5000, 200, 16, 611))
    small = dev(bna.synth_bold(1300, 90, 8, 612))
    ref = None
    with bna.Builder(0) as bl:
        for band in (1, 5, 32, 4096, 0):
            bl.set_option("tile_band", band)
            got = bl.corr_csr(b, mode="r_ge", value=0.3, precision=precision).numpy()
            bat = bl.corr_csr_batch([small, b], mode="density", value=1.5, precision=precision)
            bat = [x.numpy() for x in bat]
            if ref is None:
                ref = (got, bat)
                continue
            assert np.array_equal(got.row_ptr, ref[0].row_ptr)
            assert np.array_equal(got.col_idx, ref[0].col_idx)
            assert np.array_equal(got.val, ref[0].val), band
            for x, y in zip(bat, ref[1]):
                assert np.array_equal(x.col_idx, y.col_idx) and np.array_equal(x.val, y.val)


def _hard_series(N, T, seed):
    """Factor-model series with voxels whose products span many decades:
    spikes over a tiny background, values over 40 decades, large offsets,
    a constant voxel and a duplicated one."""
    b = bna.synth_bold(N, T, 12, seed)
    rng = np.random.default_rng(seed)
    for k in range(0, 40, 4):
        x = (rng.standard_normal(T) * 1e-7).astype(np.float32)
        x[rng.integers(T)] = 1.0
        b[:, k] = x
    for k in range(41, 60, 3):
        b[:, k] = np.exp(np.linspace(-40.0, 10.0, T) + rng.standard_normal(T)).astype(np.float32)
    for k in range(61, 80, 3):
        b[:, k] = (1e6 + rng.standard_normal(T)).astype(np.float32)
    b[:, 90] = 3.0
    b[:, 91] = b[:, 92]
    return b


@pytest.mark.parametrize("T", [240, 1200])
def test_every_pair_recomputed_is_bit_exact(builder, T):
    """A recompute band wider than the range of r makes every pair a
    candidate: every value of the CSR (r >= -2: all pairs) is then the
    exact reference value (float products, double sum in time order,
    CorMat.cpp:955-964, post_block), bit for bit, including pairs whose
    products span many decades."""
    N = 1100
    b = _hard_series(N, T, 930 + T)
    R, C, V = oracle.csr_corr(b, "r_ge", -2.0)
    res = builder.corr_csr(dev(b), mode="r_ge", value=-2.0, precision="bf16x3", delta=3.0)
    g = res.numpy()
    assert res.stats["band_candidates"] >= N * (N - 1) // 2 - N
    assert np.array_equal(g.row_ptr, R) and np.array_equal(g.col_idx, C)
    bad = np.flatnonzero(g.val.view(np.uint32) != V.view(np.uint32))
    assert len(bad) == 0, (len(bad), g.val[bad[:5]], V[bad[:5]])


def test_host_buffer_path_equals_device_path(builder):
    b = bna.synth_bold(1000, 64, 10, 13)
    h = builder.corr_csr_host(b, mode="r_gt", value=0.45)
    d = builder.corr_csr(dev(b), mode="r_gt", value=0.45).numpy()
    assert np.array_equal(h.row_ptr, d.row_ptr) and np.array_equal(h.col_idx, d.col_idx)
    assert np.array_equal(h.val, d.val)


def test_host_into_caller_buffers_and_capacity(builder):
    b = bna.synth_bold(1000, 64, 10, 13)
    d = builder.corr_csr(dev(b), mode="r_gt", value=0.45).numpy()
    rp = np.empty(1001, np.int32)
    small = np.empty(10, np.int32)
    with pytest.raises(bna.BnaError) as e:
        builder.corr_csr_host_into(b, rp, small, np.empty(10, np.float32), mode="r_gt", value=0.45)
    assert e.value.status == 13
    ci = np.empty(d.nnz, np.int32)
    va = np.empty(d.nnz, np.float32)
    nnz, st = builder.corr_csr_host_into(b, rp, ci, va, mode="r_gt", value=0.45)
    assert nnz == d.nnz and np.array_equal(rp, d.row_ptr)
    assert np.array_equal(ci, d.col_idx) and np.array_equal(va, d.val)


@pytest.mark.parametrize("mode,value,weighted", [("r_ge", 0.3, True), ("density", 2.0, True),
                                                 ("abs_ge", 0.35, False)])
def test_host_into_chunked_copies_equal_device_path(builder, mode, value, weighted):
    """The host-buffer form copies the CSR out in row-block chunks behind the
    fill pass (pinned buffers, several row blocks per chunk): same CSR as the
    device form."""
    import torch
    b = bna.synth_bold(5000, 100, 12, 17)
    d = builder.corr_csr(dev(b), mode=mode, value=value, weighted=weighted,
                         precision="bf16x3").numpy()
    pin = lambda n, dt: torch.empty(n, dtype=dt).pin_memory().numpy()
    rp = pin(5001, torch.int32)
    ci = pin(d.nnz + 100, torch.int32)
    va = pin(d.nnz + 100, torch.float32) if weighted else None
    bp = torch.from_numpy(b).pin_memory().numpy()
    nnz, st = builder.corr_csr_host_into(bp, rp, ci, va, mode=mode, value=value,
                                         precision="bf16x3")
    assert nnz == d.nnz and np.array_equal(rp, d.row_ptr)
    assert st["kernel_launches"] > 0
    assert np.array_equal(ci[:nnz], d.col_idx)
    if weighted:
        assert np.array_equal(va[:nnz], d.val)


def test_repeat_calls_are_deterministic(builder):
    b = dev(bna.synth_bold(2000, 120, 20, 5))
    r1 = builder.corr_csr(b, mode="r_gt", value=0.3).numpy()
    r2 = builder.corr_csr(b, mode="r_gt", value=0.3).numpy()
    assert np.array_equal(r1.col_idx, r2.col_idx) and np.array_equal(r1.val, r2.val)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_full_size_workload_slice(builder, precision):
    """N=45,000 x T=240 (the benchmark workload): rows of three slices equal the
    oracle; symmetry, ascending columns and no diagonal over the whole CSR."""
    import json
    w = json.load(open(os.path.join(GOLD, "workload_tau.json")))
    b = bna.synth_bold(w["N"], w["T"], w["K"], w["seed"])
    tau = w["tau_f32"]
    res = builder.corr_csr(dev(b), mode="r_ge", value=tau, precision=precision)
    g = res.numpy()
    n = w["N"]
    # about 1 % density (tau is the FP64 quantile)
    assert abs(res.nnz - 2 * w["k"]) < 0.001 * 2 * w["k"]
    rp, ci = g.row_ptr.astype(np.int64), g.col_idx
    rows = np.repeat(np.arange(n), np.diff(rp))
    assert not np.any(ci == rows)
    d = np.diff(ci)
    starts = rp[1:-1][np.diff(rp)[1:] > 0]
    ok = np.ones(len(ci), bool)
    ok[starts] = False
    assert np.all(d[ok[1:]] > 0) if len(d) else True
    key = rows.astype(np.int64) * n + ci
    tkey = ci.astype(np.int64) * n + rows
    assert np.array_equal(np.sort(key), np.sort(tkey))
    z = oracle.zscore(b)
    for r0, r1 in [(0, 96), (22500, 22560), (n - 70, n)]:
        R, C, V = oracle.rows_csr(z, "r_ge", tau, r0, r1)
        assert np.array_equal(g.row_ptr[r0:r1 + 1] - g.row_ptr[r0], R)
        assert np.array_equal(g.col_idx[g.row_ptr[r0]:g.row_ptr[r1]], C)
        assert np.max(np.abs(g.val[g.row_ptr[r0]:g.row_ptr[r1]] - V)) <= res.stats["delta"]


def test_ec_matches_oracle(builder):
    gold = np.load(os.path.join(GOLD, "ref_cases.npz"))
    for name in ["small_c1", "n1000_t64_gt", "n1500_t240_dens1"]:
        R, C, V = gold[name + "_R"], gold[name + "_C"], gold[name + "_V"]
        ec_o, lam_o, it_o, conv_o = oracle.ec(R, C, V.astype(np.float64))
        import torch
        csr = bna.CsrResult(len(R) - 1, len(C), dev(R), dev(C), dev(V), {})
        ec, lam, it, conv = builder.ec(csr)
        ec = ec.cpu().numpy()
        assert conv == conv_o
        assert abs(it - it_o) <= 1, (it, it_o)
        scale = np.max(np.abs(ec_o))
        assert np.max(np.abs(ec - ec_o)) <= 1e-5 * scale, name
        assert abs(lam - lam_o) <= 1e-5 * abs(lam_o)
        # binary graph (V := 1)
        ec_o, lam_o, it_o, _ = oracle.ec(R, C)
        csr = bna.CsrResult(len(R) - 1, len(C), dev(R), dev(C), None, {})
        ec, lam, it, _ = builder.ec(csr)
        assert np.max(np.abs(ec.cpu().numpy() - ec_o)) <= 1e-5 * np.max(np.abs(ec_o))


@pytest.mark.parametrize("n,unsorted", [(60000, False), (60000, True), (60001, False)])
def test_ec_large_graph_matches_oracle(builder, n, unsorted):
    """Graphs above the persistent kernel's size (per-iteration launches
    replayed from a graph), with columns ascending or not within a row: same
    iterations and values as the FP64 oracle.  Ascending columns take the
    column-chunked kernel; an odd n puts every other iterate at an 8-byte
    (not 16-byte) boundary, which its staging of the iterate must allow."""
    R, C, V = _random_graph(n, 40, 91)
    if unsorted:
        r = 777
        C[R[r]:R[r + 1]] = C[R[r]:R[r + 1]][::-1].copy()
        V[R[r]:R[r + 1]] = V[R[r]:R[r + 1]][::-1].copy()
    ec_o, lam_o, it_o, conv_o = oracle.ec(R, C, V.astype(np.float64))
    csr = bna.CsrResult(len(R) - 1, len(C), dev(R), dev(C), dev(V), {})
    ec, lam, it, conv = builder.ec(csr)
    ec = ec.cpu().numpy()
    assert conv == conv_o and it == it_o, (it, it_o)
    assert np.max(np.abs(ec - ec_o)) <= 1e-9 * np.max(np.abs(ec_o))
    assert abs(lam - lam_o) <= 1e-9 * abs(lam_o)
    ec_o, lam_o, it_o, _ = oracle.ec(R, C)
    csr = bna.CsrResult(len(R) - 1, len(C), dev(R), dev(C), None, {})
    ec, lam, it, _ = builder.ec(csr)
    assert it == it_o
    assert np.max(np.abs(ec.cpu().numpy() - ec_o)) <= 1e-9 * np.max(np.abs(ec_o))


@pytest.mark.parametrize("hub", [0, 600])
def test_ec_sparse_large_graph_matches_oracle(builder, hub):
    """Graphs above the persistent kernel's size with at most two entries per
    row on average (the graphs whose centrality converges slowly or never)
    sum their rows a thread per row; a row of 600 entries is summed by its
    warp.  300 iterations (neither side converges), weighted and binary:
    iterations, status and values against the FP64 oracle."""
    R, C, V = sparse_hub_graph(40000, 30000, hub, 17)
    assert len(C) <= 2 * (len(R) - 1)
    for vals in (V, None):
        ec_o, lam_o, it_o, conv_o = oracle.ec(R, C, None if vals is None else vals.astype(np.float64),
                                              max_iter=300)
        csr = bna.CsrResult(len(R) - 1, len(C), dev(R), dev(C),
                            None if vals is None else dev(vals), {})
        ec, lam, it, conv = builder.ec(csr, max_iter=300)
        ec = ec.cpu().numpy()
        assert conv == conv_o and it == it_o, (it, it_o)
        assert np.max(np.abs(ec - ec_o)) <= 1e-9 * np.max(np.abs(ec_o))
        assert abs(lam - lam_o) <= 1e-9 * abs(lam_o)


@pytest.mark.parametrize("n", [7, 20000])
def test_ec_of_a_graph_without_edges_matches_reference_order(builder, n):
    """No edges: the reference normalises before its SpMV, so the second
    iterate is exactly 0 (an empty row adds nothing, even of an infinite
    1 / lambda) and it stops there with lambda 0 (weighted-net.cu:154-189)."""
    R = np.zeros(n + 1, np.int32)
    ec_o, lam_o, it_o, _ = oracle.ec(R, np.zeros(0, np.int32))
    assert it_o == 2 and lam_o == 0.0 and not ec_o.any()
    csr = bna.CsrResult(n, 0, dev(R), dev(np.zeros(1, np.int32)), None, {})
    ec, lam, it, conv = builder.ec(csr)
    assert conv and it == 2 and lam == 0.0 and not ec.cpu().numpy().any()


def test_lead_vector_known_answer_4node(builder):
    R = np.array([0, 2, 3, 6, 8], np.int32)
    C = np.array([2, 3, 2, 0, 1, 3, 0, 2], np.int32)
    ec, lam, it, conv = builder.lead_vector(R, C)
    ec_o, lam_o, it_o, _ = oracle.ec(R, C)
    assert conv and abs(lam - lam_o) < 1e-9 and np.allclose(ec, ec_o, rtol=1e-9, atol=1e-12)
    ec2, lam2, _, _ = builder.lead_vector(R, C, np.full(8, 2.0))
    assert abs(lam2 - 2 * lam) < 1e-9


def test_ec_not_converged_reports_status(builder):
    R = np.array([0, 1, 2], np.int32)
    C = np.array([1, 0], np.int32)  # bipartite pair: +-1 eigenvalues, e2 -> 0 quickly
    csr = bna.CsrResult(2, 2, dev(R), dev(C), None, {})
    ec, lam, it, conv = builder.ec(csr, max_iter=1)
    ec_o, lam_o, it_o, conv_o = oracle.ec(R, C, max_iter=1)
    assert it == it_o == 1 and conv == conv_o


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("mode,taus", [("r_gt", (0.30, 0.35, 0.5)), ("r_ge", (0.32, 0.32, 0.4)),
                                       ("abs_ge", (0.3, 0.42))])
def test_rethreshold_equals_direct_build(builder, precision, mode, taus):
    """Several thresholds from one pass (the reference's threshold list):
    deriving the CSR at each higher tau from the lowest one gives the CSR a
    direct build at that tau gives (row_ptr / col_idx bit-exact)."""
    b = bna.synth_bold(3000, 150, 12, 41)
    b[:, 17] = 3.0  # zero-variance voxel
    base = builder.corr_csr(dev(b), mode=mode, value=taus[0], precision=precision)
    z = oracle.zscore(b)
    P = oracle.cormat_packed(z)
    for t in taus[1:]:
        d = builder.rethreshold(base, mode, t).numpy()
        R, C, V = oracle.threshold_csr(P, 3000, mode, t)
        assert np.array_equal(d.row_ptr, R) and np.array_equal(d.col_idx, C), (mode, t)
        assert np.max(np.abs(d.val - V)) <= base.stats["delta"]


def test_rethreshold_refuses_lower_tau_and_other_rules(builder):
    b = bna.synth_bold(500, 60, 8, 42)
    base = builder.corr_csr(dev(b), mode="r_gt", value=0.4, precision="bf16x3")
    for mode, t in [("r_gt", 0.3), ("abs_gt", 0.5)]:
        with pytest.raises(bna.BnaError) as e:
            builder.rethreshold(base, mode, t)
        assert e.value.status == 1
    dens = builder.corr_csr(dev(b), mode="density", value=2.0, precision="bf16x3")
    with pytest.raises(bna.BnaError):
        builder.rethreshold(dens, "r_gt", 0.5)


def _avg_subjects(N=1500, Ts=(120, 200, 160), seed=60):
    out = []
    for k, T in enumerate(Ts):
        b = bna.synth_bold(N, T, 15, seed + k)
        out.append(b)
    out[1][:, 5] = 1.0  # a zero-variance voxel in one subject
    return out


@pytest.mark.parametrize("precision", ["bf16x3", "tf32"])
@pytest.mark.parametrize("mode,value", [("r_gt", 0.25), ("density", 1.5)])
def test_average_matches_oracle(builder, precision, mode, value):
    """to_average y/yn: subjects' r summed in order, divided; thresholded.
    Plain average: float arithmetic only, so the CSR is bit-exact."""
    bolds = _avg_subjects()
    N = bolds[0].shape[1]
    A = oracle.avg_packed(bolds)
    res = builder.corr_csr_avg([dev(b) for b in bolds], mode=mode, value=value,
                               precision=precision)
    if mode == "density":
        tau, k, drop = oracle.density(A, N, value)
        R, C, V = oracle.threshold_csr(A, N, "r_ge", tau, drop=drop)
        assert res.nnz == 2 * k
    else:
        R, C, V = oracle.threshold_csr(A, N, mode, value)
    assert_csr_equal(res, R, C, V, res.stats["delta"])


def test_average_fisher_matches_oracle(builder):
    """to_average yf: Fisher z averaged, transformed back.  log/exp come from
    different math libraries on the two sides, so pairs within 1e-5 of tau
    may differ; every other pair must agree."""
    bolds = _avg_subjects(seed=70)
    N = bolds[0].shape[1]
    tau = 0.25
    A = oracle.avg_packed(bolds, fisher=True)
    R, C, V = oracle.threshold_csr(A, N, "r_gt", tau)
    g = builder.corr_csr_avg([dev(b) for b in bolds], mode="r_gt", value=tau, fisher=True,
                             precision="bf16x3").numpy()

    def pairs(rp, ci):
        rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
        return set(zip(rows.tolist(), ci.tolist()))
    diff = pairs(g.row_ptr, g.col_idx) ^ pairs(R, C)
    for i, j in diff:
        a, b = min(i, j), max(i, j)
        v = A[a * (2 * N - a - 1) // 2 + b - a - 1]
        assert abs(v - tau) <= 1e-5, (i, j, v)
    assert len(diff) <= 10


@pytest.mark.parametrize("precision", ["bf16x3", "tf32"])
@pytest.mark.parametrize("mode,value", [("r_ge", 0.35), ("abs_gt", 0.4), ("density", 1.2)])
def test_batch_equals_single_subject_builds(builder, precision, mode, value):
    """Subjects of different sizes in one persistent count pass: every CSR
    equals the one the single-subject path builds (bit-exact, values too)."""
    import torch
    shapes = [(1500, 100), (3100, 240), (700, 60), (5000, 180), (2222, 333)]
    bolds = [dev(bna.synth_bold(N, T, 12, 400 + k)) for k, (N, T) in enumerate(shapes)]
    bolds[1][:, 9] = 2.0  # a zero-variance voxel
    batch = builder.corr_csr_batch(bolds, mode=mode, value=value, precision=precision)
    for k, b in enumerate(bolds):
        one = builder.corr_csr(b, mode=mode, value=value, precision=precision).numpy()
        got = batch[k].numpy()
        assert got.nnz == one.nnz, k
        assert np.array_equal(got.row_ptr, one.row_ptr) and np.array_equal(got.col_idx, one.col_idx)
        assert np.array_equal(got.val, one.val), k


def test_batch_density_with_sampled_window(builder):
    import torch
    shapes = [(24000, 60), (2000, 120)]
    bolds = [dev(bna.synth_bold(N, T, 12, 500 + k)) for k, (N, T) in enumerate(shapes)]
    batch = builder.corr_csr_batch(bolds, mode="density", value=0.9, precision="bf16x3")
    for k, b in enumerate(bolds):
        one = builder.corr_csr(b, mode="density", value=0.9, precision="bf16x3").numpy()
        got = batch[k].numpy()
        assert got.nnz == one.nnz == bna.density_nnz(shapes[k][0], 0.9)
        assert np.array_equal(got.row_ptr, one.row_ptr) and np.array_equal(got.col_idx, one.col_idx)


def test_autotune_picks_a_form_and_auto_resolves(builder, tmp_path, monkeypatch):
    """The autotuner times both tensor-core forms and remembers the faster one;
    precision "auto" then builds with it (the same CSR as any form)."""
    monkeypatch.setenv("BNA_TUNE_CACHE", str(tmp_path / "tune.txt"))
    t = bna.Builder(0)
    try:
        best, ms = t.autotune(3000, 200, mode="r_gt", value=0.4)
        assert best in ("bf16x3", "tf32") and ms["bf16x3"] > 0 and ms["tf32"] > 0
        assert (ms[best] <= min(ms.values()))
        lines = (tmp_path / "tune.txt").read_text().split("\n")
        assert len([x for x in lines if x.strip()]) == 1
        b = dev(bna.synth_bold(3000, 200, 12, 77))
        auto = t.corr_csr(b, mode="r_gt", value=0.4, precision="auto").numpy()
        ref = t.corr_csr(b, mode="r_gt", value=0.4, precision="fp32").numpy()
        assert np.array_equal(auto.row_ptr, ref.row_ptr) and np.array_equal(auto.col_idx, ref.col_idx)
    finally:
        t.close()
    # a fresh context reads the choice from the cache file instead of tuning
    t2 = bna.Builder(0)
    try:
        t2.corr_csr(b, mode="r_gt", value=0.4, precision="auto")
        lines = (tmp_path / "tune.txt").read_text().split("\n")
        assert len([x for x in lines if x.strip()]) == 1
    finally:
        t2.close()


def test_autotune_shapes_listed_and_all_give_the_same_csr(tmp_path, monkeypatch):
    """bna_autotune_shape times every (form, band) shape, the cache line lists
    the chosen form and band with the six times, and every shape builds the
    same CSR (row_ptr / col_idx bit-exact; values within the forms' bands)."""
    monkeypatch.setenv("BNA_TUNE_CACHE", str(tmp_path / "tune.txt"))
    b = dev(bna.synth_bold(4000, 300, 12, 78))
    with bna.Builder(0) as t:
        (prec, band), times = t.autotune_shape(4000, 300, mode="r_ge", value=0.35)
        assert prec in ("bf16x3", "tf32") and band in bna.Builder.TUNE_BANDS
        assert len(times) == 6 and all(v > 0 for v in times.values())
        assert times[(prec, band)] == min(times.values())
        f = (tmp_path / "tune.txt").read_text().split()
        assert int(f[1]) == bna._lib.PRECISIONS[prec] and int(f[2]) == band and len(f) == 11
        ref = t.corr_csr(b, mode="r_ge", value=0.35, precision="fp32").numpy()
        for form, bd in times:
            t.set_option("tile_band", bd)
            g = t.corr_csr(b, mode="r_ge", value=0.35, precision=form).numpy()
            assert np.array_equal(g.row_ptr, ref.row_ptr) and np.array_equal(g.col_idx, ref.col_idx)
            assert np.max(np.abs(g.val - ref.val)) <= g.stats["delta"] + ref.stats["delta"]
        t.set_option("tile_band", 0)
        auto = t.corr_csr(b, mode="r_ge", value=0.35, precision="auto").numpy()
        assert np.array_equal(auto.col_idx, ref.col_idx)


MOD_CASES = ["planted60", "planted300", "planted1000", "noisy500", "cliques", "small_c1"]


@pytest.mark.parametrize("name", MOD_CASES)
def test_modularity_matches_reference_golden(builder, name):
    """Newman spectral modularity on the device: the reference tool's modules
    (labels from its own compiled code), Q as the oracle computes it."""
    g = np.load(os.path.join(GOLD, "modularity_ref.npz"))
    if name == "small_c1":
        ref = np.load(os.path.join(GOLD, "ref_cases.npz"))
        R, C = ref["small_c1_R"], ref["small_c1_C"]
    else:
        R, C = g[name + "_R"], g[name + "_C"]
    csr = bna.CsrResult(len(R) - 1, len(C), dev(R), dev(C), None, {})
    log = []
    labels, m, q = builder.modularity(csr, log=log)
    assert m == int(g[name + "_modules"])
    assert np.array_equal(labels.cpu().numpy(), g[name + "_labels"])
    log_o = []
    _, q_o, _, _ = oracle.modularity(R, C, log=log_o)
    assert abs(q - q_o) <= 1e-9 * abs(q_o)
    _same_rounds(log, log_o)


def _same_rounds(log, log_o):
    """Round records of the device run against the oracle's: the same rounds,
    node counts and decisions; power-step counts within one step of the
    oracle's (the FP64 sums run in another order) and eigenvalues within 1e-6."""
    assert len(log) == len(log_o)
    for a, b in zip(log, log_o):
        assert (a["round"], a["nodes"], a["divided"]) == (b["round"], b["nodes"], b["divided"])
        assert all(abs(x - y) <= 1 for x, y in zip(a["iters"], b["iters"])), (a, b)
        assert abs(a["lambda"] - b["lambda"]) <= 1e-6 * max(1.0, abs(b["lambda"])), (a, b)


def test_modularity_of_a_correlation_network(builder):
    """The modules of a thresholded correlation CSR (values ignored, as the
    reference tool reads only R and C) equal the oracle's."""
    b = bna.synth_bold(6000, 240, 12, 41)
    res = builder.corr_csr(dev(b), mode="r_gt", value=0.45, precision="bf16x3")
    h = res.numpy()
    log, log_o = [], []
    labels, m, q = builder.modularity(res, log=log)
    lab_o, q_o, m_o, _ = oracle.modularity(h.row_ptr, h.col_idx, log=log_o)
    assert m == m_o and np.array_equal(labels.cpu().numpy(), lab_o)
    assert abs(q - q_o) <= 1e-9 * abs(q_o)
    _same_rounds(log, log_o)


def test_modularity_without_edges(builder):
    R = np.zeros(7, np.int32)
    csr = bna.CsrResult(6, 0, dev(R), dev(np.zeros(1, np.int32)), None, {})
    labels, m, q = builder.modularity(csr)
    assert m == 1 and np.all(labels.cpu().numpy() == 1) and np.isnan(q)



@pytest.mark.parametrize("name", SPARSE_CASES)
def test_modularity_isolated_nodes_and_small_components(builder, name):
    """Graphs with isolated nodes, two-node components, a star and a path:
    groups whose iterate collapses to zero (|y| = 0 stops with a NaN
    iterate, as in the reference), two-node groups and retries with
    beta = -lambda; labels, Q and every round against the oracle."""
    R, C = dict(sparse_graphs())[name]
    csr = bna.CsrResult(len(R) - 1, len(C), dev(R), dev(C), None, {})
    log, log_o = [], []
    labels, m, q = builder.modularity(csr, log=log)
    lab_o, q_o, m_o, _ = oracle.modularity(R, C, log=log_o)
    assert m == m_o and np.array_equal(labels.cpu().numpy(), lab_o)
    assert abs(q - q_o) <= 1e-9 * abs(q_o)
    _same_rounds(log, log_o)
