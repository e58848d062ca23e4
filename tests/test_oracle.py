"""The oracle (CPU restatement, oracle/oracle.c) pinned against the
reference's own outputs: the golden fixtures made from the reference's
compiled CPU functions, the compiled reference itself when present, and the
known-answer inputs of the reference's drivers."""
import hashlib
import os

import numpy as np
import pytest

import cuda_newest20160331_gb300 as bna
import oracle
from sparse_graphs import SPARSE_CASES, sparse_graphs, sym_csr

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = [
    ("small_c1", 4096, 240, 20, 1, "r_ge", 0.5),
    ("n300_t33_gt", 300, 33, 20, 11, "r_gt", 0.3),
    ("n129_t240_ge", 129, 240, 20, 12, "r_ge", 0.25),
    ("n1000_t64_gt", 1000, 64, 10, 13, "r_gt", 0.45),
    ("n1500_t240_dens1", 1500, 240, 20, 14, "density", 1.0),
    ("n700_t50_dens5", 700, 50, 5, 15, "density", 5.0),
]


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(GOLD, "ref_cases.npz"))


def dup_bold(gold):
    N, T = 400, 48
    b = bna.synth_bold(N, T, 8, int(gold["dupties_seed"]))
    for k in range(6):
        b[:, N - 1 - k] = b[:, 3 * k + 1]
    assert hashlib.sha256(b.tobytes()).digest() == gold["dupties_sha"].tobytes()
    return b


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_reference_golden(gold, case):
    name, N, T, K, seed, mode, value = case
    b = bna.synth_bold(N, T, K, seed)
    assert hashlib.sha256(b.tobytes()).digest() == gold[name + "_sha"].tobytes()
    z = oracle.zscore(b)
    P = oracle.cormat_packed(z)
    if mode == "density":
        tau, k, drop = oracle.density(P, N, value)
        assert np.float32(tau) == gold[name + "_tau"]
        R, C, V = oracle.threshold_csr(P, N, "r_ge", tau, drop=drop)
        assert len(C) == 2 * k
    else:
        R, C, V = oracle.threshold_csr(P, N, mode, value)
    assert np.array_equal(R, gold[name + "_R"])
    assert np.array_equal(C, gold[name + "_C"])
    assert np.array_equal(V, gold[name + "_V"])


def test_oracle_density_ties_match_reference(gold):
    b = dup_bold(gold)
    P = oracle.cormat_packed(oracle.zscore(b))
    tau, k, drop = oracle.density(P, 400, float(gold["dupties_percent"]))
    assert len(drop) == int(gold["dupties_ndrop"]) >= 1
    R, C, V = oracle.threshold_csr(P, 400, "r_ge", tau, drop=drop)
    assert np.array_equal(R, gold["dupties_R"]) and np.array_equal(C, gold["dupties_C"])
    assert len(C) == 2 * k


def test_oracle_against_compiled_reference_random_shapes():
    if oracle.ref_w() is None:
        pytest.skip("reference tree not present on this host")
    rng = np.random.default_rng(5)
    for _ in range(4):
        N = int(rng.integers(2, 260))
        T = int(rng.integers(3, 90))
        b = bna.synth_bold(N, T, 6, int(rng.integers(1, 10**6)))
        tau = float(rng.uniform(0.05, 0.6))
        R, C, V, P = oracle.ref_csr(b, "r_gt", tau)
        R2, C2, V2 = oracle.csr_corr(b, "r_gt", tau)
        assert np.array_equal(R, R2) and np.array_equal(C, C2) and np.array_equal(V, V2)


def test_ec_known_answer_4node():
    # U/cuda_EC/cuda_EC/ecGPU.cu:223-224 (binary, symmetric)
    R = np.array([0, 2, 3, 6, 8], np.int32)
    C = np.array([2, 3, 2, 0, 1, 3, 0, 2], np.int32)
    ec, lam, it, conv = oracle.ec(R, C)
    A = np.zeros((4, 4))
    for i in range(4):
        A[i, C[R[i]:R[i + 1]]] = 1
    w, v = np.linalg.eigh(A)
    assert conv and abs(lam - w[-1]) < 1e-6
    # ec is A u-hat, so ec / lambda is the unit leading eigenvector
    assert np.allclose(np.abs(ec / lam), np.abs(v[:, -1]), atol=1e-6)


def test_ec_norm_known_answer():
    # U/cuda_EC/cuda_EC_test/kernel.cu:22: ||[2,5,2,4]|| = 7 is the first
    # lambda of a power iteration started (by this definition) at u0[i] = i;
    # on a graph whose u0 = [0,1,2,...] the first lambda is ||u0||.
    R = np.array([0, 1, 2], np.int32)
    C = np.array([1, 0], np.int32)
    ec, lam, it, conv = oracle.ec(R, C, max_iter=1)
    assert it == 1 and abs(lam - 1.0) < 1e-15
    assert np.linalg.norm([2.0, 5.0, 2.0, 4.0]) == 7.0


def test_ec_matches_dense_eigenvector_weighted(gold):
    R, C, V = gold["n1000_t64_gt_R"], gold["n1000_t64_gt_C"], gold["n1000_t64_gt_V"]
    ec, lam, it, conv = oracle.ec(R, C, V.astype(np.float64))
    N = len(R) - 1
    A = np.zeros((N, N))
    for i in range(N):
        A[i, C[R[i]:R[i + 1]]] = V[R[i]:R[i + 1]]
    w, v = np.linalg.eigh(A)
    assert conv and abs(lam - w[-1]) / w[-1] < 1e-6
    assert np.max(np.abs(ec / np.linalg.norm(ec) - np.abs(v[:, -1]))) < 1e-5


def test_three_voxel_known_answers():
    T = 64
    t = np.arange(T, dtype=np.float64)
    x = np.sin(0.3 * t) + 0.1 * t
    y = np.cos(1.7 * t)
    y -= y.mean()
    xc = x - x.mean()
    y -= (y @ xc) / (xc @ xc) * xc  # orthogonal to x after centring
    b = np.stack([x, 3.0 * x + 7.0, -x, y]).T.astype(np.float32)
    z = oracle.zscore(b)
    assert abs(oracle.pair_r(z, 0, 1) - 1.0) <= 2e-7 or oracle.pair_r(z, 0, 1) == 0.0
    assert abs(oracle.pair_r(z, 0, 2) + 1.0) <= 2e-7 or oracle.pair_r(z, 0, 2) == 0.0
    assert abs(oracle.pair_r(z, 0, 3)) < 1e-5


def test_zero_variance_voxel_is_never_an_edge():
    b = bna.synth_bold(50, 40, 5, 3)
    b[:, 7] = 2.5
    z = oracle.zscore(b)
    assert np.isnan(z[7]).all()
    R, C, V = oracle.csr_corr(b, "r_gt", 0.0)
    assert 7 not in C and R[8] == R[7]


def test_float_accumulating_mt_tool_close_to_reference():
    b = bna.synth_bold(300, 120, 20, 4)
    P = oracle.cormat_mt_f32(b, 0, 300, 4)
    P2 = oracle.cormat_packed(oracle.zscore(b))
    assert np.max(np.abs(P - P2)) < 2e-5
    r = oracle.ref_u()
    if r is not None:
        out = np.zeros_like(P)
        bb = np.ascontiguousarray(b)
        r.ref_u_cormat_cpu_mt(out.ctypes.data, bb.ctypes.data, 300, 120, 4)
        assert np.array_equal(out, P)


@pytest.mark.parametrize("fisher", [0, 1])
def test_avg_accumulation_matches_reference_post_block(fisher):
    """The averaging restatement adds a subject like the reference's
    post_block with accumulation (CorMat.cpp:847-883, fishertrans :36-42),
    including values outside [-1, 1], NaN, and r = +-1 exactly."""
    r = oracle.ref_w()
    if r is None:
        pytest.skip("reference tree not present on this host")
    import cuda_newest20160331_gb300 as bna
    N, B = 300, 128
    nbk = (N + B - 1) // B
    m = N * (N - 1) // 2
    iu, ju = np.triu_indices(N, 1)
    acc_ref = np.zeros(m, np.float32)
    acc_orc = np.zeros(m, np.float32)
    for s in range(3):
        P = oracle.cormat_packed(oracle.zscore(bna.synth_bold(N, 40, 8, 90 + s)))
        P[:: 97] = 1.0
        P[5:: 211] = -1.0
        P[7:: 389] = 1.5
        P[11:: 401] = np.nan
        # the reference's blocked layout of the upper-triangle tiles
        blocked = np.zeros(nbk * (nbk + 1) // 2 * B * B, np.float32)
        br, bc = iu // B, ju // B
        off = (br * (2 * nbk - br + 1) // 2 + bc - br) * B * B
        blocked[off + (iu % B) * B + (ju % B)] = P
        r.ref_w_post_block(acc_ref.ctypes.data, blocked.ctypes.data, N, B, fisher)
        clamp = np.where((P >= -1) & (P <= 1), P, np.float32(0)).astype(np.float32)
        oracle.lib().orc_avg_accumulate(clamp.ctypes.data, m, fisher, acc_orc.ctypes.data)
    assert np.array_equal(acc_ref, acc_orc)


MOD_CASES = ["planted60", "planted300", "planted1000", "noisy500", "cliques", "small_c1"]


def _mod_graph(name):
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "modularity_ref.npz"))
    if name == "small_c1":
        ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_cases.npz"))
        return ref["small_c1_R"], ref["small_c1_C"], g
    return g[name + "_R"], g[name + "_C"], g


@pytest.mark.parametrize("name", MOD_CASES)
def test_modularity_oracle_matches_reference_labels(name):
    """The restated spectral bisection gives the reference tool's modules
    (labels recorded from its own compiled code)."""
    R, C, g = _mod_graph(name)
    labels, q, m, _ = oracle.modularity(R, C)
    assert m == int(g[name + "_modules"])
    assert np.array_equal(labels, g[name + "_labels"])
    assert 0.0 < q < 1.0


def test_modularity_known_answer_two_cliques():
    """Two 5-cliques joined by one edge: split into the cliques, Q = 2 (10/21 - 1/4)."""
    R, C, _ = _mod_graph("cliques")
    labels, q, m, _ = oracle.modularity(R, C)
    assert m == 2 and len(set(labels[:5])) == 1 and len(set(labels[5:])) == 1
    assert labels[0] != labels[5]
    assert abs(q - 2 * (10 / 21 - 0.25)) < 1e-12


def test_modularity_oracle_against_compiled_reference_random():
    if oracle.ref_m() is None:
        pytest.skip("reference tree not present on this host")
    rng = np.random.default_rng(17)
    for _ in range(3):
        n = int(rng.integers(20, 400))
        p = float(rng.uniform(0.02, 0.2))
        up = np.triu(rng.random((n, n)) < p, 1)
        adj = up | up.T
        R = np.concatenate([[0], np.cumsum(adj.sum(1))]).astype(np.int32)
        C = np.nonzero(adj)[1].astype(np.int32)
        if len(C) == 0:
            continue
        lab_r, m_r = oracle.ref_modularity(R, C)
        lab_o, _, m_o, _ = oracle.modularity(R, C)
        assert m_r == m_o and np.array_equal(lab_r, lab_o)


def test_modularity_oracle_against_compiled_reference_random_sparse():
    """Random edge lists of 0.2 to 3 edges per node (isolated nodes, pairs,
    trees and one larger component): the reference tool's labels."""
    if oracle.ref_m() is None:
        pytest.skip("reference tree not present on this host")
    rng = np.random.default_rng(2026)
    for _ in range(10):
        n = int(rng.integers(5, 700))
        m = int(rng.integers(1, max(2, int(n * rng.uniform(0.2, 3.0)))))
        R, C = sym_csr(n, [tuple(x) for x in rng.integers(0, n, (m, 2))])
        if len(C) == 0:
            continue
        lab_r, m_r = oracle.ref_modularity(R, C)
        lab_o, _, m_o, _ = oracle.modularity(R, C)
        assert m_r == m_o and np.array_equal(lab_r, lab_o), (n, m)


@pytest.mark.parametrize("name", SPARSE_CASES)
def test_modularity_oracle_against_compiled_reference_sparse(name):
    """Isolated nodes, pairs, a star, a path and a sparse random graph: the
    restated bisection gives the reference tool's own labels.  Under the
    retry's shift the entries of isolated nodes shrink far below float's range
    and must keep their sign, which the device test of the same graphs checks."""
    if oracle.ref_m() is None:
        pytest.skip("reference tree not present on this host")
    R, C = dict(sparse_graphs())[name]
    lab_r, m_r = oracle.ref_modularity(R, C)
    lab_o, _, m_o, _ = oracle.modularity(R, C)
    assert m_r == m_o and np.array_equal(lab_r, lab_o)


def test_modularity_without_edges_is_one_module():
    labels, q, m, _ = oracle.modularity(np.zeros(5, np.int32), np.zeros(0, np.int32))
    assert m == 1 and np.all(labels == 1) and np.isnan(q)


def test_2mm_rule_restatement():
    """The oracle's BNA_THR_R_EPS rule against the 2mm tools' comparison
    written out directly (CorMat-2mm.cu:13,140,156: out > (r_thresh - ep) &&
    out <= (1 + ep), ep = 1e-6 a double, the diagonal excluded) on the raw
    values: NaN never passes, a zero-variance voxel never is an edge."""
    N = 260
    b = bna.synth_bold(N, 60, 8, 71)
    b[:, 11] = 4.0
    b[:, 40] = b[:, 2] * np.float32(3.0)
    z = oracle.zscore(b)
    P = oracle.cormat_packed(z, raw=True)
    assert np.isnan(P).sum() == N - 1
    for tau in (np.float32(0.25), np.float32(-0.3), np.float32(float(np.nanmax(P)))):
        R, C, V = oracle.threshold_csr(P, N, "r_eps", float(tau))
        want = []
        for i in range(N):
            for j in range(N):
                if i == j:
                    continue
                a, c = min(i, j), max(i, j)
                r = P[a * N - (1 + a) * a // 2 + c - (a + 1)]
                if np.float64(r) > np.float64(tau) - 1e-6 and np.float64(r) <= 1.0 + 1e-6:
                    want.append(j)
        assert np.array_equal(C, want)

