"""Generate the golden fixtures of tests/golden/ (run on the development host,
where the reference tree is present and oracle/_ref/ is built from it).

Outputs
  synth_sha256.json   sha256 of small synthetic inputs (pins the generator's bits)
  ref_cases.npz       CSR outputs of the reference's own CPU functions
                      (CorMat_cpu + FormFullGraph / FormFullGraph_s + FormCSRGraph,
                      W/CorMat/CUCorMat/CUCorMat/CorMat.cpp) on seeded inputs,
                      including the small workload (N=4096, T=240, r >= 0.5)
  workload_tau.json   tau of the N=45,000 x T=240 workload: the k-th largest
                      FP64 Pearson r, k = the reference's edge count for 1 %
                      density (CorMat.cpp:327-329)

Each reference output is also checked against the C restatement
(oracle/oracle.c) before it is written.  Usage:
  python tests/golden/make_golden.py [--skip-tau]
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import cuda_newest20160331_gb300 as bna  # noqa: E402  (generator only)
import oracle  # noqa: E402
import oracle.build  # noqa: E402

BLOCKNET = {"load_sd": 0.117, "jitter_sd": 0.08}

# (name, N, T, K, seed, mode, value) ; mode "density" takes value = percent
CASES = [
    ("small_c1", 4096, 240, 20, 1, "r_ge", 0.5),
    ("n300_t33_gt", 300, 33, 20, 11, "r_gt", 0.3),
    ("n129_t240_ge", 129, 240, 20, 12, "r_ge", 0.25),
    ("n1000_t64_gt", 1000, 64, 10, 13, "r_gt", 0.45),
    ("n1500_t240_dens1", 1500, 240, 20, 14, "density", 1.0),
    ("n700_t50_dens5", 700, 50, 5, 15, "density", 5.0),
]


def dup_input(N, T, seed):
    """Input with duplicated voxels (exact ties in r) whose self-pairs stay <= 1."""
    for s in range(seed, seed + 200):
        b = bna.synth_bold(N, T, 8, s)
        for k in range(6):
            b[:, N - 1 - k] = b[:, 3 * k + 1]
        z = oracle.zscore(b)
        ok = all(oracle.pair_r(z, 3 * k + 1, N - 1 - k) <= 1.0 for k in range(6))
        raw = [float(np.float32(np.sum((z[3 * k + 1].astype(np.float64) ** 2)))) for k in range(6)]
        if ok and all(r <= 1.0 for r in raw):
            return b, s
    raise RuntimeError("no seed without r > 1 on the duplicated pairs")


def check_and_pack(name, b, mode, value, out):
    T, N = b.shape
    z = oracle.zscore(b)
    P = oracle.cormat_packed(z)
    if mode == "density":
        tau_ref, R, Cc, V, Pr = oracle.ref_density_csr(b, value)
        tau, k, drop = oracle.density(P, N, value)
        R2, C2, V2 = oracle.threshold_csr(P, N, "r_ge", tau, drop=drop)
        assert tau == tau_ref, (name, tau, tau_ref)
        out[name + "_tau"] = np.float32(tau)
        out[name + "_ndrop"] = np.int64(len(drop))
    else:
        R, Cc, V, Pr = oracle.ref_csr(b, mode, value)
        R2, C2, V2 = oracle.threshold_csr(P, N, mode, value)
    assert np.array_equal(Pr, P), name
    assert np.array_equal(R, R2) and np.array_equal(Cc, C2) and np.array_equal(V, V2), name
    out[name + "_R"] = R
    out[name + "_C"] = Cc
    out[name + "_V"] = V
    print(f"{name}: N={N} T={T} nnz={len(Cc)}", flush=True)


def workload_tau(N=45000, T=240, K=40, seed=2, s_percent=1.0):
    """k-th largest FP64 r over i < j (blocked float64 GEMM, two passes)."""
    b = bna.synth_bold(N, T, K, seed).astype(np.float64)
    x = b.T - b.T.mean(axis=1, keepdims=True)
    z = x / np.sqrt((x * x).sum(axis=1, keepdims=True))
    k = oracle.density_k(N, s_percent)
    nbins = 1 << 20
    hist = np.zeros(nbins + 1, np.int64)
    blk = 1024

    def upper_blocks():
        for i0 in range(0, N, blk):
            i1 = min(N, i0 + blk)
            g = z[i0:i1] @ z[i0:].T
            m = np.triu(np.ones((i1 - i0, N - i0), bool), k=1)
            yield g[m]

    t0 = time.time()
    for v in upper_blocks():
        idx = np.clip(((v + 1.0) * 0.5 * nbins).astype(np.int64), 0, nbins)
        hist += np.bincount(idx, minlength=nbins + 1)
    above = np.cumsum(hist[::-1])[::-1]  # above[q] = count in bins >= q
    q = int(np.nonzero(above >= k)[0][-1])
    n_above = int(above[q + 1]) if q + 1 <= nbins else 0
    lo = q / nbins * 2.0 - 1.0
    hi = (q + 1) / nbins * 2.0 - 1.0
    cand = []
    for v in upper_blocks():
        idx = np.clip(((v + 1.0) * 0.5 * nbins).astype(np.int64), 0, nbins)
        cand.append(v[idx == q])
    cand = np.sort(np.concatenate(cand))[::-1]
    tau64 = float(cand[k - n_above - 1])
    print(f"workload tau: k={k} tau64={tau64!r} ({time.time() - t0:.1f}s)", flush=True)
    return {"N": N, "T": T, "K": K, "seed": seed, "density_percent": s_percent, "k": k,
            "tau_fp64": tau64, "tau_f32": float(np.float32(tau64)), "bin": [lo, hi]}


def main():
    oracle.build.build()
    assert oracle.ref_w() is not None, "reference CPU library not built (needs the reference tree)"
    pins = {}
    for (N, T, K, seed, kind) in [(500, 64, 20, 1, "iid"), (777, 33, 7, 9, "iid"),
                                  (1200, 40, 60, 3, "blocknet")]:
        x = bna.synth_bold(N, T, K, seed, kind=kind, **(BLOCKNET if kind == "blocknet" else {}))
        pins[f"{N},{T},{K},{seed},{kind}"] = hashlib.sha256(x.tobytes()).hexdigest()
    json.dump(pins, open(os.path.join(HERE, "synth_sha256.json"), "w"), indent=1)

    out = {}
    for name, N, T, K, seed, mode, value in CASES:
        b = bna.synth_bold(N, T, K, seed)
        out[name + "_sha"] = np.frombuffer(hashlib.sha256(b.tobytes()).digest(), np.uint8)
        check_and_pack(name, b, mode, value, out)
    b, s = dup_input(400, 48, 21)
    out["dupties_seed"] = np.int64(s)
    out["dupties_sha"] = np.frombuffer(hashlib.sha256(b.tobytes()).digest(), np.uint8)
    # a density whose k-th largest r is a tied value split by the cut, so that
    # FormFullGraph_s has to drop ties (CorMat.cpp:797-808); the percent goes
    # through the reference's own edge-count arithmetic, so search for one
    # whose k lands on the first of a tied pair
    P = oracle.cormat_packed(oracle.zscore(b))
    vals, counts = np.unique(P[P > 0.3], return_counts=True)
    tied = vals[counts >= 2]
    pct = None
    for v in tied[len(tied) // 2:]:
        k = int((P > v).sum()) + 1
        for scale in (1.0, 1.0 + 1e-7, 1.0 - 1e-7, 1.0 + 3e-7):
            cand = k * 100.0 / len(P) * scale
            if oracle.density_k(400, cand) == k:
                pct = cand
                break
        if pct is not None:
            break
    assert pct is not None
    out["dupties_percent"] = np.float64(pct)
    check_and_pack("dupties", b, "density", pct, out)
    assert out["dupties_ndrop"] >= 1
    np.savez_compressed(os.path.join(HERE, "ref_cases.npz"), **out)
    if "--skip-tau" not in sys.argv:
        json.dump(workload_tau(), open(os.path.join(HERE, "workload_tau.json"), "w"), indent=1)


if __name__ == "__main__":
    main()
