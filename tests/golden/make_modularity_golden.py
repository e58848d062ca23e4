"""Generate tests/golden/modularity_ref.npz (run on the development host,
where the reference tree is present and oracle/_ref/libref_m.so is built).

For each graph: its binary CSR (R, C) and the module labels and count that
the reference's own unweighted Newman modularity tool
(U/Newman_Modularity_CPU/Modularity_CPU/Modularity_CPU.cpp, Partition) gives
on it.  The graphs: seeded planted-partition graphs of 60 to 1,000 nodes,
two 5-cliques joined by one edge, and the binary CSR of the small workload
(ref_cases.npz small_c1, N=4096, r >= 0.5).  Each reference output is also
checked against the C restatement (oracle/oracle.c orc_modularity).
Usage:  python tests/golden/make_modularity_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
import oracle.build  # noqa: E402


def planted(n, k, p_in, p_out, seed):
    """Symmetric graph, k groups: edge probability p_in inside, p_out across."""
    rng = np.random.default_rng(seed)
    grp = rng.integers(0, k, n)
    rows, cols = [], []
    for i in range(n):
        p = np.where(grp == grp[i], p_in, p_out)
        p[i] = 0
        nb = np.nonzero(rng.random(n) < p)[0]
        nb = nb[nb > i]
        rows.append(np.full(len(nb), i))
        cols.append(nb)
    r = np.concatenate(rows + cols)
    c = np.concatenate(cols + rows)
    o = np.lexsort((c, r))
    r, c = r[o], c[o]
    R = np.zeros(n + 1, np.int64)
    np.add.at(R, r + 1, 1)
    return np.cumsum(R).astype(np.int32), c.astype(np.int32)


def two_cliques():
    edges = sorted([(i, j) for i in range(5) for j in range(5) if i != j] +
                   [(i + 5, j + 5) for i in range(5) for j in range(5) if i != j] +
                   [(4, 5), (5, 4)])
    R = np.zeros(11, np.int64)
    for a, _ in edges:
        R[a + 1] += 1
    return np.cumsum(R).astype(np.int32), np.array([b for _, b in edges], np.int32)


GRAPHS = [("planted60", (60, 2, 0.5, 0.02, 1)), ("planted300", (300, 4, 0.2, 0.01, 2)),
          ("planted1000", (1000, 6, 0.08, 0.004, 3)), ("noisy500", (500, 3, 0.05, 0.03, 4))]


def main():
    oracle.build.build()
    if oracle.ref_m() is None:
        raise SystemExit("the reference modularity tool is not built (reference tree missing)")
    out = {}
    cases = [(name, planted(*args)) for name, args in GRAPHS]
    cases.append(("cliques", two_cliques()))
    ref = np.load(os.path.join(HERE, "ref_cases.npz"))
    cases.append(("small_c1", (ref["small_c1_R"], ref["small_c1_C"])))
    for name, (R, C) in cases:
        lab_r, m_r = oracle.ref_modularity(R, C)
        lab_o, q_o, m_o, _ = oracle.modularity(R, C)
        assert m_r == m_o and np.array_equal(lab_r, lab_o), name
        if name != "small_c1":  # already in ref_cases.npz
            out[name + "_R"] = R
            out[name + "_C"] = C
        out[name + "_labels"] = lab_r
        out[name + "_modules"] = np.int32(m_r)
        print(f"{name}: N={len(R) - 1} nnz={len(C)} modules={m_r} Q={q_o:.6f}", flush=True)
    np.savez_compressed(os.path.join(HERE, "modularity_ref.npz"), **out)


if __name__ == "__main__":
    main()
