"""Small graphs with isolated nodes and tiny components, shared by the oracle
and device modularity tests: a graph of two cliques, a pair and isolated
nodes; a star beside a path; a sparse random graph of 500 nodes (many
isolated nodes, pairs and small trees)."""
import numpy as np


def sym_csr(n, edges):
    """Symmetric binary CSR (no self loops, no duplicates) of an edge list."""
    adj = [set() for _ in range(n)]
    for a, b in edges:
        if a != b:
            adj[a].add(int(b))
            adj[b].add(int(a))
    R = np.zeros(n + 1, np.int32)
    C = []
    for i in range(n):
        C += sorted(adj[i])
        R[i + 1] = len(C)
    return R, np.array(C, np.int32)


def sparse_graphs():
    e = ([(i, j) for i in range(5) for j in range(i + 1, 5)] +
         [(5 + i, 5 + j) for i in range(4) for j in range(i + 1, 4)] + [(12, 13)])
    yield "cliques_isolated", sym_csr(16, e)
    e = [(0, i) for i in range(1, 21)] + [(21 + i, 22 + i) for i in range(9)]
    yield "star_path", sym_csr(31, e)
    rng = np.random.default_rng(5)
    yield "sparse500", sym_csr(500, [tuple(x) for x in rng.integers(0, 500, (375, 2))])


SPARSE_CASES = ["cliques_isolated", "star_path", "sparse500"]


def random_graph(n, deg, seed):
    """Symmetric random graph, columns ascending per row, values in (0, 1)."""
    rng = np.random.default_rng(seed)
    i = rng.integers(0, n, n * deg // 2)
    j = rng.integers(0, n, n * deg // 2)
    keep = i != j
    i, j = i[keep], j[keep]
    w = rng.uniform(0.05, 1.0, len(i)).astype(np.float32)
    rows = np.concatenate([i, j])
    cols = np.concatenate([j, i])
    vals = np.concatenate([w, w])
    key = rows.astype(np.int64) * n + cols
    key, first = np.unique(key, return_index=True)
    rows, cols, vals = (key // n).astype(np.int32), (key % n).astype(np.int32), vals[first]
    R = np.zeros(n + 1, np.int32)
    np.add.at(R, rows + 1, 1)
    return np.cumsum(R).astype(np.int32), cols, vals


def sparse_hub_graph(n, pairs, hub, seed):
    """Symmetric graph of `pairs` random pairs plus vertex 0 joined to vertices
    1..hub (a row of `hub` entries), columns ascending, values in (0, 1)."""
    rng = np.random.default_rng(seed)
    i = np.concatenate([rng.integers(0, n, pairs), np.zeros(hub, np.int64)])
    j = np.concatenate([rng.integers(0, n, pairs), np.arange(1, hub + 1)])
    keep = i != j
    i, j = i[keep], j[keep]
    w = rng.uniform(0.05, 1.0, len(i)).astype(np.float32)
    rows = np.concatenate([i, j])
    cols = np.concatenate([j, i])
    vals = np.concatenate([w, w])
    key = rows.astype(np.int64) * n + cols
    key, first = np.unique(key, return_index=True)
    rows, cols, vals = (key // n).astype(np.int32), (key % n).astype(np.int32), vals[first]
    R = np.zeros(n + 1, np.int32)
    np.add.at(R, rows + 1, 1)
    return np.cumsum(R).astype(np.int32), cols, vals
