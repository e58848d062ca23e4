"""The timed CPU baseline (bench.py's reference arm and cpu_baseline): the
oracle's restatement of the reference's CPU tool on a row sample, CSR
assembly included, checked against the full restatement and the compiled
reference tool; its input comes from the oracle's copy of the generator,
bit-identical to the library's, so the arm loads nothing of the product."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import cuda_newest20160331_gb300 as bna
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

GEN_CASES = [
    dict(N=1000, T=100, K=10, seed=5),
    dict(N=777, T=33, K=0, seed=6),
    dict(N=3000, T=120, K=60, seed=3, kind="blocknet", load_sd=0.117, jitter_sd=0.08,
         block=500, n_net=60),
    dict(N=2100, T=50, K=7, seed=8, kind="blocknet", load_sd=0.2, jitter_sd=0.1, block=300,
         n_net=4),
]


@pytest.mark.parametrize("kw", GEN_CASES)
def test_oracle_generator_equals_library_generator(kw):
    a = oracle.synth_bold(**kw)
    b = bna.synth_bold(**kw)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_oracle_generator_rejects_bad_parameters():
    with pytest.raises(ValueError):
        oracle.synth_bold(100, 10, 3, 1, kind="blocknet", block=0)


@pytest.mark.parametrize("mode,tau", [("r_ge", 0.3), ("abs_gt", 0.25), ("r_gt", 0.4)])
def test_all_rows_sample_equals_full_tool(mode, tau):
    b = oracle.synth_bold(700, 50, 8, 9)
    bt, m2 = oracle.mt_prepare(b)
    R, C, V, secs = oracle.mt_rows_csr(bt, m2, range(700), mode, tau, 4)
    full = oracle.cormat_mt_f32(b, 0, 700, 4)
    R2, C2, V2 = oracle.threshold_csr(full, 700, mode, tau)
    assert np.array_equal(R, R2) and np.array_equal(C, C2)
    assert np.array_equal(V.view(np.uint32), V2.view(np.uint32))
    assert len(secs) == 3 and min(secs) >= 0


def test_row_sample_holds_exactly_the_sampled_pairs():
    N = 600
    b = oracle.synth_bold(N, 40, 6, 10)
    bt, m2 = oracle.mt_prepare(b)
    S = [0, 3, 50, 51, 400, N - 1]
    R, C, V, _ = oracle.mt_rows_csr(bt, m2, S, "r_ge", 0.3, 3)
    full = oracle.cormat_mt_f32(b, 0, N, 3)
    inS = np.zeros(N, bool)
    inS[S] = True
    ER, EC, EV = [0], [], []
    for i in range(N):
        for j in range(N):
            if i == j:
                continue
            a, c = min(i, j), max(i, j)
            if not inS[a]:
                continue
            r = full[a * N - (1 + a) * a // 2 + c - (a + 1)]
            if r >= np.float32(0.3):
                EC.append(j)
                EV.append(r)
        ER.append(len(EC))
    assert np.array_equal(R, ER) and np.array_equal(C, EC) and np.array_equal(V, EV)


def test_capacity_retry_gives_the_same_csr(monkeypatch):
    b = oracle.synth_bold(300, 30, 12, 4)
    bt, m2 = oracle.mt_prepare(b)
    R, C, V, _ = oracle.mt_rows_csr(bt, m2, range(300), "r_ge", 0.1, 2)
    # a direct call with a small capacity reports the size needed
    out_R = np.empty(301, np.int32)
    small = np.empty(5, np.int32)
    S = np.arange(300, dtype=np.int32)
    got = oracle.lib().orc_mt_rows_csr(bt.ctypes.data, m2.ctypes.data, 300, 30, S.ctypes.data,
                                       300, oracle.MODES["r_ge"], 0.1, 2, out_R.ctypes.data,
                                       small.ctypes.data, None, 5, None)
    assert got == -len(C) - 1 and len(C) > 5


def test_sample_matches_compiled_reference_tool():
    ru = oracle.ref_u()
    if ru is None:
        pytest.skip("the reference's CPU tool is compiled only where its sources are")
    N, T = 500, 60
    b = oracle.synth_bold(N, T, 10, 21)
    packed = np.zeros(N * (N - 1) // 2, np.float32)
    ru.ref_u_cormat_cpu_mt(packed.ctypes.data, b.ctypes.data, N, T, 4)
    adj = np.zeros(N * N, np.bool_)
    nnz = ru.ref_u_form_full_graph(adj.ctypes.data, packed.ctypes.data, N, 0.3)
    Rr = np.empty(N + 1, np.int32)
    Cr = np.empty(nnz, np.int32)
    ru.ref_u_form_csr_graph(Rr.ctypes.data, Cr.ctypes.data, adj.ctypes.data, N)
    bt, m2 = oracle.mt_prepare(b)
    R, C, V, _ = oracle.mt_rows_csr(bt, m2, range(N), "abs_gt", 0.3, 4)
    assert np.array_equal(R, Rr) and np.array_equal(C, Cr)


REF_ARM = r"""
import json, os, sys
sys.path.insert(0, os.environ["BENCH_ROOT"])
import bench
from cuda_newest20160331_gb300 import workloads
sys.argv = ["bench.py", "--impl", "reference", "--workload", "small", "--steps", "2",
            "--warmup", "1", "--cpu-seconds", "0.4"]
bench.run_reference(bench.parse())
maps = open("/proc/self/maps").read()
print("LOADED", json.dumps(sorted({l.split()[-1] for l in maps.splitlines()
                                   if l.rstrip().endswith(".so")})))
print("CONFIG", json.dumps(bench.bench_config(workloads.get("small"), 1)))
"""


def test_reference_arm_loads_no_product_library():
    env = dict(os.environ, BENCH_ROOT=ROOT)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    p = subprocess.run([sys.executable, "-c", REF_ARM], env=env, capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 0, p.stderr
    lines = p.stdout.splitlines()
    line = json.loads(next(l for l in lines if l.startswith("{")))
    loaded = json.loads(next(l for l in lines if l.startswith("LOADED"))[7:])
    config = json.loads(next(l for l in lines if l.startswith("CONFIG"))[7:])
    assert not any("libbna" in so for so in loaded), loaded
    assert any(so.endswith("liboracle.so") for so in loaded)
    assert line["impl"] == "reference" and line["unit"] == "edges/s" and line["value"] > 0
    assert line["config"] == config  # the GPU arm prints bench_config(w, world) too
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["cores"] >= 1
