"""The benchmark workloads follow the configurations they stand for: sizes,
factor counts, thresholds and the ranges of the batch and serving draws."""
import json
import os

import numpy as np

from cuda_newest20160331_gb300 import workloads

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_small_n45k_n180k():
    s = workloads.get("small")
    assert (s.N, s.T, s.K, s.mode, s.value, s.weighted) == (4096, 240, 20, "r_ge", 0.5, False)
    n = workloads.get("n45k")
    assert (n.N, n.T, n.K, n.mode, n.weighted) == (45000, 240, 40, "r_ge", True)
    # tau is the FP64 quantile that keeps 1 % of the pairs
    tau = json.load(open(os.path.join(GOLD, "workload_tau.json")))
    assert (tau["N"], tau["T"], tau["K"], tau["seed"]) == (n.N, n.T, n.K, n.seed)
    assert tau["density_percent"] == 1.0 and tau["k"] == round(0.01 * n.N * (n.N - 1) / 2)
    assert n.value == tau["tau_f32"] == float(np.float32(tau["tau_fp64"]))
    d = workloads.get("n45k_density")
    assert (d.N, d.T, d.K, d.seed, d.mode, d.value) == (n.N, n.T, n.K, n.seed, "density", 1.0)
    b = workloads.get("n180k")
    assert (b.N, b.T, b.K, b.mode, b.value, b.weighted) == (180000, 1200, 60, "r_ge", 0.4, True)
    assert b.kind == "blocknet" and b.synth["block"] == 500


def test_batch_subjects():
    subs = workloads.batch_subjects()
    assert len(subs) == 64
    assert all(20000 <= N <= 70000 and 150 <= T <= 1200 for N, T, _, _ in subs)
    assert len({seed for *_, seed in subs}) == 64  # each subject its own seed


def test_serving_requests():
    subjects, reqs = workloads.serving(1000)
    assert all(4096 <= N <= 180000 and T in (240, 600, 1200) for N, T, _, _ in subjects)
    t = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(t) > 0)
    assert 3.5 < len(reqs) / t[-1] < 4.5  # Poisson arrivals at 4 requests/s
    for r in reqs:
        assert 0 <= r.subject < len(subjects)
        if r.mode == "r_ge":
            assert 0.3 <= r.value <= 0.6
        else:
            assert r.mode == "density" and 0.1 <= r.value <= 2.0
    modes = [r.mode for r in reqs]
    assert 0.4 < modes.count("r_ge") / len(modes) < 0.6
