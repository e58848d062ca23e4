"""Synthetic workloads of the voxel-network builder (seeded factor-model BOLD;
no public dataset exists for this path and the reference's own fMRI data is
not distributed).  Sizes follow the reference's typical runs (N up to
~180k grey-matter voxels at 2 mm, T = 120 to 1200 volumes).

  small      N=4,096   T=240  K=20  r >= 0.5, binary CSR, then centrality
  n45k       N=45,000  T=240  K=40  1 % density: tau = the FP64 quantile
             (tests/golden/workload_tau.json), weighted CSR
  n45k_density  the same subject through the exact density rule (1 %)
  n180k      N=180,000 T=1200 K=60  block-network loadings (500-voxel blocks),
             tau = 0.4, weighted CSR, then centrality
  n40k_t1200 the same generator and rule at N=40,000 (a case small enough for
             detailed profiler captures)
  batch64    64 subjects, N uniform in [20,000, 70,000], T uniform in [150, 1200],
             seeds 1000 + s, 1 % density each, weighted CSRs, in one batch
  serving    Poisson arrivals at 4 requests/s; each request a subject with N
             log-uniform in [4,096, 180,000], T in {240, 600, 1200}, threshold
             r >= tau (tau uniform in [0.3, 0.6]) or a density uniform in
             [0.1 %, 2 %]; corr -> CSR -> centrality
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass, field

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TAU_FILE = os.path.join(ROOT, "tests", "golden", "workload_tau.json")


@dataclass
class Workload:
    name: str
    N: int
    T: int
    K: int
    seed: int
    mode: str
    value: float
    weighted: bool
    kind: str = "iid"
    synth: dict = field(default_factory=dict)

    def bold(self, threads: int = 0):
        from . import synth_bold
        return synth_bold(**self.synth_args(), threads=threads)

    def synth_args(self) -> dict:
        """Generator arguments (the same for the library's and the oracle's generator)."""
        return dict(N=self.N, T=self.T, K=self.K, seed=self.seed, kind=self.kind, **self.synth)

    def describe(self) -> str:
        rule = {"r_gt": "r > tau", "r_ge": "r >= tau", "abs_gt": "|r| > tau",
                "abs_ge": "|r| >= tau", "density": "density"}[self.mode]
        val = f"{self.value:g} %" if self.mode == "density" else f"tau={self.value:.6f}"
        return (f"{self.name}: N={self.N} T={self.T} K={self.K} {self.kind} loadings, "
                f"{rule} ({val}), {'weighted' if self.weighted else 'binary'} CSR")


def n45k_tau() -> float:
    return float(json.load(open(TAU_FILE))["tau_f32"])


def get(name: str) -> Workload:
    if name == "small":
        return Workload("small", 4096, 240, 20, 1, "r_ge", 0.5, False)
    if name == "n45k":
        return Workload("n45k", 45000, 240, 40, 2, "r_ge", n45k_tau(), True)
    if name == "n45k_density":
        return Workload("n45k_density", 45000, 240, 40, 2, "density", 1.0, True)
    if name == "n180k":
        return Workload("n180k", 180000, 1200, 60, 3, "r_ge", 0.4, True, kind="blocknet",
                        synth={"load_sd": 0.117, "jitter_sd": 0.08, "block": 500, "n_net": 60})
    if name == "n40k_t1200":  # the 180k network's generator at 40,000 voxels (profiling size)
        return Workload("n40k_t1200", 40000, 1200, 60, 3, "r_ge", 0.4, True, kind="blocknet",
                        synth={"load_sd": 0.117, "jitter_sd": 0.08, "block": 500, "n_net": 60})
    raise KeyError(name)


@dataclass
class ServeRequest:
    arrival: float   # seconds after the start of the run
    subject: int     # index into the subject pool
    mode: str
    value: float


def serving(n_requests: int, rate: float = 4.0, seed: int = 5000, pool: int = 24,
            n_min: int = 4096, n_max: int = 180000):
    """-> (subjects [(N, T, K, seed)], requests [ServeRequest]).

    Requests draw their subject from a pool of `pool` distinct seeded subjects
    (generating a fresh 180k x 1200 series per request would dominate the
    run); every request is computed from scratch."""
    import numpy as np
    rng = np.random.default_rng(seed)
    subjects = []
    for k in range(pool):
        N = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        T = int(rng.choice([240, 600, 1200]))
        subjects.append((N, T, 40, seed + 1 + k))
    t = 0.0
    reqs = []
    for _ in range(n_requests):
        t += float(rng.exponential(1.0 / rate))
        subj = int(rng.integers(pool))
        if rng.random() < 0.5:
            reqs.append(ServeRequest(t, subj, "r_ge", float(rng.uniform(0.3, 0.6))))
        else:
            reqs.append(ServeRequest(t, subj, "density", float(rng.uniform(0.1, 2.0))))
    return subjects, reqs


def batch_subjects(n: int = 64, seed: int = 1000, n_lo: int = 20000, n_hi: int = 70000,
                   t_lo: int = 150, t_hi: int = 1200):
    """-> [(N, T, K, seed)] of the batch workload (subject s uses seed + s)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(n_lo, n_hi + 1)), int(rng.integers(t_lo, t_hi + 1)), 40, seed + s)
            for s in range(n)]
