"""Benchmark of the voxel-network builder's hot path: correlation -> CSR.

One step = one pass of the path over the workload's BOLD already resident in
HBM: z-score, count pass, near-threshold recompute, offset scan, fill pass.
Default workload: the 180k-voxel network, N=180,000 voxels x T=1,200
(float32, seeded factor model, K=60 networks of contiguous 500-voxel blocks),
r >= 0.4 into a weighted CSR (about 1.6e8 directed entries), then eigenvector
centrality on the device-resident CSR.  The line also times the plain FP32
and TF32 forms on the same input and reports max |r - r_fp64| of each form.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision P]
                  [--workload n45k|small|n180k|n45k_density|batch64|serving]
                  [--impl reference]
                  [--serve-requests R]

The line's "serve" object is a serving sample: R requests (default 120) with
Poisson arrivals at 4/s through bna_server (continuous admission by HBM
budget), latency p50/p99 and each request's slowdown against running alone.
--workload serving runs the full case (R default 1,000) and prints its own line.

--gpus N > 1 runs under torchrun: every rank builds its own replica of the
workload (the path has no cross-GPU exchange: replicas only), barrier + max
over ranks; value = all ranks' edges / time.  --impl reference times the
reference's own multi-threaded CPU tool (correlation, FormFullGraph and
FormCSRGraph, restated in the oracle) on a bounded row sample of the same
workload, fed by the oracle's copy of the generator.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "corr→CSR edges/s & TFLOP/s, BF16-split vs FP32, same edge set; serving p50/p99"
L2_BYTES = 129 * 1024 * 1024


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--precision", default="bf16x3")
    p.add_argument("--no-plain", action="store_true", help="skip the plain FP32 comparison")
    p.add_argument("--workload", default="n180k")
    p.add_argument("--impl", default="gb300")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--modularity", default="auto", choices=["auto", "on", "off"],
                   help="Newman modularity of the step's CSR (auto: N <= 100,000)")
    p.add_argument("--serve-requests", type=int, default=None,
                   help="serving requests (default 120 in the line, 1,000 for --workload serving)")
    p.add_argument("--serve-slots", type=int, default=4)
    p.add_argument("--serve-budget-gb", type=float, default=160.0)
    p.add_argument("--serve-dump", default="", help="write per-request records (JSON) here")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(ms: float, world: int, device) -> float:
    """The slowest rank's step time, on every rank (ranks are replicas)."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_value(world: int, units_per_rank: float, ms: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's step time (ms)."""
    return world * units_per_rank / (ms / 1000.0)


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def sample_rows(N: int, n: int):
    """n rows spread evenly over [0, N) (their pairs j > i average N / 2)."""
    return sorted({min(N - 1, int((k + 0.5) * N / n)) for k in range(n)})


class CpuReference:
    """The reference's CPU tool on a bounded sample of the workload.

    U/CorMat/CorMat_CPU/CorMat/CorMat_CPU.cpp: CorMat_cpu_MT's cross terms
    (float accumulation, all host threads) for the pairs (i, j > i) of a set
    of rows spread over the matrix, then its FormFullGraph / FormCSRGraph
    steps (single-threaded, as in the reference) restricted to those pairs,
    with the workload's threshold rule and the pair values in the CSR (the
    weighted tree's FormCSRGraph).  Restated in the oracle's C; the one-time
    transpose and centring run once, outside the sample."""

    def __init__(self, w, bold_h, threads: int):
        import oracle
        self.w, self.threads, self.oracle = w, threads, oracle
        t0 = time.perf_counter()
        self.bt, self.m2 = oracle.mt_prepare(bold_h)
        self.prepare_s = time.perf_counter() - t0
        self.rate = None

    def run(self, n_rows: int) -> dict:
        w = self.w
        rows = sample_rows(w.N, n_rows)
        t0 = time.perf_counter()
        R, Cc, V, secs = self.oracle.mt_rows_csr(self.bt, self.m2, rows, w.mode, w.value,
                                                 self.threads, weighted=w.weighted)
        dt = time.perf_counter() - t0
        pairs = sum(w.N - 1 - i for i in rows)
        self.rate = pairs / dt
        return {"rows": len(rows), "pairs": pairs, "nnz": len(Cc), "seconds": dt,
                "step_seconds": [float(x) for x in secs]}

    def sample(self, seconds: float) -> dict:
        """One sample sized to take about `seconds` (from the last run's rate)."""
        w = self.w
        if self.rate is None:
            self.run(4)
        n = max(2, min(w.N, int(seconds * self.rate / max(1.0, (w.N - 1) / 2.0))))
        r = self.run(n)
        total = w.N * (w.N - 1) // 2
        r.update({
            "value": r["nnz"] / r["seconds"], "unit": "edges/s", "cores": self.threads,
            "kind": "port", "pairs_per_s": r["pairs"] / r["seconds"],
            "tflops": r["pairs"] * 2.0 * w.T / r["seconds"] / 1e12,
            "full_job_s_extrapolated": self.prepare_s + total * r["seconds"] / r["pairs"],
            "sample": (f"{r['rows']} rows spread over N={w.N} (pairs i<j with i in the sample: "
                       f"{r['pairs']}, {r['pairs'] / total:.3%} of all), T={w.T}; the reference "
                       f"CPU tool (CorMat_cpu_MT cross terms on {self.threads} threads, then "
                       f"FormFullGraph + FormCSRGraph on the sample's pairs, single-threaded as "
                       f"in the reference; {w.describe()}): {r['nnz']} directed CSR entries in "
                       f"{r['seconds']:.2f} s on {cpu_model()}; the one-time transpose and "
                       f"centring ({self.prepare_s:.1f} s) are outside the sample"),
        })
        return r


def bench_config(w, world: int) -> dict:
    """The config both arms print (the same dict for the same workload)."""
    return {"workload": w.describe(), "parallelism": f"replicas x{world} (no collective)",
            "l2": "inputs larger than L2 on the GPU arm (and a 2x L2 buffer zeroed between "
                  "timed steps, outside the events); host memory on the CPU arm"}


def max_abs_err(b, bold, bold_h, precision: str, n_tiles: int = 16, seed: int = 7) -> dict:
    """max |r - r_fp64| over sampled 128 x 128 tiles: the form's approximate r
    (bna_corr_tile_values) against r computed in FP64 from the float input
    (centred, L2-normalised, dotted in double); the diagonal is excluded."""
    import numpy as np
    T, N = bold_h.shape
    nb = (N + 127) // 128
    rng = np.random.default_rng(seed)
    tiles = {(0, 0), (nb - 1, nb - 1), (0, nb - 1)}
    while len(tiles) < min(n_tiles, nb * (nb + 1) // 2):
        I, J = sorted(int(x) for x in rng.integers(0, nb, 2))
        tiles.add((I, J))

    def z64(blk):
        x = bold_h[:, blk * 128:min(N, blk * 128 + 128)].astype(np.float64)
        x = x - x.mean(axis=0)
        return (x / np.sqrt((x * x).sum(axis=0))).T

    worst, pairs = 0.0, 0
    for I, J in sorted(tiles):
        v = b.tile_values(bold, I, J, precision=precision).cpu().numpy().astype(np.float64)
        zi, zj = z64(I), z64(J)
        r64 = zi @ zj.T
        d = np.abs(v[:r64.shape[0], :r64.shape[1]] - r64)
        if I == J:
            np.fill_diagonal(d, 0.0)
            pairs += r64.shape[0] * (r64.shape[0] - 1) // 2
        else:
            pairs += r64.size
        d = d[np.isfinite(d)]
        if d.size:
            worst = max(worst, float(d.max()))
    return {"value": worst, "tiles": len(tiles), "pairs": pairs,
            "sample": f"{len(tiles)} seeded 128x128 tiles ({pairs} pairs) against r in FP64 "
                      "from the float input"}


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def serve_run(n_requests: int, slots: int = 4, rate: float = 4.0, seed: int = 5000,
              budget: int = 160 << 30, dump: str = "") -> dict:
    """Poisson serving run through bna_server, then every request alone.

    The CSR of each request stays on the device (consumed by the centrality);
    the centrality vector comes back to a pinned host buffer."""
    import numpy as np
    import torch
    import cuda_newest20160331_gb300 as bna
    from cuda_newest20160331_gb300 import workloads
    subjects, reqs = workloads.serving(n_requests, rate, seed)
    pool = []
    for (N, T, K, sd) in subjects:
        b = bna.synth_bold(N, T, K, sd)
        pool.append(torch.from_numpy(b).pin_memory().numpy())
    n_max = max(N for N, _, _, _ in subjects)
    ecbufs = [torch.empty(n_max, dtype=torch.float64).pin_memory().numpy() for _ in range(64)]

    def submit(srv, k, r):
        N = subjects[r.subject][0]
        return srv.submit(pool[r.subject], mode=r.mode, value=r.value, precision="bf16x3",
                          csr_out=False, ec_out=ecbufs[k % 64][:N], tag=k)

    def one_pass(srv, timed_arrivals: bool):
        replies = [None] * len(reqs)
        lock = threading.Lock()
        tickets = []
        start = time.perf_counter()

        def feeder():
            for k, r in enumerate(reqs):
                if timed_arrivals:
                    d = r.arrival - (time.perf_counter() - start)
                    if d > 0:
                        time.sleep(d)
                t = submit(srv, k, r)
                with lock:
                    tickets.append((k, t))
                if not timed_arrivals:  # alone: wait before the next one
                    replies[k] = srv.wait(t)

        th = threading.Thread(target=feeder)
        th.start()
        if timed_arrivals:
            done = 0
            while done < len(reqs):
                with lock:
                    pending = tickets[done:]
                if not pending:
                    time.sleep(0.001)
                    continue
                k, t = pending[0]
                replies[k] = srv.wait(t)
                done += 1
        th.join()
        return replies, time.perf_counter() - start

    with bna.Server(0, slots=slots, hbm_budget=budget) as srv:
        # warm-up: every pool subject once (arena growth, graph capture)
        for j, (N, T, K, sd) in enumerate(subjects):
            srv.wait(srv.submit(pool[j], mode="density", value=1.0, csr_out=False,
                                ec_out=ecbufs[0][:N]))
        mixed, span = one_pass(srv, True)
        alone, _ = one_pass(srv, False)
    bad = [r.status for r in mixed + alone if r.status != 0]
    if dump:
        with open(dump, "w") as f:
            json.dump([{"k": k, "N": subjects[r.subject][0], "T": subjects[r.subject][1],
                        "mode": r.mode, "value": r.value, "arrival": r.arrival,
                        "status": m.status, "slot": m.slot, "nnz": m.nnz,
                        "sub": m.t_submit, "start": m.t_start, "done": m.t_done,
                        "corr": m.t_corr, "solo": a.latency, "solo_corr": a.t_corr - a.t_submit,
                        "iters": m.ec_iters, "stats": m.stats}
                       for k, (r, m, a) in enumerate(zip(reqs, mixed, alone))], f)
    lat = np.array([r.latency for r in mixed]) * 1000.0
    solo = np.array([r.latency for r in alone]) * 1000.0
    slow = lat / solo
    diff = [{"k": k, "N": subjects[reqs[k].subject][0], "T": subjects[reqs[k].subject][1],
             "mode": reqs[k].mode, "value": reqs[k].value, "nnz": [a.nnz, m.nnz],
             "lambda": [a.lam, m.lam], "iters": [a.ec_iters, m.ec_iters],
             "status": [a.status, m.status]}
            for k, (a, m) in enumerate(zip(alone, mixed))
            if a.nnz != m.nnz or not (a.lam == m.lam or (a.lam != a.lam and m.lam != m.lam))]
    same = not diff
    edges = sum(r.nnz for r in mixed)
    return {
        "requests": len(reqs), "rate_per_s": rate, "slots": slots,
        "budget_gb": budget / 2**30, "errors": len(bad),
        "error_status": {str(c): bad.count(c) for c in sorted(set(bad))},
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "solo_p50_ms": float(np.percentile(solo, 50)), "solo_p99_ms": float(np.percentile(solo, 99)),
        "slowdown_p50": float(np.percentile(slow, 50)), "slowdown_p99": float(np.percentile(slow, 99)),
        "p99_over_median_solo": float(np.percentile(lat, 99) / np.percentile(solo, 50)),
        "throughput_req_s": len(reqs) / span, "edges_per_s": edges / span,
        "same_results_alone_and_mixed": same,
        "differences": diff[:20],
        "sample": f"{len(reqs)} requests from {len(subjects)} seeded subjects "
                  f"(N {min(s[0] for s in subjects)}..{n_max}, T in {{240,600,1200}}), "
                  "tau U[0.3,0.6] or density U[0.1,2]%, split-BF16, CSR kept on device, "
                  "centrality to host",
    }


def batch_run(n_subjects: int, precision: str = "auto", plain: bool = True) -> dict:
    """The batch workload: all subjects through bna_corr_csr_batch (one
    persistent count pass over every subject's tiles), against each subject
    built alone with the plain FP32 form."""
    import numpy as np
    import torch
    import cuda_newest20160331_gb300 as bna
    from cuda_newest20160331_gb300 import workloads
    subs = workloads.batch_subjects(n_subjects)
    bolds = [torch.from_numpy(bna.synth_bold(N, T, K, sd)).cuda() for (N, T, K, sd) in subs]
    b = bna.Builder(0)
    stream = torch.cuda.current_stream()
    # warm-up: the autotuner's choice, arenas grown
    res = b.corr_csr_batch(bolds, mode="density", value=1.0, precision=precision, copy=False)
    chosen = res[0].stats
    names = {0: "fp32", 1: "bf16x3", 2: "tf32"}
    shape = {"form": names.get(chosen["precision"]), "tile_band": chosen["tile_band"],
             "tile": "128 x 256 (rows x columns), K block 64 BF16 x 3 products, 2 stages"
             if chosen["precision"] == 1 else "128 x 256, K block 32 TF32, 4 stages",
             "chosen_by": "bna_autotune_shape for the largest subject's size bucket"
             if precision == "auto" else "fixed by the caller"}
    times = []
    for _ in range(2):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        res = b.corr_csr_batch(bolds, mode="density", value=1.0, precision=precision, copy=False)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append((time.perf_counter() - t0) * 1000.0)
    batch_ms = min(times)
    nnz = sum(r.nnz for r in res)
    exact = all(r.nnz == bna.density_nnz(N, 1.0) for r, (N, _, _, _) in zip(res, subs))
    out = {"subjects": n_subjects, "batch_ms": batch_ms,
           "subjects_per_s": n_subjects / (batch_ms / 1000.0), "edges_per_s": nnz / (batch_ms / 1000.0),
           "exact_edge_counts": exact, "precision": precision, "shape": shape,
           "flop_algorithmic": float(sum(N * (N - 1) / 2 * 2 * T for (N, T, _, _) in subs)),
           "sample": f"{n_subjects} subjects, N {min(s[0] for s in subs)}..{max(s[0] for s in subs)}, "
                     f"T {min(s[1] for s in subs)}..{max(s[1] for s in subs)}, density 1 %, weighted"}
    out["tflops_algorithmic"] = out["flop_algorithmic"] / (batch_ms / 1000.0) / 1e12
    if plain:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for bold in bolds:
            b.corr_csr(bold, mode="density", value=1.0, precision="fp32", copy=False)
        torch.cuda.synchronize()
        pms = (time.perf_counter() - t0) * 1000.0
        out["plain_fp32_each_alone_ms"] = pms
        out["plain_fp32_subjects_per_s"] = n_subjects / (pms / 1000.0)
        out["speedup_vs_plain_fp32"] = pms / batch_ms
    b.close()
    return out


def mod_levels(log):
    """Critical path of a modularity run: rounds are the nodes of a binary
    tree visited breadth first (a division of round r numbers its children
    maxres + 1, maxres + 2); the rounds of one tree level run side by side, so
    the level's longest round (power steps of both Lead_Vector calls) bounds it."""
    level = {0: 0}
    maxres = 0
    per_level = {}
    for e in log:
        lv = level.get(e["round"], 0)
        per_level[lv] = max(per_level.get(lv, 0), sum(e["iters"]))
        if e["divided"]:
            level[maxres + 1] = level[maxres + 2] = lv + 1
            maxres += 2
    return sum(per_level.values()), len(per_level)


def modularity_run(b, csr, stream, reps: int = 2) -> dict:
    """Newman modularity of a device CSR's binary graph, CUDA-event timed."""
    import torch
    times = []
    for _ in range(reps):
        log = []
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        labels, m, q = b.modularity(csr, log=log)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    crit, levels = mod_levels(log)
    ms = statistics.median(times)
    return {"ms": ms, "modules": m, "Q": q, "rounds": len(log),
            "power_steps": sum(sum(e["iters"]) for e in log), "tree_levels": levels,
            "critical_path_steps": crit, "us_per_critical_step": ms * 1e3 / max(crit, 1),
            "labels": labels}


def modularity_small_pair(b, stream) -> dict:
    """The small workload's binary CSR (N=4,096, r >= 0.5): the device
    modularity against the reference tool's CPU arithmetic (the C restatement,
    one thread) on the same graph, whole runs on both sides."""
    import numpy as np
    import torch
    import oracle
    from cuda_newest20160331_gb300 import workloads
    ws = workloads.get("small")
    bs = torch.from_numpy(ws.bold()).cuda()
    csr = b.corr_csr(bs, mode=ws.mode, value=ws.value, precision="bf16x3", weighted=False,
                     copy=True)
    g = modularity_run(b, csr, stream, reps=1)
    h = csr.numpy()
    t0 = time.perf_counter()
    lab_o, q_o, m_o, _ = oracle.modularity(h.row_ptr, h.col_idx)
    cpu_s = time.perf_counter() - t0
    same = bool(np.array_equal(g.pop("labels").cpu().numpy(), lab_o))
    return {"workload": f"small: N={ws.N} T={ws.T} r>=0.5 binary, nnz={csr.nnz}",
            "gpu_ms": g["ms"], "cpu_ms": cpu_s * 1e3, "cpu_cores": 1, "cpu_kind": "port",
            "modules": g["modules"], "labels_equal": same,
            "critical_path_steps": g["critical_path_steps"], "power_steps": g["power_steps"]}


def load_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` on `workload` from one ncu capture
    (profiles/traffic.txt: `kernel:workload bytes` lines), or None."""
    try:
        for line in open(os.path.join(ROOT, "profiles", "traffic.txt")):
            f = line.split("#")[0].split()
            if len(f) == 2 and f[0] == f"{kernel}:{workload}":
                return int(f[1])
    except OSError:
        pass
    return None


def run_reference(args):
    """The reference's CPU path on the host cores (rank 0 only): the oracle's
    restatement of its CPU tool, fed by the oracle's copy of the generator, so
    nothing of the product library is loaded."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    import oracle
    from cuda_newest20160331_gb300 import workloads
    w = workloads.get(args.workload)
    bold = oracle.synth_bold(**w.synth_args())
    cores = host_cores()
    ref = CpuReference(w, bold, cores)
    per_step = args.cpu_seconds / max(1, args.steps)
    for _ in range(args.warmup):
        ref.sample(min(per_step, 1.0))
    samples = [ref.sample(per_step) for _ in range(args.steps)]
    v = statistics.median(s["value"] for s in samples)
    s0 = samples[len(samples) // 2]
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "edges/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * statistics.median(s["seconds"] for s in samples),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded factor model)",
        "config": bench_config(w, world),
        "precision": "f32 (float-accumulated cross terms)",
        "cpu_baseline": {"value": v, "unit": "edges/s", "cores": cores, "kind": "port",
                         "sample": s0["sample"]},
        "e2e": {"value": v, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "tflops_algorithmic": statistics.median(s["tflops"] for s in samples),
        "pairs_per_s": statistics.median(s["pairs_per_s"] for s in samples),
        "full_job_s_extrapolated": statistics.median(s["full_job_s_extrapolated"] for s in samples),
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import numpy as np
    import torch
    import cuda_newest20160331_gb300 as bna
    from cuda_newest20160331_gb300 import workloads

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if args.workload == "batch64":
        bt = batch_run(64, precision=args.precision if args.precision != "bf16x3" else "auto",
                       plain=not args.no_plain)
        if rank == 0:
            print(json.dumps({"metric": "subjects/s, 64-subject batch at 1 % density",
                              "value": bt["subjects_per_s"], "unit": "subjects/s",
                              "higher_is_better": True, "n_gpus": 1, "batch": bt}), flush=True)
        return
    if args.workload == "serving":
        sv = serve_run(1000 if args.serve_requests is None else args.serve_requests,
                       slots=args.serve_slots, dump=args.serve_dump,
                       budget=int(args.serve_budget_gb * 2**30))
        if rank == 0:
            print(json.dumps({"metric": "serving latency p50/p99 (corr -> CSR -> centrality)",
                              "value": sv["p99_ms"], "unit": "ms", "higher_is_better": False,
                              "n_gpus": 1, "serve": sv}), flush=True)
        return
    # serving first, in a fresh device state: its requests then meet only one
    # another (a builder context and its arena from the measurements below
    # would share the device with them)
    serve = None
    n_serve = 120 if args.serve_requests is None else args.serve_requests
    if rank == 0 and n_serve > 0:
        serve = serve_run(n_serve, slots=args.serve_slots, dump=args.serve_dump,
                       budget=int(args.serve_budget_gb * 2**30))
    w = workloads.get(args.workload)
    precision = args.precision
    bold_h = w.bold()
    T, N = bold_h.shape
    bold = torch.from_numpy(bold_h).to(dev)
    b = bna.Builder(local)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    def step():
        return b.corr_csr(bold, mode=w.mode, value=w.value, precision=precision,
                          weighted=w.weighted, copy=False)

    for _ in range(max(3, args.warmup)):
        res = step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    count_ms, fill_ms, stats = [], [], []
    barrier()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()  # evict L2 between steps (inputs are smaller than L2)
            starts[k].record(stream)
            res = step()
            ends[k].record(stream)
            stats.append(res.stats)
        barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = max_over_ranks(sum(step_ms) / len(step_ms), world, dev)
    nnz = res.nnz
    pairs = N * (N - 1) // 2
    flop = pairs * 2.0 * T
    value = job_value(world, nnz, ms)

    # eigenvector centrality on the device-resident CSR of the last step
    # (Lead_Vector_GPU semantics: 10,000 iterations max, stop at 1e-6)
    csr_dev = b.corr_csr(bold, mode=w.mode, value=w.value, precision=precision,
                         weighted=w.weighted, copy=True)
    ec_ms = []
    for rep in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ec_vec, lam, iters, conv = b.ec(csr_dev)
        e1.record(stream)
        torch.cuda.synchronize()
        ec_ms.append(e0.elapsed_time(e1))
    ec_info = {"ms": statistics.median(ec_ms), "iterations": iters, "lambda": lam,
               "converged": conv,
               "hbm_gbs_per_iteration": (8.0 * csr_dev.nnz + 4.0 * (N + 1) + 16.0 * N) * iters
               / (statistics.median(ec_ms) / 1000.0) / 1e9 if iters else None}
    # Newman modularity of the same CSR's binary graph (values ignored, as the
    # reference tool reads only R and C)
    if args.modularity == "on" or (args.modularity == "auto" and N <= 100000):
        mod_info = modularity_run(b, csr_dev, stream)
        mod_info.pop("labels")
        mod_info["workload"] = f"{w.name} CSR, binary view (nnz={csr_dev.nnz})"
    else:
        mod_info = {"skipped": f"N={N} above the automatic limit (--modularity on runs it)"}
    del csr_dev

    # the other forms on the same input, same edge set (3 timed steps each):
    # plain FP32 on CUDA cores, and the single-product TF32 tensor-core form
    def time_form(prec):
        for _ in range(2):
            rp = b.corr_csr(bold, mode=w.mode, value=w.value, precision=prec,
                            weighted=w.weighted, copy=False)
        pms = []
        for _ in range(3):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rp = b.corr_csr(bold, mode=w.mode, value=w.value, precision=prec,
                            weighted=w.weighted, copy=False)
            e1.record(stream)
            torch.cuda.synchronize()
            pms.append(e0.elapsed_time(e1))
        pm = statistics.median(pms)
        return {"value": rp.nnz / (pm / 1000.0), "unit": "edges/s", "ms_per_step": pm,
                "nnz": rp.nnz, "same_edge_count": rp.nnz == nnz,
                "ms_count": rp.stats["ms_count"], "ms_recompute": rp.stats["ms_recompute"],
                "band_candidates": rp.stats["band_candidates"], "band_1e6": rp.stats["band_1e6"],
                "delta": rp.stats["delta"],
                "tflops_algorithmic": flop / (pm / 1000.0) / 1e12,
                "speedup_of_chosen_form": pm / ms}

    plain = None
    if precision != "fp32" and not args.no_plain:
        plain = time_form("fp32")
    other_tc = None
    if precision in ("bf16x3", "tf32") and not args.no_plain:
        other_tc = time_form("tf32" if precision == "bf16x3" else "bf16x3")

    # end to end through the host-buffer API (bna_corr_csr_host_into): pinned
    # BOLD in, CSR out into pinned caller buffers, copies inside the timed region
    pinned = torch.from_numpy(bold_h).pin_memory()
    pin_np = pinned.numpy()
    cap = int(nnz * 1.25) + 1024
    rp_h = torch.empty(N + 1, dtype=torch.int32).pin_memory().numpy()
    ci_h = torch.empty(cap, dtype=torch.int32).pin_memory().numpy()
    va_h = torch.empty(cap, dtype=torch.float32).pin_memory().numpy() if w.weighted else None
    for _ in range(2):
        he_nnz, _ = b.corr_csr_host_into(pin_np, rp_h, ci_h, va_h, mode=w.mode, value=w.value,
                                         precision=precision)
    e2e_ms = []
    for _ in range(max(3, args.steps // 2)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        he_nnz, _ = b.corr_csr_host_into(pin_np, rp_h, ci_h, va_h, mode=w.mode, value=w.value,
                                         precision=precision)
        e2e_ms.append((time.perf_counter() - t0) * 1000.0)
    e2e = max_over_ranks(statistics.median(e2e_ms), world, dev)
    h2d = N * T * 4
    d2h = (N + 1) * 4 + he_nnz * (8 if w.weighted else 4)

    # max |r - r_fp64| of each form on sampled tiles (rewrites the context's
    # z-scores, so it runs after every use of the step's CSR)
    max_err = max_abs_err(b, bold, bold_h, precision)
    if plain is not None:
        plain["max_abs_r_minus_fp64"] = max_abs_err(b, bold, bold_h, "fp32")["value"]
    if other_tc is not None:
        other_tc["max_abs_r_minus_fp64"] = max_abs_err(
            b, bold, bold_h, "tf32" if precision == "bf16x3" else "bf16x3")["value"]

    # dominant kernel: one correlation pass (count) over all N(N-1)/2 pairs
    cnt = statistics.median(s["ms_count"] for s in stats)
    fil = statistics.median(s["ms_fill"] for s in stats)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("bf16_tflops", 1900.0)
    achieved = flop / (cnt / 1000.0) / 1e12
    roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": load_traffic(f"corr_count_{precision}", w.name),
            "kernel": f"correlation count pass ({precision})",
            "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)" if peaks else "fallback"}
    line = {
        "metric": METRIC, "value": value, "unit": "edges/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if precision == "fp32" else precision,
        "data": "synthetic (seeded factor model, device-resident input)",
        "config": bench_config(w, world),
        "precision": precision,
        "tflops_algorithmic": flop * world / (ms / 1000.0) / 1e12,
        "nnz": nnz, "stage_ms": {k: statistics.median(s[k] for s in stats) for k in
                                 ("ms_zscore", "ms_count", "ms_recompute", "ms_scan", "ms_fill")},
        "band_candidates": stats[-1]["band_candidates"], "band_1e6": stats[-1]["band_1e6"],
        "delta": stats[-1]["delta"],
        "max_abs_r_minus_fp64": max_err,
        "roofline": roof,
        "plain_fp32": plain,
        ("tf32" if precision == "bf16x3" else "bf16x3"): other_tc,
        "ec": ec_info,
        "modularity": mod_info,
        "e2e": {"value": job_value(world, he_nnz, e2e), "unit": "edges/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms": e2e},
        "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
        "clocks": clk.summary(),
    }
    if serve is not None:
        line["serve"] = serve
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        ref = CpuReference(w, bold_h, host_cores())
        cb = ref.sample(args.cpu_seconds)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        line["cpu_baseline"]["full_job_s_extrapolated"] = cb["full_job_s_extrapolated"]
        if "skipped" not in line["modularity"]:
            line["modularity"]["small_vs_cpu"] = modularity_small_pair(b, stream)
    if rank == 0:
        print(json.dumps(line), flush=True)
    b.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
