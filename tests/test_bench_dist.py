"""The multi-rank arithmetic of bench.py on CPU: two gloo ranks (replicas)
agree on the slowest rank's step time, the whole-job value counts both
ranks' units over that time, and the reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_CODE = r"""
import os, sys
sys.path.insert(0, os.environ["BENCH_ROOT"])
import torch.distributed as dist
import bench
dist.init_process_group("gloo", init_method="env://")
rank = dist.get_rank()
ms = [2.5, 4.0][rank]
worst = bench.max_over_ranks(ms, dist.get_world_size(), "cpu")
print("RESULT", rank, repr(worst), repr(bench.job_value(dist.get_world_size(), 1000, worst)))
dist.barrier()
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_take_the_slowest_time():
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), BENCH_ROOT=ROOT)
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_CODE], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(out)
    got = sorted(l.split()[1:] for o in outs for l in o.splitlines() if l.startswith("RESULT"))
    assert [g[0] for g in got] == ["0", "1"]
    for _, worst, value in got:
        assert float(worst) == 4.0  # the slower rank's step time on both ranks
        assert float(value) == 2 * 1000 / 0.004  # both ranks' units over that time


def test_single_rank_keeps_its_own_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, 1, "cpu") == 3.25
    assert bench.job_value(1, 500, 2.0) == 500 / 0.002


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.run_reference(None) is None  # returns before reading its arguments
    assert capsys.readouterr().out == ""
