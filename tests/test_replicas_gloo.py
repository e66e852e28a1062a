"""bench.py's multi-rank path on the CPU: two ranks over gloo.

Images are independent, so N GPUs run N replicas with no data-path
collective; the only cross-rank steps are the barriers around the timed
region and the max-over-ranks of the step time, after which rank 0 alone
prints the line.  These tests run those pieces as two processes on
127.0.0.1 with the gloo backend (no GPU needed).
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, os.environ["TT_ROOT"])
import torch.distributed as dist
import bench
rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo")
bench.barrier(world)
mx = bench.max_over_ranks(10.0 + 5.0 * rank, world)   # per-rank step times
mn = -bench.max_over_ranks(-(10.0 + 5.0 * rank), world)
rate = bench.job_rate(8, world, mx)
bench.barrier(world)
dist.destroy_process_group()
print(json.dumps({"rank": rank, "max": mx, "min": mn, "rate": rate}))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_ranks(script, world, extra_env=None, args=()):
    port = _free_port()
    procs = []
    for rank in range(world):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                   WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), TT_ROOT=ROOT)
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable, "-c", script, *args], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    try:
        for p in procs:
            out, err = p.communicate(timeout=120)
            assert p.returncode == 0, err
            outs.append(out)
    finally:
        for p in procs:  # a rank that failed or hung must not outlive the test
            if p.poll() is None:
                p.kill()
                p.wait()
    return outs


def test_max_over_ranks_and_barriers_two_ranks():
    outs = _run_ranks(_RANK_SCRIPT, 2)
    res = sorted((json.loads(o.strip().splitlines()[-1]) for o in outs), key=lambda r: r["rank"])
    # every rank reports the slowest rank's time (the weak-scaling clock)
    assert [r["max"] for r in res] == [15.0, 15.0]
    assert [r["min"] for r in res] == [10.0, 10.0]
    # both ranks' units over the slowest rank's time
    assert [r["rate"] for r in res] == [pytest.approx(2 * 8 / 0.015)] * 2


_REF_SCRIPT = r"""
import os, sys
sys.path.insert(0, os.environ["TT_ROOT"])
sys.argv = ["bench.py", "--impl", "reference", "--gpus", os.environ["WORLD_SIZE"]]
import bench
bench.main()
"""


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm is the host's CPU implementation: the
    other ranks exit 0 without work or output (rank 0 is not started here)."""
    port = _free_port()
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2",
               RANK="1", LOCAL_RANK="1", TT_ROOT=ROOT)
    p = subprocess.run([sys.executable, "-c", _REF_SCRIPT], env=env, capture_output=True,
                       text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""


def test_weak_scaling_job_rate():
    """value = world x per-rank units / slowest rank's step time."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_rate(8, 1, 20.0) == pytest.approx(400.0)
    # two replicas of 8 sinograms, the slower taking 25 ms: 16 per 25 ms
    assert bench.job_rate(8, 2, 25.0) == pytest.approx(640.0)
