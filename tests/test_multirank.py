"""The multi-GPU path of bench.py on CPU: two gloo ranks (replicas only -- each
rank advances its own replicas; the only collectives are the timing barrier and
max/sum over ranks, exactly as under torchrun on N GPUs)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

WORKER = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import bench
dist, rank, local, world = bench._dist_init(2)
assert world == 2 and dist is not None and dist.get_backend() == "gloo"
bench._barrier(dist)
out = {
    "rank": rank,
    "max": bench._max_over_ranks(dist, 1.5 + rank),       # timing: the slowest rank's seconds
    "sum": bench._sum_over_ranks(dist, 100.0 * (rank + 1)),  # throughput: moves of all ranks
    "streams": bench.replica_streams(4, rank).tolist(),   # per-rank RNG streams never collide
}
print(json.dumps(out), flush=True)
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _launch(code_args, port, extra_env=None):
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable] + code_args, env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True, cwd=str(ROOT)))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=240)
        assert p.returncode == 0, e
        outs.append(o)
    return outs


def test_two_ranks_reduce_like_the_benchmark():
    pytest.importorskip("torch")
    outs = _launch(["-c", WORKER, str(ROOT)], _free_port())
    res = sorted((json.loads(o.strip().splitlines()[-1]) for o in outs), key=lambda d: d["rank"])
    assert [r["max"] for r in res] == [2.5, 2.5]
    assert [r["sum"] for r in res] == [300.0, 300.0]
    assert not set(res[0]["streams"]) & set(res[1]["streams"])


def test_reference_arm_runs_on_rank_zero_only():
    """--impl reference under torchrun: rank 0 prints the line, the other rank exits without work."""
    pytest.importorskip("torch")
    outs = _launch(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
                    "--cpu-sample-seconds", "0.05"], _free_port(), extra_env={"OMP_NUM_THREADS": "1"})
    lines = [o.strip().splitlines() for o in outs]
    assert len(lines[1]) == 0
    d = json.loads(lines[0][-1])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
