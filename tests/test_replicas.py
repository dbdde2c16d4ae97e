"""Multi-GPU form (replicas, no data-path collective), on CPU with gloo:
bench's whole-job rate sums the units of all ranks over the slowest rank's
time, and the reference arm runs on rank 0 only (the others exit 0 without
work)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

WORKER = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo", init_method="env://")
# rank r processed 1000 * (r + 1) units in 100 + 50 r ms (spans: whole, part)
rate, total, spans = bench.replica_rate(1000 * (rank + 1), [100.0 + 50 * rank, 10.0 * (rank + 1)], world, "cpu")
dist.barrier()
dist.destroy_process_group()
print(json.dumps({"rank": rank, "rate": rate, "total": total, "spans": spans}))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _launch(code, world, extra_env=None, args=()):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE=str(world), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), **(extra_env or {}))
        procs.append(subprocess.Popen([sys.executable, "-c", code, str(ROOT), *args], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=180)
        assert p.returncode == 0, err[-2000:]
        outs.append(out)
    return outs


def test_replica_rate_two_ranks_gloo():
    outs = [json.loads(o.strip().splitlines()[-1]) for o in _launch(WORKER, 2)]
    for o in outs:
        assert o["total"] == 3000.0
        assert o["spans"] == [150.0, 20.0]
        assert abs(o["rate"] - 3000.0 / 0.150) < 1e-6


def test_reference_arm_runs_on_rank_zero_only():
    code = ("import sys; sys.path.insert(0, sys.argv[1]); import bench, argparse; "
            "a = argparse.Namespace(steps=1, warmup=0, gpus=2); sys.exit(bench.reference_arm(a))")
    port = _free_port()
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    p = subprocess.run([sys.executable, "-c", code, str(ROOT)], env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""
