"""The N > 1 launch path on CPU (gloo, world size 2), no GPU.

The path has no data-path collective ("replicas only": every rank runs its own replica
set); what crosses ranks is the timing: the bench reports the summed work of all ranks
over the slowest rank's time.  Checked with two gloo ranks, and the reference arm under
torchrun (rank 0 prints the one JSON line, rank 1 exits 0 without output).
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    secs, counts = bench.reduce_over_ranks(1.0 + rank, [100.0 * (rank + 1), 7.0], dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out, "r%d.json" % rank), "w") as f:
        json.dump([secs, counts], f)


def test_reduce_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        secs, counts = json.load(open(tmp_path / ("r%d.json" % r)))
        assert secs == 2.0                      # the slowest rank's time
        assert counts == [300.0, 14.0]          # every rank's work summed


def test_reference_arm_two_ranks():
    pytest.importorskip("torch")
    port = free_port()
    env = dict(os.environ, PYTHONPATH=ROOT)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--workload", "c0", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--cpu-seconds", "0.5"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port"
