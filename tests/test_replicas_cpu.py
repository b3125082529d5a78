"""The multi-GPU form of this path is replicas (the solve does not shard):
N ranks each run the whole workload and bench.py reports the slowest rank.
The host-side logic is checked here on CPU with the gloo backend, two ranks:
the max over ranks, and the reference arm printing one line from rank 0."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE="2", LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    ws, r, _ = bench.dist_setup("gloo")
    m = bench.max_over_ranks(1.5 + r, ws)
    bench.barrier(ws)
    with open(os.path.join(out_dir, "rank%d" % r), "w") as f:
        f.write("%d %r" % (ws, m))
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(_free_port(), str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        ws, m = open(tmp_path / ("rank%d" % r)).read().split()
        assert int(ws) == 2 and float(m) == 2.5


def test_reference_arm_prints_once_under_torchrun():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0"]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["unit"] == "s"
    assert d["config"]["iterations"] > 0 and d["e2e"]["h2d_bytes_per_step"] == 0
