"""The N > 1 path of bench.py on CPU: ranks are independent frame replicas
coordinated on the host over gloo (no data-path collective).  The slowest
rank sets the step time, and under torchrun the reference arm runs on rank 0
alone and prints one line."""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    out[rank] = bench.rank_max(10.0 + 5.0 * rank, world)
    dist.barrier()
    dist.destroy_process_group()


def test_rank_max_over_two_gloo_ranks():
    port = _free_port()
    # the manager process is started with spawn, not fork: this test may run
    # in a process that has already used the GPU
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
        assert dict(out) == {0: 15.0, 1: 15.0}


def test_reference_arm_under_torchrun_prints_one_line():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "1", "--particles", "3000", "--ref-budget-s", "60"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
    # whole frames timed: the line's steps is the number of frames it timed
    assert 1 <= d["steps"] <= 2 and len(d["frames_timed_s"]) == d["steps"]
