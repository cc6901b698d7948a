"""The multi-GPU path of bench.py is replicas only: every rank runs the
whole workload on its own GPU, timings are combined as the maximum over the
ranks, and whole-job throughput is all ranks' units over that time. These
tests run the rank plumbing as two gloo processes on the CPU."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # Rank r took 10 + r ms for the device loop and 20 - r ms end to end.
        got = bench.slowest_rank([10.0 + rank, 20.0 - rank], world)
        dist.barrier()
        q.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1] == [11.0, 20.0]


def test_replica_throughput_counts_every_rank():
    assert bench.slowest_rank([3.0, 4.0], 1) == [3.0, 4.0]
    # 2 ranks x 30 steps x 4 frames in 100 ms: 2400 frames/s.
    assert bench.replica_throughput(30 * 4, 2, 100.0) == pytest.approx(2400.0)


def test_reference_arm_under_torchrun_two_ranks():
    # Rank 0 alone times the reference's CPU path and prints one line; the
    # other rank exits 0 without work.
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--size", "256x144",
           "--frames", "6"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("port", "reference")
