"""The replica path of bench.py on CPU: gloo ranks and torch.distributed.run.

Independent instances are the shard unit, so ranks exchange only the timing
maximum; these tests run that exchange with world size 2 and the reference
arm under a 2-process launch, where rank 0 alone measures and prints.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [12.5, 30.0][rank]
    slowest = bench.world_max(ms, world, device="cpu")
    rate = bench.whole_job_rate(1000.0, world, slowest / 1e3)
    out.put((rank, slowest, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_world_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, slowest, rate in res:
        assert slowest == 30.0
        assert rate == pytest.approx(2 * 1000.0 / 0.030)


def test_reference_arm_under_two_rank_launch():
    """Rank 0 prints one JSON line for the whole job; rank 1 exits 0 without output."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--workload", "1d4096", "--gpus", "2", "--steps", "4", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("port", "reference")
