"""The N > 1 host path of bench.py on CPU: independent replicas under
torch.distributed with the gloo backend (world size 2), the way torchrun
launches one process per GPU.  The path has no data-path collective; the
only exchange is the max over ranks of the step times."""
import json
import os
import pathlib
import socket
import subprocess
import sys

import pytest

import bench

ROOT = pathlib.Path(__file__).resolve().parents[1]


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 5.0], world, "cpu")
        out.put((rank, got, bench.replicas_rate(world, 4096, got[0])))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    """Each rank gets every figure's maximum over both ranks, and the
    whole-job rate counts both replicas' chunks over the slowest step."""
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    for _, got, rate in res:
        assert got == [2.0, 10.0, 5.0]
        assert rate == pytest.approx(2 * 4096 / 2e-3)


def test_max_over_ranks_one_rank():
    assert bench.max_over_ranks([3, 4.5], 1, None) == [3.0, 4.5]
    assert bench.replicas_rate(1, 4096, 18.35) == pytest.approx(4096 / 0.01835)


def test_reference_arm_under_torchrun():
    """`bench.py --impl reference` launched as for N = 2: rank 0 alone times
    the CPU reference and prints one JSON line; rank 1 exits 0 without work."""
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--gpus", "2",
           "--impl", "reference", "--workload", "tiled", "--steps", "1", "--warmup", "0", "--cpu-sample", "8"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    assert lines[0]["impl"] == "reference" and lines[0]["value"] > 0
    assert lines[0]["e2e"]["h2d_bytes_per_step"] == 0
