"""The multi-rank host logic of bench.py on CPU: world_size 2 over gloo (the
bench runs one replica per GPU with a barrier and the max over ranks; every
GPU machine here has one GPU, so the path is covered on the host)."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    env = bench.dist_env()
    bench.barrier(ws)
    # each rank's device time differs; the line must carry the slowest
    t = bench.max_over_ranks(10.0 + rank, ws)
    dist.destroy_process_group()
    q.put((rank, env, t))


@pytest.mark.timeout(120)
def test_two_ranks_barrier_and_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=100) for _ in ps)
    for p in ps:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [(2, 0, 0), (2, 1, 1)]
    assert all(r[2] == 11.0 for r in res)


@pytest.mark.timeout(120)
def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's rank 0 alone times the CPU code and prints the line;
    every other rank exits 0 at once without work or output."""
    import subprocess

    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2",
               MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()))
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus",
                        "2", "--steps", "1", "--warmup", "0"], env=env, cwd=str(ROOT),
                       capture_output=True, text=True, timeout=100)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
