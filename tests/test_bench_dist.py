"""bench.py's multi-rank host logic on CPU: two gloo ranks, as torchrun would
launch them (RANK / WORLD_SIZE / MASTER_* from the environment).  The whole-job
figure is the sum of the ranks' events over the slowest rank's time; the
reference arm prints from rank 0 only."""
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


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r: wall 1 + r seconds, 100 * (r + 1) events
    wall, count = bench.reduce_over_ranks(dist, 1.0 + rank, 100 * (rank + 1))
    dist.destroy_process_group()
    q.put((rank, wall, count))


def test_reduce_over_ranks_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for _, wall, count in res:
        assert wall == 2.0 and count == 300.0


def test_reduce_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(None, 1.5, 7) == (1.5, 7.0)


@pytest.mark.timeout(300)
def test_reference_arm_rank1_prints_nothing():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--cpu-seconds", "0.5"], env=env, capture_output=True, text=True,
                       timeout=240)
    assert r.returncode == 0 and r.stdout.strip() == ""
