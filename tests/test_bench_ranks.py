"""The benchmark's multi-rank host logic on the CPU (two gloo ranks): each
rank drives its own local GPU (replicas, no data-path collective) and the
job's time is the slowest rank's, exchanged as one scalar."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, bench.device(), bench.rank_max(1.5 + rank), bench.dist_env()))
    finally:
        dist.destroy_process_group()


def test_two_ranks_pick_their_gpu_and_share_the_slowest_time():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [0, 1]           # rank i drives local GPU i
    assert [o[2] for o in out] == [2.5, 2.5]       # max over ranks
    assert [o[3] for o in out] == [(0, 0, 2), (1, 1, 2)]


def test_one_rank_needs_no_process_group(monkeypatch):
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(k, raising=False)
    import bench
    assert bench.device() == 0 and bench.rank_max(3.25) == 3.25
