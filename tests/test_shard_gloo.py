"""Multi-GPU is replicas only: streams are partitioned across ranks with no
data-path collective.  Two gloo ranks on CPU check that the partition they
compute independently covers every stream exactly once and balances work."""
import os
import socket

import pytest

from cuimg_gb300.shard import assign, stream_cost

SHAPES = [(240, 320), (640, 480), (1280, 720), (1920, 1080), (3840, 2160)]


def _streams(n=64, seed=3):
    import random
    rnd = random.Random(seed)
    out = []
    for _ in range(n):
        c, r = rnd.choice(SHAPES)
        out.append(dict(rows=r, cols=c, nscales=4, frames=60))
    return out


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = assign(_streams(), world)[rank]
    t = torch.zeros(64, dtype=torch.int64)
    t[mine] = 1
    dist.all_reduce(t)
    load = torch.tensor([sum(stream_cost(**_streams()[i]) for i in mine)], dtype=torch.float64)
    loads = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(loads, load)
    if rank == 0:
        q.put((t.tolist(), [float(x) for x in loads]))
    dist.destroy_process_group()


def test_two_gloo_ranks_partition_streams():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    counts, loads = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert counts == [1] * 64                      # every stream on exactly one rank
    assert max(loads) / min(loads) < 1.05          # balanced within 5%


def test_assign_deterministic_and_complete():
    s = _streams()
    for world in (1, 2, 3, 8):
        parts = assign(s, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(s)))
        assert parts == assign(s, world)
