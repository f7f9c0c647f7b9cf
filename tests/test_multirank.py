"""The N>1 host path on CPU: two gloo ranks plan the same jobs without communicating, score
disjoint shares that cover every job, and agree on the slowest rank's time."""
import os
import socket

import pytest

from breseq_gb300 import shard


def test_plan_covers_and_balances():
    work = [5, 1, 9, 3, 3, 7, 2, 8, 1, 4]
    for world in (1, 2, 3, 4):
        p = shard.plan(work, world)
        flat = sorted(i for r in p for i in r)
        assert flat == list(range(len(work)))
        loads = [sum(work[i] for i in r) for r in p]
        assert max(loads) - min(loads) <= max(work)
    assert shard.plan(work, 2) == shard.plan(list(work), 2)   # deterministic


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, work, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard.plan(work, world)[rank]
    fake_ms = 10.0 * (rank + 1) + sum(work[i] for i in mine) * 1e-3
    slow = shard.slowest(fake_ms)
    dist.barrier()
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{','.join(map(str, mine))};{fake_ms!r};{slow!r}\n")
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    work = [300, 120, 80, 75, 60, 40, 22, 9]
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), work, str(tmp_path)), nprocs=world, join=True)
    shares, times, slows = [], [], []
    for r in range(world):
        a, b, c = open(tmp_path / f"rank{r}.txt").read().strip().split(";")
        shares.append([int(x) for x in a.split(",") if x])
        times.append(float(b))
        slows.append(float(c))
    assert sorted(i for s in shares for i in s) == list(range(len(work)))
    assert not set(shares[0]) & set(shares[1])
    assert slows[0] == slows[1] == max(times)
