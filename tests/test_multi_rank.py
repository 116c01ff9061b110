"""The N>1 path of bench.py on CPU: two gloo ranks shard the model list with no
data-path collective and reduce only the timing (max) and counts (sum)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    sys.path[:0] = [ROOT, os.path.join(ROOT, "fedem-solvers_gb300")]
    import torch
    import torch.distributed as dist

    import bench
    from fedem_gb300 import models

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cases = models.batch_c4(40, seed=9, n_max=4000, steps=1)
    mine = bench.shard(cases, rank, world)
    load = sum(cases[k][2] for k in mine)
    t = torch.tensor([float(rank + 1), float(len(mine)), float(load)], dtype=torch.float64)
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    if rank == 0:
        out.put((float(tmax[0]), float(t[1]), float(t[2]), gathered, [c[2] for c in cases]))
    dist.destroy_process_group()


def test_two_rank_sharding_covers_every_model_once():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    tmax, nsum, loadsum, parts, sizes = res
    assert tmax == 2.0                         # max over ranks of the timings
    assert nsum == 40                          # every model counted once
    allm = sorted(parts[0] + parts[1])
    assert allm == list(range(40))             # a partition, no model on two ranks
    loads = [sum(sizes[k] for k in part) for part in parts]
    assert loadsum == sum(sizes)
    assert max(loads) <= 0.5 * sum(sizes) + max(sizes)  # balanced by element count


class _FakeSolverLib:
    """Stands in for libfedem_solver_core.so's device entry points on CPU:
    records the ordinal each rank asks for."""

    def __init__(self):
        self.asked = []
        self.cur = -1

    def fgpu_set_device(self, ordinal):
        self.asked.append(ordinal)
        self.cur = ordinal
        return 0

    def fgpu_get_device(self, dev_ref, bus, n):
        dev_ref._obj.value = self.cur
        bus.value = b"fake:%d" % self.cur
        return 0

    def fgpu_last_error(self):
        return b""


def _device_worker(rank, world, port, out):
    sys.path[:0] = [ROOT, os.path.join(ROOT, "fedem-solvers_gb300")]
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.rank_env()
    fake = _FakeSolverLib()
    dev, bus = bench.rank_device(local, fake)
    gathered = [None] * world
    dist.all_gather_object(gathered, (r, w, local, fake.asked, dev, bus))
    if rank == 0:
        out.put(gathered)
    dist.destroy_process_group()


def test_each_rank_selects_its_own_device():
    """bench.py gives the solver library each rank's LOCAL_RANK as its device
    (fgpu_set_device) before anything is created, so two ranks on one node use
    two GPUs."""
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_device_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, local, asked, dev, bus) in enumerate(res):
        assert (rank, world, local) == (r, 2, r)
        assert asked == [r] and dev == r and bus == f"fake:{r}"
