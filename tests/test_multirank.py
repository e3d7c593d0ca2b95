"""The multi-rank path of the batched workloads on CPU with two gloo ranks:
every rank computes the same flop-balanced split of the uneven batch without
communicating, the shares are disjoint and complete, and the only exchange --
a gather of per-instance scalars to rank 0 -- reassembles the whole batch."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from tncontract_gb300 import workloads as W
        specs = W.config3_specs(1, 64)
        parts = W.partition_by_flops(specs, world)
        mine = parts[rank]
        # per-instance scalars this rank would report (here: its estimated cost)
        scal = {i: W.spec_flops(specs[i]) for i in mine}
        got = [None] * world if rank == 0 else None
        dist.gather_object(scal, got, dst=0)
        views = [None] * world
        dist.all_gather_object(views, parts)
        if rank == 0:
            merged = {}
            for g in got:
                merged.update(g)
            out.put((sorted(merged), [len(p) for p in parts], all(v == parts for v in views),
                     [sum(W.spec_flops(specs[i]) for i in p) for p in parts]))
    finally:
        dist.destroy_process_group()


def test_partition_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    merged, sizes, same, loads = q.get(timeout=10)
    assert merged == list(range(64))           # complete and disjoint
    assert same                                # every rank computed the same split
    assert min(sizes) > 0
    assert max(loads) / min(loads) < 1.05      # flops balanced


def test_partition_single_rank_and_balance():
    from tncontract_gb300 import workloads as W
    specs = W.config3_specs(1, 512)
    assert W.partition_by_flops(specs, 1) == [list(range(512))]
    parts = W.partition_by_flops(specs, 8)
    assert sorted(i for p in parts for i in p) == list(range(512))
    loads = [sum(W.spec_flops(specs[i]) for i in p) for p in parts]
    assert max(loads) / min(loads) < 1.02
