"""The multi-rank path of the batched workloads on CPU with two gloo ranks:
every rank computes the same flop-balanced split of the uneven batch without
communicating, the shares are disjoint and complete, and the only exchange --
a gather of per-instance scalars to rank 0 -- reassembles the whole batch.
The end-to-end test runs the sharded executor (workloads.run_sharded) with
the engine's host control flow over the CPU stand-in of the device ops and
checks every gathered instance against the oracle."""
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


def _sharded_main(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import numpy as np
        from host_fake import cpu_ops
        from tncontract_gb300 import engine as E
        from tncontract_gb300 import workloads as W
        import tn_oracle as O
        specs = _small_specs()
        inputs = {i: O.random_mps(sp[4], sp[0], sp[1], sp[2], sp[3]) for i, sp in enumerate(specs)}

        def make_job(i):
            def job():
                N, d, chi, dt, seed = specs[i]
                st = E.SweepStats()
                sites = [torch.from_numpy(a) for a in inputs[i]]
                out, ln = E.compress(sites, chi // 2, stats=st, fold_norm=False)
                return {"bonds": [1] + [int(a.shape[2]) for a in out], "log_norm": ln,
                        "sites": [a.numpy() for a in out]}
            return job

        with cpu_ops():
            local = W.run_sharded(specs, make_job, lambda jobs: [j() for j in jobs], rank, world)
        merged = W.gather_results(local, world)
        if rank == 0:
            errs, bonds_ok = [], []
            for i, sp in enumerate(specs):
                r = merged[i]
                ref = O.svd_compress_method(O.left_canonise_qr(inputs[i]), sp[2] // 2)
                got = [a * (np.exp(r["log_norm"]) if j == 0 else 1.0) for j, a in enumerate(r["sites"])]
                errs.append(1.0 - O.fidelity(ref, got))
                bonds_ok.append(r["bonds"] == [1] + [a.shape[2] for a in ref])
                errs.append(abs(O.mps_norm(got) - O.mps_norm(ref)) / O.mps_norm(ref))
            out.put((sorted(merged), sorted(local), max(errs), all(bonds_ok)))
    finally:
        dist.destroy_process_group()


def _small_specs():
    import numpy as np
    rng = np.random.default_rng(4)
    return [(int(rng.integers(5, 11)), int(rng.choice([2, 3])), int(rng.integers(4, 11)),
             np.complex128 if b % 2 else np.float64, 7000 + b) for b in range(10)]


def test_sharded_uneven_batch_two_gloo_ranks():
    """The uneven batch run by the sharded executor on two ranks (CPU stand-in
    for the device ops): rank 0 gathers every instance's result, each equal
    to the oracle's svd_compress of that instance (fidelity, norm, bonds)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_sharded_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    merged, mine0, err, bonds_ok = q.get(timeout=10)
    assert merged == list(range(10))
    assert 0 < len(mine0) < 10            # rank 0 ran only its share
    assert err < 1e-10 and bonds_ok
