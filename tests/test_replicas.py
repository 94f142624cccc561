"""Replica sharding across ranks (host logic, gloo on CPU, world size 2).

Each rank integrates its contiguous shard of the batch (here with the CPU
oracle standing in for the engine, which needs a GPU) and the results are
gathered; the gathered batch equals the single-process run, and the
objective all-reduce equals the sum over all conditions."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from amici_gb300.replicas import shard_range


def test_shard_range_partitions():
    for n in (0, 1, 7, 1024, 1025):
        for world in (1, 2, 3, 8):
            ranges = [shard_range(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_path):
    import torch.distributed as dist

    from amici_gb300.networks import robertson_workload
    from amici_gb300.replicas import allreduce_objective, gather_shards
    from oracle.pyoracle import Oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n = 5
    w = robertson_workload(n)
    p = w.p * (1 + 0.01 * np.arange(n))[:, None]
    base = Oracle(w.model).run(w.p[:1], w.pscale, w.k[:1], w.ts[:1], rtol=1e-8, atol=1e-12)
    my = base["y"] + np.random.default_rng(1).normal(0, 0.01, base["y"].shape)
    a, b = shard_range(n, rank, world)
    r = Oracle(w.model).run(p[a:b], w.pscale, w.k[a:b], w.ts[a:b], my, rtol=1e-8, atol=1e-12, sensi=1)
    full = gather_shards({"x": r["x"], "llh": r["llh"], "sllh": r["sllh"], "status": r["status"]}, n)
    llh_sum, sllh_sum = allreduce_objective(r["llh"], r["sllh"])
    if rank == 0:
        np.savez(out_path, p=p, my=my, llh_sum=llh_sum, sllh_sum=sllh_sum, **full)
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_gather_equals_single_process(tmp_path):
    from amici_gb300.networks import robertson_workload
    from oracle.pyoracle import Oracle

    out = str(tmp_path / "gathered.npz")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    g = dict(np.load(out))
    w = robertson_workload(5)
    ref = Oracle(w.model).run(g["p"], w.pscale, w.k, w.ts, g["my"], rtol=1e-8, atol=1e-12, sensi=1)
    np.testing.assert_array_equal(g["x"], ref["x"])
    np.testing.assert_array_equal(g["llh"], ref["llh"])
    np.testing.assert_array_equal(g["sllh"], ref["sllh"])
    np.testing.assert_allclose(g["llh_sum"], ref["llh"].sum(), rtol=1e-14)
    np.testing.assert_allclose(g["sllh_sum"], ref["sllh"].sum(axis=0), rtol=1e-13)
