"""Sharding realizations over ranks (world size 2, gloo on CPU): the summed
count grids equal one process's, and the Philox draws are shard-independent."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import golden

from onekapy_gb300.shard import reduce_counts, shard_range


def test_shard_range_covers_everything_once():
    for nreal in (0, 1, 7, 100, 10001):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                f, n = shard_range(nreal, r, world)
                seen.extend(range(f, f + n))
            assert seen == list(range(nreal))
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def test_philox_draws_do_not_depend_on_the_shard(oracle_mod):
    u_all = [oracle_mod.philox_uniforms(42, r, 3) for r in range(20)]
    f, n = shard_range(20, 1, 2)
    assert [oracle_mod.philox_uniforms(42, r, 3) for r in range(f, f + n)] == u_all[f:f + n]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import oracle
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    d = golden("track_confined_u10.npz")
    g = d["grid"]
    grid = (g[0], g[1], g[2], g[3], int(g[4]), int(g[5]))
    f, n = shard_range(d["coef"].shape[0], rank, world)
    aq = np.stack([d["K"], d["n"], d["H"]], axis=1)
    r = oracle.track(d["wells"][:, :2], d["coef"][f:f + n], d["q"][f:f + n], aq[f:f + n], d["release"], grid,
                     duration=float(d["duration"]), tol=1.0, maxstep=10.0, umbra=10.0, confined=True,
                     nthreads=1)
    counts = torch.from_numpy(r["counts"])
    reg = torch.tensor([r["registered"]], dtype=torch.int64)
    reduce_counts(counts, reg)
    if rank == 0:
        out.put((counts.numpy().copy(), int(reg.item())))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_reduction_equals_single_process():
    d = golden("track_confined_u10.npz")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    counts, reg = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert reg == int(d["total_weight"])
    assert np.array_equal(counts, d["counts"])
