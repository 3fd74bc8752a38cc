"""Replicas on several GPUs, tested on the CPU: two gloo ranks each take their work-balanced
pair range of one batch, compute it (the CPU oracle stands in for the GPU engine here)
and all-gather the results; the gathered arrays equal a single-process run."""
import os
import socket

import numpy as np
import pytest

from ogx import replicas, workloads as W


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_bounds_balanced():
    b = W.powerlaw(seed=3, n_pairs=5000)
    for world in (1, 2, 3, 8):
        bd = replicas.shard_bounds(b.counts, b.pairs, world)
        assert bd[0] == 0 and bd[-1] == b.n_pairs and np.all(np.diff(bd) >= 0)
        w = b.pair_vertex_counts()
        loads = np.array([w[bd[r]:bd[r + 1]].sum() for r in range(world)])
        assert loads.max() - loads.min() <= 2 * w.max()
    assert replicas.shard(b.counts, b.pairs, 1, 0) == (0, b.n_pairs)


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    from oracle import orc
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b = W.ellipsoid(seed=12, n_pairs=3000)
        bounds = replicas.shard_bounds(b.counts, b.pairs, world)
        lo, hi = int(bounds[rank]), int(bounds[rank + 1])
        mine = orc.run(b.coords, b.offsets, b.counts, b.pairs[lo:hi], mode=orc.MODE_GJK_EPA, precision="f32")
        full = replicas.all_gather_rows(mine, bounds)
        dist.barrier()
        if rank == 0:
            np.save(out_path, full)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_equals_single_run(tmp_path):
    import torch.multiprocessing as mp
    from oracle import orc
    out = str(tmp_path / "gathered.npy")
    mp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    b = W.ellipsoid(seed=12, n_pairs=3000)
    ref = orc.run(b.coords, b.offsets, b.counts, b.pairs, mode=orc.MODE_GJK_EPA, precision="f32")
    assert got.shape == ref.shape
    for f in ("dist", "wit", "normal", "nvrtx"):
        a, r = got[f], ref[f]
        assert np.all((a == r) | (np.isnan(a) & np.isnan(r))), f
