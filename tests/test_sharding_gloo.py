"""Multi-rank host logic on CPU with the gloo backend (world size 2): shard
ranges, the reference-sharded argmin exchange and the spread-grid all-reduce
give the single-rank answer.  The per-rank distance computation here is a
numpy stand-in injected by the test (the product path has none); it checks
the decomposition, not the kernels."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from spinifel_gb300.sharding import merge_candidates, shard_range


def test_shard_ranges_cover_everything():
    for n in (0, 1, 7, 100, 101):
        for w in (1, 2, 3, 8):
            parts = [shard_range(n, r, w) for r in range(w)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[r][1] == parts[r + 1][0] for r in range(w - 1))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1


def test_merge_candidates_tie_rule():
    d = torch.tensor([[[1.0, 5.0]], [[1.0, 2.0]]])  # two ranks, one frame, k=2
    i = torch.tensor([[[9, 3]], [[4, 8]]])
    bd, bi = merge_candidates(d, i)
    assert bd.item() == 1.0 and bi.item() == 4  # equal distance -> lower index


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, refs, frames, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from spinifel_gb300.sharding import allreduce_grid, sharded_argmin

        def local_match(fr, lo, hi):
            r = refs[lo:hi]
            d = ((fr[:, None, :] - r[None, :, :]) ** 2).sum(-1)  # [n_img, hi-lo]
            k = min(4, hi - lo)
            vals, idx = torch.sort(d, dim=1, stable=True)
            return vals[:, :k].contiguous(), idx[:, :k].contiguous()

        bd, bi = sharded_argmin(local_match, frames, refs.shape[0])
        g = torch.full((5, 5, 5), float(rank + 1))
        allreduce_grid(g)
        if rank == 0:
            out["idx"] = bi.numpy().copy()
            out["dist"] = bd.numpy().copy()
            out["grid"] = float(g[0, 0, 0])
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_reference_sharded_argmin_equals_single_rank(world):
    rng = np.random.default_rng(70)
    refs = torch.as_tensor(rng.random((37, 16)))
    refs[30] = refs[3]  # duplicate across shards: the lower index must win
    frames = torch.as_tensor(rng.random((11, 16)))
    frames[0] = refs[3]
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), refs, frames, out), nprocs=world,
                       join=True, start_method="spawn")
    d = ((frames[:, None, :] - refs[None, :, :]) ** 2).sum(-1).numpy()
    np.testing.assert_array_equal(out["idx"], np.argmin(d, axis=1))
    assert out["idx"][0] == 3
    assert out["grid"] == float(sum(range(1, world + 1)))
