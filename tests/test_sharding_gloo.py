"""Multi-rank host logic on CPU with the gloo backend (world size 2): shard
ranges, the reference-sharded matching (sharding.match_sharded: offsets,
empty shards, the all-gather and the tie rule), the sharded merge set-up
(merge_setup_sharded) and the sharded direct operator with its CG
(ShardedDirectOperator, sharded_cg) give the single-rank answer.  The
per-rank GPU work (the matcher, the NUFFT adjoints, the operator's data term)
is replaced by CPU stand-ins injected by the test; the kernels themselves are
checked against the same decomposition on the GPU in
tests/test_gpu_sharding.py."""
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


class _Frames:
    """What match_sharded reads of a frame set: the frame count."""

    def __init__(self, x):
        self.x = x
        self.n = x.shape[0]


class _Shard:
    def __init__(self, r):
        self.r = r
        self.n_ref = r.shape[0]


def _cpu_best(fr, shard):
    """Stand-in for the GPU matcher: exact best per frame over the shard
    (lower index on ties), +inf / -1 without references."""
    if shard.n_ref == 0:
        return (torch.full((fr.n, 1), float("inf"), dtype=torch.float64),
                torch.full((fr.n, 1), -1, dtype=torch.int64))
    d = ((fr.x[:, None, :] - shard.r[None, :, :]) ** 2).sum(-1)
    v, i = torch.min(d, dim=1)  # first minimum: the lower index
    return v[:, None].contiguous(), i[:, None].to(torch.int64).contiguous()


class _FakeNufft:
    """Stand-in for the extern NUFFT's adjoint: a fixed linear map of the
    strengths onto an m^3 grid (its output is linear in the strengths, like a
    type 1)."""

    dtype = torch.float64

    def adjoint(self, c, H_, K_, L_, support, use_recip_sym, M):
        base = torch.arange(M ** 3, dtype=torch.float64).reshape((M,) * 3)
        s = float((c.to(torch.float64) * (1.0 + H_.to(torch.float64) ** 2)).sum())
        out = torch.cos(base * 0.1) * s
        return out * (support if not isinstance(support, (int, float)) else float(support))


class _DataOp:
    """Stand-in for a rank's direct-form data term: A_r x (a symmetric PSD
    block of the full operator)."""

    def __init__(self, A):
        self.A = A

    def apply(self, x, form=0):
        assert form == 1
        return self.A @ x


class _RegOp:
    def __init__(self, R):
        self.R = R

    def apply(self, x, form=0):
        assert form == 0
        return self.R @ x


def _worker(rank, world, port, refs, frames, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from spinifel_gb300.sharding import (ShardedDirectOperator, allreduce_grid, match_sharded,
                                             merge_setup_sharded, shard_range, sharded_argmin,
                                             sharded_cg)

        def local_match(fr, lo, hi):
            r = refs[lo:hi]
            d = ((fr[:, None, :] - r[None, :, :]) ** 2).sum(-1)  # [n_img, hi-lo]
            k = min(4, hi - lo)
            vals, idx = torch.sort(d, dim=1, stable=True)
            return vals[:, :k].contiguous(), idx[:, :k].contiguous()

        bd, bi = sharded_argmin(local_match, frames, refs.shape[0])
        g = torch.full((5, 5, 5), float(rank + 1))
        allreduce_grid(g)
        # the product matching path with its host logic (offsets, empty shard)
        lo, hi = shard_range(refs.shape[0], rank, world)
        md, mi = match_sharded(_Frames(frames), _Shard(refs[lo:hi]), lo, local=_cpu_best)
        lo1, hi1 = shard_range(1, rank, world)  # one reference: rank 1's shard is empty
        ed, ei = match_sharded(_Frames(frames), _Shard(refs[lo1:hi1]), lo1, local=_cpu_best)
        # sharded merge set-up: each rank's points, summed adjoints
        pts = torch.linspace(-1.0, 1.0, 10, dtype=torch.float64)
        plo, phi = shard_range(10, rank, world)
        Hs = pts[plo:phi]
        uc, adb = merge_setup_sharded(Hs, Hs, Hs, torch.arange(10.0)[plo:phi], 1, 3, 4,
                                      _FakeNufft())
        # sharded operator + CG: W = A_0 + A_1 + R
        gen = torch.Generator().manual_seed(71)
        B = [torch.randn(6, 6, generator=gen, dtype=torch.float64) for _ in range(world)]
        A = [b @ b.T for b in B]
        R = 0.5 * torch.eye(6, dtype=torch.float64)
        op = ShardedDirectOperator(_DataOp(A[rank]), _RegOp(R))
        rhs = torch.arange(1.0, 7.0, dtype=torch.float64)
        xs, hist = sharded_cg(op.apply, rhs, torch.zeros(6, dtype=torch.float64), 6, rtol=1e-12)
        if rank == 0:
            out["idx"] = bi.numpy().copy()
            out["dist"] = bd.numpy().copy()
            out["grid"] = float(g[0, 0, 0])
            out["m_idx"] = mi.numpy().copy()
            out["m_dist"] = md.numpy().copy()
            out["e_idx"] = ei.numpy().copy()
            out["ugrid_conv"] = uc.numpy().copy()
            out["adb"] = adb.numpy().copy()
            out["x"] = xs.numpy().copy()
            out["W"] = (sum(A) + R).numpy()
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
    # match_sharded: global indices, duplicate across shards -> the lower one
    np.testing.assert_array_equal(out["m_idx"], np.argmin(d, axis=1))
    np.testing.assert_allclose(out["m_dist"], d.min(axis=1), rtol=1e-12)
    assert out["m_idx"][0] == 3
    np.testing.assert_array_equal(out["e_idx"], np.zeros(11, dtype=np.int64))
    # merge set-up: the ranks' summed adjoints are the all-points adjoint
    pts = torch.linspace(-1.0, 1.0, 10, dtype=torch.float64)
    fake = _FakeNufft()
    np.testing.assert_allclose(out["ugrid_conv"],
                               fake.adjoint(torch.ones(10), pts, pts, pts, 1, True, 4).numpy(),
                               rtol=1e-12)
    np.testing.assert_allclose(out["adb"],
                               fake.adjoint(torch.arange(10.0), pts, pts, pts, 1, True,
                                            3).reshape(-1).numpy(), rtol=1e-12)
    # sharded CG on W = A_0 + A_1 + R: the solution of the full system
    np.testing.assert_allclose(out["W"] @ out["x"], np.arange(1.0, 7.0), rtol=1e-8)
