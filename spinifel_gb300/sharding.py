"""Multi-GPU decomposition of the hot path (one process per GPU).

* Frames sharded, references replicated ("replicas"): every rank matches its
  own frames; no data-path collective (the reference's MPI model,
  spinifel/mpi/orientation_matching.py:7-16, where each rank matches the
  images it loaded).
* References sharded: every rank matches all frames against its contiguous
  slice of the references and re-ranks its own top-k exactly; one all-gather
  of k (distance, global index) pairs per frame, then each frame's global best
  is the lexicographic minimum (distance, index) -- the same tie rule as the
  single-GPU argmin.
* Type-1 spreading with the points sharded: each rank spreads its points onto
  its own copy of the fine grid and one all-reduce (sum) combines them before
  the FFT (the reference's Reduce + Bcast of the M^3 vector,
  spinifel/mpi/work_autocorrelation.py:18-30).

The collectives go through torch.distributed (NCCL on GPUs; gloo in the CPU
tests of this module's host logic).
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [lo, hi) share of n items; shares differ by at most one."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def merge_candidates(dists: torch.Tensor, idxs: torch.Tensor):
    """dists/idxs [world, n_img, k] -> per-frame (best distance, best index),
    lexicographic on (distance, index)."""
    w, n, k = dists.shape
    d = dists.permute(1, 0, 2).reshape(n, w * k)
    i = idxs.permute(1, 0, 2).reshape(n, w * k).to(torch.int64)
    big = torch.iinfo(torch.int64).max
    i = torch.where(torch.isfinite(d), i, torch.full_like(i, big))
    # sort by index first, then a stable sort by distance keeps the lower index on ties
    oi = torch.argsort(i, dim=1, stable=True)
    d1 = torch.gather(d, 1, oi)
    i1 = torch.gather(i, 1, oi)
    od = torch.argsort(d1, dim=1, stable=True)
    best = od[:, :1]
    return torch.gather(d1, 1, best).squeeze(1), torch.gather(i1, 1, best).squeeze(1)


def all_gather_candidates(local_d: torch.Tensor, local_i: torch.Tensor, group=None):
    """[n_img, k] per rank -> [world, n_img, k] on every rank."""
    world = dist.get_world_size(group)
    out_d = [torch.empty_like(local_d) for _ in range(world)]
    out_i = [torch.empty_like(local_i) for _ in range(world)]
    dist.all_gather(out_d, local_d.contiguous(), group=group)
    dist.all_gather(out_i, local_i.contiguous(), group=group)
    return torch.stack(out_d), torch.stack(out_i)


def sharded_argmin(local_match, frames, n_ref: int, group=None):
    """Best reference per frame with the references sharded over the group.

    local_match(frames, lo, hi) -> (dist [n_img, k], index [n_img, k]) with
    exact distances and indices relative to lo; ranks that hold no
    references return +inf distances."""
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    lo, hi = shard_range(n_ref, rank, world)
    d, i = local_match(frames, lo, hi)
    i = i.to(torch.int64) + lo
    gd, gi = all_gather_candidates(d, i, group)
    return merge_candidates(gd, gi)


def allreduce_grid(grid: torch.Tensor, group=None) -> torch.Tensor:
    """Sum the ranks' partial spread grids in place."""
    dist.all_reduce(grid, op=dist.ReduceOp.SUM, group=group)
    return grid
