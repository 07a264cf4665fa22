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

The product paths: match_sharded runs the library's matcher (bf16 tensor
cores + exact FP32 re-rank, or the plain FP32 pass) on this rank's shard of
the references and merges the ranks' exact bests; merge_setup_sharded spreads
this rank's points for the merge's two type-1 NUFFTs and sums the results
over the ranks; ShardedDirectOperator applies the direct merge operator with
the points sharded (one all-reduce of the data term per application) and
sharded_cg runs scipy's CG steps on it.

The collectives go through torch.distributed (NCCL on GPUs; gloo in the CPU
tests of this module's host logic); every function that communicates takes
an optional `reduce` / `gather` so that the host logic can also be driven
without a process group.
"""
from __future__ import annotations

import math

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


def local_best(frames, refs, path: str = "bf16"):
    """This rank's exact best per frame over its reference shard `refs`
    (a matching.ReferenceSet; None or empty: no references): distances
    [n_img, 1] (float32, +inf without references) and shard-local indices
    [n_img, 1] (int64, -1 without references).  path "bf16": the tensor-core
    top-8 + exact re-rank (the plain path's answer); "fp32": the plain pass."""
    from . import matching

    n = frames.n
    dev = frames.f32.device
    if refs is None or refs.n_ref == 0:
        return (torch.full((n, 1), math.inf, dtype=torch.float32, device=dev),
                torch.full((n, 1), -1, dtype=torch.int64, device=dev))
    if path == "bf16":
        idx, d = matching.match_bf16(frames, refs)
    elif path == "fp32":
        idx, d = matching.argmin_fp32(frames.f32, refs.f32, images_sq=frames.sq,
                                      refs_sq=refs.sq)
    else:
        raise ValueError("path must be 'bf16' or 'fp32'")
    return d.reshape(n, 1), idx.to(torch.int64).reshape(n, 1)


def match_sharded(frames, refs_shard, lo: int, path: str = "bf16", group=None, local=None,
                  gather=None):
    """Best reference per frame when every rank holds the contiguous slice
    [lo, lo + refs_shard.n_ref) of the references (reference-sharded SNM,
    spinifel/mpi/orientation_matching.py:7-16 with the orientations split
    instead of the images).  Each rank matches all frames against its shard
    with the library's kernels (local_best, or `local` for a stand-in), the
    shard-local indices are offset by lo (a shard without references reports
    +inf), one all-gather of (distance, global index) per frame follows, and
    the lexicographic minimum is the single-GPU argmin (lower index on ties).
    gather(d, i) -> ([world, n, 1], [world, n, 1]) replaces the all-gather."""
    if local is None:
        d, i = local_best(frames, refs_shard, path)
    else:
        d, i = local(frames, refs_shard)
    i = torch.where(i >= 0, i + int(lo), torch.full_like(i, -1))
    d = torch.where(i >= 0, d, torch.full_like(d, math.inf))
    gd, gi = (gather or (lambda a, b: all_gather_candidates(a, b, group)))(d, i)
    return merge_candidates(gd, gi)


def merge_setup_sharded(H_, K_, L_, data, support, M: int, M_ups: int, nufft, group=None,
                        reduce=None):
    """The merge's two type-1 NUFFTs with the points sharded (each rank
    passes its own points H_, K_, L_ in radians and their data values): the
    Toeplitz kernel ugrid_conv (type 1 of ones onto M_ups modes) and A^H b
    (type 1 of the data onto M modes, times the support), each summed over
    the ranks -- the type 1 is linear in the strengths, so the sum is the
    adjoint over all points (the reference's reduce + bcast of these vectors,
    spinifel/mpi/work_autocorrelation.py:18-24).  nufft: an extern NUFFT
    object (its adjoint and precision).  Returns device tensors."""
    ones = torch.ones(H_.numel(), dtype=nufft.dtype, device=H_.device)
    ugrid_conv = nufft.adjoint(ones, H_, K_, L_, 1, True, M_ups)
    adb = nufft.adjoint(data, H_, K_, L_, support, True, M).reshape(-1)
    red = reduce or (lambda t: allreduce_grid(t, group))
    red(ugrid_conv)
    red(adb)
    return ugrid_conv, adb


class ShardedDirectOperator:
    """W x = sum over ranks of the data term S.Re T1(D T2(S.x)) over each
    rank's points + rlambda x + flambda S.reg(S.x): op_data is this rank's
    merge.MergeOperator with rlambda = flambda = 0 and its points attached
    (set_direct), op_reg an operator on the same grid with the ranks' common
    rlambda / flambda and a zero Toeplitz kernel.  One all-reduce of the data
    term per application (the reference's core_problem: Bcast of uvect,
    local ADA, reduce + bcast, spinifel/mpi/work_autocorrelation.py:27-34)."""

    def __init__(self, op_data, op_reg, group=None, reduce=None):
        self.op_data, self.op_reg = op_data, op_reg
        self.reduce = reduce or (lambda t: allreduce_grid(t, group))

    def apply(self, x: torch.Tensor) -> torch.Tensor:
        y = self.op_data.apply(x, form=1)
        self.reduce(y)
        return y + self.op_reg.apply(x, form=0)


def sharded_cg(apply, b: torch.Tensor, x0: torch.Tensor, maxiter: int, rtol: float = 1e-5):
    """scipy.sparse.linalg.cg's steps (spinifel/sequential/autocorrelation.py:217)
    in FP64 on the device for an operator given as apply(x) (every rank runs
    the same iteration on the reduced operator).  Returns x and ||r|| at the
    start of each iteration."""
    b = b.to(torch.float64).reshape(-1)
    x = x0.to(torch.float64).reshape(-1).clone()
    r = b - apply(x) if bool(x.any()) else b.clone()
    atol = rtol * float(b.norm())
    hist = []
    p = None
    rho_prev = None
    for _ in range(maxiter):
        nr = float(r.norm())
        hist.append(nr)
        if nr < atol:
            break
        rho = float(r @ r)
        p = r.clone() if p is None else r + (rho / rho_prev) * p
        q = apply(p)
        alpha = rho / float(p @ q)
        x += alpha * p
        r -= alpha * q
        rho_prev = rho
    return x, hist
