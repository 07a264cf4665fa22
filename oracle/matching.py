"""ORACLE -- test infrastructure only.

Orientation-matching semantics of the reference, restated in numpy FP64:

* sklearn_argmin: euclidean_distances(model_slices, slices) + argmin(axis=0),
  the reference's CPU branch (spinifel/sequential/nearest_neighbor.py:134-135);
  euclidean_distances computes ||x||^2 - 2 x.y + ||y||^2 (clipped at 0);
  sklearn_argmin_stream does the same over references given in blocks.
* snm_dist: SNM's dist = x2 + y2 - 2 x.y over orientation batches with the
  per-batch std rescale (spinifel/sequential/orientation_matching.py:148-179).
* knn_topk: the CUDA KNN top-k (orientation_matching_sp.cu:535-609):
  k smallest per row ascending, the lower index on ties.
* ties_equal: the parity rule for argmins -- indices must agree, or the two
  references' oracle distances must agree within a relative tolerance.
"""
from __future__ import annotations

import numpy as np


def sq_dists(a: np.ndarray, b: np.ndarray, block: int = 4096) -> np.ndarray:
    """[len(a), len(b)] squared distances ||a||^2 + ||b||^2 - 2 a.b in FP64."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    a2 = np.einsum("ij,ij->i", a, a)
    b2 = np.einsum("ij,ij->i", b, b)
    out = np.empty((a.shape[0], b.shape[0]))
    for s in range(0, a.shape[0], block):
        e = min(s + block, a.shape[0])
        out[s:e] = a2[s:e, None] + b2[None, :] - 2.0 * (a[s:e] @ b.T)
    return out


def sklearn_argmin(model_slices, slices):
    """argmin over references of the squared distance, per image (FP64)."""
    d = np.maximum(sq_dists(model_slices, slices), 0.0)  # [n_ref, n_img]
    return np.argmin(d, axis=0), d


def sklearn_argmin_stream(blocks, slices):
    """sklearn_argmin over references that arrive in blocks (an iterable of
    [B_i, P] arrays in reference order), so that no [n_ref, n_img] matrix is
    held: per image the index of the smallest euclidean_distances value
    (sqrt of the clipped GEMM form, as nearest_neighbor.py:134-135 computes
    it) and its squared distance; the lower index wins ties, as np.argmin's
    first occurrence does.  Returns (index, squared distance, references seen)."""
    y = np.asarray(slices, dtype=np.float64)
    y2 = np.einsum("ij,ij->i", y, y)
    best = np.full(y.shape[0], np.inf)
    best_sq = np.full(y.shape[0], np.inf)
    idx = np.full(y.shape[0], -1, dtype=np.int64)
    cols = np.arange(y.shape[0])
    start = 0
    for blk in blocks:
        b = np.asarray(blk, dtype=np.float64)
        d = np.einsum("ij,ij->i", b, b)[:, None] + y2[None, :] - 2.0 * (b @ y.T)
        np.maximum(d, 0.0, out=d)
        e = np.sqrt(d)
        m = np.argmin(e, axis=0)
        v = e[m, cols]
        upd = v < best
        best[upd] = v[upd]
        best_sq[upd] = d[m, cols][upd]
        idx[upd] = m[upd] + start
        start += b.shape[0]
    return idx, best_sq, start


def snm_argmin(batches, slices):
    """SNM semantics given the model-slice batches (each [B, P], unscaled)."""
    slices = np.asarray(slices, dtype=np.float64)
    std = slices.std()
    rows = []
    for b in batches:
        b = np.asarray(b, dtype=np.float64)
        b = b * (std / b.std())
        rows.append(sq_dists(b, slices))
    dist = np.concatenate(rows, axis=0)  # [n_orient, n_img]
    return np.argmin(dist, axis=0), dist


def knn_topk(dist: np.ndarray, k: int) -> np.ndarray:
    """k smallest per row, ascending by (value, index)."""
    dist = np.asarray(dist)
    order = np.lexsort((np.broadcast_to(np.arange(dist.shape[1]), dist.shape), dist), axis=1)
    return order[:, :k].astype(np.int32)


def ties_equal(idx_a, idx_b, dist, rtol=1e-6, axis_ref=0):
    """True where idx_a == idx_b or their distances agree within rtol.

    dist is [n_ref, n_img] (axis_ref=0) or [n_img, n_ref] (axis_ref=1)."""
    idx_a = np.asarray(idx_a).astype(np.int64)
    idx_b = np.asarray(idx_b).astype(np.int64)
    cols = np.arange(idx_a.size)
    if axis_ref == 0:
        da, db = dist[idx_a, cols], dist[idx_b, cols]
    else:
        da, db = dist[cols, idx_a], dist[cols, idx_b]
    return (idx_a == idx_b) | (np.abs(da - db) <= rtol * np.maximum(np.abs(da), np.abs(db)))
