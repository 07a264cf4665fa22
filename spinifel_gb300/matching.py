"""Device-level orientation matching: distances between images and reference
slices and the per-image best reference.

Plain FP32 path (the drop-in for SNM.euclidean_dist + argmin,
spinifel/sequential/orientation_matching.py:98-109,179):
    dist(i, r) = ||x_i||^2 + ||s_r||^2 - 2 x_i . s_r
computed by a SIMT FP32 tiled kernel with the argmin fused into its epilogue
(no distance matrix is stored); ties go to the lower reference index, as
numpy/cupy argmin does.
"""
from __future__ import annotations

import torch

from . import _lib


def row_sqnorm(x: torch.Tensor) -> torch.Tensor:
    _lib.require_cuda(x, "x", torch.float32)
    out = torch.empty(x.shape[0], device=x.device, dtype=torch.float32)
    _lib.call("spf_row_sqnorm_f32", _lib.ptr(x), x.shape[0], x[0].numel() if x.shape[0] else 0,
              _lib.ptr(out), _lib.stream_handle())
    return out


def ingest_u16(counts: torch.Tensor, out_f32: torch.Tensor, out_bf16=None, out_sq=None):
    """uint16 photon counts (held in an int16 or uint16 tensor) -> FP32 frames
    (and optionally bf16 frames and FP32 squared norms)."""
    if counts.dtype not in (torch.int16, torch.uint16):
        raise TypeError("counts must be a 16-bit integer tensor (uint16 bit pattern)")
    _lib.require_cuda(counts, "counts")
    _lib.require_cuda(out_f32, "out_f32", torch.float32)
    if out_f32.numel() != counts.numel():
        raise ValueError("out_f32 size differs from counts")
    n_img = counts.shape[0]
    n_pix = counts.numel() // max(n_img, 1)
    _lib.call("spf_frames_ingest_u16", _lib.ptr(counts), n_img, n_pix, _lib.ptr(out_f32),
              _lib.ptr(out_bf16), _lib.ptr(out_sq), _lib.stream_handle())
    return out_f32


class BestTracker:
    """Running (distance, index) minimum per image across reference batches."""

    def __init__(self, n_img: int, device):
        self.n_img = n_img
        self.best = torch.empty(n_img, device=device, dtype=torch.int64)
        _lib.call("spf_best_init", _lib.ptr(self.best), n_img, _lib.stream_handle())

    def update_fp32(self, img, img_sq, ref, ref_sq, ref_offset: int):
        n_pix = img.shape[1]
        if ref.shape[1] != n_pix:
            raise ValueError("images and references have different pixel counts")
        _lib.call("spf_dist_argmin_f32", _lib.ptr(img), _lib.ptr(img_sq), img.shape[0],
                  _lib.ptr(ref), _lib.ptr(ref_sq), ref.shape[0], n_pix, int(ref_offset),
                  _lib.ptr(self.best), _lib.stream_handle())

    def result(self):
        idx = torch.empty(self.n_img, device=self.best.device, dtype=torch.int32)
        dist = torch.empty(self.n_img, device=self.best.device, dtype=torch.float32)
        _lib.call("spf_best_unpack", _lib.ptr(self.best), self.n_img, _lib.ptr(idx),
                  _lib.ptr(dist), _lib.stream_handle())
        return idx, dist


def argmin_fp32(images: torch.Tensor, refs: torch.Tensor, images_sq=None, refs_sq=None):
    """Index of the nearest reference for every image (plain FP32 path)."""
    _lib.require_cuda(images, "images", torch.float32)
    _lib.require_cuda(refs, "refs", torch.float32)
    if images_sq is None:
        images_sq = row_sqnorm(images)
    if refs_sq is None:
        refs_sq = row_sqnorm(refs)
    t = BestTracker(images.shape[0], images.device)
    t.update_fp32(images, images_sq, refs, refs_sq, 0)
    return t.result()


def knn_eudist(ref: torch.Tensor, data: torch.Tensor) -> torch.Tensor:
    """[n_data, n_ref] sum over the first 16*floor(P/16) pixels of (d - r)^2."""
    if ref.dtype != data.dtype:
        raise TypeError("ref and data dtypes differ")
    name = {torch.float32: "spf_knn_eudist_f32", torch.float64: "spf_knn_eudist_f64"}[ref.dtype]
    out = torch.empty(data.shape[0], ref.shape[0], device=ref.device, dtype=ref.dtype)
    _lib.call(name, _lib.ptr(ref), _lib.ptr(data), ref.shape[0], data.shape[0], ref.shape[1],
              _lib.ptr(out), _lib.stream_handle())
    return out


def knn_topk(dist: torch.Tensor, k: int) -> torch.Tensor:
    name = {torch.float32: "spf_knn_topk_f32", torch.float64: "spf_knn_topk_f64"}[dist.dtype]
    out = torch.empty(dist.shape[0], k, device=dist.device, dtype=torch.int32)
    _lib.call(name, _lib.ptr(dist), dist.shape[0], dist.shape[1], int(k), _lib.ptr(out),
              _lib.stream_handle())
    return out
