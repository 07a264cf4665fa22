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

import ctypes

import numpy as np
import torch

from . import _lib


def row_sqnorm(x: torch.Tensor) -> torch.Tensor:
    _lib.require_cuda(x, "x", torch.float32)
    out = torch.empty(x.shape[0], device=x.device, dtype=torch.float32)
    _lib.call("spf_row_sqnorm_f32", _lib.ptr(x), x.shape[0], x[0].numel() if x.shape[0] else 0,
              _lib.ptr(out), _lib.stream_handle())
    return out


def ingest_u16(counts: torch.Tensor, out_f32: torch.Tensor, out_bf16=None, out_sq=None,
               out_n4=None):
    """uint16 photon counts (held in an int16 or uint16 tensor) -> FP32 frames
    (and optionally bf16 frames with a padded row stride, FP32 squared norms
    and sqrt(sum x^4))."""
    if counts.dtype not in (torch.int16, torch.uint16):
        raise TypeError("counts must be a 16-bit integer tensor (uint16 bit pattern)")
    _lib.require_cuda(counts, "counts")
    _lib.require_cuda(out_f32, "out_f32", torch.float32)
    if out_f32.numel() != counts.numel():
        raise ValueError("out_f32 size differs from counts")
    n_img = counts.shape[0]
    n_pix = counts.numel() // max(n_img, 1)
    ld = out_bf16.shape[-1] if out_bf16 is not None else n_pix
    _lib.call("spf_frames_ingest_u16", _lib.ptr(counts), n_img, n_pix, _lib.ptr(out_f32),
              _lib.ptr(out_bf16), ld, _lib.ptr(out_sq), _lib.ptr(out_n4), _lib.stream_handle())
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


class BestTracker64:
    """FP64 running (distance, index) minimum per image across reference
    batches, for matching at the reference's double precision: each batch's
    [n_img, n_ref] distance block (dist_f64) is folded in by
    spf_argmin_rows_f64 (lower index on ties, earlier batches kept on ties)."""

    def __init__(self, n_img: int, device):
        self.n_img = n_img
        self.best_dist = torch.empty(n_img, device=device, dtype=torch.float64)
        self.best_idx = torch.empty(n_img, device=device, dtype=torch.int64)
        _lib.call("spf_best64_init", _lib.ptr(self.best_dist), _lib.ptr(self.best_idx), n_img,
                  _lib.stream_handle())

    def update_block(self, dist: torch.Tensor, ref_offset: int):
        _lib.require_cuda(dist, "dist", torch.float64)
        if dist.dim() != 2 or dist.shape[0] != self.n_img:
            raise ValueError("dist must be [n_img, n_ref]")
        _lib.call("spf_argmin_rows_f64", _lib.ptr(dist), dist.shape[0], dist.shape[1],
                  int(ref_offset), _lib.ptr(self.best_dist), _lib.ptr(self.best_idx),
                  _lib.stream_handle())

    def update_fp64(self, img, ref, ref_offset: int, work: torch.Tensor | None = None):
        """Fold the distances of img [n_img, n_pix] to ref [n_ref, n_pix]."""
        self.update_block(dist_f64(ref, img, out=work), ref_offset)

    def result(self):
        return self.best_idx, self.best_dist


def dist_f64(ref: torch.Tensor, data: torch.Tensor, out: torch.Tensor | None = None):
    """[n_data, n_ref] sums over all pixels of (data - ref)^2 in FP64."""
    _lib.require_cuda(ref, "ref", torch.float64)
    _lib.require_cuda(data, "data", torch.float64)
    if ref.shape[0] and data.shape[0] and ref[0].numel() != data[0].numel():
        raise ValueError("images and references have different pixel counts")
    n_pix = data[0].numel() if data.shape[0] else (ref[0].numel() if ref.shape[0] else 0)
    if out is None:
        out = torch.empty(data.shape[0], ref.shape[0], device=ref.device, dtype=torch.float64)
    _lib.require_cuda(out, "out", torch.float64)
    if out.numel() != data.shape[0] * ref.shape[0]:
        raise ValueError("out has the wrong size")
    _lib.call("spf_dist_f64", _lib.ptr(ref), _lib.ptr(data), ref.shape[0], data.shape[0], n_pix,
              _lib.ptr(out), _lib.stream_handle())
    return out.view(data.shape[0], ref.shape[0])


def argmin_fp64(images: torch.Tensor, refs: torch.Tensor, batch: int = 4096):
    """Index (int64) and FP64 distance of the nearest reference for every
    image, references taken in batches of `batch` rows."""
    t = BestTracker64(images.shape[0], images.device)
    work = None
    for st in range(0, refs.shape[0], batch):
        blk = refs[st:st + batch]
        if work is None or work.numel() != images.shape[0] * blk.shape[0]:
            work = torch.empty(images.shape[0] * blk.shape[0], device=images.device,
                               dtype=torch.float64)
        t.update_fp64(images, blk, st, work)
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


# ---------------------------------------------------------------------------
# BF16 tensor-core path with exact FP32 re-rank
# ---------------------------------------------------------------------------

def gather_rows(src: torch.Tensor, rows: torch.Tensor, out: torch.Tensor | None = None,
                stream=None) -> torch.Tensor:
    """out[i] = src[rows[i]] along the first axis, with the library's gather
    kernel (rows: int64 device tensor)."""
    _lib.require_cuda(src, "src")
    rows = rows.to(torch.int64)
    _lib.require_cuda(rows, "rows")
    n = rows.numel()
    if out is None:
        out = torch.empty((n,) + tuple(src.shape[1:]), dtype=src.dtype, device=src.device)
    row_bytes = src[0].numel() * src.element_size() if src.shape[0] else 0
    _lib.call("spf_gather_rows", _lib.ptr(src), src.shape[0], row_bytes, _lib.ptr(rows), n,
              _lib.ptr(out), _lib.stream_handle(stream))
    return out


def row_norms(x: torch.Tensor):
    """(sum x^2, sqrt(sum x^4)) per row, FP32 results."""
    _lib.require_cuda(x, "x", torch.float32)
    n = x.shape[0]
    sq = torch.empty(n, device=x.device, dtype=torch.float32)
    n4 = torch.empty(n, device=x.device, dtype=torch.float32)
    _lib.call("spf_row_norms_f32", _lib.ptr(x), n, x[0].numel() if n else 0, _lib.ptr(sq),
              _lib.ptr(n4), _lib.stream_handle())
    return sq, n4


def to_bf16_padded(x: torch.Tensor, ld: int | None = None) -> torch.Tensor:
    """bf16 copy of [rows, n_pix] FP32 with a row stride that is a multiple of 8."""
    _lib.require_cuda(x, "x", torch.float32)
    n, p = x.shape
    ld = ld or (p + 7) // 8 * 8
    out = torch.empty(n, ld, device=x.device, dtype=torch.bfloat16)
    _lib.call("spf_f32_to_bf16", _lib.ptr(x), n, p, _lib.ptr(out), ld, _lib.stream_handle())
    return out


def check_device_error():
    """Raise if a bounded device wait of this library has timed out."""
    import ctypes

    code = ctypes.c_int(0)
    _lib.call("spf_device_error", _lib.stream_handle(), ctypes.byref(code))
    if code.value:
        raise _lib.SpfError(-code.value, "device", "a bounded device wait gave up")


class ReferenceSet:
    """Reference slices resident in HBM: FP32 rows (exact re-rank and the plain
    path), a bf16 copy for the tensor cores (row stride padded to 8), squared
    norms, and for the re-rank certificate the per-pixel max of s^2 and the
    largest squared norm."""

    def __init__(self, refs_f32: torch.Tensor, refs_bf16: torch.Tensor | None = None):
        _lib.require_cuda(refs_f32, "refs_f32", torch.float32)
        self.f32 = refs_f32
        self.n_ref, self.n_pix = refs_f32.shape
        self.ld = (self.n_pix + 7) // 8 * 8
        if refs_bf16 is None:
            refs_bf16 = to_bf16_padded(refs_f32, self.ld)
        if tuple(refs_bf16.shape) != (self.n_ref, self.ld):
            raise ValueError("bf16 copy must be [n_ref, ld]")
        self.bf16 = refs_bf16
        self._stats()

    def _stats(self):
        self.sq = row_sqnorm(self.f32)
        self.m2 = torch.empty(self.n_pix, dtype=torch.float32, device=self.f32.device)
        _lib.call("spf_col_maxsq_f32", _lib.ptr(self.f32), self.n_ref, self.n_pix,
                  _lib.ptr(self.m2), _lib.stream_handle())
        self.sq_max = float(self.sq.max().item()) if self.n_ref else 0.0

    def rescale(self, factor: float):
        """Multiply every slice by factor (FP32, bf16 and statistics kept consistent)."""
        self.f32 *= factor
        self.bf16.copy_(to_bf16_padded(self.f32, self.ld))
        self._stats()


class FrameSet:
    """Frames prepared for matching: FP32, bf16 (padded), norms."""

    def __init__(self, f32: torch.Tensor, ld: int | None = None, bf16=None, sq=None, n4=None):
        _lib.require_cuda(f32, "frames", torch.float32)
        self.f32 = f32
        self.n, self.n_pix = f32.shape
        self.ld = ld or (self.n_pix + 7) // 8 * 8
        self.bf16 = bf16 if bf16 is not None else to_bf16_padded(f32, self.ld)
        if sq is None or n4 is None:
            sq, n4 = row_norms(f32)
        self.sq, self.n4 = sq, n4

    @classmethod
    def from_counts(cls, counts: torch.Tensor, ld: int | None = None, out=None):
        """Frames from uint16 photon counts (int16/uint16 tensor on the device);
        `out` (a FrameSet of the same shape) is reused when given."""
        n, p = counts.shape
        ld = ld or (p + 7) // 8 * 8
        if out is None:
            dev = counts.device
            out = cls.__new__(cls)
            out.n, out.n_pix, out.ld = n, p, ld
            out.f32 = torch.empty(n, p, dtype=torch.float32, device=dev)
            out.bf16 = torch.empty(n, ld, dtype=torch.bfloat16, device=dev)
            out.sq = torch.empty(n, dtype=torch.float32, device=dev)
            out.n4 = torch.empty(n, dtype=torch.float32, device=dev)
        ingest_u16(counts, out.f32, out.bf16, out.sq, out.n4)
        return out


class _Workspace:
    def __init__(self):
        self.bufs = {}

    def get(self, name, numel, dtype, device):
        t = self.bufs.get((name, device))
        if t is None or t.numel() < numel or t.dtype != dtype:
            t = torch.empty(max(numel, 1), dtype=dtype, device=device)
            self.bufs[(name, device)] = t
        return t[:numel]


_ws = _Workspace()


def match_bf16(frames: FrameSet, refs: ReferenceSet, exact_fallback: bool = True,
               stats: dict | None = None, stream=None):
    """Best reference per frame: bf16 tensor-core distances, per-frame top-8,
    exact FP32 re-rank (bit-identical to the plain path's values); frames the
    certificate cannot settle are completed exactly from the kept per-tile
    candidate lists (spf_complete_open: list re-rank, and the range GEMM or
    the plain pass only where those lists may hide references)."""
    if frames.n_pix != refs.n_pix or frames.ld != refs.ld:
        raise ValueError("frames and references differ in pixel count")
    dev = frames.f32.device
    n_img = frames.n
    tiles = int(_lib.lib().spf_dist_topk_bf16_tiles(refs.n_ref))
    cand_d = _ws.get("cand_d", tiles * n_img * 8, torch.float32, dev)
    cand_i = _ws.get("cand_i", tiles * n_img * 8, torch.int32, dev)
    mrg_d = _ws.get("merged_d", n_img * 8, torch.float32, dev)
    mrg_i = _ws.get("merged_i", n_img * 8, torch.int32, dev)
    work = _ws.get("rerank_work", n_img, torch.float32, dev)
    idx = torch.empty(n_img, dtype=torch.int32, device=dev)
    dist = torch.empty(n_img, dtype=torch.float32, device=dev)
    unc = torch.empty(n_img, dtype=torch.int32, device=dev)
    sh = _lib.stream_handle(stream)
    _lib.call("spf_dist_topk_bf16", _lib.ptr(frames.bf16), n_img, _lib.ptr(refs.bf16), refs.n_ref,
              refs.n_pix, refs.ld, _lib.ptr(refs.sq), _lib.ptr(cand_d), _lib.ptr(cand_i), sh)
    _lib.call("spf_rerank_fp32_keep", _lib.ptr(cand_d), _lib.ptr(cand_i), tiles,
              _lib.ptr(frames.f32), _lib.ptr(frames.sq), n_img, _lib.ptr(refs.f32),
              _lib.ptr(refs.sq), _lib.ptr(refs.m2), float(refs.sq_max), refs.n_ref, refs.n_pix,
              0, _lib.ptr(work), _lib.ptr(idx), _lib.ptr(dist), _lib.ptr(unc), _lib.ptr(mrg_d),
              _lib.ptr(mrg_i), sh)
    if exact_fallback or stats is not None:
        bad = torch.nonzero(unc, as_tuple=False).flatten()
        nbad = int(bad.numel())
        if stats is not None:
            stats["uncertified"] = nbad
        if exact_fallback and nbad:
            i2 = torch.empty(nbad, dtype=torch.int32, device=dev)
            d2 = torch.empty(nbad, dtype=torch.float32, device=dev)
            hs = np.zeros(3, dtype=np.int64)
            _lib.call("spf_complete_open", _lib.ptr(cand_d), _lib.ptr(cand_i), tiles,
                      _lib.ptr(frames.bf16), _lib.ptr(frames.f32), _lib.ptr(frames.sq),
                      _lib.ptr(work), n_img, _lib.ptr(bad), nbad, _lib.ptr(refs.bf16),
                      _lib.ptr(refs.f32), _lib.ptr(refs.sq), refs.n_ref, refs.n_pix, refs.ld,
                      _lib.ptr(i2), _lib.ptr(d2), ctypes.c_void_p(hs.ctypes.data), sh)
            idx.index_copy_(0, bad, i2)
            dist.index_copy_(0, bad, d2)
            if stats is not None:
                stats["range_gemm_frames"] = int(hs[0])
                stats["range_overflow"] = int(hs[1])
    return idx, dist


RANGE_CAP = 512


def match_bf16_host(frames_u16_host: torch.Tensor, refs: ReferenceSet, chunk_frames: int = 0,
                    stream=None, stats: dict | None = None):
    """Host frames in, host indices out, in one library call
    (spf_match_bf16_host): chunked host -> device copies overlapped with the
    tensor-core matching of the previous chunk.  frames_u16_host: [n, n_pix]
    16-bit counts in host memory (pinned for the overlap).  chunk_frames > 0:
    fixed chunks; 0: fixed chunks of 2,560 frames; < 0: chunks doubling
    from -chunk_frames.  Returns numpy (indices int32, distances float32), the
    plain FP32 path's answer."""
    if frames_u16_host.is_cuda or frames_u16_host.dtype not in (torch.int16, torch.uint16):
        raise TypeError("frames must be 16-bit counts in host memory")
    if frames_u16_host.dim() != 2 or frames_u16_host.shape[1] != refs.n_pix:
        raise ValueError(f"frames must be [n, {refs.n_pix}]")
    f = frames_u16_host.contiguous()
    n = f.shape[0]
    idx = np.empty(n, dtype=np.int32)
    dist = np.empty(n, dtype=np.float32)
    st = np.zeros(3, dtype=np.int64)
    _lib.call("spf_match_bf16_host", ctypes.c_void_p(f.data_ptr()), n, _lib.ptr(refs.bf16),
              _lib.ptr(refs.f32), _lib.ptr(refs.sq), _lib.ptr(refs.m2), float(refs.sq_max),
              refs.n_ref, refs.n_pix, refs.ld, int(chunk_frames),
              ctypes.c_void_p(idx.ctypes.data), ctypes.c_void_p(dist.ctypes.data),
              ctypes.c_void_p(st.ctypes.data), _lib.stream_handle(stream))
    if stats is not None:
        stats["uncertified"] = int(st[0])
        stats["range_gemm_frames"], stats["range_overflow"] = int(st[1]), int(st[2])
    return idx, dist
