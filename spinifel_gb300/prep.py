"""Detector-data preparation with the reference's names (spinifel/prep.py):
clipping and 2^n x 2^n binning.  Frames (the per-event data that feeds
matching and serving) are binned on the GPU by spf_bin_frames_u16 in one
pass from uint16 counts; the per-detector geometry (pixel positions, index
maps; binned once) uses the numpy functions, which restate prep.py.

HDF5 input (prep.py:131-183: intensities, pixel_position_reciprocal,
pixel_index_map, orientations, volume) needs h5py, which is not a dependency
of this package; load_* read the same datasets from any mapping of dataset
name -> array (an h5py.File where h5py exists)."""
from __future__ import annotations

import numpy as np
import torch

from . import _lib


# ---- numpy restatements (geometry; prep.py:37-125) ------------------------
def bin2x2_sum(arr):
    return (arr[..., ::2, ::2] + arr[..., 1::2, ::2] + arr[..., ::2, 1::2]
            + arr[..., 1::2, 1::2])


def bin2x2_mean(arr):
    return bin2x2_sum(arr) / 4


def bin2x2_index(arr):
    arr = np.minimum(arr[..., ::2, :], arr[..., 1::2, :])
    arr = np.minimum(arr[..., ::2], arr[..., 1::2])
    return arr // 2


def bin2nx2n_sum(arr, n):
    for _ in range(n):
        arr = bin2x2_sum(arr)
    return arr


def bin2nx2n_mean(arr, n):
    for _ in range(n):
        arr = bin2x2_mean(arr)
    return arr


def bin2nx2n_index(arr, n):
    for _ in range(n):
        arr = bin2x2_index(arr)
    return arr


def clipping(arr, n):
    """Keep the low-resolution 1/2^n of each panel (prep.py:88-112)."""
    f = 2 ** n
    sa, sb = arr.shape[-2:]
    out = np.zeros(arr.shape[:-2] + (sa // f, sb // f), dtype=arr.dtype)
    if out.shape[1] == 4:
        out[..., 0, :, :] = arr[..., 0, -sa // f:, -sb // f:]
        out[..., 1, :, :] = arr[..., 1, -sa // f:, :sb // f]
        out[..., 2, :, :] = arr[..., 2, -sa // f:, -sb // f:]
        out[..., 3, :, :] = arr[..., 3, -sa // f:, :sb // f]
    elif out.shape[1] == 1:
        g = 2 * f
        out[..., 0, :, :] = arr[..., 0, sa // 2 - sa // g:sa // 2 + sa // g,
                                sb // 2 - sb // g:sb // 2 + sb // g]
    else:
        raise ValueError(f"clipping is defined for 1 or 4 panels, not {out.shape[1]}")
    return out


def clipping_index(arr, n):
    arr = clipping(arr, n)
    arr -= arr.min()
    return arr


def binning_sum(arr, settings):
    return bin2nx2n_sum(clipping(arr, settings.N_clipping), settings.N_binning)


def binning_mean(arr, settings):
    return bin2nx2n_mean(clipping(arr, settings.N_clipping), settings.N_binning)


def binning_index(arr, settings):
    return bin2nx2n_index(clipping_index(arr, settings.N_clipping), settings.N_binning)


def compute_pixel_distance(pixel_position_reciprocal):
    return np.sqrt((pixel_position_reciprocal ** 2).sum(axis=0))


def get_saxs(pixel_distance_reciprocal, mean_image):
    """Radial average in 100 bins (prep.py:13-23)."""
    qs = pixel_distance_reciprocal.flatten()
    N = 100
    q_max = qs.max()
    idx = (N * qs / q_max).astype(np.int64)
    acc = np.bincount(idx, mean_image.flatten(), N)
    wgt = np.bincount(idx, None, N)
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.linspace(0, q_max, N + 1), acc / wgt


# ---- device: frames ---------------------------------------------------------
def bin_frames(frames_u16: torch.Tensor, n_clip: int, n_bin: int, mean: bool = False,
               out: torch.Tensor | None = None) -> torch.Tensor:
    """Clip and bin [n_img, n_panels, sa, sb] uint16 (or int16 bit pattern)
    frames on the GPU -> float32 [n_img, n_panels, sa', sb']."""
    _lib.require_cuda(frames_u16, "frames_u16")
    if frames_u16.dtype not in (torch.int16, torch.uint16) or frames_u16.dim() != 4:
        raise TypeError("frames must be a 4-D 16-bit tensor [n_img, n_panels, sa, sb]")
    n, p, sa, sb = frames_u16.shape
    f = 2 ** n_clip
    ca, cb = (sa // f, sb // f) if not (p == 1 and n_clip) else \
        (2 * (sa // (2 * f)), 2 * (sb // (2 * f)))
    shape = (n, p, ca >> n_bin, cb >> n_bin)
    if out is None:
        out = torch.empty(shape, dtype=torch.float32, device=frames_u16.device)
    elif tuple(out.shape) != shape or out.dtype != torch.float32:
        raise ValueError(f"out must be float32 {shape}")
    _lib.call("spf_bin_frames_u16", _lib.ptr(frames_u16), n, p, sa, sb, int(n_clip), int(n_bin),
              int(bool(mean)), _lib.ptr(out), _lib.stream_handle())
    return out


# ---- datasets (prep.py:131-183) ---------------------------------------------
def load_pixel_position_reciprocal(source):
    ppr = np.asarray(source["pixel_position_reciprocal"][:])
    return ppr if ppr.shape[0] == 3 else np.moveaxis(ppr, -1, 0)


def load_pixel_index_map(source):
    return np.moveaxis(np.asarray(source["pixel_index_map"][:]), -1, 0)


def load_slices(source, i_start, i_end):
    data = source["intensities"]
    if data.shape[0] < i_end:
        raise ValueError(f"Not enough intensity slices (max:{data.shape[0]:d})")
    return np.asarray(data[i_start:i_end])


def load_orientations(source, i_start, i_end):
    return np.asarray(source["orientations"][i_start:i_end])
