"""Slicing and orientation matching with the reference's surface
(spinifel/sequential/orientation_matching.py):

    SNM(settings, slices_, pixel_position_reciprocal,
        pixel_distance_reciprocal, nufft).slicing_and_match(ac) -> quats   :40-186
    slicing_and_match(ac, slices_, ppr, pdr, ref_orientations=None)         :189-256

SNM keeps the data images resident on the device in FP32 with their squared
norms and global std (:65-77).  For each batch of N_batch_size reference
orientations it slices the model with the fused type-2 kernel, rescales the
batch by slices_std / batch std (:165), and folds the batch's distances
x2 + s2 - 2 x.s into a per-image running (distance, index) minimum with the
plain FP32 distance kernel (:98-109, :179), so the N_orientations x N_slices
distance matrix is never stored.  Ties go to the lower orientation index, as
argmin(axis=0) does.

With a NUFFT at the reference's own tolerance (settings.use_single_prec
False, or an explicit eps below 1e-7) the same steps run in FP64, as the
reference's float64 run does (f_type, :32-36): FP64 slicing at eps 1e-12,
the std rescale in double and FP64 distances folded per batch into an FP64
running minimum, so the argmin is the reference's own up to ties at the
rounding level of double.
"""
from __future__ import annotations

import time

import numpy as np
import torch

from .. import _arrays, geom, matching
from ..extern.nufft_ext import NUFFT
from ..settings import settings as _default_settings
from . import nearest_neighbor as nn


class SNM:
    def __init__(self, settings, slices_, pixel_position_reciprocal, pixel_distance_reciprocal,
                 nufft):
        self.N_orientations = settings.N_orientations
        self.N_batch_size = settings.N_batch_size
        self.reduced_det_shape = tuple(settings.reduced_det_shape)
        self.oversampling = settings.oversampling
        self.N_pixels = int(np.prod(self.reduced_det_shape))
        self.N = self.N_pixels * self.N_orientations
        assert self.N_orientations % self.N_batch_size == 0, \
            "N_orientations must be divisible by N_batch_size"
        self.N_slices = slices_.shape[0]
        assert tuple(slices_.shape) == (self.N_slices,) + self.reduced_det_shape
        self.reciprocal_extent = float(np.max(pixel_distance_reciprocal))
        self.pixel_position_reciprocal = pixel_position_reciprocal
        self.fp64 = bool(getattr(nufft, "fp64", False))
        dt = torch.float64 if self.fp64 else torch.float32
        self.slices_ = _arrays.to_dev(slices_, dt).reshape(self.N_slices, self.N_pixels)
        if self.fp64:
            self.slices_2 = None
            self.slices_std = self.slices_.std(unbiased=False) if self.N_slices else None
        else:
            self.slices_2 = matching.row_sqnorm(self.slices_) if self.N_slices else None
            self.slices_std = (self.slices_.double().std(unbiased=False).float()
                               if self.N_slices else None)
        self.nufft = nufft
        self.timings = {}

    def capture(self, ac):
        """Record one generation (model set-up, every orientation batch's
        slicing, std rescale, distances and running argmin) as a CUDA graph
        on a static copy of the model; match_indices_graphed then replays it
        for each new model.  The launch sequence does not depend on the
        model, so one capture serves every generation of this SNM."""
        self._g_ac = _arrays.to_dev(np.real(ac) if not _arrays.is_torch(ac) else ac,
                                    self.nufft.dtype).clone()
        self.match_indices(self._g_ac)  # plans, module loading and workspaces outside the capture
        torch.cuda.synchronize()
        self._graph = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(self._graph, stream=s):
                self._g_idx = self.match_indices(self._g_ac)
        torch.cuda.current_stream().wait_stream(s)

    def match_indices_graphed(self, ac) -> torch.Tensor:
        """match_indices by replaying the captured generation (capture first)."""
        self._g_ac.copy_(_arrays.to_dev(np.real(ac) if not _arrays.is_torch(ac) else ac,
                                        self.nufft.dtype))
        self._graph.replay()
        return self._g_idx.clone()

    def match_indices(self, ac) -> torch.Tensor:
        """Best reference orientation index per image (device int32; int64
        in FP64 mode)."""
        P = self.nufft.set_model(ac, 1)
        B = self.N_batch_size
        if self.fp64:
            buf = torch.empty(B, self.N_pixels, device=self.slices_.device, dtype=torch.float64)
            work = torch.empty(self.N_slices * B, device=self.slices_.device,
                               dtype=torch.float64)
            best = matching.BestTracker64(self.N_slices, self.slices_.device)
            for i in range(self.N_orientations // B):
                st = i * B
                self.nufft.slice_real(P, st, st + B, out=buf)
                buf *= self.slices_std / buf.std(unbiased=False)
                best.update_fp64(self.slices_, buf, st, work)
            idx, _ = best.result()
            return idx
        buf = torch.empty(B, self.N_pixels, device=self.slices_.device, dtype=torch.float32)
        best = matching.BestTracker(self.N_slices, self.slices_.device)
        for i in range(self.N_orientations // B):
            st = i * B
            self.nufft.slice_real(P, st, st + B, out=buf)
            buf *= self.slices_std / buf.double().std(unbiased=False).float()
            buf_sq = matching.row_sqnorm(buf)
            best.update_fp32(self.slices_, self.slices_2, buf, buf_sq, st)
        idx, _ = best.result()
        return idx

    def slicing_and_match(self, ac):
        st_init = time.monotonic()
        if not self.N_slices:
            return np.zeros((0, 4))
        idx = self.match_indices(ac)
        index = idx.cpu().numpy().astype(np.int64)
        self.timings["total"] = time.monotonic() - st_init
        return self.nufft.ref_orientations[index]


def slicing_and_match(ac, slices_, pixel_position_reciprocal, pixel_distance_reciprocal,
                      ref_orientations=None, settings=None, seed=None):
    """Function path: all model slices, one global std scale (:245-248), then
    nearest_neighbor (:252)."""
    settings = settings or _default_settings
    N_orientations = settings.N_orientations
    N_batch_size = settings.N_batch_size
    N_pixels = int(np.prod(settings.reduced_det_shape))
    N_slices = slices_.shape[0]
    assert tuple(slices_.shape) == (N_slices,) + tuple(settings.reduced_det_shape)
    if not N_slices:
        return np.zeros((0, 4))
    if ref_orientations is None:
        ref_orientations = geom.uniform_quaternions(N_orientations, np.random.default_rng(seed))
    else:
        N_orientations = ref_orientations.shape[0]
    assert N_orientations % N_batch_size == 0, "N_orientations must be divisible by N_batch_size"
    nufft = NUFFT(settings, pixel_position_reciprocal, pixel_distance_reciprocal,
                  ref_orientations=ref_orientations)
    P = nufft.set_model(ac, 1)
    model_slices = torch.empty(N_orientations, N_pixels, device=nufft._quats.device,
                               dtype=nufft.dtype)
    for i in range(N_orientations // N_batch_size):
        st = i * N_batch_size
        nufft.slice_real(P, st, st + N_batch_size, out=model_slices[st:st + N_batch_size])
    data = _arrays.to_dev(np.asarray(slices_).reshape(N_slices, N_pixels), nufft.dtype)
    ratio = data.double().std(unbiased=False) / model_slices.double().std(unbiased=False)
    model_slices *= ratio.to(nufft.dtype)
    index = nn.nearest_neighbor(model_slices, data, N_batch_size)
    return ref_orientations[index]
