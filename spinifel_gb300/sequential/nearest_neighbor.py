"""nearest_neighbor with the reference's surface
(spinifel/sequential/nearest_neighbor.py:103-145).

The reference's CUDA branch (detector >= 16 pixels) builds the full
[n_images, n_refs] distance matrix with the KNN module batch by batch and
takes the 1-nearest neighbour; its CPU branch uses sklearn
euclidean_distances + argmin.  Here both run on the GPU: with >= 16 pixels the
KNN-module semantics (sum of squared differences over the first
16*floor(P/16) pixels, lower index on ties); below 16 pixels the FP32
GEMM-form distance over all pixels (what the sklearn branch computes).
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _arrays, matching


def generate_weights(pixel_position_reciprocal, order=0):
    s_magnitudes = np.linalg.norm(pixel_position_reciprocal, axis=0) * 1e-10
    weights = 1.0 / (s_magnitudes ** order)
    weights /= np.sum(weights)
    return weights


def nearest_neighbor(model_slices, slices, batch_size):
    if _arrays.is_torch(slices):
        dt = torch.float64 if slices.dtype == torch.float64 else torch.float32
    else:
        dt = torch.float64 if np.asarray(slices).dtype == np.float64 else torch.float32
    ref = _arrays.to_dev(model_slices, dt)
    dat = _arrays.to_dev(slices, dt)
    n_ref, n_img = ref.shape[0], dat.shape[0]
    if dat.shape[1] >= 16:
        euDist = torch.empty(n_img, n_ref, device=ref.device, dtype=dt)
        nb = n_ref // batch_size
        for i in range(nb):
            st, en = i * batch_size, (i + 1) * batch_size
            euDist[:, st:en] = matching.knn_eudist(ref[st:en], dat)
        if nb * batch_size < n_ref:
            # the reference leaves these columns at zero (nearest_neighbor.py:115-123);
            # computing them is the only sensible drop-in behaviour
            euDist[:, nb * batch_size:] = matching.knn_eudist(ref[nb * batch_size:], dat)
        index = matching.knn_topk(euDist, 1)[:, 0]
    else:
        index, _ = matching.argmin_fp32(dat.float(), ref.float())
    return index.cpu().numpy().astype(np.int64)
