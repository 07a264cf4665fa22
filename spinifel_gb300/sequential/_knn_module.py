"""Shared body of the pyCudaKNearestNeighbors_SP / _DP modules
(spinifel/sequential/orientation_matching_sp.cu:612-737): host numpy in,
host numpy out, device compute.  Unlike the reference these check sizes,
raise on errors and print nothing."""
from __future__ import annotations

import numpy as np
import torch

from .. import matching


def _dev(deviceId: int) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("pyCudaKNearestNeighbors needs a CUDA device")
    return torch.device("cuda", int(deviceId))


def euclidean_distance(dtype, refImgs, dataImgs, numRefImgs, numDataImgs, totalPixels, deviceId):
    dev = _dev(deviceId)
    ref = np.ascontiguousarray(np.asarray(refImgs, dtype=dtype).reshape(-1))
    dat = np.ascontiguousarray(np.asarray(dataImgs, dtype=dtype).reshape(-1))
    if ref.size != numRefImgs * totalPixels or dat.size != numDataImgs * totalPixels:
        raise ValueError("array sizes do not match numRefImgs/numDataImgs/totalPixels")
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    with torch.cuda.device(dev):
        r = torch.as_tensor(ref, device=dev, dtype=tdt).reshape(numRefImgs, totalPixels)
        d = torch.as_tensor(dat, device=dev, dtype=tdt).reshape(numDataImgs, totalPixels)
        out = matching.knn_eudist(r, d)
        return out.reshape(-1).cpu().numpy()


def heap_sort(dtype, euDist, numDataImgs, numRefImgs, totalPixels, totalNN, deviceId):
    dev = _dev(deviceId)
    e = np.ascontiguousarray(np.asarray(euDist, dtype=dtype).reshape(-1))
    if e.size != numDataImgs * numRefImgs:
        raise ValueError("euDist size does not match numDataImgs * numRefImgs")
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    with torch.cuda.device(dev):
        t = torch.as_tensor(e, device=dev, dtype=tdt).reshape(numDataImgs, numRefImgs)
        idx = matching.knn_topk(t, int(totalNN))
        return idx.reshape(-1).cpu().numpy()
