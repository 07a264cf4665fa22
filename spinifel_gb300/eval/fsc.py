"""compute_fsc with the reference's signature (eval/fsc.py:67-125): the
transforms and shell sums run on the GPU (spf_eval_fsc_shells, FP64); the
0.5-crossing interpolation is the reference's scipy interp1d on the host."""
from __future__ import annotations

import numpy as np
import scipy.interpolate
import torch

from .. import _lib


def get_reciprocal_mesh(voxel_number_1d, distance_reciprocal_max, xp=np):
    """fsc.py:10-33."""
    ls = xp.linspace(-distance_reciprocal_max, distance_reciprocal_max, voxel_number_1d)
    return xp.moveaxis(xp.asarray(xp.meshgrid(ls, ls, ls, indexing="ij")), 0, -1)


def fsc_curve(volume1, volume2, distance_reciprocal_max, spacing=0.01):
    """rshell, fsc and the per-shell sums [n, 3] (Re F1 conj F2, |F1|^2, |F2|^2)."""
    M = int(np.asarray(volume1).shape[0])
    ls = np.linspace(-distance_reciprocal_max, distance_reciprocal_max, M)
    corner = np.array([[ls[0], ls[0], ls[0]]])
    smax = float(np.linalg.norm(corner, axis=-1)[0] * 1e-10)  # the mesh's largest |q|
    r_spacings = np.arange(0, smax / np.sqrt(3), spacing)
    n = len(r_spacings)
    dev = torch.device("cuda", torch.cuda.current_device())
    v1 = torch.as_tensor(np.asarray(volume1, dtype=np.float64), device=dev).contiguous()
    v2 = torch.as_tensor(np.asarray(volume2, dtype=np.float64), device=dev).contiguous()
    coord = torch.as_tensor(ls, dtype=torch.float64, device=dev)
    sums = torch.empty(max(n, 1), 3, dtype=torch.float64, device=dev)
    if n:
        _lib.call("spf_eval_fsc_shells", _lib.ptr(v1), _lib.ptr(v2), M, _lib.ptr(coord), 1e-10,
                  float(spacing), n, _lib.ptr(sums), _lib.stream_handle())
    s = sums[:n].cpu().numpy()
    with np.errstate(invalid="ignore", divide="ignore"):
        fsc = s[:, 0] / np.sqrt(s[:, 1] * s[:, 2])
    rshell = r_spacings + 0.5 * spacing
    return rshell, fsc, s


def compute_fsc(volume1, volume2, distance_reciprocal_max, spacing=0.01):
    """(resolution in Angstrom or -1, rshell, fsc), as the reference."""
    rshell, fsc, _ = fsc_curve(volume1, volume2, distance_reciprocal_max, spacing)
    f = scipy.interpolate.interp1d(fsc, rshell)
    try:
        resolution = float(1.0 / f(0.5))
    except ValueError:
        resolution = -1
    return resolution, rshell, fsc
