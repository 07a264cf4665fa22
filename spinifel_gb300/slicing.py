"""Model slices at given orientations with the reference's surface
(spinifel/slicing.py:10-95):

    gen_model_slices(ac, ref_orientations, pixel_position_reciprocal,
                     reciprocal_extent, oversampling, ac_support_size,
                     N_pixels, override_forward_with)            -> (N,)  :10-50
    gen_model_slices_batch(..., batch_size=None,
                           override_forward_with=None)             -> (N,)  :54-95

N = N_pixels * N_orientations, the slices laid out orientation-major as the
reference returns them (the real part of the type-2 NUFFT at the rotated,
normalised pixel positions).  The reference's function calls
autocorrelation.forward with arguments that function no longer takes
(:32-41); here the slices come from the fused slicing kernel, which rotates
every pixel by R(q)^-1 itself and scales by pi / (reciprocal_extent *
oversampling) (gen_nonuniform_normalized_positions, autocorrelation.py:
311-323).  override_forward_with None or "gpu" runs it; "cpu" is refused:
this package has no CPU path.  eps selects the tolerance: 1e-6 (FP32, the
default) or down to the reference's own 1e-12 (FP64 kernels, float64
slices).  ac_support_size is accepted for the signature and, as in the
reference (:27-28), defaults to the grid size; the support is 1.
Numpy inputs give numpy outputs; CUDA tensors stay on the device.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _arrays
from .nufft import make_plan


def gen_model_slices(ac, ref_orientations, pixel_position_reciprocal, reciprocal_extent,
                     oversampling, ac_support_size, N_pixels, override_forward_with=None,
                     eps: float = 1e-6):
    if override_forward_with not in (None, "gpu"):
        raise ValueError(f"override_forward_with={override_forward_with!r}: only the GPU "
                         "kernels exist here")
    q = np.asarray(ref_orientations) if not _arrays.is_torch(ref_orientations) \
        else ref_orientations
    n_orient = int(q.shape[0])
    ppr = pixel_position_reciprocal
    ppr_shape = tuple(ppr.shape)
    assert int(np.prod(ppr_shape[1:])) == int(N_pixels), "N_pixels differs from the detector"
    if ac_support_size is None:
        ac_support_size = ac.shape[0]
    g = ac.real if (_arrays.is_torch(ac) and torch.is_complex(ac)) else \
        (np.real(ac) if not _arrays.is_torch(ac) else ac)
    plan = make_plan(tuple(g.shape), eps)
    dt = plan.dtype
    plan.set_modes(_arrays.to_dev(g, dt))
    mult = float(np.pi / float(reciprocal_extent) / float(oversampling))
    det = ppr_shape[1:] if len(ppr_shape) == 4 else None
    out = plan.slice(_arrays.to_dev(q, dt), _arrays.to_dev(ppr, dt).reshape(3, -1), mult,
                     det_shape=det)
    return _arrays.like_input(out.reshape(n_orient * int(N_pixels)), ac)


def gen_model_slices_batch(ac, ref_orientations, pixel_position_reciprocal, reciprocal_extent,
                           oversampling, ac_support_size, N_pixels, batch_size=None,
                           override_forward_with=None, eps: float = 1e-6):
    n_orient = int(ref_orientations.shape[0])
    nb = n_orient if batch_size is None else int(batch_size)
    assert n_orient % nb == 0, \
        f"N_orientations ({n_orient}) must be divisible by N_batch_size ({nb})"
    parts = [gen_model_slices(ac, ref_orientations[st:st + nb], pixel_position_reciprocal,
                              reciprocal_extent, oversampling, ac_support_size, N_pixels,
                              override_forward_with, eps)
             for st in range(0, n_orient, nb)]
    if _arrays.is_torch(parts[0]):
        return torch.cat(parts)
    return np.concatenate(parts)
