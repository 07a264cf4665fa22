"""Forward (type 2) and adjoint (type 1) operators of the autocorrelation
merge, with the reference's signatures (spinifel/autocorrelation.py).

forward(ugrid, H_, K_, L_, support, use_recip_sym, N)      :32-61
adjoint(nuvect, H_, K_, L_, M, use_recip_sym=True, support=None)  :97-128
gen_nonuniform_positions / gen_nonuniform_normalized_positions   :290-323

The NUFFT runs on the GPU (libspinifel_gb300) at tolerance `eps`: FP32
kernels from the default 1e-6 (the GB300 path's specified tolerance) down to
about 1e-7, FP64 kernels below that, down to the 1e-12 in double that the
reference asks finufft for.  Inputs may be numpy arrays (results come back
as numpy) or CUDA tensors (results stay on the device).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _arrays, geom
from .nufft import NufftPlan, make_plan

DEFAULT_EPS = 1e-6
_plans: dict = {}


def plan_for(M, eps=DEFAULT_EPS) -> NufftPlan:
    m = (M, M, M) if np.ndim(M) == 0 else tuple(M)
    key = (m, float(eps), torch.cuda.current_device())
    p = _plans.get(key)
    if p is None:
        p = make_plan(m, eps)
        _plans[key] = p
    return p


def _numel(a) -> int:
    return a.numel() if _arrays.is_torch(a) else int(np.size(a))


def _max_abs(*arrs) -> float:
    return max(float(a.abs().max()) if _arrays.is_torch(a) else float(np.max(np.abs(a)))
               for a in arrs)


def forward(ugrid, H_, K_, L_, support, use_recip_sym, N, eps=DEFAULT_EPS):
    """Type 2, isign -1: nuvect_j = sum_k (ugrid*support)_k exp(-i k.(H,K,L)_j)."""
    if _numel(H_):
        assert _max_abs(H_, K_, L_) < 3 * np.pi
    if use_recip_sym:
        if _arrays.is_torch(ugrid):
            assert not torch.is_complex(ugrid) or bool((ugrid.imag == 0).all())
        else:
            assert np.all(np.isreal(ugrid))
    g = _arrays.to_dev(ugrid.real if _arrays.is_torch(ugrid) and torch.is_complex(ugrid)
                       else (np.real(ugrid) if not _arrays.is_torch(ugrid) else ugrid),
                       torch.float64)
    P = plan_for(g.shape, eps)
    P.set_modes(g, support, isign=-1, want_imag=True)
    x, y, z = (_arrays.to_dev(np.asarray(a).reshape(-1) if not _arrays.is_torch(a) else a,
                              torch.float64) for a in (H_, K_, L_))
    re, im = P.interp(x, y, z, want_imag=True)
    out = torch.complex(re, im)
    assert out.numel() == N
    return _arrays.like_input(out, ugrid)


# from this many points on, the adjoint bin-sorts them once and spreads with
# the sorted kernel (points sharing a footprint cell summed in registers)
# instead of one thread per point with global atomics
SORTED_SPREAD_MIN_POINTS = 1 << 21


def adjoint(nuvect, H_, K_, L_, M, use_recip_sym=True, support=None, eps=DEFAULT_EPS,
            isign=+1, plan=None, sort=None):
    """Type 1 onto M^3 (isign +1), times support, real part, divided by M^3.
    sort: None picks the sorted spreading for large point sets; True / False
    forces it on or off."""
    if _numel(H_):
        assert _max_abs(H_, K_, L_) < 3 * np.pi
    P = plan if plan is not None else plan_for(M, eps)
    x, y, z = (_arrays.to_dev(np.asarray(a).reshape(-1) if not _arrays.is_torch(a) else a,
                              P.dtype) for a in (H_, K_, L_))
    c = nuvect if _arrays.is_torch(nuvect) else torch.as_tensor(np.asarray(nuvect))
    c = c.to(_arrays.device()).reshape(-1)
    cre = (c.real if torch.is_complex(c) else c).to(P.dtype).contiguous()
    cim = c.imag.to(P.dtype).contiguous() if torch.is_complex(c) else None
    use_sorted = (x.numel() >= SORTED_SPREAD_MIN_POINTS) if sort is None else bool(sort)
    use_sorted = use_sorted and P.supports_sort
    if use_sorted:
        P.sort_points(x, y, z)

    def spread(values):
        if use_sorted:
            P.spread_sorted(values)
        else:
            P.spread(x, y, z, values)

    P.spread_zero()
    spread(cre)
    fr_re, fr_im = P.finish(isign, want_imag=True)
    re, im = fr_re, fr_im
    if cim is not None and bool((cim != 0).any()):
        P.spread_zero()
        spread(cim)
        fi_re, fi_im = P.finish(isign, want_imag=True)
        re = fr_re - fi_im
        im = fr_im + fi_re
    if support is not None:
        s = _arrays.to_dev(support, P.dtype) if not isinstance(support, (int, float)) else support
        re = re * s
        im = im * s
    out = re if use_recip_sym else torch.complex(re, im)
    out = out / float(M) ** 3
    return _arrays.like_input(out, nuvect)


def gen_nonuniform_positions(orientations, pixel_position_reciprocal):
    if orientations.shape[0] > 0:
        return geom.hkl(orientations, pixel_position_reciprocal)
    print("WARNING: gen_nonuniform_positions got empty orientation - returning h,k,l for "
          "Null rotation")
    return geom.hkl(np.zeros((0, 4)), pixel_position_reciprocal)


def gen_nonuniform_normalized_positions(orientations, pixel_position_reciprocal,
                                        reciprocal_extent, oversampling):
    H, K, L = gen_nonuniform_positions(orientations, pixel_position_reciprocal)
    s = np.pi / reciprocal_extent / oversampling
    return H.flatten() * s, K.flatten() * s, L.flatten() * s
