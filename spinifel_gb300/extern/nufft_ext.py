"""NUFFT operator object with the reference's surface
(spinifel/extern/nufft_ext.py:36-327):

    NUFFT(settings, pixel_position_reciprocal, pixel_distance_reciprocal,
          images_per_rank=None)
    .forward(ugrid, st, en, support, use_recip_sym, N) -> complex (N,)
    .adjoint(nuvect, H_, K_, L_, support, use_reciprocal_symmetry, M) -> M^3
    .update_fields(n_images_per_rank)
    .ref_orientations

Differences by design: the reference precomputes H, K, L of every reference
pixel on the host (nufft_ext.py:136-144; 78.6 GB at 1e5 x 65,536) and copies a
batch to the device per call; here the reference quaternions and the pixel
positions live on the device and the kernel rotates each pixel itself.
Reference orientations come from a seeded uniform sampler (skopi is not
available), or are passed in.

Precision follows the reference's settings: with use_single_prec (the
default) the NUFFTs run in FP32 at eps = 1e-6; without it they run in FP64 at
the reference's own eps = 1e-12 (nufft_ext.py:62) and the slices come back
in float64, as the reference's f_type = float64 run has them
(sequential/orientation_matching.py:32-36).  An explicit eps overrides this
(below 1e-7 the FP64 kernels are used).
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _arrays, geom
from ..nufft import FP32_EPS_FLOOR, make_plan

DEFAULT_EPS = 1e-6
REFERENCE_EPS = 1e-12


class NUFFT:
    def __init__(self, settings, pixel_position_reciprocal, pixel_distance_reciprocal,
                 images_per_rank=None, ref_orientations=None, eps=None, seed=None):
        self.N_orientations = settings.N_orientations
        self.N_batch_size = settings.N_batch_size
        self.reduced_det_shape = tuple(settings.reduced_det_shape)
        self.oversampling = settings.oversampling
        self.N_pixels = int(np.prod(self.reduced_det_shape))
        self.N_images = settings.N_images_per_rank if images_per_rank is None else images_per_rank
        if eps is None:
            eps = DEFAULT_EPS if getattr(settings, "use_single_prec", True) else REFERENCE_EPS
        self.eps = float(eps)
        self.fp64 = self.eps < FP32_EPS_FLOOR
        self.isign = -1
        ppr = np.asarray(pixel_position_reciprocal, dtype=np.float64)
        self.pixel_position_reciprocal = ppr
        if ref_orientations is None:
            rng = np.random.default_rng(seed)
            ref_orientations = geom.uniform_quaternions(self.N_orientations, rng)
        self.ref_orientations = np.asarray(ref_orientations)
        assert self.ref_orientations.shape == (self.N_orientations, 4)
        self.reciprocal_extent = float(np.max(pixel_distance_reciprocal))
        self.mult = np.pi / (self.oversampling * self.reciprocal_extent)
        # every rotated pixel lies within |q| <= max|q|, so |HKL| <= pi/oversampling
        assert float(np.sqrt((ppr ** 2).sum(axis=0)).max()) * self.mult < 3 * np.pi
        dev = _arrays.device()
        self._quats = torch.as_tensor(self.ref_orientations, dtype=torch.float32, device=dev)
        self._ppr = torch.as_tensor(ppr.reshape(3, -1), dtype=torch.float32, device=dev)
        if self.fp64:
            self._quats64 = torch.as_tensor(self.ref_orientations, dtype=torch.float64,
                                            device=dev)
            self._ppr64 = torch.as_tensor(ppr.reshape(3, -1), dtype=torch.float64, device=dev)
        self._plans = {}

    @property
    def dtype(self):
        """Device dtype of the slices: float64 at the reference's eps."""
        return torch.float64 if self.fp64 else torch.float32

    def plan(self, M):
        m = (M, M, M) if np.ndim(M) == 0 else tuple(M)
        p = self._plans.get(m)
        if p is None:
            p = self._plans[m] = make_plan(m, self.eps)
        return p

    def update_fields(self, n_images_per_rank):
        self.N_images = n_images_per_rank

    def set_model(self, ugrid, support=1):
        """Load the model for slicing (type 2 set-up); returns the plan."""
        g = ugrid
        if _arrays.is_torch(g) and torch.is_complex(g):
            g = g.real
        elif not _arrays.is_torch(g):
            g = np.real(g)
        g = _arrays.to_dev(g, self.dtype)
        P = self.plan(g.shape)
        P.set_modes(g, support, isign=self.isign, want_imag=False)
        return P

    def slice_real(self, P, st: int, en: int, out=None, out_bf16=None):
        """Real part of the type 2 at reference orientations st:en, [en-st, N_pixels]
        (float64 from an FP64 plan)."""
        if P.dtype == torch.float64:
            return P.slice(self._quats64[st:en], self._ppr64, self.mult, out=out)
        det = self.reduced_det_shape if len(self.reduced_det_shape) == 3 else None
        return P.slice(self._quats[st:en], self._ppr, self.mult, out=out, out_bf16=out_bf16,
                       det_shape=det)

    def forward(self, ugrid, st, en, support, use_recip_sym, N):
        if use_recip_sym:
            if _arrays.is_torch(ugrid):
                assert not torch.is_complex(ugrid) or bool((ugrid.imag == 0).all())
            else:
                assert np.all(np.isreal(ugrid))
        g = _arrays.to_dev(ugrid.real if _arrays.is_torch(ugrid) and torch.is_complex(ugrid)
                           else (np.real(ugrid) if not _arrays.is_torch(ugrid) else ugrid),
                           self.dtype)
        P = self.plan(g.shape)
        P.set_modes(g, support, isign=self.isign, want_imag=True)
        H, K, L = geom.hkl(self.ref_orientations[st:en], self.pixel_position_reciprocal)
        x, y, z = (torch.as_tensor(a.reshape(-1) * self.mult, dtype=self.dtype,
                                   device=g.device) for a in (H, K, L))
        re, im = P.interp(x, y, z, want_imag=True)
        assert re.numel() == N
        return torch.complex(re, im)

    def adjoint(self, nuvect, H_, K_, L_, support, use_reciprocal_symmetry, M):
        """Type 1 onto M^3 (isign -1), times support, real part, / M^3
        (nufft_ext.py:287-327); returns a device tensor."""
        from .. import autocorrelation as ac

        assert tuple(np.shape(H_)) == tuple(np.shape(K_)) == tuple(np.shape(L_))
        c = nuvect if _arrays.is_torch(nuvect) else torch.as_tensor(np.asarray(nuvect),
                                                                    device=_arrays.device())
        out = ac.adjoint(c, H_, K_, L_, M, use_recip_sym=use_reciprocal_symmetry,
                         support=support, eps=self.eps, isign=self.isign, plan=self.plan(M))
        return out
