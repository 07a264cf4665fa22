"""Merge with the reference's surface
(spinifel/sequential/autocorrelation.py:35-225):

    Merge(settings, slices_, pixel_position_reciprocal,
          pixel_distance_reciprocal, nufft).solve_ac(generation,
          orientations=None, ac_estimate=None) -> ac (M^3, real)

The linear system is the reference's: W = conv + rlambda I + flambda reg
with the Toeplitz kernel from the type 1 of ones onto the M_ups grid, and
d = A^H b + rlambda x0, solved by CG with scipy's stopping rule (rtol 1e-5,
maxiter = solve_ac_maxiter).  Everything after the orientation -> (H, K, L)
step stays on the device: the type-1 NUFFTs, the FFT convolution and a
device-resident CG whose vectors and dot products are FP64.
form="direct" applies W through type 2 -> type 1 NUFFTs every iteration
instead of the Toeplitz FFT (same operator for centrosymmetric x).

With a NUFFT at the reference's own tolerance (use_single_prec off: FP64 at
eps 1e-12) the two type-1 NUFFTs run in FP64 and the Toeplitz product in
FP64 too, so the solve is the reference's double-precision one; otherwise
the NUFFTs and the product are FP32 (CG vectors and dots FP64 either way).
"""
from __future__ import annotations

import numpy as np
import torch
from scipy.ndimage import gaussian_filter

from .. import _arrays, geom
from ..merge import MergeOperator, antisupport


class Merge:
    def __init__(self, settings, slices_, pixel_position_reciprocal, pixel_distance_reciprocal,
                 nufft, form: str = "toeplitz", seed=None):
        self.M = settings.M
        self.N_images = slices_.shape[0]
        self.N = int(np.prod(slices_.shape))
        self.reciprocal_extent = float(np.max(pixel_distance_reciprocal))
        self.use_reciprocal_symmetry = True
        self.maxiter = settings.solve_ac_maxiter
        self.oversampling = settings.oversampling
        self.M_ups = settings.M_ups
        self.pixel_position_reciprocal = np.array(pixel_position_reciprocal)
        self.mult = np.pi / (self.reciprocal_extent * settings.oversampling)
        self.rlambda = 1 / self.N / 1000
        self.flambda = 1e3
        self.data = _arrays.to_dev(np.asarray(slices_, dtype=np.float64).reshape(-1)
                                   if not _arrays.is_torch(slices_) else slices_.reshape(-1),
                                   torch.float64)
        self.F_antisupport = antisupport(self.M, settings.oversampling)
        self.nufft = nufft
        self.form = form
        self.rng = np.random.default_rng(seed)
        self.iterations = 0
        self.residuals = None
        self.op = None

    def get_non_uniform_positions(self, orientations):
        if orientations.shape[0] == 0:
            print("WARNING: gen_nonuniform_positions got empty orientation - returning h,k,l "
                  "for Null rotation")
        return geom.hkl(np.asarray(orientations).reshape(-1, 4), self.pixel_position_reciprocal)

    def setup_linops(self, H, K, L, ac_support, x0, orientations=None):
        dev = _arrays.device()
        fp64 = bool(getattr(self.nufft, "fp64", False))
        dt = torch.float64 if fp64 else torch.float32
        H_, K_, L_ = (torch.as_tensor(np.asarray(a).reshape(-1) * self.mult, dtype=dt,
                                      device=dev) for a in (H, K, L))
        ones = torch.ones(H_.numel(), dtype=dt, device=dev)
        ugrid_conv = self.nufft.adjoint(ones, H_, K_, L_, 1, self.use_reciprocal_symmetry,
                                        self.M_ups)
        sup = torch.as_tensor(np.asarray(ac_support, dtype=np.float32), device=dev)
        op = MergeOperator(self.M, self.M_ups, self.rlambda, self.flambda, sup,
                           self.F_antisupport)
        op.set_kernel(ugrid_conv, fp64=fp64)
        if self.form == "direct":
            assert orientations is not None
            # a plan of its own: the operator keeps its bin-sorted points for
            # the whole solve, while the adjoints below sort on the shared one
            from ..nufft import NufftPlan

            plan = NufftPlan(self.M, max(self.nufft.eps, 1e-6))
            det = tuple(self.pixel_position_reciprocal.shape[1:])
            op.set_direct(plan, torch.as_tensor(orientations, dtype=torch.float32, device=dev),
                          torch.as_tensor(self.pixel_position_reciprocal.reshape(3, -1),
                                          dtype=torch.float32, device=dev), self.mult,
                          det_shape=det if len(det) == 3 else None)
        sup_t = sup.to(dt) if fp64 else sup
        uvect_ADb = self.nufft.adjoint(self.data, H_, K_, L_, sup_t,
                                       self.use_reciprocal_symmetry, self.M).reshape(-1)
        d = uvect_ADb.double() + self.rlambda * x0
        self.op = op
        return op, d

    def solve_ac(self, generation, orientations=None, ac_estimate=None):
        if orientations is None:
            orientations = geom.uniform_quaternions(self.N_images, self.rng)
        H, K, L = self.get_non_uniform_positions(orientations)
        if ac_estimate is None:
            ac_support = np.ones((self.M,) * 3)
            ac_estimate = np.zeros((self.M,) * 3)
        else:
            ac_estimate = np.asarray(ac_estimate, dtype=np.float64)
            ac_smoothed = gaussian_filter(ac_estimate, 0.5)
            ac_support = (ac_smoothed > 1e-12).astype(np.float64)
            ac_estimate = ac_estimate * ac_support
        dev = _arrays.device()
        x0 = torch.as_tensor(ac_estimate.reshape(-1), dtype=torch.float64, device=dev)
        op, d = self.setup_linops(H, K, L, ac_support, x0, orientations)
        form = op.DIRECT if self.form == "direct" else op.TOEPLITZ
        x, iters, hist = op.cg(d, x0, self.maxiter, rtol=1e-5, form=form)
        self.iterations = int(iters.item())
        self.residuals = hist[:self.iterations].cpu().numpy() if hist is not None else None
        return x.reshape((self.M,) * 3).cpu().numpy()
