"""The MPI merge's regularisation sweep on one GPU
(spinifel/mpi/autocorrelation.py:40-214, class MergeMPI).

The reference runs one CG per MPI rank r with
    rlambda_r = M^3 / N * 2**(r - size / 2),   flambda_r = 1e5 * 10**(r - size // 2)
(N = number of data values), the Toeplitz kernel transform without the 1/M^3
of the sequential merge, and the antisupport |q| rounded to 4 decimals > pi
on linspace(-pi, pi, M)^3; rank 0 gathers (rank, rlambda, ||x||, ||W x - d||)
and keeps, in generation 0, the largest rlambda among the solutions whose norm
is at least the mean norm, and later the smallest ||x|| + ||W x - d||; every
rank then receives that solution.  Here the `size` systems are one batched
device CG (spf_merge_cg_sweep) and the same rule picks the result.
"""
from __future__ import annotations

import numpy as np
import torch
from scipy.ndimage import gaussian_filter

from .. import _arrays, geom
from ..merge import MergeOperator


def antisupport_mpi(M: int) -> np.ndarray:
    """mpi/autocorrelation.py:75-79."""
    lu = np.linspace(-np.pi, np.pi, M)
    Hu, Ku, Lu = np.meshgrid(lu, lu, lu, indexing="ij")
    return np.around(np.sqrt(Hu ** 2 + Ku ** 2 + Lu ** 2), 4) > np.pi


def lambdas(M: int, N: int, size: int):
    """(rlambda_r, flambda_r) for ranks r = 0 .. size-1 (mpi/autocorrelation.py:64-67)."""
    r = np.arange(size)
    return (M ** 3 / N * 2.0 ** (r - size / 2), 1e5 * np.power(10.0, r - size // 2))


def choose(generation: int, lambdas_r, v1s, v2s) -> int:
    """Rank 0's choice (mpi/autocorrelation.py:188-196)."""
    v1s, v2s, lambdas_r = (np.asarray(a) for a in (v1s, v2s, lambdas_r))
    if generation == 0:
        idx = v1s >= np.mean(v1s)
        imax = np.argmax(lambdas_r[idx])
        return int(np.arange(len(v1s), dtype=int)[idx][imax])
    return int(np.argmin(v1s + v2s))


class MergeMPI:
    """Drop-in for spinifel.mpi.autocorrelation.MergeMPI with the ranks' sweep
    run as `size` batched systems on this GPU."""

    def __init__(self, settings, slices_, pixel_position_reciprocal, pixel_distance_reciprocal,
                 nufft, size: int = 8, seed=None):
        self.M = settings.M
        self.Mquat = settings.Mquat
        self.M_ups = self.M * 2
        self.N_images = slices_.shape[0]
        self.N = int(np.prod(slices_.shape))
        self.Mtot = self.M ** 3
        self.size = int(size)
        self.maxiter = settings.solve_ac_maxiter
        self.reciprocal_extent = float(np.max(pixel_distance_reciprocal))
        self.mult = np.pi / self.reciprocal_extent
        self.use_reciprocal_symmetry = True
        self.pixel_position_reciprocal = np.array(pixel_position_reciprocal)
        self.rlambdas, self.flambdas = lambdas(self.M, self.N, self.size)
        self.F_antisupport = antisupport_mpi(self.M)
        self.data = _arrays.to_dev(np.asarray(slices_, dtype=np.float64).reshape(-1)
                                   if not _arrays.is_torch(slices_) else slices_.reshape(-1))
        self.nufft = nufft
        self.rng = np.random.default_rng(seed)
        self.ref_rank = -1
        self.summary = None
        self.iterations = None

    def solve_ac(self, generation, orientations=None, ac_estimate=None):
        if orientations is None:
            orientations = geom.uniform_quaternions(self.N_images, self.rng)
        H, K, L = geom.hkl(np.asarray(orientations).reshape(-1, 4),
                           self.pixel_position_reciprocal)
        if ac_estimate is None:
            ac_support = np.ones((self.M,) * 3)
            ac_estimate = np.zeros((self.M,) * 3)
        else:
            ac_estimate = np.asarray(ac_estimate, dtype=np.float64)
            ac_support = (gaussian_filter(ac_estimate, 0.5) > 1e-12).astype(np.float64)
            ac_estimate = ac_estimate * ac_support
        dev = _arrays.device()
        H_, K_, L_ = (torch.as_tensor(np.asarray(a).reshape(-1) * self.mult, dtype=torch.float32,
                                      device=dev) for a in (H, K, L))
        ones = torch.ones(H_.numel(), dtype=torch.float32, device=dev)
        ugrid_conv = self.nufft.adjoint(ones, H_, K_, L_, 1, self.use_reciprocal_symmetry,
                                        self.M_ups)
        sup = torch.as_tensor(np.asarray(ac_support, dtype=np.float32), device=dev)
        op = MergeOperator(self.M, self.M_ups, 0.0, 0.0, sup, self.F_antisupport)
        op.set_kernel(ugrid_conv)
        adb = self.nufft.adjoint(self.data, H_, K_, L_, sup, self.use_reciprocal_symmetry,
                                 self.M).reshape(-1).double()
        x0 = torch.as_tensor(ac_estimate.reshape(-1), dtype=torch.float64, device=dev)
        x, norms, iters, _ = op.cg_sweep(self.rlambdas, self.flambdas, adb, x0, self.maxiter,
                                         rtol=1e-5, conv_factor=float(self.Mtot))
        nrm = norms.cpu().numpy()
        v1s, v2s = nrm[:, 0], nrm[:, 1]
        self.summary = [(r, self.rlambdas[r], v1s[r], v2s[r]) for r in range(self.size)]
        self.ref_rank = choose(generation, self.rlambdas, v1s, v2s)
        self.iterations = iters.cpu().numpy()
        op.close()
        return x[self.ref_rank].reshape((self.M,) * 3).cpu().numpy()
