"""ORACLE -- test infrastructure only.

FP64 numpy/scipy restatement of the autocorrelation merge
(spinifel/sequential/autocorrelation.py:35-225, class Merge):

  ugrid_conv = adjoint(ones, H, K, L, support=1, M_ups) (real, / M_ups^3)  :158-166
  F_conv     = fftn(ifftshift(ugrid_conv)) / M^3                          :168-169
  W x        = conv(x) + rlambda x + flambda fourier_reg(x)               :171-177
    conv(x)  = crop_M( fftshift(ifftn(fftn(ifftshift(pad_{M_ups}(x S))) F_conv)) ) S, real
    reg(x)   = fftshift(ifftn(fftn(ifftshift(x S)) ifftshift(F_antisupport))) S, real
  d          = adjoint(data, H, K, L, support=S, M) + rlambda x0          :184-193
  x          = cg(W, d, x0, maxiter)                                       :217

with rlambda = 1 / N / 1000, flambda = 1e3 (:61-62), N = number of data
values, F_antisupport = |q| > pi / oversampling on linspace(-pi, pi, M)^3
(:78-81).  The adjoint is the FP64 ES NUFFT of oracle/nufft.py.
"""
from __future__ import annotations

import numpy as np
from scipy.ndimage import gaussian_filter
from scipy.sparse.linalg import LinearOperator, cg

from . import nufft as onufft


def antisupport(M: int, oversampling: int) -> np.ndarray:
    lu = np.linspace(-np.pi, np.pi, M)
    Hu, Ku, Lu = np.meshgrid(lu, lu, lu, indexing="ij")
    return np.sqrt(Hu ** 2 + Ku ** 2 + Lu ** 2) > np.pi / oversampling


def support_from_estimate(ac_estimate: np.ndarray) -> np.ndarray:
    """spinifel/sequential/autocorrelation.py:209-210."""
    return (gaussian_filter(ac_estimate, 0.5) > 1e-12).astype(np.float64)


def cg_recurrence(matvec, b, x0, maxiter, rtol=1e-5):
    """scipy.sparse.linalg.cg's iteration without a preconditioner, step for
    step (r = b - A x0; rho = r.r; p = r + (rho / rho_prev) p; q = A p;
    alpha = rho / p.q; x += alpha p; r -= alpha q; stop when ||r|| <
    rtol ||b||), returning also ||r|| at the start of every iteration (the
    recurrence residual the device CG records)."""
    b = np.asarray(b, dtype=np.float64)
    x = np.array(x0, dtype=np.float64, copy=True)
    r = b - matvec(x) if np.any(x) else b.copy()
    atol = rtol * np.linalg.norm(b)
    hist = []
    p = None
    rho_prev = None
    for it in range(maxiter):
        nr = np.linalg.norm(r)
        hist.append(float(nr))
        if nr < atol:
            break
        rho = float(r @ r)
        p = r.copy() if p is None else r + (rho / rho_prev) * p
        q = matvec(p)
        alpha = rho / float(p @ q)
        x += alpha * p
        r -= alpha * q
        rho_prev = rho
    return x, np.array(hist)


class MergeOracle:
    def __init__(self, M, M_ups, N, oversampling=1, maxiter=100, eps=1e-12, workers=None):
        self.M, self.M_ups, self.N = M, M_ups, N
        self.rlambda = 1.0 / N / 1000.0
        self.flambda = 1e3
        self.maxiter = maxiter
        self.eps = eps
        self.F_antisupport = antisupport(M, oversampling)
        self.iterations = 0
        self.residuals = []
        # workers: threads for scipy.fft (same FP64 transforms, for the large
        # grids); None keeps numpy's FFT, the one the reference calls
        self.workers = workers

    def _fftn(self, a):
        if self.workers is None:
            return np.fft.fftn(a)
        import scipy.fft as sfft

        return sfft.fftn(a, workers=self.workers)

    def _ifftn(self, a):
        if self.workers is None:
            return np.fft.ifftn(a)
        import scipy.fft as sfft

        return sfft.ifftn(a, workers=self.workers)

    def conv(self, x, F_conv, S):
        M, Mu = self.M, self.M_ups
        ups = np.zeros((Mu,) * 3)
        ups[:M, :M, :M] = x.reshape((M,) * 3) * S
        out = np.fft.fftshift(self._ifftn(self._fftn(np.fft.ifftshift(ups)) * F_conv))
        return (out[:M, :M, :M] * S).real.reshape(-1)

    def reg(self, x, S):
        M = self.M
        g = x.reshape((M,) * 3) * S
        F = self._fftn(np.fft.ifftshift(g))
        r = np.fft.fftshift(self._ifftn(F * np.fft.ifftshift(self.F_antisupport)))
        return (r * S).real.reshape(-1)

    def W(self, x, F_conv, S):
        x = np.real(x)
        return self.conv(x, F_conv, S) + self.rlambda * x + self.flambda * self.reg(x, S)

    def kernel(self, H_, K_, L_):
        """F_conv from the type 1 of ones onto the M_ups grid."""
        ones = np.ones(np.size(H_))
        ugrid_conv = onufft.adjoint(ones, H_, K_, L_, self.M_ups, True, None, eps=self.eps)
        return np.fft.fftn(np.fft.ifftshift(ugrid_conv)) / self.M ** 3

    def rhs(self, data, H_, K_, L_, S, x0):
        adb = onufft.adjoint(np.asarray(data, dtype=np.float64).reshape(-1), H_, K_, L_, self.M,
                             True, S, eps=self.eps)
        return adb.reshape(-1) + self.rlambda * x0

    def solve(self, data, H_, K_, L_, ac_support, x0, maxiter=None, rtol=1e-5):
        F_conv = self.kernel(H_, K_, L_)
        S = ac_support

        def W(u):
            u = np.real(u)
            return self.conv(u, F_conv, S) + self.rlambda * u + self.flambda * self.reg(u, S)

        d = self.rhs(data, H_, K_, L_, S, x0)
        n = self.M ** 3
        A = LinearOperator(dtype=np.float64, shape=(n, n), matvec=W)
        self.iterations = 0
        self.residuals = []

        def cb(xk):
            self.iterations += 1
            self.residuals.append(float(np.linalg.norm(d - W(xk))))

        x, info = cg(A, d, x0=x0.copy(), maxiter=maxiter or self.maxiter, rtol=rtol, callback=cb)
        return x.reshape((self.M,) * 3), info, F_conv, d


def antisupport_mpi(M: int) -> np.ndarray:
    """spinifel/mpi/autocorrelation.py:75-79: |q| rounded to 4 decimals > pi."""
    lu = np.linspace(-np.pi, np.pi, M)
    Hu, Ku, Lu = np.meshgrid(lu, lu, lu, indexing="ij")
    return np.around(np.sqrt(Hu ** 2 + Ku ** 2 + Lu ** 2), 4) > np.pi


def mpi_sweep(data, H_, K_, L_, ac_support, x0, M, size, maxiter, generation, eps=1e-12):
    """The MPI merge (spinifel/mpi/autocorrelation.py:40-214) for ranks
    0..size-1 in sequence: rank r solves with rlambda = M^3/N 2^(r - size/2),
    flambda = 1e5 10^(r - size//2), the kernel transform without 1/M^3 and
    the rounded antisupport; then rank 0's choice.  Returns (x of the chosen
    rank, chosen rank, summary rows (rank, rlambda, ||x||, ||W x - d||))."""
    N = np.asarray(data).size
    mo = MergeOracle(M, 2 * M, N, 1, maxiter, eps)
    mo.F_antisupport = antisupport_mpi(M)
    F_conv = mo.kernel(H_, K_, L_) * M ** 3  # the MPI kernel is not divided by M^3
    S = ac_support
    adb = onufft.adjoint(np.asarray(data, dtype=np.float64).reshape(-1), H_, K_, L_, M, True, S,
                         eps=eps).reshape(-1)
    n = M ** 3
    xs, rows = [], []
    for r in range(size):
        rl = M ** 3 / N * 2 ** (r - size / 2)
        fl = 1e5 * pow(10, r - size // 2)

        def W(u, rl=rl, fl=fl):
            u = np.real(u)
            return mo.conv(u, F_conv, S) + rl * u + fl * mo.reg(u, S)

        d = adb + rl * x0
        A = LinearOperator(dtype=np.float64, shape=(n, n), matvec=W)
        x, info = cg(A, d, x0=x0.copy(), maxiter=maxiter, rtol=1e-5)
        xs.append(x)
        rows.append((r, rl, float(np.linalg.norm(x)), float(np.linalg.norm(W(x) - d))))
    rows = np.array(rows)
    v1s, v2s, lam = rows[:, 2], rows[:, 3], rows[:, 1]
    if generation == 0:
        idx = v1s >= np.mean(v1s)
        iref = int(np.arange(size)[idx][np.argmax(lam[idx])])
    else:
        iref = int(np.argmin(v1s + v2s))
    return xs[iref].reshape((M,) * 3), iref, rows
