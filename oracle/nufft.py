"""ORACLE -- test infrastructure only (never imported by the product path).

FP64 CPU restatement of the 3D type-1 / type-2 NUFFT used by Spinifel
(spinifel/extern/nufft_ext.py:248-327 and :420-487, spinifel/autocorrelation.py
:32-61 and :97-128).  The library the reference calls (finufft 1.1.2 / 2.1.0,
cufinufft 1.1 / 1.2, accepted at spinifel/extern/__init__.py:89-104) is an
un-vendored git submodule, so the published exponential-of-semicircle method
is restated here: spread/interpolate with phi(z) = exp(beta(sqrt(1-z^2)-1)) on
a grid upsampled by sigma, FFT, divide by the kernel's Fourier transform.

Conventions pinned by tests (and by the direct sums in nufft_oracle.c):
  * modes k = -floor(m/2) .. ceil(m/2)-1 on each axis, C-ordered arrays;
  * the first coordinate (H) runs along axis 0;
  * type 2: c_j = sum_k f_k exp(isign i k.x_j); type 1 the adjoint sum.

Spread and interpolation are C (oracle/nufft_oracle.c, OpenMP); FFTs are numpy.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def lib():
    """Load (building if needed) the C oracle."""
    global _LIB
    if _LIB is None:
        from oracle import build as _b

        path = _b.build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        i64 = ctypes.c_int64
        ci = ctypes.c_int
        L.orc_interp.argtypes = [ci, ci, ci, dp, i64, dp, dp, dp, ci, ctypes.c_double, dp]
        L.orc_spread.argtypes = [ci, ci, ci, dp, i64, dp, dp, dp, dp, ci, ctypes.c_double]
        L.orc_nudft_t2.argtypes = [ci, ci, ci, dp, i64, dp, dp, dp, ci, dp]
        L.orc_nudft_t1.argtypes = [ci, ci, ci, dp, i64, dp, dp, dp, ci, dp]
        L.orc_knn_eudist.argtypes = [dp, dp, i64, i64, i64, dp]
        L.orc_es_kernel.argtypes = [ctypes.c_double, ctypes.c_double]
        L.orc_es_kernel.restype = ctypes.c_double
        for f in (L.orc_interp, L.orc_spread, L.orc_nudft_t2, L.orc_nudft_t1, L.orc_knn_eudist):
            f.restype = None
        _LIB = L
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


# ----------------------------------------------------------------------------
# kernel parameters (published ES choices, restated)
# ----------------------------------------------------------------------------

def kernel_width(eps: float) -> int:
    """Spread width w for tolerance eps at upsampling 2: ceil(-log10(eps/10))."""
    w = int(math.ceil(-math.log10(eps / 10.0)))
    return max(2, min(16, w))


def kernel_beta(w: int, sigma: float = 2.0) -> float:
    """ES shape parameter beta for width w and upsampling sigma."""
    if sigma == 2.0:
        bon = {2: 2.20, 3: 2.26, 4: 2.38}.get(w, 2.30)
        return bon * w
    return 0.97 * math.pi * w * (1.0 - 1.0 / (2.0 * sigma))


def next_smooth_even(n: int) -> int:
    """Smallest even integer >= n whose only prime factors are 2, 3, 5."""
    n = max(2, int(n))
    if n % 2:
        n += 1
    while True:
        m = n
        for p in (2, 3, 5):
            while m % p == 0:
                m //= p
        if m == 1:
            return n
        n += 2


def fine_size(m: int, w: int, sigma: float = 2.0) -> int:
    return next_smooth_even(max(int(math.ceil(sigma * m)), 2 * w))


def deconv_factors(m: int, n: int, w: int, beta: float) -> np.ndarray:
    """p(k) = int_{-w/2}^{w/2} phi(2t/w) cos(k h t) dt, h = 2 pi / n, for the
    modes k = -floor(m/2) .. ; Gauss-Legendre on [0, w/2] (phi is even)."""
    xq, wq = np.polynomial.legendre.leggauss(4 * w + 40)
    t = 0.25 * w * (xq + 1.0)  # [0, w/2]
    wt = 0.25 * w * wq
    z = 2.0 * t / w
    phi = np.exp(beta * (np.sqrt(np.maximum(1.0 - z * z, 0.0)) - 1.0))
    k = np.arange(m) - (m // 2)
    h = 2.0 * np.pi / n
    return 2.0 * (np.cos(np.outer(k * h, t)) * (phi * wt)).sum(axis=1)


class Params:
    def __init__(self, m, eps=1e-12, sigma=2.0):
        self.m = tuple(int(v) for v in (m if np.ndim(m) else (m, m, m)))
        self.eps = eps
        self.sigma = sigma
        self.w = kernel_width(eps) if sigma == 2.0 else kernel_width_sigma(eps, sigma)
        self.beta = kernel_beta(self.w, sigma)
        self.n = tuple(fine_size(mi, self.w, sigma) for mi in self.m)
        self.p = [deconv_factors(mi, ni, self.w, self.beta) for mi, ni in zip(self.m, self.n)]


def kernel_width_sigma(eps: float, sigma: float) -> int:
    """Width for a general upsampling factor: error ~ exp(-pi w sqrt(1-1/sigma))."""
    w = int(math.ceil(math.log(1.0 / eps) / (math.pi * math.sqrt(1.0 - 1.0 / sigma))))
    return max(2, min(16, w))


def _coords(x, y, z):
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64).ravel())
    y = np.ascontiguousarray(np.asarray(y, dtype=np.float64).ravel())
    z = np.ascontiguousarray(np.asarray(z, dtype=np.float64).ravel())
    assert x.shape == y.shape == z.shape
    return x, y, z


def _mode_index(m, n):
    """Fine-grid index of each centred mode k = -floor(m/2).. (k mod n)."""
    return (np.arange(m) - (m // 2)) % n


# ----------------------------------------------------------------------------
# type 2 / type 1
# ----------------------------------------------------------------------------

def nufft3d2(x, y, z, f, isign=-1, eps=1e-12, sigma=2.0):
    """c_j = sum_k f_k exp(isign i k.x_j); f complex/real (m1, m2, m3)."""
    x, y, z = _coords(x, y, z)
    f = np.asarray(f)
    P = Params(f.shape, eps, sigma)
    b = np.zeros(P.n, dtype=np.complex128)
    pk = P.p[0][:, None, None] * P.p[1][None, :, None] * P.p[2][None, None, :]
    i0, i1, i2 = (_mode_index(mi, ni) for mi, ni in zip(P.m, P.n))
    b[np.ix_(i0, i1, i2)] = f / pk
    if isign < 0:
        U = np.fft.fftn(b)
    else:
        U = np.fft.ifftn(b) * float(np.prod(P.n))
    U = np.ascontiguousarray(U)
    out = np.empty(x.size, dtype=np.complex128)
    lib().orc_interp(P.n[0], P.n[1], P.n[2], _p(U.view(np.float64)), x.size,
                     _p(x), _p(y), _p(z), P.w, P.beta, _p(out.view(np.float64)))
    return out


def nufft3d1(x, y, z, c, m, isign=+1, eps=1e-12, sigma=2.0):
    """f_k = sum_j c_j exp(isign i k.x_j) onto m = (m1, m2, m3) centred modes."""
    x, y, z = _coords(x, y, z)
    c = np.ascontiguousarray(np.asarray(c, dtype=np.complex128).ravel())
    P = Params(m, eps, sigma)
    G = np.zeros(P.n, dtype=np.complex128)
    lib().orc_spread(P.n[0], P.n[1], P.n[2], _p(G.view(np.float64)), x.size,
                     _p(x), _p(y), _p(z), _p(c.view(np.float64)), P.w, P.beta)
    if isign < 0:
        Gh = np.fft.fftn(G)
    else:
        Gh = np.fft.ifftn(G) * float(np.prod(P.n))
    i0, i1, i2 = (_mode_index(mi, ni) for mi, ni in zip(P.m, P.n))
    pk = P.p[0][:, None, None] * P.p[1][None, :, None] * P.p[2][None, None, :]
    return Gh[np.ix_(i0, i1, i2)] / pk


def nudft3d2(x, y, z, f, isign=-1):
    """Exact direct sum for type 2 (ground truth; O(npts m^3))."""
    x, y, z = _coords(x, y, z)
    f = np.ascontiguousarray(np.asarray(f, dtype=np.complex128))
    out = np.empty(x.size, dtype=np.complex128)
    m1, m2, m3 = f.shape
    lib().orc_nudft_t2(m1, m2, m3, _p(f.view(np.float64)), x.size, _p(x), _p(y), _p(z),
                       int(isign), _p(out.view(np.float64)))
    return out


def nudft3d1(x, y, z, c, m, isign=+1):
    """Exact direct sum for type 1 (ground truth)."""
    x, y, z = _coords(x, y, z)
    c = np.ascontiguousarray(np.asarray(c, dtype=np.complex128).ravel())
    m1, m2, m3 = (m, m, m) if np.ndim(m) == 0 else m
    f = np.empty((m1, m2, m3), dtype=np.complex128)
    lib().orc_nudft_t1(m1, m2, m3, _p(c.view(np.float64)), x.size, _p(x), _p(y), _p(z),
                       int(isign), _p(f.view(np.float64)))
    return f


# ----------------------------------------------------------------------------
# the reference's operator glue, restated
# ----------------------------------------------------------------------------

def forward(ugrid, H_, K_, L_, support, use_recip_sym, N, eps=1e-12):
    """spinifel/autocorrelation.py:32-61: support multiply, type 2 isign -1."""
    assert np.max(np.abs(np.array([H_, K_, L_]))) < 3 * np.pi
    ugrid = np.array(ugrid, dtype=np.complex128)
    if use_recip_sym:
        assert np.all(np.isreal(ugrid))
    if support is not None:
        ugrid = ugrid * support
    out = nufft3d2(H_, K_, L_, ugrid, -1, eps)
    assert out.size == N
    return out


def adjoint(nuvect, H_, K_, L_, M, use_recip_sym=True, support=None, isign=+1, eps=1e-12):
    """spinifel/autocorrelation.py:97-128 and nufft_ext.py:287-327: type 1 onto
    M^3, support multiply, real part, divided by M^3."""
    assert np.max(np.abs(np.array([H_, K_, L_]))) < 3 * np.pi
    ugrid = nufft3d1(H_, K_, L_, nuvect, (M, M, M), isign, eps)
    if support is not None:
        ugrid = ugrid * support
    if use_recip_sym:
        ugrid = ugrid.real
    return ugrid / M ** 3


def knn_eudist(ref, data):
    """Reference CUDA KNN distance semantics (orientation_matching_sp.cu:22-519)
    in FP64: [n_data, n_ref] sums over the first 16*floor(P/16) pixels."""
    ref = np.ascontiguousarray(ref, dtype=np.float64)
    data = np.ascontiguousarray(data, dtype=np.float64)
    out = np.empty((data.shape[0], ref.shape[0]), dtype=np.float64)
    lib().orc_knn_eudist(_p(ref), _p(data), ref.shape[0], data.shape[0], data.shape[1], _p(out))
    return out
