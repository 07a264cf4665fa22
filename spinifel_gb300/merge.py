"""Device objects of the autocorrelation merge: the W operator (Toeplitz or
direct form) and the FP64 device-resident CG (libspinifel_gb300 spf_merge_*)."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .nufft import NufftPlan


def antisupport(M: int, oversampling: int) -> np.ndarray:
    """F_antisupport of spinifel/sequential/autocorrelation.py:78-81."""
    lu = np.linspace(-np.pi, np.pi, M)
    Hu, Ku, Lu = np.meshgrid(lu, lu, lu, indexing="ij")
    return np.sqrt(Hu ** 2 + Ku ** 2 + Lu ** 2) > np.pi / oversampling


class MergeOperator:
    """W x = S.conv(S.x) + rlambda x + flambda S.reg(S.x) on an M^3 grid."""

    TOEPLITZ, DIRECT = 0, 1

    def __init__(self, M: int, M_ups: int, rlambda: float, flambda: float,
                 support: torch.Tensor, F_antisupport, device=None):
        self.device = support.device
        self.M, self.M_ups = M, M_ups
        self.support = support.to(torch.float32).contiguous()
        self.anti = torch.as_tensor(np.asarray(F_antisupport, dtype=np.float32),
                                    device=self.device).contiguous()
        h = ctypes.c_void_p()
        _lib.call("spf_merge_create", M, M_ups, float(rlambda), float(flambda),
                  _lib.ptr(self.support), _lib.ptr(self.anti), ctypes.byref(h))
        self._h = h
        L = ctypes.c_int()
        _lib.call("spf_merge_info", h, ctypes.byref(L))
        self.fft_size = L.value
        self._keep = []
        self.has_direct = False

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().spf_merge_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_kernel(self, ugrid_conv: torch.Tensor, fp64: bool | None = None):
        """ugrid_conv: real M_ups^3 (type 1 of ones onto M_ups modes / M_ups^3).
        fp64 (default: ugrid_conv is float64) runs the Toeplitz product in
        FP64, as the reference's double-precision run does."""
        if fp64 is None:
            fp64 = ugrid_conv.dtype == torch.float64
        if fp64:
            u = ugrid_conv.to(device=self.device, dtype=torch.float64).contiguous()
            _lib.call("spf_merge_set_kernel_f64", self._h, _lib.ptr(u), u.shape[0],
                      _lib.stream_handle())
        else:
            u = ugrid_conv.to(device=self.device, dtype=torch.float32).contiguous()
            _lib.call("spf_merge_set_kernel", self._h, _lib.ptr(u), u.shape[0],
                      _lib.stream_handle())
        self.fp64 = bool(fp64)
        torch.cuda.current_stream().synchronize()

    def set_direct(self, plan: NufftPlan, quats: torch.Tensor, ppr: torch.Tensor, scale: float,
                   weights: torch.Tensor | None = None, det_shape: tuple | None = None):
        quats = quats.to(device=self.device, dtype=torch.float32).contiguous()
        if det_shape is None and ppr.dim() == 4:
            det_shape = tuple(ppr.shape[1:])
        ppr = ppr.to(device=self.device, dtype=torch.float32).contiguous().reshape(3, -1)
        if weights is not None:
            weights = weights.to(device=self.device, dtype=torch.float32).contiguous()
        d = tuple(det_shape) if det_shape is not None and len(det_shape) == 3 else (0, 0, 0)
        _lib.call("spf_merge_set_direct", self._h, plan.handle, _lib.ptr(quats), quats.shape[0],
                  _lib.ptr(ppr), ppr.shape[1], int(d[0]), int(d[1]), int(d[2]), float(scale),
                  _lib.ptr(weights))
        self._keep = [plan, quats, ppr, weights]
        self.has_direct = True

    def apply(self, x: torch.Tensor, form: int = 0) -> torch.Tensor:
        x = x.to(device=self.device, dtype=torch.float64).contiguous().reshape(-1)
        y = torch.empty_like(x)
        _lib.call("spf_merge_apply", self._h, int(form), _lib.ptr(x), _lib.ptr(y),
                  _lib.stream_handle())
        return y

    def cg_into(self, b: torch.Tensor, x: torch.Tensor, hist: torch.Tensor | None,
                iters: torch.Tensor, maxiter: int, rtol: float = 1e-5, form: int = 0,
                x0_is_zero: bool = False):
        """CG into preallocated device tensors with no host synchronisation, so
        the call can be captured in a CUDA graph (x holds x0 on entry)."""
        _lib.call("spf_merge_cg", self._h, int(form), _lib.ptr(b), _lib.ptr(x), int(x0_is_zero),
                  int(maxiter), float(rtol), _lib.ptr(hist), _lib.ptr(iters),
                  _lib.stream_handle())

    def cg(self, b: torch.Tensor, x0: torch.Tensor, maxiter: int, rtol: float = 1e-5,
           form: int = 0, history: bool = True):
        b = b.to(device=self.device, dtype=torch.float64).contiguous().reshape(-1)
        x = x0.to(device=self.device, dtype=torch.float64).clone().contiguous().reshape(-1)
        hist = torch.zeros(max(maxiter, 1), dtype=torch.float64, device=self.device) \
            if history else None
        iters = torch.zeros(1, dtype=torch.int32, device=self.device)
        x0_zero = int(not bool(x.any()))
        _lib.call("spf_merge_cg", self._h, int(form), _lib.ptr(b), _lib.ptr(x), x0_zero,
                  int(maxiter), float(rtol), _lib.ptr(hist), _lib.ptr(iters),
                  _lib.stream_handle())
        return x, iters, hist

    def cg_sweep(self, rlambdas, flambdas, adb: torch.Tensor, x0: torch.Tensor | None,
                 maxiter: int, rtol: float = 1e-5, conv_factor: float = 1.0,
                 history: bool = False):
        """All (rlambda_l, flambda_l) systems in one batched device CG
        (Toeplitz form): returns x [n, M^3], norms [n, 2] = (||x_l||,
        ||W_l x_l - d_l||), iterations [n] and, if asked, residual histories."""
        rl = np.ascontiguousarray(rlambdas, dtype=np.float64)
        fl = np.ascontiguousarray(flambdas, dtype=np.float64)
        if rl.shape != fl.shape or rl.ndim != 1:
            raise ValueError("rlambdas and flambdas must be 1-D of the same length")
        nl = rl.size
        n = self.M ** 3
        adb = adb.to(device=self.device, dtype=torch.float64).contiguous().reshape(-1)
        if x0 is not None:
            x0 = x0.to(device=self.device, dtype=torch.float64).contiguous().reshape(-1)
        x = torch.empty(nl, n, dtype=torch.float64, device=self.device)
        norms = torch.empty(nl, 2, dtype=torch.float64, device=self.device)
        iters = torch.zeros(nl, dtype=torch.int32, device=self.device)
        hist = torch.zeros(nl, max(maxiter, 1), dtype=torch.float64, device=self.device) \
            if history else None
        P = ctypes.POINTER(ctypes.c_double)
        _lib.call("spf_merge_cg_sweep", self._h, nl, float(conv_factor),
                  rl.ctypes.data_as(P), fl.ctypes.data_as(P), _lib.ptr(adb), _lib.ptr(x0),
                  _lib.ptr(x), int(maxiter), float(rtol), _lib.ptr(norms), _lib.ptr(hist),
                  _lib.ptr(iters), _lib.stream_handle())
        return x, norms, iters, hist
