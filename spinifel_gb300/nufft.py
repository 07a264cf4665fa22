"""Device NUFFT plans (type 2 interpolation / type 1 spreading, ES kernel).

NufftPlan owns an FP32 `spf_nufft_plan` (tolerances down to about 1e-7);
NufftPlan64 owns an FP64 `spf_nufft64_plan` for tighter tolerances, down to
the reference's own eps = 1e-12 in double (spinifel/extern/nufft_ext.py:62).
make_plan(m, eps) picks the one the tolerance needs.  All arrays are torch
CUDA tensors; calls are asynchronous on the current torch stream.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

import torch

from . import _lib


# finest tolerance the FP32 plan resolves; below it make_plan returns an FP64 plan
FP32_EPS_FLOOR = 1e-7


def make_plan(m, eps: float = 1e-6, upsampfac: float = 2.0, device=None):
    """The FP32 plan for eps >= FP32_EPS_FLOOR, the FP64 plan below it."""
    cls = NufftPlan if float(eps) >= FP32_EPS_FLOOR else NufftPlan64
    return cls(m, eps, upsampfac, device)


class NufftPlan:
    dtype = torch.float32
    supports_sort = True

    def __init__(self, m, eps: float = 1e-6, upsampfac: float = 2.0,
                 device: torch.device | int | None = None):
        if isinstance(m, int):
            m = (m, m, m)
        self.m = tuple(int(v) for v in m)
        self.eps = float(eps)
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None \
            else torch.device("cuda", device if isinstance(device, int) else device.index or 0)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("spf_nufft_plan_create", self.m[0], self.m[1], self.m[2], self.eps,
                      float(upsampfac), ctypes.byref(h))
        self._h = h
        n = (ctypes.c_int * 3)()
        npad = (ctypes.c_int * 3)()
        w = ctypes.c_int()
        beta = ctypes.c_double()
        _lib.call("spf_nufft_plan_info", h, n, ctypes.byref(w), ctypes.byref(beta), npad)
        self.n_fine = tuple(n)
        self.n_padded = tuple(npad)
        self.width = w.value
        self.beta = beta.value
        self.has_modes = False

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            with torch.cuda.device(self.device):
                _lib.lib().spf_nufft_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- type 2 ---------------------------------------------------------
    def set_modes(self, modes: torch.Tensor, support: torch.Tensor | None = None,
                  isign: int = -1, want_imag: bool = False):
        modes = modes.to(device=self.device, dtype=torch.float32).contiguous()
        if tuple(modes.shape) != self.m:
            raise ValueError(f"modes shape {tuple(modes.shape)} != plan modes {self.m}")
        sup = None
        if support is not None and not (isinstance(support, (int, float)) and support == 1):
            sup = torch.as_tensor(support, device=self.device, dtype=torch.float32)
            sup = sup.expand(self.m).contiguous()
        _lib.call("spf_nufft_t2_set_modes", self._h, _lib.ptr(modes), _lib.ptr(sup), int(isign),
                  int(bool(want_imag)), _lib.stream_handle())
        self._keep = (modes, sup)
        self.has_modes = True
        self.has_imag = bool(want_imag)

    def interp(self, x: torch.Tensor, y: torch.Tensor, z: torch.Tensor, want_imag=False):
        x, y, z = (t.to(device=self.device, dtype=torch.float32).contiguous().reshape(-1)
                   for t in (x, y, z))
        n = x.numel()
        re = torch.empty(n, device=self.device, dtype=torch.float32)
        im = torch.empty(n, device=self.device, dtype=torch.float32) if want_imag else None
        _lib.call("spf_nufft_t2_interp", self._h, _lib.ptr(x), _lib.ptr(y), _lib.ptr(z), n,
                  _lib.ptr(re), _lib.ptr(im), _lib.stream_handle())
        return re, im

    def slice(self, quats: torch.Tensor, ppr: torch.Tensor, scale: float,
              out: torch.Tensor | None = None, out_bf16: torch.Tensor | None = None,
              det_shape: tuple | None = None):
        """Slices [n_orient, n_pix] (real part) at the given orientations.
        With det_shape = (n_panels, nx, ny) the patch-staged kernel is used."""
        quats = quats.to(device=self.device, dtype=torch.float32).contiguous()
        if det_shape is None and ppr.dim() == 4:
            det_shape = tuple(ppr.shape[1:])
        ppr = ppr.to(device=self.device, dtype=torch.float32).contiguous().reshape(3, -1)
        n_o, n_p = quats.shape[0], ppr.shape[1]
        if out is None:
            out = torch.empty(n_o, n_p, device=self.device, dtype=torch.float32)
        _lib.require_cuda(out, "out", torch.float32)
        if out.numel() != n_o * n_p:
            raise ValueError("out has the wrong size")
        if out_bf16 is not None:
            _lib.require_cuda(out_bf16, "out_bf16", torch.bfloat16)
        if det_shape is not None and len(det_shape) == 3 and int(np.prod(det_shape)) == n_p:
            _lib.call("spf_slice_t2_det", self._h, _lib.ptr(quats), n_o, _lib.ptr(ppr),
                      int(det_shape[0]), int(det_shape[1]), int(det_shape[2]), float(scale),
                      _lib.ptr(out), _lib.ptr(out_bf16), _lib.stream_handle())
        else:
            _lib.call("spf_slice_t2", self._h, _lib.ptr(quats), n_o, _lib.ptr(ppr), n_p,
                      float(scale), _lib.ptr(out), _lib.ptr(out_bf16), _lib.stream_handle())
        return out

    # ---- type 1 ---------------------------------------------------------
    def spread_zero(self):
        _lib.call("spf_nufft_t1_zero", self._h, _lib.stream_handle())

    def spread(self, x, y, z, c):
        x, y, z, c = (t.to(device=self.device, dtype=torch.float32).contiguous().reshape(-1)
                      for t in (x, y, z, c))
        _lib.call("spf_nufft_t1_spread", self._h, _lib.ptr(x), _lib.ptr(y), _lib.ptr(z),
                  _lib.ptr(c), x.numel(), _lib.stream_handle())

    # from this many points on, spread_orient bin-sorts the points and uses
    # the sorted spreading (points sharing a footprint cell summed in
    # registers); below it, the patch or thread-per-point kernels
    SORTED_MIN_POINTS = 1 << 21

    def spread_orient(self, quats, ppr, scale, c, det_shape: tuple | None = None,
                      sort: bool | None = None):
        quats = quats.to(device=self.device, dtype=torch.float32).contiguous()
        if det_shape is None and ppr.dim() == 4:
            det_shape = tuple(ppr.shape[1:])
        ppr = ppr.to(device=self.device, dtype=torch.float32).contiguous().reshape(3, -1)
        c = c.to(device=self.device, dtype=torch.float32).contiguous()
        if c.numel() != quats.shape[0] * ppr.shape[1]:
            raise ValueError("strengths must be n_orient * n_pix")
        if sort is None:
            sort = c.numel() >= self.SORTED_MIN_POINTS
        if sort:
            self._sorted_points = (quats, ppr)
            _lib.call("spf_nufft_sort_orient", self._h, _lib.ptr(quats), quats.shape[0],
                      _lib.ptr(ppr), ppr.shape[1], float(scale), _lib.stream_handle())
            _lib.call("spf_nufft_spread_sorted", self._h, _lib.ptr(c), _lib.stream_handle())
        elif det_shape is not None and len(det_shape) == 3 and \
                int(np.prod(det_shape)) == ppr.shape[1]:
            _lib.call("spf_nufft_t1_spread_det", self._h, _lib.ptr(quats), quats.shape[0],
                      _lib.ptr(ppr), int(det_shape[0]), int(det_shape[1]), int(det_shape[2]),
                      float(scale), _lib.ptr(c), _lib.stream_handle())
        else:
            _lib.call("spf_nufft_t1_spread_orient", self._h, _lib.ptr(quats), quats.shape[0],
                      _lib.ptr(ppr), ppr.shape[1], float(scale), _lib.ptr(c),
                      _lib.stream_handle())

    def sort_points(self, x, y, z):
        """Bin-sort explicit points (radians) once for spread_sorted; the
        coordinate tensors are kept alive by the plan."""
        x, y, z = (t.to(device=self.device, dtype=torch.float32).contiguous().reshape(-1)
                   for t in (x, y, z))
        self._sorted_points = (x, y, z)
        _lib.call("spf_nufft_sort_points", self._h, _lib.ptr(x), _lib.ptr(y), _lib.ptr(z),
                  x.numel(), _lib.stream_handle())

    def spread_sorted(self, c=None):
        """Type-1 spreading of c (or ones) over the points of the last sort
        (sort_points or the orientation sort), into the type-1 accumulator."""
        if c is not None:
            c = c.to(device=self.device, dtype=torch.float32).contiguous().reshape(-1)
        _lib.call("spf_nufft_spread_sorted", self._h, _lib.ptr(c) if c is not None else None,
                  _lib.stream_handle())

    def finish(self, isign: int = 1, want_imag=False):
        re = torch.empty(self.m, device=self.device, dtype=torch.float32)
        im = torch.empty(self.m, device=self.device, dtype=torch.float32) if want_imag else None
        _lib.call("spf_nufft_t1_finish", self._h, int(isign), _lib.ptr(re), _lib.ptr(im),
                  _lib.stream_handle())
        return re, im


class NufftPlan64:
    """FP64 type 2 / type 1 at explicit points and FP64 slicing at
    orientation points (thread per point; quaternions, pixel positions and
    the rotation in double).  Same call surface as NufftPlan for the methods
    it has; no bin-sorted passes."""

    dtype = torch.float64
    supports_sort = False

    def __init__(self, m, eps: float = 1e-12, upsampfac: float = 2.0,
                 device: torch.device | int | None = None):
        if isinstance(m, int):
            m = (m, m, m)
        self.m = tuple(int(v) for v in m)
        self.eps = float(eps)
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None \
            else torch.device("cuda", device if isinstance(device, int) else device.index or 0)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("spf_nufft64_plan_create", self.m[0], self.m[1], self.m[2], self.eps,
                      float(upsampfac), ctypes.byref(h))
        self._h = h
        n = (ctypes.c_int * 3)()
        npad = (ctypes.c_int * 3)()
        w = ctypes.c_int()
        beta = ctypes.c_double()
        _lib.call("spf_nufft64_plan_info", h, n, ctypes.byref(w), ctypes.byref(beta), npad)
        self.n_fine = tuple(n)
        self.n_padded = tuple(npad)
        self.width = w.value
        self.beta = beta.value
        self.has_modes = False

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            with torch.cuda.device(self.device):
                _lib.lib().spf_nufft64_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _f64(self, t):
        return torch.as_tensor(t).to(device=self.device, dtype=torch.float64).contiguous()

    def set_modes(self, modes, support=None, isign: int = -1, want_imag: bool = False):
        modes = self._f64(modes)
        if tuple(modes.shape) != self.m:
            raise ValueError(f"modes shape {tuple(modes.shape)} != plan modes {self.m}")
        sup = None
        if support is not None and not (isinstance(support, (int, float)) and support == 1):
            sup = self._f64(support).expand(self.m).contiguous()
        _lib.call("spf_nufft64_t2_set_modes", self._h, _lib.ptr(modes), _lib.ptr(sup),
                  int(isign), int(bool(want_imag)), _lib.stream_handle())
        self._keep = (modes, sup)
        self.has_modes = True
        self.has_imag = bool(want_imag)

    def interp(self, x, y, z, want_imag=False):
        x, y, z = (self._f64(t).reshape(-1) for t in (x, y, z))
        n = x.numel()
        re = torch.empty(n, device=self.device, dtype=torch.float64)
        im = torch.empty(n, device=self.device, dtype=torch.float64) if want_imag else None
        _lib.call("spf_nufft64_t2_interp", self._h, _lib.ptr(x), _lib.ptr(y), _lib.ptr(z), n,
                  _lib.ptr(re), _lib.ptr(im), _lib.stream_handle())
        return re, im

    def slice(self, quats, ppr, scale: float, out: torch.Tensor | None = None,
              out_bf16=None, det_shape: tuple | None = None):
        """FP64 slices [n_orient, n_pix] (real part) at the given orientations
        (det_shape is accepted for symmetry with NufftPlan and not needed)."""
        if out_bf16 is not None:
            raise ValueError("the FP64 plan writes no bf16 copy")
        quats = self._f64(quats)
        ppr = self._f64(ppr).reshape(3, -1)
        n_o, n_p = quats.shape[0], ppr.shape[1]
        if out is None:
            out = torch.empty(n_o, n_p, device=self.device, dtype=torch.float64)
        _lib.require_cuda(out, "out", torch.float64)
        if out.numel() != n_o * n_p:
            raise ValueError("out has the wrong size")
        _lib.call("spf_slice_t2_f64", self._h, _lib.ptr(quats), n_o, _lib.ptr(ppr), n_p,
                  float(scale), _lib.ptr(out), _lib.stream_handle())
        return out

    def spread_zero(self):
        _lib.call("spf_nufft64_t1_zero", self._h, _lib.stream_handle())

    def spread(self, x, y, z, c):
        x, y, z, c = (self._f64(t).reshape(-1) for t in (x, y, z, c))
        _lib.call("spf_nufft64_t1_spread", self._h, _lib.ptr(x), _lib.ptr(y), _lib.ptr(z),
                  _lib.ptr(c), x.numel(), _lib.stream_handle())

    def finish(self, isign: int = 1, want_imag=False):
        re = torch.empty(self.m, device=self.device, dtype=torch.float64)
        im = torch.empty(self.m, device=self.device, dtype=torch.float64) if want_imag else None
        _lib.call("spf_nufft64_t1_finish", self._h, int(isign), _lib.ptr(re), _lib.ptr(im),
                  _lib.stream_handle())
        return re, im
