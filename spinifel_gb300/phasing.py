"""Device-resident phase retrieval (ER / HIO / shrink-wrap) over the C ABI
spf_phase_*: the state (rho_, support_, amplitudes_) stays on the GPU for the
whole schedule; only the recentring reads three integers back.  FP64 with
cuFFT D2Z / Z2D, as the reference's double-precision run
(spinifel/sequential/phasing.py)."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib

METHODS = {None: 0, "std": 0, "max": 1}


class Phaser:
    """Phase-retrieval state for an M^3 grid on the current CUDA device."""

    def __init__(self, M: int, device=None):
        self.device = torch.device(device) if device is not None else \
            torch.device("cuda", torch.cuda.current_device())
        self.M = int(M)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("spf_phase_create", self.M, ctypes.byref(h))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            _lib.call("spf_phase_destroy", self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _dev(self, a, dtype):
        t = torch.as_tensor(np.asarray(a) if not isinstance(a, torch.Tensor) else a)
        t = t.to(device=self.device, dtype=dtype).contiguous()
        if tuple(t.shape) != (self.M,) * 3:
            raise ValueError(f"expected an {self.M}^3 array, got {tuple(t.shape)}")
        return t

    def set_ac(self, ac):
        """amplitudes_ and ac_filt_ from a centred autocorrelation."""
        ac = self._dev(np.real(ac) if not isinstance(ac, torch.Tensor) else ac, torch.float64)
        _lib.call("spf_phase_set_ac", self._h, _lib.ptr(ac), _lib.stream_handle())

    def create_support(self, Mquat: int):
        _lib.call("spf_phase_create_support", self._h, int(Mquat), _lib.stream_handle())

    def set_state(self, rho_=None, support_=None):
        r = self._dev(rho_, torch.float64) if rho_ is not None else None
        s = self._dev(support_, torch.uint8) if support_ is not None else None
        _lib.call("spf_phase_set_state", self._h, _lib.ptr(r), _lib.ptr(s), _lib.stream_handle())
        torch.cuda.current_stream(self.device).synchronize()

    def state(self):
        """(rho_ float64, support_ bool) as device tensors."""
        r = torch.empty((self.M,) * 3, dtype=torch.float64, device=self.device)
        s = torch.empty((self.M,) * 3, dtype=torch.uint8, device=self.device)
        _lib.call("spf_phase_get_state", self._h, _lib.ptr(r), _lib.ptr(s), _lib.stream_handle())
        return r, s.bool()

    def er(self, n_loops: int, rho_max: float = np.inf):
        _lib.call("spf_phase_er", self._h, int(n_loops), float(rho_max), _lib.stream_handle())

    def hio(self, n_loops: int, beta: float, rho_max: float = np.inf):
        _lib.call("spf_phase_hio", self._h, int(n_loops), float(beta), float(rho_max),
                  _lib.stream_handle())

    def shrink_wrap(self, sigma: float = 1.0, method=None, weight: float = 1.0,
                    cutoff: float = 0.05):
        if method not in METHODS:
            raise ValueError(f"Invalid method: {method}. Options are 'std' or 'max'.")
        _lib.call("spf_phase_shrink_wrap", self._h, float(sigma), METHODS[method], float(weight),
                  float(cutoff), _lib.stream_handle())

    def run(self, n_phase_loops: int, nER: int, nHIO: int, beta: float, method=None,
            weight: float = 1.0, cutoff: float = 0.05, rho_max: float = np.inf):
        if method not in METHODS:
            raise ValueError(f"Invalid method: {method}. Options are 'std' or 'max'.")
        _lib.call("spf_phase_run", self._h, int(n_phase_loops), int(nER), int(nHIO), float(beta),
                  float(rho_max), METHODS[method], float(weight), float(cutoff),
                  _lib.stream_handle())

    def finish(self):
        """Recenter, then the phased autocorrelation (device, centred); also
        returns the three recentring shifts."""
        out = torch.empty((self.M,) * 3, dtype=torch.float64, device=self.device)
        sh = (ctypes.c_int * 3)()
        _lib.call("spf_phase_finish", self._h, _lib.ptr(out), sh, _lib.stream_handle())
        return out, list(sh)
