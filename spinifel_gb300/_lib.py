"""ctypes binding of libspinifel_gb300.so (the C ABI in include/spinifel_gb300.h).

The product path has no CPU fallback: if the library is missing or cannot be
loaded, every call raises.  Calls pass device pointers (torch tensors'
data_ptr()) and the current torch CUDA stream; a non-zero status raises
SpfError with the library's own message.  ctypes releases the GIL for the
duration of each foreign call.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libspinifel_gb300.so")

SPF_OK = 0
SPF_ERR_ARG = -1
SPF_ERR_OOM = -2
SPF_ERR_TIMEOUT = -3
SPF_ERR_LAUNCH = -4
SPF_ERR_CUDA = -5
SPF_ERR_UNSUPPORTED = -6

SPF_TUNE_BF16_GROUP_M = 1
SPF_TUNE_FP32_GROUP_M = 2
SPF_TUNE_BF16_GRID = 3
SPF_TUNE_PRIME_DFT = 4
SPF_TUNE_SLICE_SHAPE = 5
SPF_TUNE_SORT_ITEM = 6
SPF_TUNE_STATIC_ABORT_TEST = 7


class SpfError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: status {status}: {msg}")
        self.status = status


_c_void_p = ctypes.c_void_p
_i64 = ctypes.c_int64
_int = ctypes.c_int
_dbl = ctypes.c_double

# name -> argtypes (restype int unless listed in _RESTYPES)
SIGNATURES = {
    "spf_version": [],
    "spf_status_string": [_int],
    "spf_last_error": [],
    "spf_launch_count": [],
    "spf_device_error": [_c_void_p, ctypes.POINTER(_int)],
    "spf_selftest_bounded_wait": [_i64, _c_void_p, _c_void_p],
    "spf_tune_set": [_int, _i64],
    "spf_tune_get": [_int, ctypes.POINTER(_i64)],
    "spf_nufft_plan_create": [_int, _int, _int, _dbl, _dbl, ctypes.POINTER(_c_void_p)],
    "spf_nufft_plan_destroy": [_c_void_p],
    "spf_nufft_plan_info": [_c_void_p, ctypes.POINTER(_int), ctypes.POINTER(_int),
                            ctypes.POINTER(_dbl), ctypes.POINTER(_int)],
    "spf_nufft_t2_set_modes": [_c_void_p, _c_void_p, _c_void_p, _int, _int, _c_void_p],
    "spf_nufft_t2_interp": [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _i64, _c_void_p,
                            _c_void_p, _c_void_p],
    "spf_slice_t2": [_c_void_p, _c_void_p, _i64, _c_void_p, _i64, _dbl, _c_void_p, _c_void_p,
                     _c_void_p],
    "spf_slice_t2_det": [_c_void_p, _c_void_p, _i64, _c_void_p, _int, _int, _int, _dbl, _c_void_p,
                         _c_void_p, _c_void_p],
    "spf_nufft_t1_zero": [_c_void_p, _c_void_p],
    "spf_nufft_t1_spread": [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, _i64,
                            _c_void_p],
    "spf_nufft_t1_spread_orient": [_c_void_p, _c_void_p, _i64, _c_void_p, _i64, _dbl, _c_void_p,
                                   _c_void_p],
    "spf_nufft_t1_finish": [_c_void_p, _int, _c_void_p, _c_void_p, _c_void_p],
    "spf_nufft_interp_spread_orient": [_c_void_p, _c_void_p, _i64, _c_void_p, _i64, _dbl,
                                       _c_void_p, _c_void_p],
    "spf_merge_create": [_int, _int, _dbl, _dbl, _c_void_p, _c_void_p, ctypes.POINTER(_c_void_p)],
    "spf_merge_destroy": [_c_void_p],
    "spf_merge_info": [_c_void_p, ctypes.POINTER(_int)],
    "spf_merge_set_kernel": [_c_void_p, _c_void_p, _int, _c_void_p],
    "spf_merge_set_kernel_f64": [_c_void_p, _c_void_p, _int, _c_void_p],
    "spf_merge_set_direct": [_c_void_p, _c_void_p, _c_void_p, _i64, _c_void_p, _i64, _int, _int,
                             _int, _dbl, _c_void_p],
    "spf_nufft_sort_orient": [_c_void_p, _c_void_p, _i64, _c_void_p, _i64, _dbl, _c_void_p],
    "spf_nufft_sort_points": [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _i64, _c_void_p],
    "spf_nufft_interp_spread_sorted": [_c_void_p, _c_void_p, _c_void_p],
    "spf_nufft_spread_sorted": [_c_void_p, _c_void_p, _c_void_p],
    "spf_nufft_t1_spread_det": [_c_void_p, _c_void_p, _i64, _c_void_p, _int, _int, _int, _dbl,
                                _c_void_p, _c_void_p],
    "spf_nufft_interp_spread_det": [_c_void_p, _c_void_p, _i64, _c_void_p, _int, _int, _int, _dbl,
                                    _c_void_p, _c_void_p],
    "spf_merge_apply": [_c_void_p, _int, _c_void_p, _c_void_p, _c_void_p],
    "spf_merge_cg": [_c_void_p, _int, _c_void_p, _c_void_p, _int, _int, _dbl, _c_void_p,
                     _c_void_p, _c_void_p],
    "spf_knn_eudist_f32": [_c_void_p, _c_void_p, _i64, _i64, _i64, _c_void_p, _c_void_p],
    "spf_knn_eudist_f64": [_c_void_p, _c_void_p, _i64, _i64, _i64, _c_void_p, _c_void_p],
    "spf_knn_topk_f32": [_c_void_p, _i64, _i64, _int, _c_void_p, _c_void_p],
    "spf_knn_topk_f64": [_c_void_p, _i64, _i64, _int, _c_void_p, _c_void_p],
    "spf_frames_ingest_u16": [_c_void_p, _i64, _i64, _c_void_p, _c_void_p, _i64, _c_void_p,
                              _c_void_p, _c_void_p],
    "spf_row_sqnorm_f32": [_c_void_p, _i64, _i64, _c_void_p, _c_void_p],
    "spf_best_init": [_c_void_p, _i64, _c_void_p],
    "spf_dist_argmin_f32": [_c_void_p, _c_void_p, _i64, _c_void_p, _c_void_p, _i64, _i64, _i64,
                            _c_void_p, _c_void_p],
    "spf_best_unpack": [_c_void_p, _i64, _c_void_p, _c_void_p, _c_void_p],
    "spf_dist_topk_bf16_tiles": [_i64],
    "spf_dist_topk_bf16_tile_refs": [],
    "spf_dist_topk_bf16": [_c_void_p, _i64, _c_void_p, _i64, _i64, _i64, _c_void_p, _c_void_p,
                           _c_void_p, _c_void_p],
    "spf_rerank_fp32": [_c_void_p, _c_void_p, _i64, _c_void_p, _c_void_p, _i64, _c_void_p,
                        _c_void_p, _c_void_p, ctypes.c_float, _i64, _i64, _i64, _c_void_p,
                        _c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p],
    "spf_col_maxsq_f32": [_c_void_p, _i64, _i64, _c_void_p, _c_void_p],
    "spf_dist_range_bf16": [_c_void_p, _i64, _c_void_p, _i64, _i64, _i64, _c_void_p, _c_void_p,
                            _c_void_p, _c_void_p, _int, _c_void_p],
    "spf_match_bf16_static": [_c_void_p, _c_void_p, _c_void_p, _i64, _c_void_p, _c_void_p,
                              _c_void_p, _c_void_p, ctypes.c_float, _i64, _i64, _i64, _c_void_p,
                              _c_void_p, _c_void_p, _c_void_p],
    "spf_rerank_list_fp32": [_c_void_p, _c_void_p, _int, _c_void_p, _c_void_p, _i64, _c_void_p,
                             _c_void_p, _i64, _i64, _c_void_p, _c_void_p],
    "spf_row_norms_f32": [_c_void_p, _i64, _i64, _c_void_p, _c_void_p, _c_void_p],
    "spf_f32_to_bf16": [_c_void_p, _i64, _i64, _c_void_p, _i64, _c_void_p],
    "spf_gather_rows": [_c_void_p, _i64, _i64, _c_void_p, _i64, _c_void_p, _c_void_p],
    "spf_spread_t1": [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, _i64, _int,
                      _c_void_p, _c_void_p, _c_void_p],
    "spf_fft_deconv": [_c_void_p, _int, _int, _c_void_p, _c_void_p, _c_void_p, _c_void_p,
                       _c_void_p],
    "spf_dist_argmin_fp32": [_c_void_p, _c_void_p, _i64, _c_void_p, _c_void_p, _i64, _i64,
                             _c_void_p, _c_void_p, _c_void_p, _c_void_p],
    "spf_cg_solve": [_c_void_p, _int, _c_void_p, _c_void_p, _int, _int, _dbl, _c_void_p,
                     _c_void_p, _c_void_p],
    "spf_serve_clock": [],
    "spf_serve_create": [_int, _c_void_p, _c_void_p, _c_void_p, _c_void_p, ctypes.c_float, _i64,
                         _i64, _i64, _int, _i64, _int, _i64, ctypes.POINTER(_c_void_p)],
    "spf_serve_submit": [_c_void_p, _c_void_p, _i64, _c_void_p, _c_void_p, _dbl,
                         ctypes.POINTER(_i64)],
    "spf_serve_wait": [_c_void_p, _i64, _i64, ctypes.POINTER(_int)],
    "spf_serve_stats": [_c_void_p, ctypes.POINTER(_dbl), _int],
    "spf_serve_latencies": [_c_void_p, ctypes.POINTER(_dbl), _i64, ctypes.POINTER(_i64)],
    "spf_serve_destroy": [_c_void_p],
    "spf_merge_cg_sweep": [_c_void_p, _int, _dbl, ctypes.POINTER(_dbl), ctypes.POINTER(_dbl),
                           _c_void_p, _c_void_p, _c_void_p, _int, _dbl, _c_void_p, _c_void_p,
                           _c_void_p, _c_void_p],
    "spf_eval_score_rotations": [_c_void_p, _c_void_p, _int, _c_void_p, _i64, _c_void_p,
                                 _c_void_p],
    "spf_eval_rotate_volume": [_c_void_p, _int, _c_void_p, _i64, _c_void_p, _c_void_p],
    "spf_eval_fsc_shells": [_c_void_p, _c_void_p, _int, _c_void_p, _dbl, _dbl, _int, _c_void_p,
                            _c_void_p],
    "spf_bin_frames_u16": [_c_void_p, _i64, _int, _int, _int, _int, _int, _int, _c_void_p,
                           _c_void_p],
    "spf_scatter_rows": [_c_void_p, _i64, _c_void_p, _i64, _c_void_p, _i64, _c_void_p],
    "spf_rerank_fp32_keep": [_c_void_p, _c_void_p, _i64, _c_void_p, _c_void_p, _i64, _c_void_p,
                             _c_void_p, _c_void_p, ctypes.c_float, _i64, _i64, _i64, _c_void_p,
                             _c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p],
    "spf_scan_band_bf16": [_c_void_p, _c_void_p, _i64, _i64, _c_void_p, _i64, _c_void_p,
                           _c_void_p, _c_void_p, _int, _c_void_p],
    "spf_complete_open": [_c_void_p, _c_void_p, _i64, _c_void_p, _c_void_p, _c_void_p,
                          _c_void_p, _i64, _c_void_p, _i64, _c_void_p, _c_void_p, _c_void_p,
                          _i64, _i64, _i64, _c_void_p, _c_void_p, _c_void_p, _c_void_p],
    "spf_match_bf16_host": [_c_void_p, _i64, _c_void_p, _c_void_p, _c_void_p, _c_void_p,
                            ctypes.c_float, _i64, _i64, _i64, _i64, _c_void_p, _c_void_p,
                            _c_void_p, _c_void_p],
    "spf_nufft64_plan_create": [_int, _int, _int, _dbl, _dbl, ctypes.POINTER(_c_void_p)],
    "spf_nufft64_plan_destroy": [_c_void_p],
    "spf_nufft64_plan_info": [_c_void_p, ctypes.POINTER(_int), ctypes.POINTER(_int),
                              ctypes.POINTER(_dbl), ctypes.POINTER(_int)],
    "spf_nufft64_t2_set_modes": [_c_void_p, _c_void_p, _c_void_p, _int, _int, _c_void_p],
    "spf_nufft64_t2_interp": [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _i64, _c_void_p,
                              _c_void_p, _c_void_p],
    "spf_slice_t2_f64": [_c_void_p, _c_void_p, _i64, _c_void_p, _i64, _dbl, _c_void_p,
                         _c_void_p],
    "spf_nufft64_t1_zero": [_c_void_p, _c_void_p],
    "spf_nufft64_t1_spread": [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, _i64,
                              _c_void_p],
    "spf_nufft64_t1_finish": [_c_void_p, _int, _c_void_p, _c_void_p, _c_void_p],
    "spf_dist_f64": [_c_void_p, _c_void_p, _i64, _i64, _i64, _c_void_p, _c_void_p],
    "spf_best64_init": [_c_void_p, _c_void_p, _i64, _c_void_p],
    "spf_argmin_rows_f64": [_c_void_p, _i64, _i64, _i64, _c_void_p, _c_void_p, _c_void_p],
    "spf_phase_create": [_int, ctypes.POINTER(_c_void_p)],
    "spf_phase_destroy": [_c_void_p],
    "spf_phase_set_ac": [_c_void_p, _c_void_p, _c_void_p],
    "spf_phase_create_support": [_c_void_p, _int, _c_void_p],
    "spf_phase_set_state": [_c_void_p, _c_void_p, _c_void_p, _c_void_p],
    "spf_phase_get_state": [_c_void_p, _c_void_p, _c_void_p, _c_void_p],
    "spf_phase_er": [_c_void_p, _int, _dbl, _c_void_p],
    "spf_phase_hio": [_c_void_p, _int, _dbl, _dbl, _c_void_p],
    "spf_phase_shrink_wrap": [_c_void_p, _dbl, _int, _dbl, _dbl, _c_void_p],
    "spf_phase_run": [_c_void_p, _int, _int, _int, _dbl, _dbl, _int, _dbl, _dbl, _c_void_p],
    "spf_phase_finish": [_c_void_p, _c_void_p, ctypes.POINTER(_int), _c_void_p],
}

_RESTYPES = {
    "spf_version": ctypes.c_char_p,
    "spf_status_string": ctypes.c_char_p,
    "spf_last_error": ctypes.c_char_p,
    "spf_launch_count": ctypes.c_uint64,
    "spf_dist_topk_bf16_tiles": ctypes.c_int64,
    "spf_dist_topk_bf16_tile_refs": ctypes.c_int64,
    "spf_serve_clock": ctypes.c_double,
}

_lock = threading.Lock()
_lib = None


def header_symbols() -> list[str]:
    """Function names declared in include/spinifel_gb300.h."""
    import re

    hdr = os.path.join(HERE, "..", "include", "spinifel_gb300.h")
    text = open(hdr).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(spf_[a-z0-9_]+)\s*\(", text)))


def load(path: str | None = None):
    """Load the library (no build).  Raises if it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise ImportError(
                f"libspinifel_gb300.so not found at {p}; run "
                "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)")
        L = ctypes.CDLL(p)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _lib = L
        return _lib


def lib():
    return _lib if _lib is not None else load()


def call(name: str, *args):
    """Invoke an int-returning entry point and raise on a non-zero status."""
    L = lib()
    st = getattr(L, name)(*args)
    if st != SPF_OK:
        msg = L.spf_last_error().decode(errors="replace")
        raise SpfError(st, name, msg)
    return st


def launch_count() -> int:
    return int(lib().spf_launch_count())


def ptr(t: torch.Tensor | None):
    """Device pointer of a contiguous tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_contiguous():
        raise ValueError("tensor must be contiguous")
    return ctypes.c_void_p(t.data_ptr())


def stream_handle(stream: torch.cuda.Stream | None = None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def require_cuda(t: torch.Tensor, name: str, dtype=None):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
