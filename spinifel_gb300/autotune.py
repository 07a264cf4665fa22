"""Autotuner for the launch parameters and tile shapes of the hot kernels.

The tensor-core kernel is persistent (one CTA per SM by default) and walks
its (image tile, reference tile) pairs in groups of GROUP_M image tiles, so
that the CTAs resident at one time share image and reference rows in L2; the
plain FP32 kernel rasterises the same way.  The best group size (and the
persistent grid size) depends on the shape, so it is measured: each candidate
is launched on the caller's real operands and timed with CUDA events, and the
fastest is kept through spf_tune_set and cached in a JSON file keyed by
device, kernel and shape (SPF_TUNE_CACHE overrides the file's location).
Results do not depend on these parameters (only the order in which tiles are
visited changes), so tuning never changes an answer.

The fused NUFFT kernels are tuned the same way: the tile shape of the
panel-detector slicing kernel (patch and warp block, SPF_TUNE_SLICE_SHAPE;
every shape gives the same bits) and the work-item size of the bin-sorted
interpolate / spread passes (SPF_TUNE_SORT_ITEM; the points of an item are
summed in another grouping, so sums may differ in the last bits).
"""
from __future__ import annotations

import json
import math
import os
import threading

import torch

from . import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
_lock = threading.Lock()


def _cache_path():
    return os.environ.get("SPF_TUNE_CACHE", os.path.join(HERE, "_tuned.json"))


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(d):
    p = _cache_path()
    tmp = p + f".tmp{os.getpid()}"
    try:
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


def _bucket(n: int) -> int:
    return 1 << max(0, int(math.ceil(math.log2(max(n, 1)))))


def _key(kind, n_img, n_ref, n_pix):
    name = torch.cuda.get_device_name()
    return f"{name}|{kind}|{_bucket(n_img)}|{_bucket(n_ref)}|{n_pix}"


def _time(fn, reps):
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def tune_bf16(frames, refs, group_sizes=(4, 8, 16, 32), grids=(0,), reps=2, force=False):
    """Pick SPF_TUNE_BF16_GROUP_M / SPF_TUNE_BF16_GRID for spf_dist_topk_bf16
    on these operands; returns {"group_m", "grid", "ms", "trials"}."""
    key = _key("bf16", frames.n, refs.n_ref, refs.n_pix)
    with _lock:
        cache = _load()
        if not force and key in cache:
            best = cache[key]
            _lib.call("spf_tune_set", _lib.SPF_TUNE_BF16_GROUP_M, int(best["group_m"]))
            _lib.call("spf_tune_set", _lib.SPF_TUNE_BF16_GRID, int(best["grid"]))
            return dict(best, cached=True)
        tiles = int(_lib.lib().spf_dist_topk_bf16_tiles(refs.n_ref))
        dev = frames.f32.device
        cd = torch.empty(tiles * frames.n * 8, dtype=torch.float32, device=dev)
        ci = torch.empty(tiles * frames.n * 8, dtype=torch.int32, device=dev)

        def run():
            _lib.call("spf_dist_topk_bf16", _lib.ptr(frames.bf16), frames.n, _lib.ptr(refs.bf16),
                      refs.n_ref, refs.n_pix, refs.ld, _lib.ptr(refs.sq), _lib.ptr(cd),
                      _lib.ptr(ci), _lib.stream_handle())

        trials = []
        for gm in group_sizes:
            for gr in grids:
                _lib.call("spf_tune_set", _lib.SPF_TUNE_BF16_GROUP_M, int(gm))
                _lib.call("spf_tune_set", _lib.SPF_TUNE_BF16_GRID, int(gr))
                trials.append({"group_m": gm, "grid": gr, "ms": _time(run, reps)})
        best = min(trials, key=lambda t: t["ms"])
        _lib.call("spf_tune_set", _lib.SPF_TUNE_BF16_GROUP_M, int(best["group_m"]))
        _lib.call("spf_tune_set", _lib.SPF_TUNE_BF16_GRID, int(best["grid"]))
        rec = {"group_m": best["group_m"], "grid": best["grid"], "ms": best["ms"],
               "trials": trials}
        cache[key] = rec
        _save(cache)
        return dict(rec, cached=False)


def tune_fp32(frames_f32, frames_sq, refs, group_sizes=(4, 8, 16), reps=1, force=False,
              max_frames=2048):
    """Pick SPF_TUNE_FP32_GROUP_M for the plain FP32 kernel (timed on at most
    max_frames frames)."""
    from .matching import BestTracker

    n = min(frames_f32.shape[0], max_frames)
    key = _key("fp32", n, refs.n_ref, refs.n_pix)
    with _lock:
        cache = _load()
        if not force and key in cache:
            _lib.call("spf_tune_set", _lib.SPF_TUNE_FP32_GROUP_M, int(cache[key]["group_m"]))
            return dict(cache[key], cached=True)
        x, sq = frames_f32[:n].contiguous(), frames_sq[:n].contiguous()
        tr = BestTracker(n, x.device)

        def run():
            tr.update_fp32(x, sq, refs.f32, refs.sq, 0)

        trials = []
        for gm in group_sizes:
            _lib.call("spf_tune_set", _lib.SPF_TUNE_FP32_GROUP_M, int(gm))
            trials.append({"group_m": gm, "ms": _time(run, reps)})
        best = min(trials, key=lambda t: t["ms"])
        _lib.call("spf_tune_set", _lib.SPF_TUNE_FP32_GROUP_M, int(best["group_m"]))
        rec = {"group_m": best["group_m"], "ms": best["ms"], "trials": trials}
        cache[key] = rec
        _save(cache)
        return dict(rec, cached=False)


SLICE_SHAPES = {0: "16x16 patch, 4x8 warps", 1: "16x16 patch, 8x4 warps",
                2: "8x32 patch, 2x16 warps", 3: "8x32 patch, 4x8 warps",
                4: "32x8 patch, 8x4 warps", 5: "32x8 patch, 16x2 warps",
                6: "16x16 patch, 4x8 warps, stride search",
                7: "16x16 patch, 8x4 warps, stride search"}


def tune_slice(plan, quats, ppr, scale: float, det_shape, reps=2, force=False):
    """Pick SPF_TUNE_SLICE_SHAPE for spf_slice_t2_det on this model grid and
    detector (quats: the orientations to time on, a few thousand suffice);
    returns {"shape", "tile", "ms", "trials"}."""
    name = torch.cuda.get_device_name()
    key = f"{name}|slice|{plan.n_fine}|w{plan.width}|{tuple(det_shape)}"
    with _lock:
        cache = _load()
        if not force and key in cache:
            best = cache[key]
            _lib.call("spf_tune_set", _lib.SPF_TUNE_SLICE_SHAPE, int(best["shape"]))
            return dict(best, cached=True)
        out = torch.empty(quats.shape[0], int(ppr[0].numel()), device=quats.device)
        trials = {}
        for code in SLICE_SHAPES:
            _lib.call("spf_tune_set", _lib.SPF_TUNE_SLICE_SHAPE, code)
            trials[code] = _time(lambda: plan.slice(quats, ppr, scale, out=out,
                                                    det_shape=det_shape), reps)
        code = min(trials, key=trials.get)
        _lib.call("spf_tune_set", _lib.SPF_TUNE_SLICE_SHAPE, code)
        best = {"shape": code, "tile": SLICE_SHAPES[code], "ms": trials[code]}
        cache[key] = best
        _save(cache)
        return dict(best, trials={SLICE_SHAPES[k]: v for k, v in trials.items()}, cached=False)


def tune_sort_item(plan, sort_fn, pass_fn, sizes=(2048, 4096, 8192), reps=2,
                   force=False, tag=""):
    """Pick SPF_TUNE_SORT_ITEM (points per work item of the bin-sorted
    passes): for each size sort_fn() re-sorts the points and pass_fn() is
    timed; the best size is set and the points re-sorted with it.  Returns
    {"items", "ms", "trials"}."""
    name = torch.cuda.get_device_name()
    key = f"{name}|sort_item|{plan.n_fine}|w{plan.width}|{tag}"
    with _lock:
        cache = _load()
        if not force and key in cache:
            best = cache[key]
            _lib.call("spf_tune_set", _lib.SPF_TUNE_SORT_ITEM, int(best["items"]))
            sort_fn()
            return dict(best, cached=True)
        trials = {}
        for n in sizes:
            _lib.call("spf_tune_set", _lib.SPF_TUNE_SORT_ITEM, int(n))
            sort_fn()
            trials[n] = _time(pass_fn, reps)
        n = min(trials, key=trials.get)
        _lib.call("spf_tune_set", _lib.SPF_TUNE_SORT_ITEM, int(n))
        sort_fn()
        best = {"items": n, "ms": trials[n]}
        cache[key] = best
        _save(cache)
        return dict(best, trials=trials, cached=False)
