"""spf_match_bf16_static: matching for callers that cannot allocate device
memory (a data-acquisition process whose GPU memory is fixed at start-up, or
a plug-in whose host application owns the device memory).  Called through
the C ABI, it must give exactly what the allocating entry points
(spf_dist_topk_bf16 + spf_rerank_fp32) give, on two calls in a row with
different frames, without taking device memory after its first call and
without a device error, and must reject sizes beyond its static scratch.
This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _allocating(lib_mod, fr, rs):
    L = lib_mod
    tiles = int(L.lib().spf_dist_topk_bf16_tiles(rs.n_ref))
    dev = fr.f32.device
    cd = torch.empty(tiles * fr.n * 8, dtype=torch.float32, device=dev)
    ci = torch.empty(tiles * fr.n * 8, dtype=torch.int32, device=dev)
    work = torch.empty(fr.n, dtype=torch.float32, device=dev)
    idx = torch.empty(fr.n, dtype=torch.int32, device=dev)
    dist = torch.empty(fr.n, dtype=torch.float32, device=dev)
    unc = torch.empty(fr.n, dtype=torch.int32, device=dev)
    sh = L.stream_handle()
    L.call("spf_dist_topk_bf16", L.ptr(fr.bf16), fr.n, L.ptr(rs.bf16), rs.n_ref, rs.n_pix, rs.ld,
           L.ptr(rs.sq), L.ptr(cd), L.ptr(ci), sh)
    L.call("spf_rerank_fp32", L.ptr(cd), L.ptr(ci), tiles, L.ptr(fr.f32), L.ptr(fr.sq), fr.n,
           L.ptr(rs.f32), L.ptr(rs.sq), L.ptr(rs.m2), float(rs.sq_max), rs.n_ref, rs.n_pix, 0,
           L.ptr(work), L.ptr(idx), L.ptr(dist), L.ptr(unc), None, sh)
    torch.cuda.synchronize()
    return idx, dist, unc


def _static(lib_mod, fr, rs, idx, dist, unc):
    L = lib_mod
    L.call("spf_match_bf16_static", L.ptr(fr.bf16), L.ptr(fr.f32), L.ptr(fr.sq), fr.n,
           L.ptr(rs.bf16), L.ptr(rs.f32), L.ptr(rs.sq), L.ptr(rs.m2), float(rs.sq_max), rs.n_ref,
           rs.n_pix, rs.ld, L.ptr(idx), L.ptr(dist), L.ptr(unc), L.stream_handle())
    torch.cuda.synchronize()


def test_static_scratch_entry_point_matches_allocating_path(lib):
    from spinifel_gb300 import _lib, matching

    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(90)
    n_ref, n_pix = 3000, 2048
    refs = rng.gamma(0.5, 1.0, (n_ref, n_pix)).astype(np.float32)
    rs = matching.ReferenceSet(torch.as_tensor(refs, device=dev))
    frames = []
    for n in (300, 77):  # two calls in a row, different frames and sizes
        pick = rng.integers(0, n_ref, n)
        x = torch.as_tensor(rng.poisson(refs[pick]).astype(np.float32), device=dev)
        frames.append(matching.FrameSet(x))
    outs = [(torch.empty(f.n, dtype=torch.int32, device=dev),
             torch.empty(f.n, dtype=torch.float32, device=dev),
             torch.empty(f.n, dtype=torch.int32, device=dev)) for f in frames]
    torch.cuda.synchronize()
    free_before = None
    for k, (fr, out) in enumerate(zip(frames, outs)):
        _static(_lib, fr, rs, *out)
        if k == 0:
            free_before = torch.cuda.mem_get_info(dev)[0]
    free_after = torch.cuda.mem_get_info(dev)[0]
    assert free_after == free_before  # no device memory taken by the second call
    code = ctypes.c_int(-1)
    _lib.call("spf_device_error", _lib.stream_handle(), ctypes.byref(code))
    assert code.value == 0  # no bounded wait gave up (the static path's word included)
    for idx, _, _ in outs:
        assert bool((idx >= 0).all())  # no frame was marked void
    for fr, (idx, dist, unc) in zip(frames, outs):
        ridx, rdist, runc = _allocating(_lib, fr, rs)
        assert torch.equal(idx, ridx)
        assert torch.equal(dist, rdist)
        assert torch.equal(unc, runc)


def test_static_scratch_call_replays_from_a_cuda_graph(lib):
    """The static entry point recorded in a CUDA graph (after a first call on
    the device, which looks up the scratch and sets the kernel attributes)
    and replayed on new frame contents copied into the same buffers gives
    exactly the allocating path's answer for those frames."""
    from spinifel_gb300 import _lib, matching

    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(92)
    n_ref, n_pix, n = 2000, 1024, 150
    refs = rng.gamma(0.5, 1.0, (n_ref, n_pix)).astype(np.float32)
    rs = matching.ReferenceSet(torch.as_tensor(refs, device=dev))

    def frames():
        pick = rng.integers(0, n_ref, n)
        x = torch.as_tensor(rng.poisson(refs[pick]).astype(np.float32), device=dev)
        return matching.FrameSet(x)

    fr, fr_b = frames(), frames()
    out = (torch.empty(n, dtype=torch.int32, device=dev),
           torch.empty(n, dtype=torch.float32, device=dev),
           torch.empty(n, dtype=torch.int32, device=dev))
    _static(_lib, fr, rs, *out)  # first call on the device: outside the capture
    L = _lib
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        L.call("spf_match_bf16_static", L.ptr(fr.bf16), L.ptr(fr.f32), L.ptr(fr.sq), fr.n,
               L.ptr(rs.bf16), L.ptr(rs.f32), L.ptr(rs.sq), L.ptr(rs.m2), float(rs.sq_max),
               rs.n_ref, rs.n_pix, rs.ld, L.ptr(out[0]), L.ptr(out[1]), L.ptr(out[2]),
               L.stream_handle())
    fr.f32.copy_(fr_b.f32)
    fr.bf16.copy_(fr_b.bf16)
    fr.sq.copy_(fr_b.sq)
    g.replay()
    torch.cuda.synchronize()
    code = ctypes.c_int(-1)
    _lib.call("spf_device_error", _lib.stream_handle(), ctypes.byref(code))
    assert code.value == 0
    ridx, rdist, runc = _allocating(_lib, fr_b, rs)
    assert torch.equal(out[0], ridx) and torch.equal(out[1], rdist)
    assert torch.equal(out[2], runc)


def test_static_scratch_abort_is_reported_and_voids_the_call(lib):
    """A GEMM that gave up a bounded wait (recorded by the library's test hook
    right after the GEMM, as the kernel's own timeout path records it): every
    frame of the call comes back void (index -1, distance NaN, uncertified)
    and spf_device_error reports SPF_ERR_TIMEOUT once; the next call is
    exact again."""
    from spinifel_gb300 import _lib, matching

    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(91)
    n_ref, n_pix = 1000, 1024
    refs = rng.gamma(0.5, 1.0, (n_ref, n_pix)).astype(np.float32)
    rs = matching.ReferenceSet(torch.as_tensor(refs, device=dev))
    pick = rng.integers(0, n_ref, 50)
    fr = matching.FrameSet(torch.as_tensor(rng.poisson(refs[pick]).astype(np.float32), device=dev))
    out = (torch.zeros(fr.n, dtype=torch.int32, device=dev),
           torch.zeros(fr.n, dtype=torch.float32, device=dev),
           torch.zeros(fr.n, dtype=torch.int32, device=dev))
    code = ctypes.c_int(-1)
    _lib.call("spf_device_error", _lib.stream_handle(), ctypes.byref(code))  # start clean
    _lib.call("spf_tune_set", _lib.SPF_TUNE_STATIC_ABORT_TEST, 1)
    try:
        _static(_lib, fr, rs, *out)
    finally:
        _lib.call("spf_tune_set", _lib.SPF_TUNE_STATIC_ABORT_TEST, 0)
    idx, dist, unc = out
    assert bool((idx == -1).all())
    assert bool(torch.isnan(dist).all())
    assert bool((unc == 1).all())
    _lib.call("spf_device_error", _lib.stream_handle(), ctypes.byref(code))
    assert code.value == -_lib.SPF_ERR_TIMEOUT
    _lib.call("spf_device_error", _lib.stream_handle(), ctypes.byref(code))
    assert code.value == 0  # reported once, then cleared
    _static(_lib, fr, rs, *out)
    ridx, rdist, runc = _allocating(_lib, fr, rs)
    assert torch.equal(out[0], ridx) and torch.equal(out[1], rdist)
    assert torch.equal(out[2], runc)


def test_static_scratch_entry_point_rejects_oversize(lib):
    from spinifel_gb300 import _lib

    L = _lib.lib()
    # 4097 frames: more than the scratch holds; rejected before any device work
    st = L.spf_match_bf16_static(ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16),
                                 4097, ctypes.c_void_p(16), ctypes.c_void_p(16),
                                 ctypes.c_void_p(16), ctypes.c_void_p(16), 1.0, 1000, 64, 64,
                                 ctypes.c_void_p(16), None, None, None)
    assert st == _lib.SPF_ERR_ARG
    assert b"static scratch limit" in L.spf_last_error()
    # 2000 frames x 200,000 references: 893 tiles * 2000 > 262,144
    st = L.spf_match_bf16_static(ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16),
                                 2000, ctypes.c_void_p(16), ctypes.c_void_p(16),
                                 ctypes.c_void_p(16), ctypes.c_void_p(16), 1.0, 200_000, 64, 64,
                                 ctypes.c_void_p(16), None, None, None)
    assert st == _lib.SPF_ERR_ARG
    assert b"static scratch limit" in L.spf_last_error()
