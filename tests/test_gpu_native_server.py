"""The native continuous-batching server (spf_serve_* through the C ABI):
every request's indices and distances are exactly those of the plain FP32
pass (spf_dist_argmin_fp32) on the same frames, whether the frames were
settled by the top-8 certificate, by the range list, or by the overflow pass
over all references; pinned and pageable inputs, both paths, a tight HBM
budget, and arrival-based latencies."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def world(lib):
    from spinifel_gb300 import matching

    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(70)
    n_ref, n_pix = 3000, 2048
    refs = rng.gamma(0.5, 1.0, (n_ref, n_pix)).astype(np.float32)
    # a cluster of 40 near-copies (the range list settles their frames) and
    # one of 700 near-copies (more than the list holds: the overflow pass)
    refs[100:140] = refs[100] * (1 + 1e-4 * rng.standard_normal((40, n_pix))).astype(np.float32)
    refs[1000:1700] = refs[1000] * (1 + 1e-5 * rng.standard_normal((700, n_pix))).astype(
        np.float32)
    pick = rng.integers(0, n_ref, 1200)
    pick[:30] = 100
    pick[30:36] = 1000
    frames = np.minimum(rng.poisson(refs[pick] * 4.0), 65535).astype(np.uint16)
    rs = matching.ReferenceSet(torch.as_tensor(refs, device=dev))
    return dict(rs=rs, frames=frames, dev=dev)


def _plain(world, frames_u16):
    """Plain FP32 matching of the same frames through spf_dist_argmin_fp32."""
    from spinifel_gb300 import _lib, matching

    dev = world["dev"]
    rs = world["rs"]
    c = torch.as_tensor(frames_u16.astype(np.int32), device=dev).to(torch.int16)
    fs = matching.FrameSet.from_counts(c)
    n = fs.n
    best = torch.empty(n, dtype=torch.int64, device=dev)
    idx = torch.empty(n, dtype=torch.int32, device=dev)
    dist = torch.empty(n, dtype=torch.float32, device=dev)
    _lib.call("spf_dist_argmin_fp32", _lib.ptr(fs.f32), _lib.ptr(fs.sq), n, _lib.ptr(rs.f32),
              _lib.ptr(rs.sq), rs.n_ref, rs.n_pix, _lib.ptr(best), _lib.ptr(idx), _lib.ptr(dist),
              _lib.stream_handle())
    torch.cuda.synchronize()
    return idx.cpu().numpy(), dist.cpu().numpy()


def _submit_all(srv, frames, sizes, pinned):
    bounds = np.cumsum([0] + sizes)
    futs = []
    for i in range(len(sizes)):
        t = torch.from_numpy(frames[bounds[i]:bounds[i + 1]].view(np.int16).copy())
        if pinned:
            t = t.pin_memory()
        futs.append(srv.submit(t))
    return bounds, futs


@pytest.mark.parametrize("pinned", [True, False])
def test_native_server_equals_plain_fp32(world, pinned):
    from spinifel_gb300.serving import NativeOrientationServer

    sizes = [36, 1, 7, 128, 300, 2, 256, 33, 64, 200, 5, 168]
    with NativeOrientationServer(world["rs"], slot_frames=512, n_slots=3) as srv:
        bounds, futs = _submit_all(srv, world["frames"], sizes, pinned)
        res = [(f.result(timeout=120), f.distances.copy()) for f in futs]
        st = srv.stats
        lat = srv.latency_ms()
    pidx, pdist = _plain(world, world["frames"][:bounds[-1]])
    for i, (idx, dist) in enumerate(res):
        np.testing.assert_array_equal(idx, pidx[bounds[i]:bounds[i + 1]])
        np.testing.assert_array_equal(dist, pdist[bounds[i]:bounds[i + 1]])
    assert st["requests"] == len(sizes) and st["frames"] == bounds[-1]
    assert st["launches"] < len(sizes)        # requests were batched together
    assert st["uncertified"] >= 36            # the two clusters' frames were open
    assert st["range_overflow"] >= 6          # the 700-copy cluster overflowed the list
    assert lat.shape == (len(sizes),) and np.all(lat > 0)
    assert st["p50_ms"] <= st["p99_ms"]


def test_native_server_plain_path_and_tight_budget(world):
    from spinifel_gb300.serving import NativeOrientationServer

    sizes = [100, 50, 100, 100, 30]
    pidx, pdist = _plain(world, world["frames"][:sum(sizes)])
    per_frame = None
    with NativeOrientationServer(world["rs"], slot_frames=256, n_slots=2, path="fp32") as srv:
        bounds, futs = _submit_all(srv, world["frames"], sizes, True)
        got = np.concatenate([f.result(timeout=120) for f in futs])
    np.testing.assert_array_equal(got, pidx)
    # room for 120 frames in flight: slots of 256 are never full
    from spinifel_gb300 import _lib

    tiles = int(_lib.lib().spf_dist_topk_bf16_tiles(world["rs"].n_ref))
    rs = world["rs"]
    per_frame = rs.n_pix * 6 + rs.ld * 2 + 16 + tiles * 64 + 16
    with NativeOrientationServer(world["rs"], slot_frames=256, n_slots=3,
                                 hbm_budget=120 * per_frame) as srv:
        bounds, futs = _submit_all(srv, world["frames"], sizes, True)
        got = np.concatenate([f.result(timeout=120) for f in futs])
        assert srv.stats["launches"] >= 4
    np.testing.assert_array_equal(got, pidx)


def test_native_server_rejects_bad_requests(world):
    from spinifel_gb300 import _lib
    from spinifel_gb300.serving import NativeOrientationServer

    with NativeOrientationServer(world["rs"], slot_frames=64, n_slots=1) as srv:
        big = torch.zeros(65, world["rs"].n_pix, dtype=torch.int16)
        with pytest.raises(_lib.SpfError):
            srv.submit(big)
        flag = ctypes.c_int(0)
        st = _lib.lib().spf_serve_wait(srv._h, 12345, 0, ctypes.byref(flag))
        assert st == _lib.SPF_ERR_ARG and flag.value == 0
        ok = srv.submit(torch.from_numpy(world["frames"][:3].view(np.int16).copy()))
        assert ok.result(timeout=60).shape == (3,)


@pytest.mark.parametrize("chunk", [0, -100, 300, 1200])
def test_host_batch_call_equals_plain_fp32(world, chunk):
    """spf_match_bf16_host (chunked copies overlapped with matching, each
    chunk's open frames completed from its kept tile lists): indices and
    distances equal the plain FP32 pass, the open frames included."""
    from spinifel_gb300 import matching

    frames = world["frames"]
    host = torch.from_numpy(frames.view(np.int16).copy()).pin_memory()
    st = {}
    idx, dist = matching.match_bf16_host(host, world["rs"], chunk_frames=chunk, stats=st)
    pidx, pdist = _plain(world, frames)
    np.testing.assert_array_equal(idx, pidx)
    np.testing.assert_array_equal(dist, pdist)
    assert st["uncertified"] >= 36 and st["range_overflow"] >= 6
