"""BF16 tensor-core distances (tcgen05) with fused top-8 and the exact FP32
re-rank.  The candidate distances are checked against a torch FP64 product of
the same bf16-rounded operands (relative tolerance 1e-5 of the distance
scale), and the final argmin against the plain FP32 path and the FP64 oracle
(identical, or a tie within 1e-6 relative)."""
import numpy as np
import pytest
import torch

from oracle import matching as om

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev(lib):
    return torch.device("cuda", 0)


def _raw_candidates(frames, refs):
    from spinifel_gb300 import _lib

    tiles = int(_lib.lib().spf_dist_topk_bf16_tiles(refs.n_ref))
    cd = torch.empty(tiles * frames.n * 8, dtype=torch.float32, device=frames.f32.device)
    ci = torch.empty(tiles * frames.n * 8, dtype=torch.int32, device=frames.f32.device)
    _lib.call("spf_dist_topk_bf16", _lib.ptr(frames.bf16), frames.n, _lib.ptr(refs.bf16),
              refs.n_ref, refs.n_pix, refs.ld, _lib.ptr(refs.sq), _lib.ptr(cd), _lib.ptr(ci),
              _lib.stream_handle())
    torch.cuda.synchronize()
    return cd.view(tiles, frames.n, 8), ci.view(tiles, frames.n, 8)


@pytest.mark.parametrize("shape", [(128, 256, 64), (130, 600, 256), (300, 1000, 1000),
                                   (7, 3, 8), (129, 224, 72), (64, 449, 200)])
def test_tcgen05_tile_topk_matches_torch(dev, shape):
    from spinifel_gb300 import matching

    n_img, n_ref, n_pix = shape
    g = torch.Generator(device="cpu").manual_seed(40)
    x = torch.rand(n_img, n_pix, generator=g).to(dev)
    s = torch.rand(n_ref, n_pix, generator=g).to(dev)
    fr = matching.FrameSet(x)
    rs = matching.ReferenceSet(s)
    cd, ci = _raw_candidates(fr, rs)
    matching.check_device_error()
    xb = fr.bf16[:, :n_pix].double()
    sb = rs.bf16[:, :n_pix].double()
    approx = rs.sq.double()[None, :] - 2.0 * xb @ sb.T  # [n_img, n_ref]
    scale = float(approx.abs().max())
    tiles = cd.shape[0]
    from spinifel_gb300 import _lib

    tile_refs = int(_lib.lib().spf_dist_topk_bf16_tile_refs())
    assert tiles == -(-n_ref // tile_refs)
    for t in range(tiles):
        lo, hi = t * tile_refs, min((t + 1) * tile_refs, n_ref)
        k = min(8, hi - lo)
        ref_vals, ref_idx = torch.sort(approx[:, lo:hi], dim=1, stable=True)
        got_d = cd[t, :, :k].double()
        got_i = ci[t, :, :k].long()
        # values agree (FP32 accumulation vs FP64)
        assert float((got_d - ref_vals[:, :k]).abs().max()) <= 1e-5 * scale
        # the value the kernel reports for each index is that index's distance
        recomputed = torch.gather(approx, 1, got_i)
        assert float((recomputed - got_d).abs().max()) <= 1e-5 * scale
        if k < 8:
            assert bool((ci[t, :, k:] == 2**31 - 1).all())


@pytest.mark.parametrize("shape", [(500, 3000, 1024), (129, 1000, 4096), (64, 257, 40)])
def test_bf16_rerank_argmin_equals_plain_fp32(dev, shape):
    from spinifel_gb300 import matching

    n_img, n_ref, n_pix = shape
    rng = np.random.default_rng(41)
    refs = rng.random((n_ref, n_pix)).astype(np.float32)
    # frames near some references, plus noise: realistic gaps
    pick = rng.integers(0, n_ref, n_img)
    imgs = (refs[pick] + 0.3 * rng.random((n_img, n_pix))).astype(np.float32)
    x = torch.as_tensor(imgs, device=dev)
    s = torch.as_tensor(refs, device=dev)
    fr, rs = matching.FrameSet(x), matching.ReferenceSet(s)
    st = {}
    idx, dist = matching.match_bf16(fr, rs, stats=st)
    matching.check_device_error()
    pidx, pdist = matching.argmin_fp32(x, s)
    oidx, od = om.sklearn_argmin(refs, imgs)
    assert np.all(om.ties_equal(idx.cpu().numpy(), oidx, od))
    assert np.all(om.ties_equal(idx.cpu().numpy(), pidx.cpu().numpy(), od))
    assert st["uncertified"] <= n_img


def test_bf16_poisson_frames_certify(dev):
    """Integer photon counts are exact in bf16; most frames should certify."""
    from spinifel_gb300 import matching

    rng = np.random.default_rng(42)
    n_ref, n_img, n_pix = 2000, 256, 4096
    refs = rng.gamma(0.5, 1.0, (n_ref, n_pix)).astype(np.float32)
    pick = rng.integers(0, n_ref, n_img)
    imgs = rng.poisson(refs[pick]).astype(np.float32)
    x = torch.as_tensor(imgs, device=dev)
    s = torch.as_tensor(refs, device=dev)
    fr, rs = matching.FrameSet(x), matching.ReferenceSet(s)
    st = {}
    idx, _ = matching.match_bf16(fr, rs, stats=st)
    oidx, od = om.sklearn_argmin(refs, imgs)
    assert np.all(om.ties_equal(idx.cpu().numpy(), oidx, od))
    assert st["uncertified"] < n_img // 2


def test_range_completion_when_gaps_are_tiny(dev):
    """References in clusters of near-duplicates: the top-8 certificate cannot
    separate them, the range query + list re-rank must still give exactly the
    plain FP32 argmin."""
    from spinifel_gb300 import matching

    rng = np.random.default_rng(43)
    base = rng.gamma(0.5, 1.0, (60, 2048)).astype(np.float32)
    refs = np.repeat(base, 12, axis=0) * (1 + 1e-4 * rng.standard_normal((720, 2048))).astype(
        np.float32)
    refs = refs.astype(np.float32)
    pick = rng.integers(0, 720, 300)
    imgs = rng.poisson(refs[pick]).astype(np.float32)
    x = torch.as_tensor(imgs, device=dev)
    s = torch.as_tensor(refs, device=dev)
    fr, rs = matching.FrameSet(x), matching.ReferenceSet(s)
    st = {}
    idx, dist = matching.match_bf16(fr, rs, stats=st)
    pidx, pdist = matching.argmin_fp32(x, s)
    assert st["uncertified"] > 0
    assert torch.equal(idx, pidx)
    assert torch.equal(dist, pdist)  # bit-identical distances


def test_rerank_distances_bit_identical_to_plain(dev):
    from spinifel_gb300 import matching

    rng = np.random.default_rng(44)
    refs = rng.random((700, 1000)).astype(np.float32)
    imgs = (refs[rng.integers(0, 700, 200)] + 0.2 * rng.random((200, 1000))).astype(np.float32)
    x = torch.as_tensor(imgs, device=dev)
    s = torch.as_tensor(refs, device=dev)
    idx, dist = matching.match_bf16(matching.FrameSet(x), matching.ReferenceSet(s))
    pidx, pdist = matching.argmin_fp32(x, s)
    assert torch.equal(idx, pidx) and torch.equal(dist, pdist)


def test_autotuner_picks_a_candidate_and_never_changes_results(dev, tmp_path, monkeypatch):
    from spinifel_gb300 import _lib, autotune, matching

    monkeypatch.setenv("SPF_TUNE_CACHE", str(tmp_path / "tuned.json"))
    rng = np.random.default_rng(45)
    refs = rng.random((1500, 1024)).astype(np.float32)
    imgs = (refs[rng.integers(0, 1500, 400)] + 0.3 * rng.random((400, 1024))).astype(np.float32)
    fr = matching.FrameSet(torch.as_tensor(imgs, device=dev))
    rs = matching.ReferenceSet(torch.as_tensor(refs, device=dev))
    base, _ = matching.match_bf16(fr, rs)
    try:
        rec = autotune.tune_bf16(fr, rs, group_sizes=(1, 2, 16), grids=(0, 64))
        assert rec["group_m"] in (1, 2, 16) and rec["grid"] in (0, 64) and not rec["cached"]
        assert len(rec["trials"]) == 6
        for gm, gr in ((1, 64), (2, 0), (16, 0)):
            _lib.call("spf_tune_set", _lib.SPF_TUNE_BF16_GROUP_M, gm)
            _lib.call("spf_tune_set", _lib.SPF_TUNE_BF16_GRID, gr)
            idx, _ = matching.match_bf16(fr, rs)
            assert torch.equal(idx, base)
        rec2 = autotune.tune_bf16(fr, rs)
        assert rec2["cached"] and rec2["group_m"] == rec["group_m"]
    finally:
        _lib.call("spf_tune_set", _lib.SPF_TUNE_BF16_GROUP_M, 0)
        _lib.call("spf_tune_set", _lib.SPF_TUNE_BF16_GRID, 0)


def test_bf16_paths_accept_empty_inputs(dev):
    """No frames: the tensor-core path, the one-call host path and the static
    entry point all return empty answers (and launch nothing that fails)."""
    import ctypes

    from spinifel_gb300 import _lib, matching

    g = torch.Generator(device="cpu").manual_seed(41)
    rs = matching.ReferenceSet(torch.rand(300, 64, generator=g).to(dev))
    fr = matching.FrameSet(torch.empty(0, 64, device=dev))
    idx, dist = matching.match_bf16(fr, rs)
    assert idx.numel() == 0 and dist.numel() == 0
    h_idx, h_dist = matching.match_bf16_host(torch.empty(0, 64, dtype=torch.int16).pin_memory(),
                                             rs)
    assert h_idx.size == 0 and h_dist.size == 0
    L = _lib.lib()
    assert L.spf_match_bf16_static(ctypes.c_void_p(16), ctypes.c_void_p(16),
                                   ctypes.c_void_p(16), 0, ctypes.c_void_p(16),
                                   ctypes.c_void_p(16), ctypes.c_void_p(16),
                                   ctypes.c_void_p(16), 1.0, 300, 64, 64, ctypes.c_void_p(16),
                                   None, None, None) == _lib.SPF_OK
    matching.check_device_error()
