"""Parity of the CUDA NUFFT kernels (type 2 interpolation / slicing, type 1
spreading) with the FP64 oracle; tolerance: relative L2 error <= 1e-5 at
eps = 1e-6 (FP32 on the device)."""
import os

import numpy as np
import pytest
import torch

from oracle import nufft as onufft
from tests.golden import cases

pytestmark = pytest.mark.gpu
TOL = 1e-5
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.fixture(scope="module")
def dev(lib):
    return torch.device("cuda", 0)


def t(a, dev, dtype=torch.float32):
    return torch.as_tensor(np.asarray(a), dtype=dtype, device=dev)


@pytest.mark.parametrize("m", [(9, 9, 9), (10, 11, 12), (21, 21, 21)])
@pytest.mark.parametrize("isign", [-1, 1])
def test_type2_interp_matches_direct_sum(dev, m, isign):
    from spinifel_gb300.nufft import NufftPlan

    rng = np.random.default_rng(10)
    f = rng.standard_normal(m)
    x, y, z = rng.uniform(-3 * np.pi + 1e-3, 3 * np.pi - 1e-3, (3, 3000)).astype(np.float32)
    P = NufftPlan(m, 1e-6)
    P.set_modes(t(f, dev), isign=isign, want_imag=True)
    re, im = P.interp(t(x, dev), t(y, dev), t(z, dev), want_imag=True)
    got = re.cpu().numpy() + 1j * im.cpu().numpy()
    exact = onufft.nudft3d2(x, y, z, f, isign)
    assert rel(got, exact) < TOL


def test_type2_support_multiplies_modes(dev):
    from spinifel_gb300.nufft import NufftPlan

    rng = np.random.default_rng(11)
    m = (11, 11, 11)
    f = rng.standard_normal(m)
    sup = (rng.random(m) > 0.5).astype(np.float64)
    x, y, z = rng.uniform(-np.pi, np.pi, (3, 1000)).astype(np.float32)
    P = NufftPlan(m, 1e-6)
    P.set_modes(t(f, dev), t(sup, dev))
    re, _ = P.interp(t(x, dev), t(y, dev), t(z, dev))
    assert rel(re.cpu().numpy(), onufft.nudft3d2(x, y, z, f * sup, -1).real) < TOL


@pytest.mark.parametrize("m", [(9, 9, 9), (8, 10, 7), (30, 30, 30)])
@pytest.mark.parametrize("isign", [-1, 1])
def test_type1_spread_matches_direct_sum(dev, m, isign):
    from spinifel_gb300.nufft import NufftPlan

    rng = np.random.default_rng(12)
    x, y, z = rng.uniform(-3 * np.pi + 1e-3, 3 * np.pi - 1e-3, (3, 4000)).astype(np.float32)
    c = rng.standard_normal(4000).astype(np.float32)
    P = NufftPlan(m, 1e-6)
    P.spread_zero()
    P.spread(t(x, dev), t(y, dev), t(z, dev), t(c, dev))
    re, im = P.finish(isign, want_imag=True)
    got = re.cpu().numpy() + 1j * im.cpu().numpy()
    exact = onufft.nudft3d1(x, y, z, c, m, isign)
    assert rel(got, exact) < TOL


def test_one_call_type1_and_fft_deconv_stage(dev):
    """spf_spread_t1 (zero + spread + finish in one call) against the direct
    sum, and spf_fft_deconv's two directions against the calls they stand for."""
    from spinifel_gb300 import _lib
    from spinifel_gb300.nufft import NufftPlan

    rng = np.random.default_rng(13)
    m = (12, 11, 10)
    x, y, z = rng.uniform(-3 * np.pi + 1e-3, 3 * np.pi - 1e-3, (3, 3000)).astype(np.float32)
    c = rng.standard_normal(3000).astype(np.float32)
    P = NufftPlan(m, 1e-6)
    xt, yt, zt, ct = (t(v, dev) for v in (x, y, z, c))
    re = torch.empty(m, dtype=torch.float32, device=dev)
    im = torch.empty(m, dtype=torch.float32, device=dev)
    sh = _lib.stream_handle()
    _lib.call("spf_spread_t1", P.handle, _lib.ptr(xt), _lib.ptr(yt), _lib.ptr(zt), _lib.ptr(ct),
              3000, 1, _lib.ptr(re), _lib.ptr(im), sh)
    got = re.cpu().numpy() + 1j * im.cpu().numpy()
    assert rel(got, onufft.nudft3d1(x, y, z, c, m, 1)) < TOL
    # type 1 stage: spread, then spf_fft_deconv == spf_nufft_t1_finish
    P.spread_zero()
    P.spread(xt, yt, zt, ct)
    re2 = torch.empty_like(re)
    _lib.call("spf_fft_deconv", P.handle, 1, 1, None, None, _lib.ptr(re2), None, sh)
    assert rel(re2.cpu().numpy(), re.cpu().numpy()) < 1e-6  # float atomics: order may differ
    # type 2 stage: spf_fft_deconv then interpolation == set_modes then interpolation
    f = t(rng.standard_normal(m), dev)
    _lib.call("spf_fft_deconv", P.handle, 2, -1, _lib.ptr(f), None, None, None, sh)
    a, _ = P.interp(xt, yt, zt)
    P.set_modes(f, isign=-1)
    b, _ = P.interp(xt, yt, zt)
    assert torch.equal(a, b)
    with pytest.raises(_lib.SpfError):
        _lib.call("spf_fft_deconv", P.handle, 1, 1, _lib.ptr(f), None, _lib.ptr(re2), None, sh)


def test_type1_is_adjoint_of_type2(dev):
    from spinifel_gb300.nufft import NufftPlan

    rng = np.random.default_rng(13)
    m = (12, 12, 12)
    f = rng.standard_normal(m)
    x, y, z = rng.uniform(-np.pi, np.pi, (3, 5000)).astype(np.float32)
    c = rng.standard_normal(5000).astype(np.float32)
    P = NufftPlan(m, 1e-6)
    P.set_modes(t(f, dev), isign=-1, want_imag=True)
    re, im = P.interp(t(x, dev), t(y, dev), t(z, dev), want_imag=True)
    P.spread_zero()
    P.spread(t(x, dev), t(y, dev), t(z, dev), t(c, dev))
    fr, fi = P.finish(+1, want_imag=True)
    lhs = np.vdot(c, re.cpu().numpy() + 1j * im.cpu().numpy())
    rhs = np.vdot(fr.cpu().numpy() + 1j * fi.cpu().numpy(), f)
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def _slice_case(M, det, n_orient, seed):
    from spinifel_gb300 import geom, synth

    rng = np.random.default_rng(seed)
    model = synth.intensity_model(M, seed=seed)
    ppr, pdr = geom.flat_detector(*det)
    quats = geom.uniform_quaternions(n_orient, rng).astype(np.float32)
    return model, ppr, pdr, quats


def _oracle_slices(model, ppr, pdr, quats, eps=1e-12):
    from spinifel_gb300 import geom

    mult = np.pi / pdr.max()
    H, K, L = geom.hkl(quats.astype(np.float64), ppr)
    return onufft.nufft3d2(H.reshape(-1) * mult, K.reshape(-1) * mult, L.reshape(-1) * mult,
                           model, -1, eps).real.reshape(len(quats), -1)


def test_slice_matches_oracle_config1_geometry(dev):
    """41^3 model, 4 x 32 x 32 detector (the CPU-runnable configuration)."""
    from spinifel_gb300.nufft import NufftPlan

    model, ppr, pdr, quats = _slice_case(41, (4, 32, 32), 300, 20)
    P = NufftPlan(41, 1e-6)
    P.set_modes(t(model, dev))
    bf = torch.empty(300, ppr[0].size, dtype=torch.bfloat16, device=dev)
    got = P.slice(t(quats, dev), t(ppr.reshape(3, -1), dev), np.pi / pdr.max(), out_bf16=bf)
    exact = _oracle_slices(model, ppr, pdr, quats)
    assert rel(got.cpu().numpy(), exact) < TOL
    assert torch.equal(bf, got.to(torch.bfloat16))


def test_slice_full_size_subset_and_linearity(dev):
    """81^3 model, 4 x 128 x 128 detector: a subset of orientations against the
    oracle, and linearity in the model at full batch size."""
    from spinifel_gb300.nufft import NufftPlan

    model, ppr, pdr, quats = _slice_case(81, (4, 128, 128), 512, 21)
    ppr_t = t(ppr.reshape(3, -1), dev)
    mult = np.pi / pdr.max()
    P = NufftPlan(81, 1e-6)
    P.set_modes(t(model, dev))
    full = P.slice(t(quats, dev), ppr_t, mult)
    sub = [0, 7, 511]
    exact = _oracle_slices(model, ppr, pdr, quats[sub], eps=1e-9)
    assert rel(full[sub].cpu().numpy(), exact) < TOL
    rng = np.random.default_rng(22)
    g = rng.standard_normal(model.shape)
    P.set_modes(t(g, dev))
    sg = P.slice(t(quats, dev), ppr_t, mult)
    P.set_modes(t(2.0 * model - 3.0 * g, dev))
    comb = P.slice(t(quats, dev), ppr_t, mult)
    lin = 2.0 * full.double() - 3.0 * sg.double()
    assert float((comb.double() - lin).norm() / lin.norm()) < 1e-6


@pytest.mark.parametrize("det", [(4, 32, 32), (4, 128, 128), (2, 20, 37)])
def test_patch_slicing_identical_to_point_slicing(dev, det):
    """spf_slice_t2_det (shared-memory patches) gives the same bits as
    spf_slice_t2 (thread per point), ragged patches included, with every
    tile shape the autotuner chooses from."""
    from spinifel_gb300 import _lib
    from spinifel_gb300.nufft import NufftPlan

    model, ppr, pdr, quats = _slice_case(81, det, 64, 25)
    ppr_t = t(ppr.reshape(3, -1), dev)
    P = NufftPlan(81, 1e-6)
    P.set_modes(t(model, dev))
    a = P.slice(t(quats, dev), ppr_t, np.pi / pdr.max())
    try:
        for shape in range(8):
            _lib.call("spf_tune_set", _lib.SPF_TUNE_SLICE_SHAPE, shape)
            b = P.slice(t(quats, dev), ppr_t, np.pi / pdr.max(), det_shape=det)
            assert torch.equal(a, b), shape
    finally:
        _lib.call("spf_tune_set", _lib.SPF_TUNE_SLICE_SHAPE, 0)


def test_spread_orient_equals_spread_points(dev):
    from spinifel_gb300 import geom
    from spinifel_gb300.nufft import NufftPlan

    model, ppr, pdr, quats = _slice_case(15, (4, 16, 16), 20, 23)
    mult = np.pi / pdr.max()
    rng = np.random.default_rng(24)
    c = rng.poisson(2.0, (20, ppr[0].size)).astype(np.float32)
    P = NufftPlan(15, 1e-6)
    P.spread_zero()
    P.spread_orient(t(quats, dev), t(ppr.reshape(3, -1), dev), mult, t(c, dev))
    a, _ = P.finish(+1)
    H, K, L = geom.hkl(quats.astype(np.float64), ppr)
    P.spread_zero()
    P.spread(*(t(v.reshape(-1) * mult, dev) for v in (H, K, L)), t(c, dev))
    b, _ = P.finish(+1)
    assert rel(a.cpu().numpy(), b.cpu().numpy()) < 1e-5


@pytest.mark.parametrize("det", [(4, 16, 16), (4, 128, 128), (2, 20, 37)])
def test_patch_spreading_equals_point_spreading(dev, det):
    from spinifel_gb300.nufft import NufftPlan

    model, ppr, pdr, quats = _slice_case(41, det, 24, 26)
    mult = np.pi / pdr.max()
    rng = np.random.default_rng(27)
    c = t(rng.poisson(2.0, (24, ppr[0].size)).astype(np.float32), dev)
    ppr_t = t(ppr.reshape(3, -1), dev)
    P = NufftPlan(41, 1e-6)
    out = []
    for shape in (None, det):
        P.spread_zero()
        P.spread_orient(t(quats, dev), ppr_t, mult, c, det_shape=shape)
        out.append(P.finish(+1)[0].cpu().numpy())
    # two FP32 accumulation orders (shared-memory box then flush, vs direct
    # atomics) over ~1.6e6 points: equal within the NUFFT tolerance
    assert rel(out[1], out[0]) < TOL
    # the fused interpolate-then-spread operator, point vs patch kernels
    from spinifel_gb300 import _lib

    P.set_modes(t(model, dev))
    res = []
    for patch in (False, True):
        P.spread_zero()
        if patch:
            _lib.call("spf_nufft_interp_spread_det", P.handle, _lib.ptr(t(quats, dev)), 24,
                      _lib.ptr(ppr_t), det[0], det[1], det[2], float(mult), None,
                      _lib.stream_handle())
        else:
            _lib.call("spf_nufft_interp_spread_orient", P.handle, _lib.ptr(t(quats, dev)), 24,
                      _lib.ptr(ppr_t), ppr_t.shape[1], float(mult), None, _lib.stream_handle())
        res.append(P.finish(+1)[0].cpu().numpy())
    assert rel(res[1], res[0]) < TOL


def test_sorted_interp_spread_equals_unsorted(dev):
    from spinifel_gb300 import _lib
    from spinifel_gb300.nufft import NufftPlan

    det = (4, 64, 64)
    model, ppr, pdr, quats = _slice_case(41, det, 40, 28)
    mult = float(np.pi / pdr.max())
    ppr_t = t(ppr.reshape(3, -1), dev)
    q_t = t(quats, dev)
    w = t(np.random.default_rng(29).random((40, ppr[0].size)).astype(np.float32), dev)
    P = NufftPlan(41, 1e-6)
    P.set_modes(t(model, dev))
    P.spread_zero()
    _lib.call("spf_nufft_interp_spread_orient", P.handle, _lib.ptr(q_t), 40, _lib.ptr(ppr_t),
              ppr_t.shape[1], mult, _lib.ptr(w), _lib.stream_handle())
    a = P.finish(+1)[0].cpu().numpy()
    _lib.call("spf_nufft_sort_orient", P.handle, _lib.ptr(q_t), 40, _lib.ptr(ppr_t), ppr_t.shape[1],
              mult, _lib.stream_handle())
    P.spread_zero()
    _lib.call("spf_nufft_interp_spread_sorted", P.handle, _lib.ptr(w), _lib.stream_handle())
    b = P.finish(+1)[0].cpu().numpy()
    from spinifel_gb300 import matching

    matching.check_device_error()  # no point fell outside its bin's box
    assert rel(b, a) < TOL


def test_operator_glue_matches_reference_golden(dev):
    """autocorrelation.forward / adjoint against the reference's own glue
    (support, real part, / M^3) run on the FP64 oracle."""
    from spinifel_gb300 import autocorrelation as ac

    ugrid, sup, H_, K_, L_, nuv = cases.ops_inputs()
    g = np.load(os.path.join(GOLD, "golden_ops.npz"))
    fwd = ac.forward(ugrid.copy(), H_, K_, L_, sup, True, H_.size)
    adj = ac.adjoint(nuv, H_, K_, L_, cases.OPS["M"], True, sup)
    assert rel(fwd, g["forward"]) < TOL
    assert rel(adj, g["adjoint"]) < TOL
    assert adj.dtype in (np.float32, np.float64) and adj.shape == (15, 15, 15)


@pytest.mark.parametrize("with_values", [True, False])
def test_sorted_spread_of_explicit_points_equals_unsorted(dev, with_values):
    """spf_nufft_sort_points + spf_nufft_spread_sorted (bin-sorted, runs of
    points with the same footprint cell summed in registers) equals the
    thread-per-point type-1 spreading, with values and with ones (NULL)."""
    from spinifel_gb300 import geom
    from spinifel_gb300.nufft import NufftPlan

    model, ppr, pdr, quats = _slice_case(31, (4, 32, 32), 60, 41)
    mult = np.pi / pdr.max()
    H, K, L = geom.hkl(quats.astype(np.float64), ppr)
    x, y, z = (t(v.reshape(-1) * mult, dev) for v in (H, K, L))
    rng = np.random.default_rng(42)
    c = t(rng.poisson(2.0, x.numel()).astype(np.float32), dev) if with_values else \
        torch.ones(x.numel(), dtype=torch.float32, device=dev)
    P = NufftPlan(31, 1e-6)
    P.spread_zero()
    P.spread(x, y, z, c)
    a, _ = P.finish(+1)
    P.sort_points(x, y, z)
    P.spread_zero()
    P.spread_sorted(c if with_values else None)
    b, _ = P.finish(+1)
    from spinifel_gb300 import matching

    matching.check_device_error()  # no point fell outside its bin's box
    assert rel(b.cpu().numpy(), a.cpu().numpy()) < 1e-6


def test_adjoint_sorted_matches_oracle(dev):
    """autocorrelation.adjoint with the sorted spreading forced on equals the
    FP64 oracle's adjoint (the reference's glue) at the NUFFT tolerance."""
    from spinifel_gb300 import autocorrelation as ac
    from spinifel_gb300 import geom

    model, ppr, pdr, quats = _slice_case(21, (4, 16, 16), 30, 43)
    mult = np.pi / pdr.max()
    H, K, L = (v.reshape(-1) * mult for v in geom.hkl(quats.astype(np.float64), ppr))
    nuv = np.random.default_rng(44).standard_normal(H.size)
    got = ac.adjoint(nuv, H, K, L, 21, True, None, sort=True)
    want = onufft.adjoint(nuv, H, K, L, 21, True, None)
    assert rel(np.asarray(got), np.asarray(want)) < TOL


def test_spread_orient_sorted_equals_patch(dev):
    """NufftPlan.spread_orient with the bin sort + sorted spreading (what it
    picks for large point sets) equals the patch kernel on the same points."""
    from spinifel_gb300.nufft import NufftPlan

    model, ppr, pdr, quats = _slice_case(41, (4, 32, 32), 50, 45)
    mult = np.pi / pdr.max()
    ppr_t = t(ppr.reshape(3, -1), dev)
    q_t = t(quats, dev)
    c = t(np.random.default_rng(46).poisson(1.5, (50, ppr[0].size)).astype(np.float32), dev)
    P = NufftPlan(41, 1e-6)
    out = []
    for sort in (False, True):
        P.spread_zero()
        P.spread_orient(q_t, ppr_t, mult, c.reshape(-1), det_shape=(4, 32, 32), sort=sort)
        out.append(P.finish(+1)[0].cpu().numpy())
    from spinifel_gb300 import matching

    matching.check_device_error()
    assert rel(out[1], out[0]) < 1e-6


@pytest.mark.parametrize("eps,tol", [(1e-6, TOL), (1e-12, 1e-10)])
def test_gen_model_slices_matches_oracle(dev, eps, tol):
    """slicing.gen_model_slices (the reference's signature) and its batched
    form against the oracle's type 2 at the normalised rotated positions."""
    from spinifel_gb300 import geom
    from spinifel_gb300.slicing import gen_model_slices, gen_model_slices_batch

    model, ppr, pdr, quats = _slice_case(21, (4, 16, 16), 12, 90)
    n_pix = ppr[0].size
    s = gen_model_slices(model, quats, ppr, pdr.max(), 1, None, n_pix, None, eps=eps)
    H, K, L = geom.hkl(quats, ppr)
    mult = np.pi / pdr.max()
    want = onufft.nufft3d2(H.reshape(-1) * mult, K.reshape(-1) * mult, L.reshape(-1) * mult,
                           model, -1, 1e-12).real
    assert s.shape == (12 * n_pix,)
    assert rel(s, want) < tol
    sb = gen_model_slices_batch(model, quats, ppr, pdr.max(), 1, None, n_pix, batch_size=4,
                                eps=eps)
    np.testing.assert_array_equal(sb, s)
    with pytest.raises(ValueError):
        gen_model_slices(model, quats, ppr, pdr.max(), 1, None, n_pix, "cpu")


def test_sorted_pass_item_size_keeps_the_operator(dev):
    """The bin-sorted direct operator split into work items of 512, 1,024,
    4,096 or 8,192 points (SPF_TUNE_SORT_ITEM; the default is 2,048) gives
    the default's result to rounding, and reports no device error."""
    from spinifel_gb300 import _lib
    from spinifel_gb300.nufft import NufftPlan

    model, ppr, pdr, quats = _slice_case(31, (4, 32, 32), 120, 46)
    q, ppr_t = t(quats, dev), t(ppr.reshape(3, -1), dev)
    mult = np.pi / pdr.max()
    P = NufftPlan(31, 1e-6)
    P.set_modes(t(model, dev))
    res = {}
    try:
        for n in (0, 512, 1024, 4096, 8192):
            _lib.call("spf_tune_set", _lib.SPF_TUNE_SORT_ITEM, n)
            _lib.call("spf_nufft_sort_orient", P.handle, _lib.ptr(q), q.shape[0],
                      _lib.ptr(ppr_t), ppr_t.shape[1], float(mult), _lib.stream_handle())
            P.spread_zero()
            _lib.call("spf_nufft_interp_spread_sorted", P.handle, None, _lib.stream_handle())
            res[n] = P.finish(+1)[0].cpu().numpy()
    finally:
        _lib.call("spf_tune_set", _lib.SPF_TUNE_SORT_ITEM, 0)
    from spinifel_gb300 import matching

    matching.check_device_error()
    for n in (512, 1024, 4096, 8192):
        assert rel(res[n], res[0]) < 1e-6


# Every kernel width the FP32 plan compiles (w = ceil(-log10(eps / 10)): 3 .. 8),
# not only the w = 7 of eps 1e-6: type 2 and type 1 against the direct sums with
# a tolerance that follows eps (the kernel's error) above FP32's floor, the
# bin-sorted spreading against the per-point spreading, and the patch slicing
# (every tile shape, the stride search included) bit for bit against the
# per-point slicing.
WIDTH_EPS = [(1e-2, 3), (1e-3, 4), (1e-4, 5), (1e-5, 6), (1e-7, 8)]


def _width_tol(eps):
    return max(20.0 * eps, 1e-5)


@pytest.mark.parametrize("eps,w", WIDTH_EPS)
def test_type2_and_type1_every_width(dev, eps, w):
    from spinifel_gb300.nufft import NufftPlan

    rng = np.random.default_rng(60 + w)
    m = (13, 12, 11)
    P = NufftPlan(m, eps)
    assert P.width == w
    f = rng.standard_normal(m)
    x, y, z = rng.uniform(-3 * np.pi + 1e-3, 3 * np.pi - 1e-3, (3, 2000)).astype(np.float32)
    P.set_modes(t(f, dev), isign=-1, want_imag=True)
    re, im = P.interp(t(x, dev), t(y, dev), t(z, dev), want_imag=True)
    got = re.cpu().numpy() + 1j * im.cpu().numpy()
    assert rel(got, onufft.nudft3d2(x, y, z, f, -1)) < _width_tol(eps)
    c = rng.standard_normal(2000).astype(np.float32)
    P.spread_zero()
    P.spread(t(x, dev), t(y, dev), t(z, dev), t(c, dev))
    re1, im1 = P.finish(+1, want_imag=True)
    exact1 = onufft.nudft3d1(x, y, z, c, m, +1)
    g1 = re1.cpu().numpy() + 1j * im1.cpu().numpy()
    assert rel(g1, exact1) < _width_tol(eps)
    # the bin-sorted pass over the same points gives the same sums (up to the
    # order of the float additions)
    P.sort_points(t(x, dev), t(y, dev), t(z, dev))
    P.spread_zero()
    P.spread_sorted(t(c, dev))
    re2, im2 = P.finish(+1, want_imag=True)
    g2 = re2.cpu().numpy() + 1j * im2.cpu().numpy()
    assert rel(g2, g1) < 1e-5


@pytest.mark.parametrize("eps,w", WIDTH_EPS)
def test_patch_slicing_every_width_and_shape(dev, eps, w):
    from spinifel_gb300 import _lib
    from spinifel_gb300.nufft import NufftPlan

    det = (2, 20, 37)
    model, ppr, pdr, quats = _slice_case(41, det, 24, 30 + w)
    ppr_t = t(ppr.reshape(3, -1), dev)
    P = NufftPlan(41, eps)
    assert P.width == w
    P.set_modes(t(model, dev))
    mult = np.pi / pdr.max()
    a = P.slice(t(quats, dev), ppr_t, mult)
    exact = _oracle_slices(model, ppr, pdr, quats)
    assert rel(a.cpu().numpy().astype(np.float64), exact) < _width_tol(eps)
    try:
        for shape in range(8):
            _lib.call("spf_tune_set", _lib.SPF_TUNE_SLICE_SHAPE, shape)
            b = P.slice(t(quats, dev), ppr_t, mult, det_shape=det)
            assert torch.equal(a, b), shape
    finally:
        _lib.call("spf_tune_set", _lib.SPF_TUNE_SLICE_SHAPE, 0)
