"""FP64 NUFFT and FP64 matching at the reference's own precision (eps 1e-12 in
double, spinifel/extern/nufft_ext.py:62; float64 distances when
use_single_prec is off, spinifel/sequential/orientation_matching.py:32-36).

Tolerances: the FP64 kernels against the exact direct sums and against the
FP64 oracle at eps 1e-12: relative L2 <= 1e-10; distances: relative 1e-12;
argmin: identical, a different pick counted as equal only when its oracle
distance is within 1e-6 relative of the oracle's minimum."""
import os

import numpy as np
import pytest
import torch

from oracle import matching as om
from oracle import nufft as onufft
from tests.golden import cases

pytestmark = pytest.mark.gpu
TOL64 = 1e-10
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.fixture(scope="module")
def dev(lib):
    return torch.device("cuda", 0)


def t(a, dev, dtype=torch.float64):
    return torch.as_tensor(np.asarray(a), dtype=dtype, device=dev)


@pytest.mark.parametrize("m", [(9, 9, 9), (10, 11, 12), (21, 21, 21)])
@pytest.mark.parametrize("isign", [-1, 1])
def test_fp64_type2_matches_direct_sum(dev, m, isign):
    from spinifel_gb300.nufft import NufftPlan64

    rng = np.random.default_rng(60)
    f = rng.standard_normal(m)
    x, y, z = rng.uniform(-3 * np.pi + 1e-3, 3 * np.pi - 1e-3, (3, 2000))
    P = NufftPlan64(m, 1e-12)
    assert P.width == 13
    P.set_modes(t(f, dev), isign=isign, want_imag=True)
    re, im = P.interp(t(x, dev), t(y, dev), t(z, dev), want_imag=True)
    got = re.cpu().numpy() + 1j * im.cpu().numpy()
    assert rel(got, onufft.nudft3d2(x, y, z, f, isign)) < TOL64


@pytest.mark.parametrize("m", [(9, 9, 9), (10, 11, 12)])
@pytest.mark.parametrize("isign", [-1, 1])
def test_fp64_type1_matches_direct_sum(dev, m, isign):
    from spinifel_gb300.nufft import NufftPlan64

    rng = np.random.default_rng(61)
    x, y, z = rng.uniform(-np.pi, np.pi, (3, 1500))
    c = rng.standard_normal(1500)
    P = NufftPlan64(m, 1e-12)
    P.spread_zero()
    P.spread(t(x, dev), t(y, dev), t(z, dev), t(c, dev))
    re, im = P.finish(isign, want_imag=True)
    got = re.cpu().numpy() + 1j * im.cpu().numpy()
    assert rel(got, onufft.nudft3d1(x, y, z, c, m, isign)) < TOL64


@pytest.mark.parametrize("eps,tol", [(1e-9, 1e-8), (1e-14, 1e-12)])
def test_fp64_tolerance_scales(dev, eps, tol):
    from spinifel_gb300.nufft import NufftPlan64

    rng = np.random.default_rng(62)
    f = rng.standard_normal((12, 12, 12))
    x, y, z = rng.uniform(-np.pi, np.pi, (3, 1000))
    P = NufftPlan64(12, eps)
    P.set_modes(t(f, dev), isign=-1, want_imag=True)
    re, im = P.interp(t(x, dev), t(y, dev), t(z, dev), want_imag=True)
    got = re.cpu().numpy() + 1j * im.cpu().numpy()
    assert rel(got, onufft.nudft3d2(x, y, z, f, -1)) < tol


def _slice_case(M, det, n_orient, seed):
    from spinifel_gb300 import geom, synth

    rng = np.random.default_rng(seed)
    model = synth.intensity_model(M, seed=seed)
    ppr, pdr = geom.flat_detector(*det)
    return model, ppr, pdr, geom.uniform_quaternions(n_orient, rng)


def test_fp64_slicing_matches_oracle_and_direct_sum(dev):
    """41^3 model, 4 x 32 x 32 detector: the FP64 slices against the oracle's
    eps-1e-12 slices (all of them) and the exact direct sum (a subset)."""
    from spinifel_gb300 import geom
    from spinifel_gb300.nufft import make_plan

    model, ppr, pdr, quats = _slice_case(41, (4, 32, 32), 40, 63)
    mult = np.pi / pdr.max()
    P = make_plan(41, 1e-12)
    assert P.dtype == torch.float64
    P.set_modes(t(model, dev))
    got = P.slice(t(quats, dev), t(ppr.reshape(3, -1), dev), mult).cpu().numpy()
    H, K, L = (v.reshape(len(quats), -1) * mult for v in geom.hkl(quats, ppr))
    want = onufft.nufft3d2(H.ravel(), K.ravel(), L.ravel(), model, -1, 1e-12).real
    assert rel(got.ravel(), want) < TOL64
    sub = slice(0, 3)
    exact = onufft.nudft3d2(H[sub].ravel(), K[sub].ravel(), L[sub].ravel(), model, -1).real
    assert rel(got[sub].ravel(), exact) < TOL64


def test_fp64_operator_glue_matches_reference_golden(dev):
    """autocorrelation.forward / adjoint at eps 1e-12 against the reference's
    own glue run on the FP64 oracle at eps 1e-12."""
    from spinifel_gb300 import autocorrelation as ac

    ugrid, sup, H_, K_, L_, nuv = cases.ops_inputs()
    g = np.load(os.path.join(GOLD, "golden_ops.npz"))
    fwd = ac.forward(ugrid.copy(), H_, K_, L_, sup, True, H_.size, eps=1e-12)
    adj = ac.adjoint(nuv, H_, K_, L_, cases.OPS["M"], True, sup, eps=1e-12)
    assert fwd.dtype == np.complex128 and adj.dtype == np.float64
    assert rel(fwd, g["forward"]) < TOL64
    assert rel(adj, g["adjoint"]) < TOL64


@pytest.mark.parametrize("n_img,n_ref,n_pix", [(37, 300, 1024), (5, 129, 33), (1, 1, 1)])
def test_fp64_distances_and_running_argmin(dev, n_img, n_ref, n_pix):
    """spf_dist_f64 over all pixels (ragged tails included) against numpy,
    and the batched running argmin (planted exact ties: the lower index
    wins, also across batches) against numpy's argmin."""
    from spinifel_gb300 import matching

    rng = np.random.default_rng(64 + n_pix)
    ref = rng.random((n_ref, n_pix))
    img = rng.random((n_img, n_pix))
    if n_ref > 200:
        ref[200] = ref[3]          # tie across batches of 128
        ref[10] = ref[7]           # tie within one batch
        img[0] = ref[3] + 1e-3
        img[1] = ref[7] - 1e-3
    d = matching.dist_f64(t(ref, dev), t(img, dev)).cpu().numpy()
    want = ((img[:, None, :] - ref[None, :, :]) ** 2).sum(axis=2)
    np.testing.assert_allclose(d, want, rtol=1e-12, atol=0)
    idx, dist = matching.argmin_fp64(t(img, dev), t(ref, dev), batch=128)
    np.testing.assert_array_equal(idx.cpu().numpy(), want.argmin(axis=1))
    np.testing.assert_allclose(dist.cpu().numpy(), want.min(axis=1), rtol=1e-12)


def test_fp64_empty_inputs(dev):
    from spinifel_gb300 import matching

    idx, dist = matching.argmin_fp64(torch.empty(0, 8, dtype=torch.float64, device=dev),
                                     torch.rand(4, 8, dtype=torch.float64, device=dev))
    assert idx.numel() == 0 and dist.numel() == 0
    idx, _ = matching.argmin_fp64(torch.rand(3, 8, dtype=torch.float64, device=dev),
                                  torch.empty(0, 8, dtype=torch.float64, device=dev))
    assert (idx.cpu() == -1).all()


def _snm_settings(**kw):
    from spinifel_gb300 import Settings

    s = cases.SNM
    return Settings(N_orientations=s["n_orient"], N_batch_size=s["batch"],
                    det_shape=s["det_shape"], N_clipping=0, N_binning=0, **kw)


def test_snm_fp64_identical_to_reference_golden(dev):
    """SNM.slicing_and_match with use_single_prec off (FP64 slicing at eps
    1e-12, FP64 distances) against the reference's own SNM run in float64:
    every frame's index identical or tied within 1e-6 relative."""
    from spinifel_gb300.extern.nufft_ext import NUFFT
    from spinifel_gb300.sequential.orientation_matching import SNM

    ac, ppr, pdr, quats, slices_ = cases.snm_inputs()
    g = np.load(os.path.join(GOLD, "golden_snm.npz"))
    st = _snm_settings(use_single_prec=False)
    nufft = NUFFT(st, ppr, pdr, ref_orientations=quats)
    assert nufft.fp64 and nufft.eps == 1e-12
    snm = SNM(st, slices_, ppr, pdr, nufft)
    q = snm.slicing_and_match(ac)
    idx = np.array([np.flatnonzero((quats == v).all(axis=1))[0] for v in q])
    ok = om.ties_equal(idx, g["index"], g["dist"], rtol=1e-6)
    assert ok.all(), f"{(~ok).sum()} of {ok.size} frames differ beyond 1e-6 ties"


def test_function_path_fp64_identical_to_reference_golden(dev):
    from spinifel_gb300.sequential.orientation_matching import slicing_and_match

    ac, ppr, pdr, quats, slices_ = cases.snm_inputs()
    gold = np.load(os.path.join(GOLD, "golden_sam.npz"))["index"]
    q = slicing_and_match(ac, slices_, ppr, pdr, ref_orientations=quats,
                          settings=_snm_settings(use_single_prec=False))
    idx = np.array([np.flatnonzero((quats == v).all(axis=1))[0] for v in q])
    np.testing.assert_array_equal(idx, gold)
