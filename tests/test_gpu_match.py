"""Parity of the plain matching kernels with the oracle and with golden
outputs of the reference's own code.  Argmin rule: indices identical, or the
two references' oracle distances equal within 1e-6 relative (a tie)."""
import os

import numpy as np
import pytest
import torch

from oracle import matching as om
from oracle import nufft as onufft
from tests.golden import cases

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def dev(lib):
    return torch.device("cuda", 0)


def test_knn_module_sp_dp_match_test_OM_golden(dev):
    """tests/test_OM.py:51-76 with a fixed seed: 512 model slices x 1024 images
    x 16,384 pixels; SP and DP argmins equal the sklearn argmin."""
    from spinifel_gb300.sequential import pyCudaKNearestNeighbors_DP as dp
    from spinifel_gb300.sequential import pyCudaKNearestNeighbors_SP as sp

    model_slices, slices = cases.nn_inputs()
    gold = np.load(os.path.join(GOLD, "golden_nn.npz"))["index"]
    _, dist = om.sklearn_argmin(model_slices, slices)
    for mod in (sp, dp):
        eu = mod.cudaEuclideanDistance(model_slices.flatten(), slices.flatten(),
                                       model_slices.shape[0], slices.shape[0], slices.shape[1], 0)
        idx = mod.cudaHeapSort(eu, slices.shape[0], model_slices.shape[0], slices.shape[1], 1, 0)
        assert np.all(om.ties_equal(idx, gold, dist)), mod.__name__


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("shape", [(130, 257, 37), (5, 3, 16), (128, 128, 100), (1, 1, 15)])
def test_knn_eudist_values(dev, dtype, shape):
    from spinifel_gb300 import matching

    n_ref, n_data, n_pix = shape
    rng = np.random.default_rng(30)
    ref = rng.random((n_ref, n_pix)).astype(dtype)
    data = rng.random((n_data, n_pix)).astype(dtype)
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    got = matching.knn_eudist(torch.as_tensor(ref, device=dev, dtype=tdt),
                              torch.as_tensor(data, device=dev, dtype=tdt)).cpu().numpy()
    exact = onufft.knn_eudist(ref, data)
    tol = 1e-5 if dtype == np.float32 else 1e-12
    np.testing.assert_allclose(got, exact, rtol=tol, atol=tol)


@pytest.mark.parametrize("k", [1, 3, 8, 32])
def test_knn_topk_with_ties(dev, k):
    from spinifel_gb300 import matching

    rng = np.random.default_rng(31)
    dist = rng.integers(0, 20, (77, 300)).astype(np.float32)  # many exact ties
    got = matching.knn_topk(torch.as_tensor(dist, device=dev), k).cpu().numpy()
    np.testing.assert_array_equal(got, om.knn_topk(dist, k))


@pytest.mark.parametrize("shape", [(300, 1000, 256), (129, 77, 1001), (1, 1, 3), (64, 5000, 64)])
def test_argmin_fp32_matches_oracle(dev, shape):
    from spinifel_gb300 import matching

    n_img, n_ref, n_pix = shape
    rng = np.random.default_rng(32)
    imgs = rng.random((n_img, n_pix)).astype(np.float32)
    refs = rng.random((n_ref, n_pix)).astype(np.float32)
    idx, dmin = matching.argmin_fp32(torch.as_tensor(imgs, device=dev),
                                     torch.as_tensor(refs, device=dev))
    oidx, d = om.sklearn_argmin(refs, imgs)
    assert np.all(om.ties_equal(idx.cpu().numpy(), oidx, d))
    np.testing.assert_allclose(dmin.cpu().numpy(), d[oidx, np.arange(n_img)], rtol=1e-4,
                               atol=1e-3)


def test_argmin_fp32_duplicate_references_take_lower_index(dev):
    from spinifel_gb300 import matching

    rng = np.random.default_rng(33)
    refs = rng.random((300, 64)).astype(np.float32)
    refs[250] = refs[17]  # exact duplicate: equal distances for every image
    imgs = refs[[17, 17, 3]] + 0.001 * rng.random((3, 64)).astype(np.float32)
    idx, _ = matching.argmin_fp32(torch.as_tensor(imgs, device=dev),
                                  torch.as_tensor(refs, device=dev))
    assert idx.cpu().tolist() == [17, 17, 3]


def test_argmin_fp32_batches_offsets(dev):
    from spinifel_gb300 import matching

    rng = np.random.default_rng(34)
    imgs = torch.as_tensor(rng.random((50, 96)), dtype=torch.float32, device=dev)
    refs = torch.as_tensor(rng.random((1000, 96)), dtype=torch.float32, device=dev)
    whole, _ = matching.argmin_fp32(imgs, refs)
    tr = matching.BestTracker(50, dev)
    isq, rsq = matching.row_sqnorm(imgs), matching.row_sqnorm(refs)
    for st in range(0, 1000, 300):
        tr.update_fp32(imgs, isq, refs[st:st + 300].contiguous(), rsq[st:st + 300].contiguous(),
                       st)
    batched, _ = tr.result()
    assert torch.equal(whole, batched)


def test_nearest_neighbor_matches_reference_golden(dev):
    from spinifel_gb300.sequential.nearest_neighbor import nearest_neighbor

    model_slices, slices = cases.nn_inputs()
    gold = np.load(os.path.join(GOLD, "golden_nn.npz"))["index"]
    _, dist = om.sklearn_argmin(model_slices, slices)
    idx = nearest_neighbor(model_slices.astype(np.float32), slices.astype(np.float32), 128)
    assert np.all(om.ties_equal(idx, gold, dist))


def _snm_settings():
    from spinifel_gb300 import Settings

    s = cases.SNM
    return Settings(N_orientations=s["n_orient"], N_batch_size=s["batch"],
                    det_shape=s["det_shape"], N_clipping=0, N_binning=0)


def test_snm_matches_reference_golden(dev):
    """SNM.slicing_and_match on the fast FP32 path (eps 1e-6 slices, FP32
    distances) against the reference's float64 SNM run: the slice error
    (about 1e-6 relative) may reorder near-ties, so 98% of frames must tie at
    1e-5 and all at 1e-3.  At the reference's own precision the indices are
    identical (tests/test_gpu_fp64.py)."""
    from spinifel_gb300.extern.nufft_ext import NUFFT
    from spinifel_gb300.sequential.orientation_matching import SNM

    ac, ppr, pdr, quats, slices_ = cases.snm_inputs()
    g = np.load(os.path.join(GOLD, "golden_snm.npz"))
    st = _snm_settings()
    nufft = NUFFT(st, ppr, pdr, ref_orientations=quats)
    snm = SNM(st, slices_, ppr, pdr, nufft)
    q = snm.slicing_and_match(ac)
    idx = np.array([np.flatnonzero((quats == v).all(axis=1))[0] for v in q])
    ok = om.ties_equal(idx, g["index"], g["dist"], rtol=1e-5)
    assert ok.mean() >= 0.98 and np.all(om.ties_equal(idx, g["index"], g["dist"], rtol=1e-3))


def test_function_path_matches_reference_golden(dev):
    """The function path on the fast FP32 path; identical at the reference's
    own precision in tests/test_gpu_fp64.py."""
    from spinifel_gb300.sequential.orientation_matching import slicing_and_match

    ac, ppr, pdr, quats, slices_ = cases.snm_inputs()
    gold = np.load(os.path.join(GOLD, "golden_sam.npz"))["index"]
    q = slicing_and_match(ac, slices_, ppr, pdr, ref_orientations=quats, settings=_snm_settings())
    idx = np.array([np.flatnonzero((quats == v).all(axis=1))[0] for v in q])
    assert (idx == gold).mean() >= 0.98


def test_empty_inputs(dev):
    from spinifel_gb300 import matching

    e = torch.empty(0, 16, device=dev)
    r = torch.rand(10, 16, device=dev)
    idx, d = matching.argmin_fp32(e, r)
    assert idx.numel() == 0
    assert matching.knn_eudist(r, e).shape == (0, 10)


@pytest.mark.parametrize("dtype,shape", [(torch.bfloat16, (50, 64)), (torch.float32, (50, 7)),
                                         (torch.float32, (9, 1)), (torch.int16, (30, 3))])
def test_gather_rows_matches_indexing(dev, dtype, shape):
    from spinifel_gb300 import matching

    g = torch.Generator(device="cpu").manual_seed(3)
    src = (torch.rand(shape, generator=g) * 100).to(dtype).to(dev)
    rows = torch.tensor([3, 0, 49 % shape[0], 3, shape[0] - 1], dtype=torch.int64, device=dev)
    out = matching.gather_rows(src, rows)
    assert torch.equal(out, src[rows])


@pytest.mark.parametrize("n_pix,ld", [(4096, 4096), (1003, 1008)])
def test_frame_ingest_exact(lib, n_pix, ld):
    """uint16 counts -> FP32, bf16 (zero-padded to ld), squared norm and
    4-norm: FP32 and bf16 exactly as converted by torch, the squared norm
    the exactly rounded integer sum, on the vector (16-byte) and the scalar
    path, counts up to 65535."""
    from spinifel_gb300 import matching

    rng = np.random.default_rng(33)
    c = rng.integers(0, 65536, (37, n_pix)).astype(np.uint16)
    c[0, :] = 65535
    dev = torch.device("cuda", 0)
    t = torch.as_tensor(c.view(np.int16), device=dev)
    f32 = torch.empty(37, n_pix, device=dev)
    bf = torch.empty(37, ld, dtype=torch.bfloat16, device=dev)
    sq = torch.empty(37, device=dev)
    n4 = torch.empty(37, device=dev)
    matching.ingest_u16(t, f32, bf, sq, n4)
    torch.cuda.synchronize()
    ref = c.astype(np.float32)
    np.testing.assert_array_equal(f32.cpu().numpy(), ref)
    rb = torch.zeros(37, ld, dtype=torch.bfloat16)
    rb[:, :n_pix] = torch.as_tensor(ref).to(torch.bfloat16)
    assert torch.equal(bf.cpu(), rb)
    exact = (c.astype(np.int64) ** 2).sum(axis=1)
    np.testing.assert_array_equal(sq.cpu().numpy(), exact.astype(np.float32))
    s4 = ((c.astype(np.float64) ** 2) ** 2).sum(axis=1)
    np.testing.assert_allclose(n4.cpu().numpy(), np.sqrt(s4).astype(np.float32), rtol=1e-6)
