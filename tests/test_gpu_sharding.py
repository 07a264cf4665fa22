"""The sharded product paths with the library's kernels, two shards emulated
in one process (every GPU run here uses one GPU): the collectives are
replaced by the in-process sum / gather of the other shard's result, so what
runs is the kernels on each shard plus the host logic of
spinifel_gb300.sharding.  Tolerances: matching identical to the
unsharded bf16 path (index and exact FP32 distance); merge set-up and direct
operator within 1e-6 relative L2 of the unsharded FP32 computation (the
shards' partial sums are added in another order); the sharded CG solution
within 1e-5 of the unsharded device CG."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float((a - b).norm() / b.norm())


@pytest.fixture(scope="module")
def dev(lib):
    return torch.device("cuda", 0)


def test_reference_sharded_matching_equals_whole_set(dev):
    from spinifel_gb300 import matching
    from spinifel_gb300.sharding import local_best, match_sharded

    rng = np.random.default_rng(80)
    n_ref, n_pix = 1500, 1024
    refs = torch.as_tensor(rng.gamma(0.5, 1.0, (n_ref, n_pix)).astype(np.float32), device=dev)
    refs[1200] = refs[17]  # duplicate across the shards: index 17 must win
    pick = rng.integers(0, n_ref, 200)
    x = torch.as_tensor(rng.poisson(refs[pick].cpu().numpy()).astype(np.float32), device=dev)
    x[0] = refs[17]
    fr = matching.FrameSet(x)
    whole_idx, whole_d = matching.match_bf16(fr, matching.ReferenceSet(refs.contiguous()))
    k = 700
    sh0 = matching.ReferenceSet(refs[:k].contiguous())
    sh1 = matching.ReferenceSet(refs[k:].contiguous())
    for path in ("bf16", "fp32"):
        d1, i1 = local_best(fr, sh1, path)
        gather = lambda d, i: (torch.stack([d, d1]), torch.stack([i, i1 + k]))  # noqa: E731
        bd, bi = match_sharded(fr, sh0, 0, path=path, gather=gather)
        assert torch.equal(bi.to(torch.int32), whole_idx)
        assert torch.equal(bd, whole_d)
        assert int(bi[0]) == 17
    # a rank without references reports +inf and never wins
    de, ie = local_best(fr, None)
    gather = lambda d, i: (torch.stack([d, de]), torch.stack([i, ie]))  # noqa: E731
    bd, bi = match_sharded(fr, matching.ReferenceSet(refs.contiguous()), 0, gather=gather)
    assert torch.equal(bi.to(torch.int32), whole_idx)


def _points(M, n_frames, seed):
    from spinifel_gb300 import geom

    rng = np.random.default_rng(seed)
    ppr, pdr = geom.flat_detector(4, 16, 16)
    q = geom.uniform_quaternions(n_frames, rng)
    return q, ppr, pdr, rng


def test_sharded_merge_setup_and_direct_operator(dev):
    from spinifel_gb300 import Settings, geom
    from spinifel_gb300.extern.nufft_ext import NUFFT
    from spinifel_gb300.merge import MergeOperator, antisupport
    from spinifel_gb300.nufft import NufftPlan
    from spinifel_gb300.sharding import ShardedDirectOperator, merge_setup_sharded, sharded_cg

    M, n_frames = 21, 40
    q, ppr, pdr, rng = _points(M, n_frames, 81)
    st = Settings(det_shape=(4, 16, 16), N_clipping=0, N_binning=0, M_override=M,
                  N_orientations=n_frames, N_batch_size=n_frames)
    nufft = NUFFT(st, ppr, pdr, ref_orientations=q)
    mult = np.pi / pdr.max()
    H, K, L = (torch.as_tensor(v.reshape(-1) * mult, dtype=torch.float32, device=dev)
               for v in geom.hkl(q, ppr))
    data = torch.as_tensor(rng.poisson(2.0, H.numel()).astype(np.float32), device=dev)
    sup = torch.ones((M,) * 3, dtype=torch.float32, device=dev)
    half = (n_frames // 2) * ppr[0].size
    # set-up: each shard's adjoints, summed
    uc1, adb1 = merge_setup_sharded(H[half:], K[half:], L[half:], data[half:], sup, M, 2 * M,
                                    nufft, reduce=lambda t: None)
    uc1, adb1 = uc1.clone(), adb1.clone()
    other = iter([uc1, adb1])
    uc, adb = merge_setup_sharded(H[:half], K[:half], L[:half], data[:half], sup, M, 2 * M,
                                  nufft, reduce=lambda t: t.add_(next(other)))
    uc_all = nufft.adjoint(torch.ones_like(data), H, K, L, 1, True, 2 * M)
    adb_all = nufft.adjoint(data, H, K, L, sup, True, M).reshape(-1)
    assert rel(uc, uc_all) < 1e-6 and rel(adb, adb_all) < 1e-6
    # direct operator with the points sharded
    N = data.numel()
    rl, fl = 1.0 / N / 1000.0, 1e3
    qt = torch.as_tensor(q, dtype=torch.float32, device=dev)
    ppr_t = torch.as_tensor(ppr.reshape(3, -1), dtype=torch.float32, device=dev)

    def data_op(sl):
        op = MergeOperator(M, 2 * M, 0.0, 0.0, sup, antisupport(M, 1))
        op.set_kernel(torch.zeros((2 * M,) * 3, dtype=torch.float32, device=dev))
        op.set_direct(NufftPlan(M, 1e-6), qt[sl], ppr_t, mult)
        return op

    op0, op1 = data_op(slice(0, n_frames // 2)), data_op(slice(n_frames // 2, n_frames))
    op_reg = MergeOperator(M, 2 * M, rl, fl, sup, antisupport(M, 1))
    op_reg.set_kernel(torch.zeros((2 * M,) * 3, dtype=torch.float32, device=dev))
    full = MergeOperator(M, 2 * M, rl, fl, sup, antisupport(M, 1))
    full.set_kernel(uc_all.float())
    full.set_direct(NufftPlan(M, 1e-6), qt, ppr_t, mult)
    cur = {}
    sharded = ShardedDirectOperator(op0, op_reg,
                                    reduce=lambda y: y.add_(op1.apply(cur["x"], form=1)))

    def apply(x):
        cur["x"] = x
        return sharded.apply(x)

    v = torch.randn((M,) * 3, dtype=torch.float64, device=dev)
    v = (0.5 * (v + torch.flip(v, dims=(0, 1, 2)))).reshape(-1)
    assert rel(apply(v), full.apply(v, form=1)) < 1e-6
    b = adb_all.double()
    xs, hist = sharded_cg(apply, b, torch.zeros_like(b), 12, rtol=1e-30)
    xf, _, hf = full.cg(b, torch.zeros_like(b), 12, rtol=1e-30, form=1)
    assert rel(xs, xf) < 1e-5
    np.testing.assert_allclose(hist[:3], hf[:3].cpu().numpy(), rtol=1e-5)
