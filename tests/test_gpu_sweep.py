"""The regularisation sweep (spf_merge_cg_sweep): every system of the batched
solve equals the single-system device CG with the same lambdas, and the
MergeMPI mirror reproduces the reference's MPI merge run with 4 ranks
(golden: same chosen rank in generation 0 and 1, per-rank solution norms
within 1e-4, chosen solution within 1e-3 rel-L2, the tolerance of the
sequential merge: FP32 operator on the device, FP64 in the reference)."""
import os

import numpy as np
import pytest
import torch

from oracle import merge as omerge
from oracle import nufft as onufft
from tests.golden import cases

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def setup(lib):
    from spinifel_gb300 import Settings, geom
    from spinifel_gb300.extern.nufft_ext import NUFFT

    data, ppr, pdr, orient, ac_est = cases.merge_inputs()
    M = cases.MERGE["M"]
    st = Settings(det_shape=cases.MERGE["det_shape"], N_clipping=0, N_binning=0, M_override=M,
                  solve_ac_maxiter=100, N_orientations=len(orient), N_batch_size=len(orient))
    nufft = NUFFT(st, ppr, pdr, ref_orientations=orient)
    return dict(data=data, ppr=ppr, pdr=pdr, orient=orient, ac_est=ac_est, M=M, st=st,
                nufft=nufft)


def test_batched_systems_equal_single_solves(setup):
    from spinifel_gb300 import geom
    from spinifel_gb300.merge import MergeOperator, antisupport

    dev = torch.device("cuda", 0)
    M = setup["M"]
    H, K, L = geom.hkl(setup["orient"], setup["ppr"])
    mult = np.pi / setup["pdr"].max()
    H, K, L = (a.reshape(-1) * mult for a in (H, K, L))
    S = omerge.support_from_estimate(setup["ac_est"])
    ugrid_conv = onufft.adjoint(np.ones(H.size), H, K, L, 2 * M, True, None)
    adb = onufft.adjoint(setup["data"].reshape(-1), H, K, L, M, True, S).reshape(-1)
    x0 = torch.as_tensor((setup["ac_est"] * S).reshape(-1), device=dev)
    rls = np.array([1e-6, 1e-4, 1e-2])
    fls = np.array([10.0, 1e3, 1e4])
    St = torch.as_tensor(S, dtype=torch.float32, device=dev)
    op = MergeOperator(M, 2 * M, 0.0, 0.0, St, antisupport(M, 1))
    op.set_kernel(torch.as_tensor(ugrid_conv, dtype=torch.float32, device=dev))
    adb_t = torch.as_tensor(adb, device=dev)
    x, norms, iters, hist = op.cg_sweep(rls, fls, adb_t, x0, 40, history=True)
    for l in range(3):
        single = MergeOperator(M, 2 * M, rls[l], fls[l], St, antisupport(M, 1))
        single.set_kernel(torch.as_tensor(ugrid_conv, dtype=torch.float32, device=dev))
        d = adb_t + rls[l] * x0
        xs, it, h = single.cg(d, x0, 40)
        assert int(iters[l]) == int(it.item())
        assert rel(x[l].cpu().numpy(), xs.cpu().numpy()) < 1e-6
        np.testing.assert_allclose(hist[l, :int(it.item())].cpu().numpy(),
                                   h[:int(it.item())].cpu().numpy(), rtol=1e-6)
        # the reported norms
        xn = float(xs.norm())
        rn = float((single.apply(xs) - d).norm())
        assert abs(norms[l, 0].item() - xn) <= 1e-9 * xn
        assert abs(norms[l, 1].item() - rn) <= 1e-3 * rn + 1e-12 * float(d.norm())
        single.close()
    op.close()


@pytest.mark.parametrize("gen", [0, 1])
def test_merge_mpi_mirror_matches_reference_golden(setup, gen):
    from spinifel_gb300.mpi.autocorrelation import MergeMPI

    g = np.load(os.path.join(GOLD, "golden_sweep.npz"))
    m = MergeMPI(setup["st"], setup["data"], setup["ppr"], setup["pdr"], setup["nufft"],
                 size=cases.SWEEP["size"])
    est = None if gen == 0 else setup["ac_est"].copy()
    ac = m.solve_ac(gen, setup["orient"], est)
    summ = g[f"summary_gen{gen}"]
    assert m.ref_rank == int(g[f"ref_rank_gen{gen}"])
    got = np.array(m.summary)
    np.testing.assert_allclose(got[:, 1], summ[:, 1], rtol=1e-12)  # lambdas
    np.testing.assert_allclose(got[:, 2], summ[:, 2], rtol=1e-4)   # ||x||
    assert rel(ac, g[f"ac_gen{gen}"]) < 1e-3


@pytest.mark.parametrize("M,n_sys", [(31, 3), (151, 2)])
def test_prime_grid_sweep_equals_single_solves(lib, M, n_sys):
    """On a prime grid the sweep's regulariser is the Rader DFT: batched over
    all systems while their buffers fit in L2 together (M = 31), system by
    system otherwise (M = 151).  Either way every system's iterates equal
    the single-system CG's."""
    from spinifel_gb300.merge import MergeOperator, antisupport

    dev = torch.device("cuda", 0)
    g = torch.arange(2 * M, device=dev, dtype=torch.float32) - M
    kern = torch.exp(-(g[:, None, None] ** 2 + g[None, :, None] ** 2 + g[None, None, :] ** 2)
                     / (0.05 * M * M)).contiguous()
    St = torch.ones((M,) * 3, dtype=torch.float32, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(M)
    adb = torch.randn(M ** 3, dtype=torch.float64, device=dev, generator=gen)
    x0 = torch.zeros_like(adb)
    rls = np.array([1e-3, 1e-2, 1e-1])[:n_sys]
    fls = np.array([10.0, 1e3, 1e2])[:n_sys]
    iters_n = 6
    op = MergeOperator(M, 2 * M, 0.0, 0.0, St, antisupport(M, 1))
    op.set_kernel(kern)
    x, norms, iters, _ = op.cg_sweep(rls, fls, adb, x0, iters_n, rtol=1e-30)
    for l in range(n_sys):
        single = MergeOperator(M, 2 * M, rls[l], fls[l], St, antisupport(M, 1))
        single.set_kernel(kern)
        xs, it, _ = single.cg(adb + rls[l] * x0, x0, iters_n, rtol=1e-30)
        assert int(iters[l]) == int(it.item()) == iters_n
        assert rel(x[l].cpu().numpy(), xs.cpu().numpy()) < 1e-7
        single.close()
    op.close()
