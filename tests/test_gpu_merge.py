"""The merge operator and device CG against the FP64 oracle restatement and
the reference's own Merge.solve_ac (golden, run on the FP64 NUFFT oracle).
Tolerances: FP32 operator rel-L2 <= 1e-5; on the fast FP32 path (type-1
NUFFTs at eps 1e-6, FP32 Toeplitz product) the CG solution is within 1e-3 of
the reference's after the same number of iterations (the eps-1e-6 kernel and
right-hand side, amplified by the ill-conditioned system); at the reference's
own precision (FP64 NUFFTs at eps 1e-12, FP64 product) within 1e-5 (it
agrees to about 1e-13) and the FP64 operator within 1e-12."""
import os

import numpy as np
import pytest
import torch

from oracle import merge as omerge
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
                  solve_ac_maxiter=cases.MERGE["maxiter"], N_orientations=len(orient),
                  N_batch_size=len(orient))
    nufft = NUFFT(st, ppr, pdr, ref_orientations=orient)
    H, K, L = geom.hkl(orient, ppr)
    mult = np.pi / pdr.max()
    return dict(data=data, ppr=ppr, pdr=pdr, orient=orient, ac_est=ac_est, M=M, st=st,
                nufft=nufft, H=H * mult, K=K * mult, L=L * mult)


def _operator(setup, S, flambda=None):
    from spinifel_gb300.merge import MergeOperator, antisupport

    M = setup["M"]
    dev = torch.device("cuda", 0)
    mo = omerge.MergeOracle(M, 2 * M, setup["data"].size)
    if flambda is not None:
        mo.flambda = flambda
    op = MergeOperator(M, 2 * M, mo.rlambda, mo.flambda,
                       torch.as_tensor(S, dtype=torch.float32, device=dev), antisupport(M, 1))
    ones = np.ones(setup["H"].size)
    from oracle import nufft as onufft

    ugrid_conv = onufft.adjoint(ones, setup["H"], setup["K"], setup["L"], 2 * M, True, None)
    op.set_kernel(torch.as_tensor(ugrid_conv, dtype=torch.float32, device=dev))
    return op, mo, mo.kernel(setup["H"], setup["K"], setup["L"])


def test_toeplitz_operator_matches_oracle(setup):
    M = setup["M"]
    S = omerge.support_from_estimate(setup["ac_est"])
    S[0, 1, 2] = 0.0
    op, mo, F_conv = _operator(setup, S)
    rng = np.random.default_rng(50)
    x = rng.standard_normal(M ** 3)
    got = op.apply(torch.as_tensor(x, device="cuda")).cpu().numpy()
    ref = mo.conv(x, F_conv, S) + mo.rlambda * x + mo.flambda * mo.reg(x, S)
    assert rel(got, ref) < 1e-5
    # the data (convolution) term alone, which flambda = 1e3 dwarfs in the sum
    op0, mo0, F0 = _operator(setup, S, flambda=0.0)
    got0 = op0.apply(torch.as_tensor(x, device="cuda")).cpu().numpy() - mo0.rlambda * x
    assert rel(got0, mo0.conv(x, F0, S)) < 1e-5


def test_direct_form_equals_toeplitz_for_centrosymmetric_x(setup):
    from spinifel_gb300.nufft import NufftPlan

    M = setup["M"]
    S = np.ones((M,) * 3)
    op, mo, _ = _operator(setup, S)
    dev = torch.device("cuda", 0)
    plan = NufftPlan(M, 1e-6)
    op.set_direct(plan, torch.as_tensor(setup["orient"], device=dev),
                  torch.as_tensor(setup["ppr"].reshape(3, -1), device=dev),
                  float(np.pi / setup["pdr"].max()))
    rng = np.random.default_rng(51)
    x = rng.standard_normal((M,) * 3)
    x = 0.5 * (x + x[::-1, ::-1, ::-1])  # centrosymmetric
    xt = torch.as_tensor(x.reshape(-1).copy(), device=dev)
    a = op.apply(xt, form=0).cpu().numpy()
    b = op.apply(xt, form=1).cpu().numpy()
    assert rel(b, a) < 1e-5


def test_solve_ac_matches_reference_golden(setup):
    from spinifel_gb300.sequential.autocorrelation import Merge

    g = np.load(os.path.join(GOLD, "golden_merge.npz"))
    merge = Merge(setup["st"], setup["data"], setup["ppr"], setup["pdr"], setup["nufft"])
    ac = merge.solve_ac(0, setup["orient"], setup["ac_est"].copy())
    assert merge.iterations == int(g["iterations"])
    assert rel(ac, g["ac"]) < 1e-3
    # residuals decrease overall
    r = merge.residuals
    assert r[-1] < r[0]


def test_solve_ac_direct_form_close_to_toeplitz(setup):
    from spinifel_gb300.sequential.autocorrelation import Merge

    a = Merge(setup["st"], setup["data"], setup["ppr"], setup["pdr"], setup["nufft"])
    b = Merge(setup["st"], setup["data"], setup["ppr"], setup["pdr"], setup["nufft"],
              form="direct")
    xa = a.solve_ac(0, setup["orient"], setup["ac_est"].copy())
    xb = b.solve_ac(0, setup["orient"], setup["ac_est"].copy())
    assert a.iterations == b.iterations
    assert rel(xb, xa) < 1e-3


def test_cg_stops_on_rtol(setup):
    """The device CG stops by scipy's rule (||r|| < rtol ||b||) before
    maxiter, and then the true residual is below that threshold."""
    M = setup["M"]
    S = np.ones((M,) * 3)
    op, mo, _ = _operator(setup, S)
    rng = np.random.default_rng(52)
    xs = rng.standard_normal((M,) * 3)
    xs = 0.5 * (xs + xs[::-1, ::-1, ::-1])
    dev = torch.device("cuda", 0)
    b = op.apply(torch.as_tensor(xs.reshape(-1).copy(), device=dev))
    x, iters, hist = op.cg(b, torch.zeros_like(b), maxiter=400, rtol=0.05)
    n = int(iters.item())
    assert 0 < n < 400
    h = hist.cpu().numpy()
    assert h[n] < 0.05 * float(b.norm()) <= h[n - 1]
    r = b - op.apply(x)
    assert float(r.norm() / b.norm()) < 0.06


def test_cg_solve_captured_in_a_cuda_graph(setup):
    """The whole CG solve (operator FFTs included) is one graph; replaying it
    gives the eagerly computed solution bit for bit."""
    M = setup["M"]
    S = omerge.support_from_estimate(setup["ac_est"])
    op, mo, _ = _operator(setup, S)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(53)
    xs = rng.standard_normal((M,) * 3)
    xs = 0.5 * (xs + xs[::-1, ::-1, ::-1])
    b = op.apply(torch.as_tensor(xs.reshape(-1).copy(), device=dev))
    x = torch.zeros_like(b)
    hist = torch.zeros(12, dtype=torch.float64, device=dev)
    iters = torch.zeros(1, dtype=torch.int32, device=dev)
    op.cg_into(b, x, hist, iters, 12, 1e-9, x0_is_zero=True)
    torch.cuda.synchronize()
    eager = x.clone()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        x.zero_()
        with torch.cuda.graph(g, stream=s):
            op.cg_into(b, x, hist, iters, 12, 1e-9, x0_is_zero=True)
    torch.cuda.current_stream().wait_stream(s)
    x.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert int(iters.item()) == 12
    assert torch.equal(x, eager)


def _reg_only(M, S, v, prime_dft):
    """flambda * S.reg(S.v) of the Toeplitz operator (zero convolution kernel,
    rlambda 0), with the regulariser's DFT chosen by SPF_TUNE_PRIME_DFT."""
    from spinifel_gb300 import _lib
    from spinifel_gb300.merge import MergeOperator, antisupport

    dev = torch.device("cuda", 0)
    _lib.call("spf_tune_set", _lib.SPF_TUNE_PRIME_DFT, prime_dft)
    try:
        op = MergeOperator(M, 2 * M, 0.0, 1.0, torch.as_tensor(S, dtype=torch.float32, device=dev),
                           antisupport(M, 1))
    finally:
        _lib.call("spf_tune_set", _lib.SPF_TUNE_PRIME_DFT, 0)
    op.set_kernel(torch.zeros((2 * M,) * 3, dtype=torch.float32, device=dev))
    out = op.apply(torch.as_tensor(v.reshape(-1), device=dev)).cpu().numpy()
    op.close()
    return out


@pytest.mark.parametrize("M", [31, 41])
def test_prime_grid_regulariser_matches_fp64_oracle(lib, M):
    """A prime model grid (M - 1 smooth) runs the regulariser as Rader DFTs:
    S.Re(ifftn(fftn(S.x) . ifftshift(F_anti))) equals the oracle's numpy FP64
    result to 1e-12, and the cuFFT path to 1e-12."""
    rng = np.random.default_rng(M)
    S = (rng.random((M,) * 3) > 0.2).astype(np.float64)
    v = rng.standard_normal((M,) * 3)
    mo = omerge.MergeOracle(M, 2 * M, 1000, oversampling=1)
    want = mo.reg(v.reshape(-1), S)
    rader = _reg_only(M, S, v, 1)
    cufft = _reg_only(M, S, v, 2)
    assert rel(rader, want) < 1e-12
    assert rel(cufft, want) < 1e-12
    assert rel(rader, cufft) < 1e-12


def test_prime_grid_regulariser_151(lib):
    """At the 151^3 merge grid the Rader path equals cuFFT's Bluestein path."""
    M = 151
    rng = np.random.default_rng(151)
    S = np.ones((M,) * 3)
    v = rng.standard_normal((M,) * 3)
    assert rel(_reg_only(M, S, v, 1), _reg_only(M, S, v, 2)) < 1e-12


def test_fp64_toeplitz_operator_matches_oracle(setup):
    """spf_merge_set_kernel_f64: the Toeplitz product in FP64 (D2Z / Z2D)
    equals the oracle's numpy FP64 operator to 1e-12."""
    from spinifel_gb300.merge import MergeOperator, antisupport
    from oracle import nufft as onufft

    M = setup["M"]
    S = omerge.support_from_estimate(setup["ac_est"])
    dev = torch.device("cuda", 0)
    mo = omerge.MergeOracle(M, 2 * M, setup["data"].size)
    op = MergeOperator(M, 2 * M, mo.rlambda, mo.flambda,
                       torch.as_tensor(S, dtype=torch.float32, device=dev), antisupport(M, 1))
    ugrid_conv = onufft.adjoint(np.ones(setup["H"].size), setup["H"], setup["K"], setup["L"],
                                2 * M, True, None)
    op.set_kernel(torch.as_tensor(ugrid_conv, dtype=torch.float64, device=dev))
    assert op.fp64
    F_conv = mo.kernel(setup["H"], setup["K"], setup["L"])
    x = np.random.default_rng(54).standard_normal(M ** 3)
    got = op.apply(torch.as_tensor(x, device=dev)).cpu().numpy()
    want = mo.conv(x, F_conv, S) + mo.rlambda * x + mo.flambda * mo.reg(x, S)
    assert rel(got, want) < 1e-12
    op0 = MergeOperator(M, 2 * M, mo.rlambda, 0.0,
                        torch.as_tensor(S, dtype=torch.float32, device=dev), antisupport(M, 1))
    op0.set_kernel(torch.as_tensor(ugrid_conv, dtype=torch.float64, device=dev))
    got0 = op0.apply(torch.as_tensor(x, device=dev)).cpu().numpy() - mo.rlambda * x
    assert rel(got0, mo.conv(x, F_conv, S)) < 1e-12


def test_solve_ac_fp64_matches_reference_golden(lib):
    """Merge.solve_ac at the reference's precision (use_single_prec off: FP64
    type-1 NUFFTs at eps 1e-12, FP64 Toeplitz product, FP64 CG) against the
    reference's own solve_ac: same iteration count, solution within 1e-5
    relative L2 (it agrees to about 1e-10)."""
    from spinifel_gb300 import Settings
    from spinifel_gb300.extern.nufft_ext import NUFFT
    from spinifel_gb300.sequential.autocorrelation import Merge

    data, ppr, pdr, orient, ac_est = cases.merge_inputs()
    M = cases.MERGE["M"]
    st = Settings(det_shape=cases.MERGE["det_shape"], N_clipping=0, N_binning=0, M_override=M,
                  solve_ac_maxiter=cases.MERGE["maxiter"], N_orientations=len(orient),
                  N_batch_size=len(orient), use_single_prec=False)
    nufft = NUFFT(st, ppr, pdr, ref_orientations=orient)
    assert nufft.fp64
    g = np.load(os.path.join(GOLD, "golden_merge.npz"))
    merge = Merge(st, data, ppr, pdr, nufft)
    ac = merge.solve_ac(0, orient, ac_est.copy())
    assert merge.iterations == int(g["iterations"])
    err = rel(ac, g["ac"])
    print(f"FP64 merge vs the reference's solve_ac: rel-L2 {err:.2e}")
    assert err < 1e-5


def test_direct_form_cg_captured_in_a_cuda_graph(setup):
    """The direct-form CG (type 2 -> type 1 over the bin-sorted points every
    iteration) recorded as one CUDA graph: its replay gives the eager
    solution.  The spreading adds in the order its atomics land, and this
    system's CG (flambda = 1e3 against rlambda = 1/N/1000) amplifies that
    rounding over the iterations: two eager solves differ by about 1e-5
    relative after 10 iterations, so replay and eager are held to 1e-3 and
    the first operator application to 1e-6."""
    from spinifel_gb300.nufft import NufftPlan

    M = setup["M"]
    S = np.ones((M,) * 3)
    op, mo, _ = _operator(setup, S)
    dev = torch.device("cuda", 0)
    op.set_direct(NufftPlan(M, 1e-6), torch.as_tensor(setup["orient"], device=dev),
                  torch.as_tensor(setup["ppr"].reshape(3, -1), device=dev),
                  float(np.pi / setup["pdr"].max()))
    rng = np.random.default_rng(55)
    xs = rng.standard_normal((M,) * 3)
    xs = 0.5 * (xs + xs[::-1, ::-1, ::-1])
    b = op.apply(torch.as_tensor(xs.reshape(-1).copy(), device=dev), form=1)
    x = torch.zeros_like(b)
    hist = torch.zeros(10, dtype=torch.float64, device=dev)
    iters = torch.zeros(1, dtype=torch.int32, device=dev)
    op.cg_into(b, x, hist, iters, 10, 1e-12, form=1, x0_is_zero=True)
    torch.cuda.synchronize()
    eager, eager_hist = x.clone(), hist.clone()
    x.zero_()
    op.cg_into(b, x, hist, iters, 10, 1e-12, form=1, x0_is_zero=True)
    torch.cuda.synchronize()
    print(f"two eager direct-form solves differ by {float((x - eager).norm() / eager.norm()):.2e}")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        x.zero_()
        with torch.cuda.graph(g, stream=s):
            op.cg_into(b, x, hist, iters, 10, 1e-12, form=1, x0_is_zero=True)
    torch.cuda.current_stream().wait_stream(s)
    for _ in range(2):
        x.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert int(iters.item()) == 10
        assert float((x - eager).norm() / eager.norm()) < 1e-3
        # ||b|| and ||r_1|| = ||b - alpha W b||: one application of W
        np.testing.assert_allclose(hist[:2].cpu().numpy(), eager_hist[:2].cpu().numpy(),
                                   rtol=1e-6)
