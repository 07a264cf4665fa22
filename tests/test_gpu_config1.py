"""The CPU-runnable configuration end to end: a 41^3 float64 model, 4 x 32 x 32
detector, 2,000 reference orientations sliced by type 2 at eps 1e-12 in the
FP64 oracle, 500 Poisson frames (mean 2 photons/pixel) at other orientations.

* SNM at the reference's precision (use_single_prec off: FP64 type 2 at eps
  1e-12, FP64 distances) must give the oracle's argmin on every frame
  (identical, or a tie within 1e-6 relative of the oracle distances).
* The fast FP32 path (type 2 at eps 1e-6, plain FP32 and bf16 + re-rank)
  must give the oracle's argmin on its own FP32 slices, and on this case also
  the eps-1e-12 argmin on every frame (ties within 1e-6); in general it may
  differ where the slice error moves two distances across each other."""
import numpy as np
import pytest
import torch

from oracle import matching as om
from oracle import nufft as onufft

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(lib):
    from spinifel_gb300 import geom, synth

    rng = np.random.default_rng(20261203)
    M = 41
    model = synth.intensity_model(M, seed=20261203)
    ppr, pdr = geom.flat_detector(4, 32, 32)
    ref_q = geom.uniform_quaternions(2000, rng)
    img_q = geom.uniform_quaternions(500, rng)
    mult = np.pi / pdr.max()

    def slices(q):
        H, K, L = geom.hkl(q, ppr)
        return onufft.nufft3d2(H.reshape(-1) * mult, K.reshape(-1) * mult, L.reshape(-1) * mult,
                               model, -1, 1e-12).real.reshape(len(q), -1)

    imgs = synth.poisson_images(slices(img_q), 2.0, rng).astype(np.float64)
    ref = slices(ref_q)
    return dict(model=model, ppr=ppr, pdr=pdr, ref_q=ref_q, imgs=imgs, ref=ref)


def test_config1_snm_fp64_identical_to_the_oracle(case):
    from spinifel_gb300 import Settings
    from spinifel_gb300.extern.nufft_ext import NUFFT
    from spinifel_gb300.sequential.orientation_matching import SNM

    st = Settings(N_orientations=2000, N_batch_size=500, det_shape=(4, 32, 32), N_clipping=0,
                  N_binning=0, M_override=41, use_single_prec=False)
    nufft = NUFFT(st, case["ppr"], case["pdr"], ref_orientations=case["ref_q"])
    snm = SNM(st, case["imgs"].reshape(500, 4, 32, 32), case["ppr"], case["pdr"], nufft)
    gidx = snm.match_indices(case["model"]).cpu().numpy()
    oidx, dist = om.snm_argmin([case["ref"][i:i + 500] for i in range(0, 2000, 500)],
                               case["imgs"])
    ok = om.ties_equal(gidx, oidx, dist, rtol=1e-6)
    assert ok.all(), f"{(~ok).sum()} of 500 frames differ beyond 1e-6 ties"

    # the FP64 slices themselves against the oracle's eps-1e-12 slices
    P = nufft.set_model(case["model"], 1)
    raw = nufft.slice_real(P, 0, 500).cpu().numpy()
    rel = np.linalg.norm(raw - case["ref"][:500]) / np.linalg.norm(case["ref"][:500])
    assert rel < 1e-10, rel


def test_config1_snm_plain_and_bf16_match_the_oracle(case):
    from spinifel_gb300 import Settings, matching
    from spinifel_gb300.extern.nufft_ext import NUFFT
    from spinifel_gb300.sequential.orientation_matching import SNM

    st = Settings(N_orientations=2000, N_batch_size=500, det_shape=(4, 32, 32), N_clipping=0,
                  N_binning=0, M_override=41)
    nufft = NUFFT(st, case["ppr"], case["pdr"], ref_orientations=case["ref_q"])
    snm = SNM(st, case["imgs"].reshape(500, 4, 32, 32), case["ppr"], case["pdr"], nufft)
    gidx = snm.match_indices(case["model"]).cpu().numpy()

    # the same slices the matcher used (type 2 at eps 1e-6 on the GPU), unscaled
    dev = torch.device("cuda", 0)
    P = nufft.set_model(case["model"], 1)
    raw = torch.empty(2000, 4096, device=dev)
    for b in range(4):
        nufft.slice_real(P, b * 500, (b + 1) * 500, out=raw[b * 500:(b + 1) * 500])
    torch.cuda.synchronize()
    g_slices = raw.double().cpu().numpy()
    rel = np.linalg.norm(g_slices - case["ref"], axis=1) / np.linalg.norm(case["ref"], axis=1)
    assert rel.max() < 5e-6, rel.max()

    # 1) matching on the GPU's own slices: the oracle's SNM argmin in FP64, ties
    #    within the FP32 rounding of a 4,096-term distance
    oidx_g, dist_g = om.snm_argmin([g_slices[i:i + 500] for i in range(0, 2000, 500)],
                                   case["imgs"])
    ok = om.ties_equal(gidx, oidx_g, dist_g, rtol=1e-5)
    assert ok.all(), f"{(~ok).sum()} frames differ beyond FP32 ties"

    # 2) against the exact slices (eps 1e-12): a different pick is allowed only
    #    where the slice error moves the two distances across each other
    oidx, dist = om.snm_argmin([case["ref"][i:i + 500] for i in range(0, 2000, 500)],
                               case["imgs"])
    cols = np.arange(500)
    delta = np.abs(dist - dist_g)
    slack = delta[gidx, cols] + delta[oidx, cols] + 1e-5 * dist[oidx, cols]
    assert (dist[gidx, cols] - dist[oidx, cols] <= slack).all()
    same = om.ties_equal(gidx, oidx, dist, rtol=1e-6)
    print(f"FP32 eps-1e-6 path: {same.mean():.3f} of frames equal the eps-1e-12 argmin (ties 1e-6)")
    assert same.all()

    # 3) bf16 tensor cores + re-rank on the same scaled slices: the plain
    #    FP32 argmin exactly
    refs = raw.clone()
    for b in range(4):
        blk = refs[b * 500:(b + 1) * 500]
        blk *= snm.slices_std / blk.double().std(unbiased=False).float()
    fr = matching.FrameSet(snm.slices_)
    rs = matching.ReferenceSet(refs.contiguous())
    bidx, _ = matching.match_bf16(fr, rs)
    pidx, _ = matching.argmin_fp32(snm.slices_, rs.f32, images_sq=snm.slices_2, refs_sq=rs.sq)
    assert torch.equal(bidx, pidx)
    assert om.ties_equal(bidx.cpu().numpy(), oidx_g, dist_g, rtol=1e-5).all()
