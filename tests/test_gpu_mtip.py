"""The whole M-TIP loop on the GPU (sequential/main.py's structure: merge
with random orientations, phase, then per generation match -> merge ->
phase) on a small synthetic problem with a known answer: 2,000 Poisson
images (mean 50 photons/pixel) of the intensity of a 12-blob density at
random orientations, M = 21, a 4 x 16 x 16 detector, 4,000 reference
orientations.  The reference's integration test judges convergence by the
FSC of the aligned density; here, after 6 generations, the phased
autocorrelation must correlate > 0.85 with the true one, and the density,
aligned to the truth (both hands), > 0.8."""
import numpy as np
import pytest

from oracle import nufft as onufft

pytestmark = pytest.mark.gpu


def test_mtip_reconstructs_synthetic_density(lib):
    from spinifel_gb300 import Settings, geom, synth
    from spinifel_gb300.eval.align import align_volumes
    from spinifel_gb300.eval.fsc import compute_fsc
    from spinifel_gb300.sequential.main import main

    Mquat, n_img = 5, 2000
    M = 4 * Mquat + 1
    rng = np.random.default_rng(5)
    rho_true = synth.density_blobs(M, rng, n_blobs=12)
    F = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(rho_true)))
    ac_true = np.fft.fftshift(np.fft.ifftn(np.fft.ifftshift(np.abs(F) ** 2)).real)
    det = (4, 16, 16)
    ppr, pdr = geom.flat_detector(*det)
    q = geom.uniform_quaternions(n_img, rng)
    H, K, L = geom.hkl(q, ppr)
    mult = np.pi / pdr.max()
    sl = onufft.nufft3d2(H.reshape(-1) * mult, K.reshape(-1) * mult, L.reshape(-1) * mult,
                         ac_true, -1, 1e-9).real.reshape(n_img, *det)
    imgs = synth.poisson_images(sl, 50.0, rng).astype(np.float32)
    st = Settings(Mquat_override=Mquat, det_shape=det, N_clipping=0, N_binning=0,
                  N_orientations=4000, N_batch_size=1000, N_images_per_rank=n_img,
                  solve_ac_maxiter=100)
    ac_phased, support_, rho_, ori, timings = main(st, ppr, pdr, imgs, n_generations=6, seed=1)
    assert ac_phased.shape == (M, M, M) and np.isfinite(ac_phased).all()
    assert ori.shape == (n_img, 4) and len(timings) == 6
    assert np.corrcoef(ac_phased.ravel(), ac_true.ravel())[0, 1] > 0.85
    r_vol, m2, cc = align_volumes(np.fft.fftshift(rho_), rho_true, n_iterations=6, n_search=300)
    assert cc > 0.8
    res, _, fsc = compute_fsc(m2, r_vol, 1e10 / 9.0)
    assert fsc[1] > 0.9  # the lowest-resolution shell
