"""Seeded inputs of the golden cases, shared by make_golden.py (which runs the
reference on them) and the tests (which run spinifel_gb300 on them).  Only
numpy is used, so the inputs are identical on every machine."""
from __future__ import annotations

import numpy as np

QUAT_SEED = 7001

NN = dict(seed=7002, n_ref=512, n_img=1024, n_pix=16384)  # tests/test_OM.py:51-56 shape
SNM = dict(seed=7003, M=21, det_shape=(4, 16, 16), n_orient=300, batch=100, n_images=64,
           photons=2.0)
OPS = dict(seed=7004, M=15, npts=2000)
MERGE = dict(seed=7005, M=15, det_shape=(4, 8, 8), n_images=40, maxiter=20, photons=2.0)
PREP = dict(seed=7009, frames4=(3, 4, 32, 48), frames1=(2, 1, 40, 56), n_clip=1, n_bin=2)
EVAL = dict(seed=7008, M=21, dmax=0.25e10, spacing=0.01, n_search=60, n_iterations=4)
SWEEP = dict(size=4)  # MPI ranks of the regularisation sweep, on MERGE's inputs
PHASE = dict(seed=7006, Mquat=5, nER=4, nHIO=3, N_phase_loops=2, beta=0.9)


def nn_inputs():
    rng = np.random.default_rng(NN["seed"])
    model_slices = rng.random((NN["n_ref"], NN["n_pix"]))
    slices = rng.random((NN["n_img"], NN["n_pix"]))
    return model_slices, slices


def _geometry(det_shape):
    from spinifel_gb300 import geom

    return geom.flat_detector(det_shape[0], det_shape[1], det_shape[2])


def _images(model, quats, ppr, pdr, photons, rng):
    from oracle import nufft as onufft
    from spinifel_gb300 import geom

    mult = np.pi / pdr.max()
    H, K, L = geom.hkl(quats, ppr)
    s = onufft.nufft3d2(H.reshape(-1) * mult, K.reshape(-1) * mult, L.reshape(-1) * mult,
                        model, -1, 1e-12).real
    s = np.maximum(s, 0).reshape((len(quats),) + ppr.shape[1:])
    lam = s * (photons / s.mean())
    return rng.poisson(lam).astype(np.float64)


def snm_inputs():
    from spinifel_gb300 import geom, synth

    rng = np.random.default_rng(SNM["seed"])
    ac = synth.intensity_model(SNM["M"], seed=SNM["seed"])
    ppr, pdr = _geometry(SNM["det_shape"])
    quats = geom.uniform_quaternions(SNM["n_orient"], rng)
    img_q = geom.uniform_quaternions(SNM["n_images"], rng)
    slices_ = _images(ac, img_q, ppr, pdr, SNM["photons"], rng)
    return ac, ppr, pdr, quats, slices_


def ops_inputs():
    rng = np.random.default_rng(OPS["seed"])
    M = OPS["M"]
    ugrid = rng.standard_normal((M, M, M))
    sup = (rng.random((M, M, M)) > 0.3).astype(np.float64)
    H_, K_, L_ = rng.uniform(-np.pi, np.pi, (3, OPS["npts"]))
    nuv = rng.standard_normal(OPS["npts"])
    return ugrid, sup, H_, K_, L_, nuv


def merge_inputs():
    from spinifel_gb300 import geom, synth

    rng = np.random.default_rng(MERGE["seed"])
    model = synth.intensity_model(MERGE["M"], seed=MERGE["seed"])
    ppr, pdr = _geometry(MERGE["det_shape"])
    orient = geom.uniform_quaternions(MERGE["n_images"], rng)
    data = _images(model, orient, ppr, pdr, MERGE["photons"], rng)
    ac_est = model.copy()
    return data, ppr, pdr, orient, ac_est


def phase_inputs():
    """A centred autocorrelation of a compact density of 6 Gaussian blobs on
    the M^3 grid (M = 4 Mquat + 1) and a uniform random starting density."""
    c = PHASE
    M = 4 * c["Mquat"] + 1
    rng = np.random.default_rng(c["seed"])
    ax = np.arange(M) - M // 2
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    rho = np.zeros((M, M, M))
    for _ in range(6):
        cen = rng.uniform(-M / 8, M / 8, 3)
        sig = rng.uniform(0.8, 1.6)
        rho += rng.uniform(0.5, 1.0) * np.exp(
            -((X - cen[0]) ** 2 + (Y - cen[1]) ** 2 + (Z - cen[2]) ** 2) / (2 * sig ** 2))
    F = np.fft.fftn(np.fft.ifftshift(rho))
    ac = np.fft.fftshift(np.fft.ifftn(np.abs(F) ** 2).real)
    rho0 = rng.random((M, M, M))
    return ac, rho0


def eval_inputs():
    """Two M^3 densities of the same 8 Gaussian blobs, the second with the
    blob centres rotated by a fixed quaternion and 2% noise, and the samplers
    the alignment search draws from: uniform_quat(n) / random_quat(n) share a
    seeded Shoemake stream (they stand in for skopi's samplers), randn is a
    seeded numpy RandomState."""
    from spinifel_gb300 import geom

    c = EVAL
    M = c["M"]
    rng = np.random.default_rng(c["seed"])
    ax = np.arange(M) - M // 2
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    cen = rng.uniform(-M / 6, M / 6, (8, 3))
    sig = rng.uniform(1.0, 2.0, 8)
    amp = rng.uniform(0.5, 1.0, 8)
    q = np.array([0.9, 0.2, -0.3, 0.25])
    q /= np.linalg.norm(q)
    R = geom.quaternion2rot3d(q)

    def density(cs):
        d = np.zeros((M, M, M))
        for k in range(8):
            d += amp[k] * np.exp(-((X - cs[k, 0]) ** 2 + (Y - cs[k, 1]) ** 2 +
                                   (Z - cs[k, 2]) ** 2) / (2 * sig[k] ** 2))
        return d

    v1 = density(cen)
    v2 = density(cen @ R.T) + 0.02 * rng.standard_normal((M, M, M))
    qrng = np.random.default_rng(c["seed"] + 1)
    sampler = lambda n: geom.uniform_quaternions(n, qrng)  # noqa: E731
    randn = np.random.RandomState(c["seed"] + 2).randn
    return v1, v2, sampler, sampler, randn


def prep_inputs():
    """Photon counts of a four-panel and a one-panel detector (as float64,
    the dtype the reference bins), a four-panel pixel index map and pixel
    positions for the SAXS profile."""
    c = PREP
    rng = np.random.default_rng(c["seed"])
    f4 = rng.poisson(3.0, c["frames4"]).astype(np.float64)
    f1 = rng.poisson(3.0, c["frames1"]).astype(np.float64)
    _, p, a, b = c["frames4"]
    ii, jj = np.meshgrid(np.arange(a), np.arange(b), indexing="ij")
    index_map = np.stack([np.broadcast_to(ii, (p, a, b)), np.broadcast_to(jj, (p, a, b))]) + 3
    ppr = rng.standard_normal((3,) + c["frames4"][1:])
    return f4, f1, index_map.astype(np.int64), ppr
