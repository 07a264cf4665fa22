"""Seeded synthetic inputs with the shapes and value distributions of the
Spinifel workloads (the reference's own data, e.g. 3iyf_sim_10k.h5, is not
available):

* model: |FFT(density)|^2 on an M^3 grid (modes centred at M//2), the density
  being 20 Gaussian blobs (sigma ~ U(1, 3) voxels, amplitude ~ U(0.5, 1),
  centres uniform in the inner half of the box), normalised to max 1;
* detector: 4 flat panels at 0.2 m, 300 um pixels, lambda 2.5 A;
* orientations: uniform random quaternions;
* images: Poisson counts of slices scaled to a mean photon count per pixel.
"""
from __future__ import annotations

import numpy as np

from . import geom

DEFAULT_SEED = 20261203


def density_blobs(M: int, rng: np.random.Generator, n_blobs: int = 20) -> np.ndarray:
    ax = np.arange(M) - M // 2
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    rho = np.zeros((M, M, M))
    for _ in range(n_blobs):
        c = rng.uniform(-M / 4, M / 4, 3)
        s = rng.uniform(1.0, 3.0)
        a = rng.uniform(0.5, 1.0)
        rho += a * np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / (2 * s * s))
    return rho


def intensity_model(M: int, seed: int = DEFAULT_SEED, dtype=np.float64) -> np.ndarray:
    rng = np.random.default_rng(seed)
    rho = density_blobs(M, rng)
    F = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(rho)))
    I = np.abs(F) ** 2
    I /= I.max()
    return I.astype(dtype)


def detector(n_panels: int = 4, nx: int = 32, ny: int = 32):
    return geom.flat_detector(n_panels, nx, ny)


def poisson_images(slices: np.ndarray, mean_photons: float, rng: np.random.Generator):
    """uint16 Poisson counts with the given mean photons per pixel."""
    s = np.maximum(np.asarray(slices, dtype=np.float64), 0.0)
    lam = s * (mean_photons / max(s.mean(), 1e-300))
    return np.minimum(rng.poisson(lam), 65535).astype(np.uint16)
