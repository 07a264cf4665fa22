"""Rotations, orientation sampling and detector geometry.

* quaternion2rot3d: batched [w, x, y, z] -> 3x3 rotation, the formula of
  eval/geom.py:9-48 (skopi's quaternion2rot3d in batch form).  Spinifel slices
  with the inverse rotation (spinifel/extern/nufft_ext.py:59-60).
* uniform_quaternions: seeded uniform sampling of SO(3) (Shoemake 1992,
  "Uniform random rotations", Graphics Gems III), standing in for skopi's
  get_uniform_quat / get_random_quat, which are not available here.
* hkl: the einsum("ijk,klmn->jilmn", R^-1, ppr) of
  spinifel/autocorrelation.py:302 and nufft_ext.py:136-142.
* flat_detector: a flat multi-panel detector on the Ewald sphere,
  q = (p_hat - z_hat) / lambda.
"""
from __future__ import annotations

import numpy as np


def quaternion2rot3d(quat: np.ndarray) -> np.ndarray:
    quat = np.asarray(quat, dtype=np.float64)
    single = quat.ndim == 1
    q = quat.reshape(-1, 4)
    q0, q1, q2, q3 = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((q.shape[0], 3, 3))
    R[:, 0, 0] = 1.0 - 2.0 * (q2 * q2 + q3 * q3)
    R[:, 0, 1] = 2.0 * (q1 * q2 - q0 * q3)
    R[:, 0, 2] = 2.0 * (q1 * q3 + q0 * q2)
    R[:, 1, 0] = 2.0 * (q1 * q2 + q0 * q3)
    R[:, 1, 1] = 1.0 - 2.0 * (q1 * q1 + q3 * q3)
    R[:, 1, 2] = 2.0 * (q2 * q3 - q0 * q1)
    R[:, 2, 0] = 2.0 * (q1 * q3 - q0 * q2)
    R[:, 2, 1] = 2.0 * (q2 * q3 + q0 * q1)
    R[:, 2, 2] = 1.0 - 2.0 * (q1 * q1 + q2 * q2)
    return R[0] if single else R


def inverse_rotmats(quats: np.ndarray) -> np.ndarray:
    """R^-1 for each quaternion (R is orthogonal, so R^-1 = R^T)."""
    R = quaternion2rot3d(quats)
    return np.swapaxes(R, -1, -2)


def uniform_quaternions(n: int, rng: np.random.Generator) -> np.ndarray:
    """n uniform random unit quaternions [w, x, y, z] with w >= 0."""
    u1, u2, u3 = rng.random((3, n))
    a = np.sqrt(1.0 - u1)
    b = np.sqrt(u1)
    q = np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                  b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)], axis=1)
    q[q[:, 0] < 0] *= -1.0
    return q


def hkl(quats: np.ndarray, pixel_position_reciprocal: np.ndarray):
    """H, K, L with shape (n_orient,) + detector shape."""
    Rinv = inverse_rotmats(np.asarray(quats).reshape(-1, 4))
    H, K, L = np.einsum("ijk,klmn->jilmn", Rinv, pixel_position_reciprocal)
    return H, K, L


def flat_detector(n_panels: int = 4, nx: int = 32, ny: int = 32, distance: float = 0.2,
                  pixel: float = 300e-6, wavelength: float = 2.5e-10, gap_px: float = 1.0):
    """Pixel positions in reciprocal space (3, n_panels, nx, ny) [1/m] and
    their lengths (n_panels, nx, ny), for panels tiled 2 x 2 around the beam
    (n_panels = 4) or stacked in a row otherwise."""
    ix = (np.arange(nx) + 0.5) * pixel
    iy = (np.arange(ny) + 0.5) * pixel
    g = gap_px * pixel
    pos = np.empty((3, n_panels, nx, ny))
    for p in range(n_panels):
        if n_panels == 4:
            sx = 1.0 if p in (0, 3) else -1.0
            sy = 1.0 if p in (0, 1) else -1.0
            X = sx * (g + ix)[:, None] * np.ones((1, ny))
            Y = sy * (g + iy)[None, :] * np.ones((nx, 1))
        else:
            X = (ix - nx * pixel / 2)[:, None] + (p - n_panels / 2) * nx * pixel * 1.05
            X = X * np.ones((1, ny))
            Y = (iy - ny * pixel / 2)[None, :] * np.ones((nx, 1))
        pos[0, p], pos[1, p], pos[2, p] = X, Y, distance
    norm = np.sqrt((pos ** 2).sum(axis=0))
    unit = pos / norm
    q = unit.copy()
    q[2] -= 1.0
    q /= wavelength
    dist = np.sqrt((q ** 2).sum(axis=0))
    return q, dist
