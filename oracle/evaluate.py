"""Oracle (test infrastructure only): numpy/scipy restatement of the
reference's reconstruction-quality tools, eval/fsc.py (Fourier shell
correlation) and eval/align.py + eval/geom.py (volume alignment by a
coarse-to-fine rotation search scored with the Pearson correlation).
The random samplers the reference takes from skopi and numpy's global
generator are arguments here: uniform_quat(n), random_quat(n), randn(n)."""
from __future__ import annotations

import numpy as np
import scipy.interpolate
from scipy import ndimage


# ---- eval/fsc.py --------------------------------------------------------
def reciprocal_mesh(M, dmax):
    """fsc.py:10-33: (M, M, M, 3) mesh of linspace(-dmax, dmax, M)."""
    ls = np.linspace(-dmax, dmax, M)
    return np.moveaxis(np.asarray(np.meshgrid(ls, ls, ls, indexing="ij")), 0, -1)


def fsc_shells(vol1, vol2, dmax, spacing=0.01):
    """The shell sums of compute_fsc (fsc.py:67-125): rshell, numerator,
    |F1|^2 and |F2|^2 sums per shell, and the FSC curve."""
    mesh = reciprocal_mesh(vol1.shape[0], dmax)
    smags = np.linalg.norm(mesh, axis=-1).reshape(-1) * 1e-10
    r_spacings = np.arange(0, smags.max() / np.sqrt(3), spacing)
    ft1 = np.fft.fftshift(np.fft.fftn(vol1)).reshape(-1)
    ft2 = np.conjugate(np.fft.fftshift(np.fft.fftn(vol2)).reshape(-1))
    rshell = np.zeros(len(r_spacings))
    fsc = np.zeros(len(r_spacings))
    sums = np.zeros((len(r_spacings), 3))
    for i, r in enumerate(r_spacings):
        idx = np.where((smags > r) & (smags < r + spacing))[0]
        num = np.sum(ft1[idx] * ft2[idx])
        a, b = np.sum(np.abs(ft1[idx]) ** 2), np.sum(np.abs(ft2[idx]) ** 2)
        sums[i] = (num.real, a, b)
        rshell[i] = r + 0.5 * spacing
        fsc[i] = num.real / np.sqrt(a * b)
    return rshell, fsc, sums


def resolution_from_fsc(rshell, fsc):
    """The 0.5 crossing of compute_fsc (fsc.py:117-125), -1 when it does not exist."""
    f = scipy.interpolate.interp1d(fsc, rshell)
    try:
        return float(1.0 / f(0.5))
    except ValueError:
        return -1.0


def compute_fsc(vol1, vol2, dmax, spacing=0.01):
    rshell, fsc, _ = fsc_shells(vol1, vol2, dmax, spacing)
    return resolution_from_fsc(rshell, fsc), rshell, fsc


# ---- eval/geom.py -------------------------------------------------------
def quaternion2rot3d(quat):
    """geom.py:8-45, batched."""
    q = np.asarray(quat, dtype=np.float64)
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.zeros((q.shape[0], 3, 3))
    R[:, 0, 0] = 1. - 2. * (y * y + z * z)
    R[:, 0, 1] = 2. * (x * y - w * z)
    R[:, 0, 2] = 2. * (x * z + w * y)
    R[:, 1, 0] = 2. * (x * y + w * z)
    R[:, 1, 1] = 1. - 2. * (x * x + z * z)
    R[:, 1, 2] = 2. * (y * z - w * x)
    R[:, 2, 0] = 2. * (x * z - w * y)
    R[:, 2, 1] = 2. * (y * z + w * x)
    R[:, 2, 2] = 1. - 2. * (x * x + y * y)
    return R


def axis_angle_to_quaternion(axis, theta):
    """geom.py:47-69."""
    axis = axis / np.linalg.norm(axis, axis=1)[:, None]
    half = theta / 2
    q = np.zeros((len(theta), 4))
    q[:, 0] = np.cos(half)
    q[:, 1:] = np.sin(half)[:, None] * axis
    return q


def quaternion_product(q1, q0):
    """geom.py:71-97: rotation by q0 followed by q1."""
    p0, p1, p2, p3 = q1[:, 0], q1[:, 1], q1[:, 2], q1[:, 3]
    r0, r1, r2, r3 = q0[:, 0], q0[:, 1], q0[:, 2], q0[:, 3]
    return np.array([r0 * p0 - r1 * p1 - r2 * p2 - r3 * p3,
                     r0 * p1 + r1 * p0 - r2 * p3 + r3 * p2,
                     r0 * p2 + r1 * p3 + r2 * p0 - r3 * p1,
                     r0 * p3 - r1 * p2 + r2 * p1 + r3 * p0]).T


def preferred_orientation_quat(num_pts, sigma, base_quat, random_quat, randn):
    """geom.py:99-135 with the samplers passed in."""
    if base_quat is None:
        base_quat = np.array(random_quat(1))
    base = np.tile(base_quat, num_pts).reshape(num_pts, 4)
    R_random = quaternion2rot3d(np.array(random_quat(num_pts)))
    rot_axis = np.matmul(np.array([0, 0, 1.0]), R_random)
    theta = sigma * randn(num_pts)
    pref = axis_angle_to_quaternion(theta[:, None] * rot_axis, theta)
    return quaternion_product(pref, base)


# ---- eval/align.py ------------------------------------------------------
def rotate_volume(vol, quat):
    """align.py:36-67."""
    M = vol.shape[0]
    lin = np.arange(M)
    coords = np.meshgrid(lin, lin, lin)
    h = int(M / 2)
    xyz = np.vstack([coords[0].reshape(-1) - h, coords[1].reshape(-1) - h,
                     coords[2].reshape(-1) - h])
    T = np.dot(quaternion2rot3d(quat), xyz) + h
    new_xyz = np.array([T[:, 1, :].flatten(), T[:, 0, :].flatten(), T[:, 2, :].flatten()])
    out = ndimage.map_coordinates(vol, new_xyz, order=1)
    return out.reshape((quat.shape[0], M, M, M))


def center_volume(vol):
    """align.py:69-86."""
    old = np.array(ndimage.center_of_mass(vol))
    new = np.array(np.array(vol.shape) / 2).astype(int)
    return ndimage.shift(vol, -1 * (old - new))


def pearson_cc(a, b):
    """align.py:88-110."""
    vx = a - a.mean(axis=-1)[:, None]
    vy = b - b.mean(axis=-1)[:, None]
    return np.sum(vx * vy, axis=1) / (np.sqrt(np.sum(vx ** 2, axis=1)) *
                                      np.sqrt(np.sum(vy ** 2, axis=1)))


def score_deformations(mrc1, mrc2, quats):
    """align.py:112-146 (rotations only)."""
    w = rotate_volume(mrc1, quats)
    return pearson_cc(w.reshape(w.shape[0], -1), np.expand_dims(mrc2.flatten(), axis=0))


def scan_orientations_fine(mrc1, mrc2, opt_q, prev, random_quat, randn, n_iterations=10,
                           n_search=420, score=score_deformations):
    """align.py:148-189."""
    sigmas = 2 - 0.2 * np.arange(1, 10)
    for n in range(1, n_iterations):
        quat = preferred_orientation_quat(n_search - 1, float(sigmas[n - 1]), opt_q,
                                          random_quat, randn)
        quat = np.vstack((opt_q, quat))
        ccs = score(mrc1, mrc2, quat)
        if np.max(ccs) < prev:
            break
        opt_q = quat[np.argmax(ccs)]
        prev = np.max(ccs)
    return opt_q, prev


def scan_orientations(mrc1, mrc2, uniform_quat, random_quat, randn, n_iterations=10,
                      n_search=420, nscs=1, score=score_deformations):
    """align.py:191-237."""
    quat = np.array(uniform_quat(n_search))
    ccs = score(mrc1, mrc2, quat)
    order = np.argsort(ccs)[::-1]
    qs, cs = np.zeros((nscs, 4)), np.zeros(nscs)
    for n in range(nscs):
        qs[n], cs[n] = scan_orientations_fine(mrc1, mrc2, quat[order[n]], ccs[order[n]],
                                              random_quat, randn, n_iterations, n_search, score)
    return qs[np.argmax(cs)], np.max(cs)


def align_volumes(mrc1, mrc2, uniform_quat, random_quat, randn, zoom=1, sigma=0,
                  n_iterations=10, n_search=420, nscs=1, score=score_deformations):
    """align.py:239-334 without the MRC output; returns (r_vol,
    mrc2_centred, final_cc, opt_q, inverted)."""
    mrc1, mrc2 = center_volume(np.array(mrc1)), center_volume(np.array(mrc2))
    m1o, m2o = mrc1.copy(), mrc2.copy()
    if zoom != 1:
        mrc1 = ndimage.zoom(mrc1, (zoom, zoom, zoom))
        mrc2 = ndimage.zoom(mrc2, (zoom, zoom, zoom))
    if sigma != 0:
        mrc1 = ndimage.gaussian_filter(mrc1, sigma=sigma)
        mrc2 = ndimage.gaussian_filter(mrc2, sigma=sigma)
    q1, c1 = scan_orientations(mrc1, mrc2, uniform_quat, random_quat, randn, n_iterations,
                               n_search, nscs, score)
    q2, c2 = scan_orientations(np.flip(mrc1, [0, 1, 2]), mrc2, uniform_quat, random_quat, randn,
                               n_iterations, n_search, nscs, score)
    if c1 > c2:
        opt_q, invert = q1, False
    else:
        opt_q, invert = q2, True
    if invert:
        m1o = np.flip(m1o, [0, 1, 2])
    r_vol = rotate_volume(m1o, np.expand_dims(opt_q, axis=0))[0]
    final = pearson_cc(np.expand_dims(r_vol.flatten(), 0), np.expand_dims(m2o.flatten(), 0))[0]
    return r_vol, m2o, final, opt_q, invert
