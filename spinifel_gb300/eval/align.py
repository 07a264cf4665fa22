"""Volume alignment with the reference's surface (eval/align.py,
eval/geom.py): a coarse search over uniform rotations, then rounds of
samples around the best one with a shrinking spread, for both hands.  Every
candidate set is scored on the GPU by spf_eval_score_rotations, which samples
the rotated volume trilinearly on the fly and returns the Pearson
correlations without storing rotated copies.

The samplers are arguments: the reference draws the coarse set from
skopi.get_uniform_quat, the spread axes from skopi.get_random_quat and the
angles from numpy's global generator (geom.py:99-135); here uniform_quat(n),
random_quat(n) and randn(n) default to a seeded Shoemake sampler and a seeded
numpy RandomState.  center_volume (a cubic-spline shift, once per alignment)
and the optional zoom / Gaussian prefilter run on the host with
scipy.ndimage, as in the reference's CPU branch."""
from __future__ import annotations

import numpy as np
import torch
from scipy import ndimage

from .. import _lib, geom as _geom


def _dev():
    return torch.device("cuda", torch.cuda.current_device())


def _t(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=_dev())


def quaternion2rot3d(quat):
    q = np.asarray(quat, dtype=np.float64)
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((q.shape[0], 3, 3))
    R[:, 0] = np.stack([1. - 2. * (y * y + z * z), 2. * (x * y - w * z), 2. * (x * z + w * y)], 1)
    R[:, 1] = np.stack([2. * (x * y + w * z), 1. - 2. * (x * x + z * z), 2. * (y * z - w * x)], 1)
    R[:, 2] = np.stack([2. * (x * z - w * y), 2. * (y * z + w * x), 1. - 2. * (x * x + y * y)], 1)
    return R


def axis_angle_to_quaternion(axis, theta):
    axis = axis / np.linalg.norm(axis, axis=1)[:, None]
    q = np.zeros((len(theta), 4))
    q[:, 0] = np.cos(theta / 2)
    q[:, 1:] = np.sin(theta / 2)[:, None] * axis
    return q


def quaternion_product(q1, q0):
    """Rotation by q0 followed by q1 (geom.py:71-97)."""
    p0, p1, p2, p3 = q1.T
    r0, r1, r2, r3 = q0.T
    return np.array([r0 * p0 - r1 * p1 - r2 * p2 - r3 * p3, r0 * p1 + r1 * p0 - r2 * p3 + r3 * p2,
                     r0 * p2 + r1 * p3 + r2 * p0 - r3 * p1,
                     r0 * p3 - r1 * p2 + r2 * p1 + r3 * p0]).T


def get_preferred_orientation_quat(num_pts, sigma, base_quat=None, random_quat=None, randn=None):
    random_quat, randn = _samplers(None, random_quat, randn)[1:]
    if base_quat is None:
        base_quat = np.array(random_quat(1))
    base = np.tile(base_quat, num_pts).reshape(num_pts, 4)
    R_random = quaternion2rot3d(np.array(random_quat(num_pts)))
    rot_axis = np.matmul(np.array([0, 0, 1.0]), R_random)
    theta = sigma * randn(num_pts)
    return quaternion_product(axis_angle_to_quaternion(theta[:, None] * rot_axis, theta), base)


_default = {}


def _samplers(uniform_quat, random_quat, randn):
    if not _default:
        rng = np.random.default_rng(20261203)
        _default["q"] = lambda n: _geom.uniform_quaternions(n, rng)
        _default["randn"] = np.random.RandomState(20261203).randn
    return (uniform_quat or _default["q"], random_quat or _default["q"],
            randn or _default["randn"])


def rotate_volume(vol, quat):
    """Rotated copies [n_quat, M, M, M] (align.py:36-67), on the GPU."""
    vol = np.asarray(vol, dtype=np.float64)
    quat = np.atleast_2d(np.asarray(quat, dtype=np.float64))
    M = vol.shape[0]
    out = torch.empty(quat.shape[0], M, M, M, dtype=torch.float64, device=_dev())
    v, q = _t(vol), _t(quat)
    _lib.call("spf_eval_rotate_volume", _lib.ptr(v), M, _lib.ptr(q), quat.shape[0],
              _lib.ptr(out), _lib.stream_handle())
    return out.cpu().numpy()


def score_deformations(mrc1, mrc2, warp):
    """Pearson correlation of mrc1 rotated by each quaternion with mrc2
    (align.py:112-146); rotations only, as the reference implements."""
    warp = np.atleast_2d(np.asarray(warp, dtype=np.float64))
    if warp.shape[-1] != 4:
        raise NotImplementedError("only rotations (quaternions) are scored")
    M = np.asarray(mrc1).shape[0]
    v1, v2, q = _t(mrc1), _t(mrc2), _t(warp)
    cc = torch.empty(warp.shape[0], dtype=torch.float64, device=_dev())
    _lib.call("spf_eval_score_rotations", _lib.ptr(v1), _lib.ptr(v2), M, _lib.ptr(q),
              warp.shape[0], _lib.ptr(cc), _lib.stream_handle())
    return cc.cpu().numpy()


def pearson_cc(arr1, arr2):
    vx = arr1 - arr1.mean(axis=-1)[:, None]
    vy = arr2 - arr2.mean(axis=-1)[:, None]
    return np.sum(vx * vy, axis=1) / (np.sqrt(np.sum(vx ** 2, axis=1)) *
                                      np.sqrt(np.sum(vy ** 2, axis=1)))


def center_volume(vol):
    old = np.array(ndimage.center_of_mass(vol))
    new = np.array(np.array(vol.shape) / 2).astype(int)
    return ndimage.shift(vol, -1 * (old - new))


def scan_orientations_fine(mrc1, mrc2, opt_q, prev_score, n_iterations=10, n_search=420,
                           random_quat=None, randn=None):
    sigmas = 2 - 0.2 * np.arange(1, 10)
    for n in range(1, n_iterations):
        quat = get_preferred_orientation_quat(n_search - 1, float(sigmas[n - 1]), opt_q,
                                              random_quat, randn)
        quat = np.vstack((opt_q, quat))
        ccs = score_deformations(mrc1, mrc2, quat)
        if np.max(ccs) < prev_score:
            break
        opt_q = quat[np.argmax(ccs)]
        prev_score = np.max(ccs)
    return opt_q, prev_score


def scan_orientations(mrc1, mrc2, n_iterations=10, n_search=420, nscs=1, uniform_quat=None,
                      random_quat=None, randn=None):
    uniform_quat, random_quat, randn = _samplers(uniform_quat, random_quat, randn)
    quat = np.array(uniform_quat(n_search))
    ccs = score_deformations(mrc1, mrc2, quat)
    order = np.argsort(ccs)[::-1]
    qs, cs = np.zeros((nscs, 4)), np.zeros(nscs)
    for n in range(nscs):
        qs[n], cs[n] = scan_orientations_fine(mrc1, mrc2, quat[order[n]], ccs[order[n]],
                                              n_iterations, n_search, random_quat, randn)
    return qs[np.argmax(cs)], np.max(cs)


def flip(arr, orien):
    return np.flip(arr, orien)


def align_volumes(mrc1, mrc2, zoom=1, sigma=0, n_iterations=10, n_search=420, nscs=1,
                  output=None, voxel_size=None, uniform_quat=None, random_quat=None, randn=None):
    """(r_vol, mrc2_centred, final_cc) as the reference (align.py:239-334).
    Writing an MRC file (output) needs the mrcfile package."""
    samplers = _samplers(uniform_quat, random_quat, randn)
    mrc1, mrc2 = center_volume(np.array(mrc1)), center_volume(np.array(mrc2))
    m1o, m2o = mrc1.copy(), mrc2.copy()
    if zoom != 1:
        mrc1 = ndimage.zoom(mrc1, (zoom, zoom, zoom))
        mrc2 = ndimage.zoom(mrc2, (zoom, zoom, zoom))
    if sigma != 0:
        mrc1 = ndimage.gaussian_filter(mrc1, sigma=sigma)
        mrc2 = ndimage.gaussian_filter(mrc2, sigma=sigma)
    q1, c1 = scan_orientations(mrc1, mrc2, n_iterations, n_search, nscs, *samplers)
    q2, c2 = scan_orientations(flip(mrc1, [0, 1, 2]), mrc2, n_iterations, n_search, nscs,
                               *samplers)
    opt_q, invert = (q1, False) if c1 > c2 else (q2, True)
    if invert:
        m1o = flip(m1o, [0, 1, 2])
    r_vol = rotate_volume(m1o, np.expand_dims(opt_q, axis=0))[0]
    final_cc = pearson_cc(np.expand_dims(r_vol.flatten(), 0), np.expand_dims(m2o.flatten(), 0))[0]
    if output is not None:
        import mrcfile  # noqa: F401  (absent here; the reference's save_mrc needs it)

        raise NotImplementedError("MRC output needs the mrcfile package")
    return r_vol, m2o, final_cc
