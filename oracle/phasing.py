"""Oracle (test infrastructure only): FP64 numpy/scipy restatement of the
reference's phase retrieval, spinifel/sequential/phasing.py, with the
settings singleton replaced by arguments.  Trailing underscores mean
ifftshifted arrays (phasing.py:27-40).  Imported only by tests, smoke() and
the CPU baseline of bench.py."""
from __future__ import annotations

import numpy as np
from scipy.ndimage import gaussian_filter


def center_of_mass(rho_, hkl_, M):
    """phasing.py:45-58."""
    rho_ = np.abs(rho_)
    num = (rho_ * hkl_).sum(axis=(1, 2, 3))
    den = rho_.sum()
    return np.round(num / den * M / 2)


def recenter(rho_, support_, M):
    """phasing.py:62-80; returns the three shifts."""
    ls = np.linspace(-1, 1, M + 1)
    ls = (ls[:-1] + ls[1:]) / 2
    hkl_list = np.meshgrid(ls, ls, ls, indexing="ij")
    hkl_ = np.stack([np.fft.ifftshift(c) for c in hkl_list])
    vect = center_of_mass(rho_, hkl_, M)
    shifts = []
    for i in range(3):
        shift = int(vect[i])
        rho_[:] = np.roll(rho_, -shift, i)
        support_[:] = np.roll(support_, -shift, i)
        shifts.append(shift)
    return shifts


def create_support_(ac_, M, Mquat):
    """phasing.py:84-107."""
    sl = slice(Mquat, -Mquat)
    square = np.zeros((M, M, M), dtype=np.bool_)
    square[sl, sl, sl] = 1
    square_ = np.fft.ifftshift(square)
    thresh_ = ac_ > 1e-2 * ac_.max()
    return np.logical_and(square_, thresh_)


def step_phase(rho_, amplitudes_, amp_mask_, support_):
    """phasing.py:173-189."""
    rho_hat_ = np.fft.fftn(rho_)
    phases_ = np.angle(rho_hat_)
    rho_hat_mod_ = np.where(amp_mask_, amplitudes_ * np.exp(1j * phases_), rho_hat_)
    rho_mod_ = np.fft.ifftn(rho_hat_mod_).real
    support_star_ = np.logical_and(support_, rho_mod_ > 0)
    return rho_mod_, support_star_


def ER(rho_, amplitudes_, amp_mask_, support_, rho_max):
    """phasing.py:130-147."""
    rho_mod_, star_ = step_phase(rho_, amplitudes_, amp_mask_, support_)
    rho_[:] = np.where(star_, rho_mod_, 0)
    rho_[rho_mod_ > rho_max] = rho_max


def HIO(beta, rho_, amplitudes_, amp_mask_, support_, rho_max):
    """phasing.py:151-169."""
    rho_mod_, star_ = step_phase(rho_, amplitudes_, amp_mask_, support_)
    rho_[:] = np.where(star_, rho_mod_, rho_ - beta * rho_mod_)
    over = rho_mod_ > rho_max
    rho_[over] += 2 * beta * rho_mod_[over] - rho_max


def shrink_wrap(sigma, rho_, support_, method=None, weight=1.0, cutoff=0.05):
    """phasing.py:193-221."""
    rho_abs_ = np.absolute(rho_)
    rho_gauss_ = gaussian_filter(rho_abs_, mode="wrap", sigma=sigma, truncate=2)
    method = method or "std"
    if method == "std":
        threshold = np.std(rho_gauss_) * weight
    elif method == "max":
        threshold = rho_abs_.max() * cutoff * weight
    else:
        raise ValueError(method)
    support_[:] = rho_gauss_ > threshold


def prepare(ac, M, Mquat):
    """The amplitude and support set-up at the top of phase() (phasing.py:248-262)."""
    ac_filt = gaussian_filter(np.maximum(np.asarray(ac).real, 0), mode="constant", sigma=1,
                              truncate=2)
    ac_filt_ = np.fft.ifftshift(ac_filt)
    amplitudes_ = np.sqrt(np.abs(np.fft.fftn(ac_filt_)))
    amp_mask_ = np.ones((M, M, M), dtype=np.bool_)
    amp_mask_[0, 0, 0] = 0
    return ac_filt_, amplitudes_, amp_mask_


def phase(ac, Mquat, support_=None, rho_=None, nER=10, nHIO=5, beta=0.9, N_phase_loops=5,
          method=None, weight=1.0, rng=None):
    """phase() of phasing.py:225-314 with the settings as arguments; returns
    (ac_phased, support_, rho_, shifts)."""
    M = 4 * Mquat + 1
    ac_filt_, amplitudes_, amp_mask_ = prepare(ac, M, Mquat)
    if support_ is None:
        support_ = create_support_(ac_filt_, M, Mquat)
    support_ = np.array(support_, dtype=np.bool_)
    if rho_ is None:
        rng = rng or np.random.default_rng()
        rho_ = support_ * rng.random(support_.shape)
    rho_ = np.array(rho_, dtype=np.float64)
    rho_max = np.inf
    for _ in range(N_phase_loops):
        for _ in range(nER):
            ER(rho_, amplitudes_, amp_mask_, support_, rho_max)
        for _ in range(nHIO):
            HIO(beta, rho_, amplitudes_, amp_mask_, support_, rho_max)
        for _ in range(nER):
            ER(rho_, amplitudes_, amp_mask_, support_, rho_max)
        shrink_wrap(1, rho_, support_, method=method, weight=weight)
    for _ in range(nER):
        ER(rho_, amplitudes_, amp_mask_, support_, rho_max)
    shifts = recenter(rho_, support_, M)
    intensities_phased_ = np.abs(np.fft.fftn(rho_)) ** 2
    ac_phased = np.fft.fftshift(np.abs(np.fft.ifftn(intensities_phased_)))
    return ac_phased.astype(np.float64), support_, rho_, shifts
