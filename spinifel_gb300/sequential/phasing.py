"""Drop-in for spinifel.sequential.phasing (spinifel/sequential/phasing.py):
phase() with the reference's signature and return values, its loop
functions over a device-resident Phaser, and the schedule
N_phase_loops x (ER, HIO, ER, shrink-wrap) + ER run on the GPU in FP64.

Difference: the reference seeds the starting density with the unseeded
xp.random.rand when rho_ is None (phasing.py:264-265); here the generator can
be passed (rng), defaulting to an unseeded numpy Generator."""
from __future__ import annotations

import numpy as np

from ..phasing import Phaser
from ..settings import settings as _default_settings


def create_support_(ac_, M, Mquat, generation=0, phaser: Phaser | None = None):
    """support_ from the region of strong (filtered, shifted) ACF signal in
    the central cube (phasing.py:84-107); ac_ is the ifftshifted filtered ACF
    kept by the phaser's set_ac, so phaser is required."""
    if phaser is None:
        raise ValueError("create_support_ needs the Phaser that holds ac_filt_")
    phaser.create_support(Mquat)
    return phaser.state()[1]


def ER_loop(n_loops, phaser: Phaser, rho_max=np.inf):
    phaser.er(n_loops, rho_max)


def HIO_loop(n_loops, beta, phaser: Phaser, rho_max=np.inf):
    phaser.hio(n_loops, beta, rho_max)


def shrink_wrap(sigma, phaser: Phaser, method=None, weight=1.0, cutoff=0.05):
    phaser.shrink_wrap(sigma, method, weight, cutoff)


def phase(generation, ac, support_=None, rho_=None, method=None, weight=1.0, settings=None,
          rng=None):
    """Phase retrieval of the autocorrelation `ac` (phasing.py:225-314).
    Returns (ac_phased float64 [M,M,M] centred, support_ bool, rho_ float64),
    numpy arrays, as the reference does."""
    st = settings or _default_settings
    Mquat = st.Mquat
    M = 4 * Mquat + 1
    ac = np.asarray(ac)
    if ac.shape != (M, M, M):
        raise ValueError(f"ac must be {M}^3 (M = 4 Mquat + 1), got {ac.shape}")
    ph = Phaser(M)
    try:
        ph.set_ac(np.real(ac).astype(np.float64))
        if support_ is None:
            ph.create_support(Mquat)
            sup = None
        else:
            sup = np.asarray(support_).astype(np.uint8)
        if rho_ is None:
            s = ph.state()[1].cpu().numpy() if sup is None else sup.astype(bool)
            rng = rng or np.random.default_rng()
            rho_ = s * rng.random(s.shape)
        ph.set_state(np.asarray(rho_, dtype=np.float64), sup)
        ph.run(st.N_phase_loops, st.nER, st.nHIO, st.beta, method=method, weight=weight,
               cutoff=0.05)
        ac_phased, _ = ph.finish()
        rho_d, sup_d = ph.state()
        return (ac_phased.cpu().numpy(), sup_d.cpu().numpy(), rho_d.cpu().numpy())
    finally:
        ph.close()
