"""Phase retrieval on the GPU (spf_phase_* through the C ABI) against the
FP64 oracle and the reference's own phase() output.  Tolerance: relative L2
1e-9 after the full schedule (cuFFT and pocketfft round differently; ER/HIO
are non-expansive, so the differences stay at rounding level), 1e-12 for a
single step; supports must agree exactly."""
import os

import numpy as np
import pytest
import torch

from oracle import phasing as oph
from tests.golden import cases

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.fixture(scope="module")
def dev(lib):
    return torch.device("cuda", 0)


def test_phase_matches_reference_golden(dev):
    from spinifel_gb300 import Settings
    from spinifel_gb300.sequential.phasing import phase

    p = cases.PHASE
    ac, rho0 = cases.phase_inputs()
    st = Settings(Mquat_override=p["Mquat"], nER=p["nER"], nHIO=p["nHIO"],
                  N_phase_loops=p["N_phase_loops"], beta=p["beta"])
    acp, sup, rho = phase(0, ac, None, rho0, settings=st)
    g = np.load(os.path.join(GOLD, "golden_phase.npz"))
    assert np.array_equal(sup, g["support_"].astype(bool))
    assert rel(rho, g["rho_"]) < 1e-9
    assert rel(acp, g["ac_phased"]) < 1e-9


def _state(M, rng, Mquat):
    ax = np.arange(M) - M // 2
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    rho = np.exp(-(X ** 2 + (Y - 1) ** 2 + (Z + 1) ** 2) / 6.0) + 0.3 * rng.random((M, M, M))
    F = np.fft.fftn(np.fft.ifftshift(rho))
    ac = np.fft.fftshift(np.fft.ifftn(np.abs(F) ** 2).real)
    return ac, rng.random((M, M, M))


@pytest.mark.parametrize("M", [21, 24])
def test_single_steps_match_oracle(dev, M):
    """One ER, one HIO, and both shrink-wrap methods from the same state, on
    an odd (reference) and an even grid."""
    from spinifel_gb300.phasing import Phaser

    rng = np.random.default_rng(81)
    Mquat = M // 4
    ac, rho0 = _state(M, rng, Mquat)
    ac_filt_, amp_, mask_ = oph.prepare(ac, M, Mquat)
    sup0 = oph.create_support_(ac_filt_, M, Mquat)
    ph = Phaser(M)
    ph.set_ac(ac)
    ph.create_support(Mquat)
    _, s = ph.state()
    assert np.array_equal(s.cpu().numpy(), sup0)

    for step in ("er", "hio"):
        ph.set_state(rho0, sup0)
        r = rho0.copy()
        if step == "er":
            ph.er(1)
            oph.ER(r, amp_, mask_, sup0, np.inf)
        else:
            ph.hio(1, 0.9)
            oph.HIO(0.9, r, amp_, mask_, sup0, np.inf)
        got, _ = ph.state()
        assert rel(got.cpu().numpy(), r) < 1e-12, step

    # rho_max clipping
    ph.set_state(rho0, sup0)
    r = rho0.copy()
    ph.hio(1, 0.9, rho_max=0.5)
    oph.HIO(0.9, r, amp_, mask_, sup0, 0.5)
    assert rel(ph.state()[0].cpu().numpy(), r) < 1e-12

    for method in ("std", "max"):
        ph.set_state(rho0, sup0)
        s = sup0.copy()
        ph.shrink_wrap(1.0, method=method, weight=1.0, cutoff=0.05)
        oph.shrink_wrap(1.0, rho0.copy(), s, method=method, weight=1.0, cutoff=0.05)
        assert np.array_equal(ph.state()[1].cpu().numpy(), s), method
    ph.close()


def test_finish_recenters_and_is_reproducible(dev):
    from spinifel_gb300.phasing import Phaser

    rng = np.random.default_rng(82)
    M, Mquat = 21, 5
    ac, _ = _state(M, rng, Mquat)
    # a blob away from the origin of the shifted grid, so recentring moves it
    X, Y, Z = np.meshgrid(*(np.arange(M) - 3,) * 3, indexing="ij")
    rho0 = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 4.0)
    sup0 = rho0 > 0.1
    outs = []
    for _ in range(2):
        ph = Phaser(M)
        ph.set_ac(ac)
        ph.set_state(rho0, sup0)
        ph.run(1, 2, 2, 0.9)
        out, sh = ph.finish()
        r, s = ph.state()
        outs.append((out.cpu().numpy(), sh, r.cpu().numpy(), s.cpu().numpy()))
        ph.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and outs[0][1] == outs[1][1]
    # against the oracle's schedule and recentring
    _, amp_, mask_ = oph.prepare(ac, M, Mquat)
    r = rho0.copy()
    s = sup0.copy()
    for _ in range(2):
        oph.ER(r, amp_, mask_, s, np.inf)
    for _ in range(2):
        oph.HIO(0.9, r, amp_, mask_, s, np.inf)
    for _ in range(2):
        oph.ER(r, amp_, mask_, s, np.inf)
    oph.shrink_wrap(1, r, s)
    for _ in range(2):
        oph.ER(r, amp_, mask_, s, np.inf)
    shifts = oph.recenter(r, s, M)
    acp = np.fft.fftshift(np.abs(np.fft.ifftn(np.abs(np.fft.fftn(r)) ** 2)))
    assert outs[0][1] == shifts
    assert np.array_equal(outs[0][3], s)
    assert rel(outs[0][2], r) < 1e-10
    assert rel(outs[0][0], acp) < 1e-10


def test_phaser_rejects_bad_arguments(dev):
    from spinifel_gb300 import _lib
    from spinifel_gb300.phasing import Phaser

    ph = Phaser(9)
    with pytest.raises(_lib.SpfError):  # method 7 does not exist
        _lib.call("spf_phase_shrink_wrap", ph.handle, 1.0, 7, 1.0, 0.05, _lib.stream_handle())
    with pytest.raises(ValueError):
        ph.shrink_wrap(1.0, method="median")
    with pytest.raises(_lib.SpfError):
        ph.create_support(5)  # 2 * Mquat >= M
    with pytest.raises(ValueError):
        ph.set_state(np.zeros((8, 8, 8)))
    ph.close()
