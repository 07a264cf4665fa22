"""FSC and volume alignment on the GPU against the reference's own eval/fsc.py
and eval/align.py outputs (golden, numpy/scipy branch) on the same volumes and
sampler streams.  Tolerances: FP64 on both sides; rotation samples 1e-12
absolute, correlations and FSC 1e-9 relative; the alignment search makes the
same choices, so its result matches to 1e-9."""
import os

import numpy as np
import pytest

from tests.golden import cases

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def gold(lib):
    return np.load(os.path.join(GOLD, "golden_eval.npz"))


def test_fsc_matches_reference(gold):
    from spinifel_gb300.eval.fsc import compute_fsc

    c = cases.EVAL
    v1, v2, *_ = cases.eval_inputs()
    res, rshell, fsc = compute_fsc(v1, v2, c["dmax"], spacing=c["spacing"])
    np.testing.assert_allclose(rshell, gold["rshell"], rtol=0, atol=0)
    ok = ~np.isnan(gold["fsc"])
    assert np.array_equal(np.isnan(fsc), ~ok)  # empty shells are NaN on both sides
    np.testing.assert_allclose(fsc[ok], gold["fsc"][ok], rtol=1e-9, atol=1e-12)
    assert abs(res - float(gold["resolution"])) <= 1e-9 * abs(res)


def test_rotation_and_scores_match_reference(gold):
    from spinifel_gb300.eval.align import rotate_volume, score_deformations

    v1, v2, uniform_quat, _, _ = cases.eval_inputs()
    quats = uniform_quat(12)
    np.testing.assert_array_equal(quats, gold["quats"])
    np.testing.assert_allclose(rotate_volume(v1, quats[:3]), gold["rot"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(score_deformations(v1, v2, quats), gold["ccs"], rtol=1e-9)


def test_align_volumes_matches_reference(gold):
    from spinifel_gb300.eval.align import align_volumes

    c = cases.EVAL
    v1, v2, uniform_quat, random_quat, randn = cases.eval_inputs()
    uniform_quat(12)  # the golden run drew these first
    r_vol, m2, final_cc = align_volumes(v1, v2, n_iterations=c["n_iterations"],
                                        n_search=c["n_search"], uniform_quat=uniform_quat,
                                        random_quat=random_quat, randn=randn)
    np.testing.assert_allclose(m2, gold["mrc2"], rtol=0, atol=1e-12)
    assert abs(final_cc - float(gold["final_cc"])) < 1e-9
    np.testing.assert_allclose(r_vol, gold["r_vol"], rtol=0, atol=1e-9)


def test_rotation_round_trip_and_fsc_like_reference_test(lib):
    """The shape of the reference's tests/test_FSC.py with a synthetic 81^3
    density (its PDB-derived density needs skopi): rotate by q^-1 and back by
    q, correlation > 0.85 as there; the blob density has less high-resolution
    content than the PDB map, so instead of the 1.25 x 9 Angstrom bound the
    FSC curve and resolution must equal the FP64 oracle's on the same
    volumes."""
    from oracle import evaluate as oev
    from spinifel_gb300 import geom
    from spinifel_gb300.eval.align import rotate_volume
    from spinifel_gb300.eval.fsc import compute_fsc

    M, res_target = 81, 9.0
    rng = np.random.default_rng(91)
    ax = np.arange(M) - M // 2
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    ref = np.zeros((M, M, M))
    for _ in range(30):
        c = rng.uniform(-M / 5, M / 5, 3)
        ref += rng.uniform(0.5, 1) * np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 +
                                              (Z - c[2]) ** 2) / (2 * rng.uniform(1.5, 3) ** 2))
    q = geom.uniform_quaternions(1, rng)
    q_inv = q * np.array([1, -1, -1, -1])
    back = rotate_volume(rotate_volume(ref, q_inv)[0], q)
    assert np.corrcoef(ref.flatten(), back.flatten())[0, 1] > 0.85
    res, _, fsc = compute_fsc(ref, back[0], 1e10 / res_target, 0.01)
    with np.errstate(invalid="ignore"):
        res_o, _, fsc_o = oev.compute_fsc(ref, back[0], 1e10 / res_target, 0.01)
    ok = ~np.isnan(fsc_o)
    np.testing.assert_allclose(fsc[ok], fsc_o[ok], rtol=1e-9, atol=1e-12)
    assert res > 0 and abs(res - res_o) <= 1e-9 * res
