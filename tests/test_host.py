"""Host-side logic that needs no GPU: settings, geometry, synthetic inputs,
and the C ABI library (it loads, exports every declared symbol, and rejects
bad arguments before touching the device)."""
import ctypes

import numpy as np
import pytest

from spinifel_gb300 import Settings, geom, synth


def test_settings_derived_values():
    s = Settings()
    assert s.Mquat == 20 and s.M == 81 and s.M_ups == 162
    assert Settings(oversampling=2).M == 161
    assert Settings(det_shape=(4, 512, 512)).reduced_det_shape == (4, 16, 16)
    assert Settings(det_shape=(4, 128, 128), N_clipping=0, N_binning=0).reduced_det_shape == \
        (4, 128, 128)
    assert Settings(M_override=151).M_ups == 302


def test_rotations_orthonormal_and_inverse():
    rng = np.random.default_rng(0)
    q = geom.uniform_quaternions(100, rng)
    np.testing.assert_allclose(np.linalg.norm(q, axis=1), 1.0, atol=1e-12)
    R = geom.quaternion2rot3d(q)
    np.testing.assert_allclose(R @ np.swapaxes(R, 1, 2), np.broadcast_to(np.eye(3), R.shape),
                               atol=1e-12)
    np.testing.assert_allclose(np.linalg.det(R), 1.0, atol=1e-12)
    Rinv = geom.inverse_rotmats(q)
    np.testing.assert_allclose(Rinv, np.linalg.inv(R), atol=1e-12)


def test_hkl_matches_reference_einsum():
    rng = np.random.default_rng(1)
    q = geom.uniform_quaternions(5, rng)
    ppr, _ = geom.flat_detector(4, 3, 2)
    H, K, L = geom.hkl(q, ppr)
    Rinv = np.array([np.linalg.inv(geom.quaternion2rot3d(x)) for x in q])
    H2, K2, L2 = np.einsum("ijk,klmn->jilmn", Rinv, ppr)
    np.testing.assert_allclose(H, H2)
    np.testing.assert_allclose(L, L2)


def test_detector_and_model():
    ppr, pdr = geom.flat_detector(4, 32, 32)
    assert ppr.shape == (3, 4, 32, 32) and pdr.shape == (4, 32, 32)
    np.testing.assert_allclose(np.sqrt((ppr ** 2).sum(0)), pdr)
    # Ewald sphere: |q + k0|^2 == |k0|^2
    k0 = 1 / 2.5e-10
    np.testing.assert_allclose(ppr[0] ** 2 + ppr[1] ** 2 + (ppr[2] + k0) ** 2, k0 ** 2, rtol=1e-10)
    I = synth.intensity_model(15, seed=3)
    assert I.shape == (15, 15, 15) and I.max() == 1.0 and I.min() >= 0
    np.testing.assert_allclose(I, I[::-1, ::-1, ::-1], rtol=1e-9, atol=1e-12)  # Friedel


def test_library_exports_every_header_symbol(lib):
    from spinifel_gb300 import _lib

    declared = _lib.header_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), f"{name} declared in the header but not exported"
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"
    assert lib.spf_version().decode().startswith("spinifel_gb300")


def test_library_rejects_bad_arguments_without_a_device(lib):
    from spinifel_gb300 import _lib

    h = ctypes.c_void_p()
    assert lib.spf_nufft_plan_create(0, 8, 8, 1e-6, 2.0, ctypes.byref(h)) == _lib.SPF_ERR_ARG
    assert b"bad mode counts" in lib.spf_last_error()
    assert lib.spf_nufft_plan_create(8, 8, 8, 0.0, 2.0, ctypes.byref(h)) == _lib.SPF_ERR_ARG
    assert lib.spf_knn_topk_f32(None, 4, 10, 0, None, None) == _lib.SPF_ERR_ARG
    assert lib.spf_knn_topk_f32(None, 4, 10, 33, None, None) == _lib.SPF_ERR_ARG
    assert lib.spf_dist_argmin_f32(None, None, -1, None, None, 4, 4, 0, None, None) == \
        _lib.SPF_ERR_ARG
    # empty inputs are a no-op, not an error
    assert lib.spf_knn_eudist_f32(None, None, 0, 5, 16, None, None) == _lib.SPF_OK
    assert lib.spf_status_string(_lib.SPF_ERR_TIMEOUT) == b"device wait timed out"


def test_tunables_validated_without_a_device(lib):
    """spf_tune_set / spf_tune_get (host-side): the prime-grid regulariser
    switch takes 0 (default), 1 (Rader) or 2 (cuFFT); unknown parameters and
    out-of-range values are rejected; 0 restores the built-in default."""
    from spinifel_gb300 import _lib

    v = ctypes.c_int64(-1)
    assert lib.spf_tune_set(_lib.SPF_TUNE_PRIME_DFT, 3) == _lib.SPF_ERR_ARG
    assert lib.spf_tune_set(_lib.SPF_TUNE_PRIME_DFT, -1) == _lib.SPF_ERR_ARG
    assert lib.spf_tune_set(8, 1) == _lib.SPF_ERR_ARG
    assert lib.spf_tune_set(_lib.SPF_TUNE_STATIC_ABORT_TEST, 2) == _lib.SPF_ERR_ARG
    assert lib.spf_tune_set(_lib.SPF_TUNE_SLICE_SHAPE, 8) == _lib.SPF_ERR_ARG
    assert lib.spf_tune_set(_lib.SPF_TUNE_SORT_ITEM, 100) == _lib.SPF_ERR_ARG
    assert lib.spf_tune_set(_lib.SPF_TUNE_SORT_ITEM, 8193) == _lib.SPF_ERR_ARG
    for param, value in ((_lib.SPF_TUNE_SLICE_SHAPE, 7), (_lib.SPF_TUNE_SORT_ITEM, 1024),
                         (_lib.SPF_TUNE_STATIC_ABORT_TEST, 1)):
        assert lib.spf_tune_set(param, value) == _lib.SPF_OK
        assert lib.spf_tune_get(param, ctypes.byref(v)) == _lib.SPF_OK and v.value == value
        assert lib.spf_tune_set(param, 0) == _lib.SPF_OK
    assert lib.spf_tune_set(_lib.SPF_TUNE_PRIME_DFT, 2) == _lib.SPF_OK
    assert lib.spf_tune_get(_lib.SPF_TUNE_PRIME_DFT, ctypes.byref(v)) == _lib.SPF_OK
    assert v.value == 2
    assert lib.spf_tune_set(_lib.SPF_TUNE_PRIME_DFT, 0) == _lib.SPF_OK


def test_named_entry_points_and_server_reject_bad_arguments_without_a_device(lib):
    from spinifel_gb300 import _lib

    E = _lib.SPF_ERR_ARG
    srv = ctypes.c_void_p()
    P = ctypes.c_void_p(16)
    args = [0, P, P, P, P, 1.0, 1000, 64, 64]
    assert lib.spf_serve_create(*args, 2, 64, 2, 0, ctypes.byref(srv)) == E      # bad path
    assert b"path" in lib.spf_last_error()
    assert lib.spf_serve_create(0, None, P, P, None, 1.0, 1000, 64, 64, 0, 64, 2, 0,
                                ctypes.byref(srv)) == E                          # bf16 refs missing
    assert lib.spf_serve_create(*args[:7], 60, 60, 0, 64, 2, 0, ctypes.byref(srv)) == E  # ld % 8
    assert lib.spf_serve_create(*args, 0, 0, 2, 0, ctypes.byref(srv)) == E       # no slot frames
    assert lib.spf_serve_create(*args, 0, 64, 17, 0, ctypes.byref(srv)) == E     # too many slots
    assert srv.value is None
    t = ctypes.c_int64()
    flag = ctypes.c_int()
    assert lib.spf_serve_submit(None, P, 1, None, None, -1.0, ctypes.byref(t)) == E
    assert lib.spf_serve_wait(None, 1, 0, ctypes.byref(flag)) == E
    assert lib.spf_serve_stats(None, None, 0) == E
    assert lib.spf_serve_destroy(None) == _lib.SPF_OK
    c0 = lib.spf_serve_clock()
    assert lib.spf_serve_clock() >= c0 > 0
    # the scope-table names: argument checks before any device work
    assert lib.spf_fft_deconv(None, 2, -1, P, None, None, None, None) == E       # no plan
    assert lib.spf_spread_t1(None, P, P, P, P, 10, 1, P, None, None) == E
    assert lib.spf_cg_solve(None, 0, P, P, 1, 10, 1e-5, None, None, None) == E
    assert lib.spf_dist_argmin_fp32(None, None, 0, None, None, 5, 16, None, None, None,
                                    None) == _lib.SPF_OK                         # empty: no-op
    assert lib.spf_dist_argmin_fp32(P, P, 4, P, P, 5, 16, P, None, None, None) == E


def test_product_path_has_no_cpu_fallback(tmp_path):
    from spinifel_gb300 import _lib

    with pytest.raises(ImportError, match="no CPU fallback"):
        _lib._lib_backup = _lib._lib
        try:
            _lib._lib = None
            _lib.load(str(tmp_path / "missing.so"))
        finally:
            _lib._lib = _lib._lib_backup


def test_adjoint_dispatch_sorted_spreading_by_size(monkeypatch):
    """autocorrelation.adjoint sorts the points once and spreads with the
    sorted kernel from SORTED_SPREAD_MIN_POINTS points on (twice for complex
    values, one sort), and spreads point by point below it; sort=True/False
    overrides.  Host logic only: a recording stand-in replaces the plan."""
    import torch

    from spinifel_gb300 import _arrays
    from spinifel_gb300 import autocorrelation as ac

    monkeypatch.setattr(_arrays, "device", lambda: torch.device("cpu"))
    M = 4

    class Rec:
        dtype = torch.float32
        supports_sort = True

        def __init__(self):
            self.calls = []

        def sort_points(self, x, y, z):
            self.calls.append("sort")

        def spread_sorted(self, c):
            self.calls.append("spread_sorted")

        def spread(self, x, y, z, c):
            self.calls.append("spread")

        def spread_zero(self):
            self.calls.append("zero")

        def finish(self, isign, want_imag=False):
            return torch.zeros(M ** 3), torch.zeros(M ** 3)

    class Rec64(Rec):  # the FP64 plan has no sorted passes
        dtype = torch.float64
        supports_sort = False

    def run(n, values, cls=Rec, **kw):
        P = cls()
        xyz = [np.zeros(n, dtype=np.float32) for _ in range(3)]
        ac.adjoint(values(n), *xyz, M, plan=P, **kw)
        return P.calls

    big = ac.SORTED_SPREAD_MIN_POINTS
    real = lambda n: np.ones(n, dtype=np.float32)  # noqa: E731
    cplx = lambda n: np.ones(n, dtype=np.complex64) * (1 + 1j)  # noqa: E731
    assert run(big, real) == ["sort", "zero", "spread_sorted"]
    assert run(big - 1, real) == ["zero", "spread"]
    assert run(big, cplx) == ["sort", "zero", "spread_sorted", "zero", "spread_sorted"]
    assert run(10, real, sort=True) == ["sort", "zero", "spread_sorted"]
    assert run(big, real, sort=False) == ["zero", "spread"]
    assert run(big, real, cls=Rec64) == ["zero", "spread"]
    assert run(10, real, cls=Rec64, sort=True) == ["zero", "spread"]


def test_spread_orient_dispatch_by_size(monkeypatch):
    """NufftPlan.spread_orient: bin sort + sorted spreading from
    SORTED_MIN_POINTS points on, the patch kernel (panel detector) or the
    per-point kernel below; the plan keeps the sorted points' tensors."""
    import torch

    from spinifel_gb300 import _lib
    from spinifel_gb300.nufft import NufftPlan

    calls = []
    monkeypatch.setattr(_lib, "call", lambda name, *a: calls.append(name))
    monkeypatch.setattr(_lib, "stream_handle", lambda *a: None)
    P = object.__new__(NufftPlan)
    P._h = None
    P.device = torch.device("cpu")

    def run(n_orient, n_pix, det=None, **kw):
        calls.clear()
        q = torch.zeros(n_orient, 4)
        ppr = torch.zeros(3, n_pix)
        c = torch.zeros(n_orient * n_pix)
        P.spread_orient(q, ppr, 1.0, c, det_shape=det, **kw)
        return list(calls)

    n_pix = 4 * 32 * 32
    big = -(-NufftPlan.SORTED_MIN_POINTS // n_pix)  # orientations reaching the threshold
    assert run(big, n_pix, (4, 32, 32)) == ["spf_nufft_sort_orient", "spf_nufft_spread_sorted"]
    assert len(P._sorted_points) == 2
    assert run(2, n_pix, (4, 32, 32)) == ["spf_nufft_t1_spread_det"]
    assert run(2, n_pix) == ["spf_nufft_t1_spread_orient"]
    assert run(2, n_pix, sort=True) == ["spf_nufft_sort_orient", "spf_nufft_spread_sorted"]
