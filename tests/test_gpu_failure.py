"""Failure detection without a GPU fault: a bounded device wait that can
never complete gives up after its limit, reports SPF_ERR_TIMEOUT through the
device error word, and the context stays usable for the next launch; host
errors (bad arguments) are raised before any device work."""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives(lib):
    from spinifel_gb300 import _lib, matching

    dev = torch.device("cuda", 0)
    res = torch.zeros(2, dtype=torch.int32, device=dev)
    _lib.call("spf_selftest_bounded_wait", 200, _lib.ptr(res), _lib.stream_handle())
    torch.cuda.synchronize()
    gave_up, waited_ms = res.tolist()
    assert gave_up == 0 and 190 <= waited_ms < 2000
    with pytest.raises(_lib.SpfError) as ei:
        matching.check_device_error()
    assert ei.value.status == _lib.SPF_ERR_TIMEOUT
    matching.check_device_error()  # the word was reset
    # the context is still usable
    x = torch.rand(8, 64, device=dev)
    idx, _ = matching.argmin_fp32(x, x.clone())
    assert idx.tolist() == list(range(8))


def test_bad_arguments_raise_on_the_host(lib):
    from spinifel_gb300 import _lib, matching

    with pytest.raises(_lib.SpfError) as ei:
        matching.knn_topk(torch.zeros(3, 4, device="cuda"), 5)  # k > n_ref
    assert ei.value.status == _lib.SPF_ERR_ARG
    with pytest.raises(_lib.SpfError):
        _lib.call("spf_selftest_bounded_wait", 0, ctypes.c_void_p(16), None)
