"""The continuous-batching server: every request's result is the same alone
and in the mix (identical indices), equals the plain FP32 argmin up to 1e-6
relative ties, admission respects the HBM budget, and bad requests fail on
the host without touching the device."""
import numpy as np
import pytest
import torch

from oracle import matching as om

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def world(lib):
    from spinifel_gb300 import matching

    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(60)
    n_ref, n_pix = 3000, 4096
    refs = rng.gamma(0.5, 1.0, (n_ref, n_pix)).astype(np.float32)
    pick = rng.integers(0, n_ref, 1500)
    frames = np.minimum(rng.poisson(refs[pick]), 65535).astype(np.int32)
    frames16 = torch.as_tensor(np.where(frames > 32767, frames - 65536, frames).astype(np.int16))
    rs = matching.ReferenceSet(torch.as_tensor(refs, device=dev))
    return dict(refs=refs, rs=rs, frames=frames.astype(np.float32), frames16=frames16, dev=dev)


def _alone(world, lo, hi):
    from spinifel_gb300 import matching

    x = torch.as_tensor(world["frames"][lo:hi], device=world["dev"])
    idx, _ = matching.match_bf16(matching.FrameSet(x), world["rs"])
    return idx.cpu().numpy()


def test_results_same_alone_and_in_the_mix(world):
    from spinifel_gb300.serving import OrientationServer

    rng = np.random.default_rng(61)
    sizes = [1, 7, 128, 300, 2, 512, 33, 64, 200, 5]
    bounds = np.cumsum([0] + sizes)
    with OrientationServer(world["rs"], slot_frames=512, n_slots=3) as srv:
        futs = [srv.submit(world["frames16"][bounds[i]:bounds[i + 1]].pin_memory())
                for i in range(len(sizes))]
        mixed = [f.result(timeout=60) for f in futs]
        stats = dict(srv.stats)
    assert stats["launches"] < len(sizes)  # requests were batched together
    _, d = om.sklearn_argmin(world["refs"], world["frames"][:bounds[-1]])
    for i in range(len(sizes)):
        alone = _alone(world, bounds[i], bounds[i + 1])
        np.testing.assert_array_equal(mixed[i], alone)
        oidx = np.argmin(d[:, bounds[i]:bounds[i + 1]], axis=0)
        assert np.all(om.ties_equal(mixed[i], oidx, d[:, bounds[i]:bounds[i + 1]]))


def test_plain_path_server_matches(world):
    from spinifel_gb300.serving import OrientationServer

    with OrientationServer(world["rs"], slot_frames=256, n_slots=2, path="fp32") as srv:
        a = srv.submit(world["frames16"][:100]).result(timeout=60)
    _, d = om.sklearn_argmin(world["refs"], world["frames"][:100])
    assert np.all(om.ties_equal(a, np.argmin(d, axis=0), d))


def test_admission_respects_hbm_budget(world):
    from spinifel_gb300.serving import OrientationServer

    # budget for 300 frames in flight: a 512-frame slot can never be filled
    srv = OrientationServer(world["rs"], slot_frames=512, n_slots=3, hbm_budget=None)
    per = srv.per_frame_bytes
    srv.close()
    with OrientationServer(world["rs"], slot_frames=512, n_slots=3, hbm_budget=300 * per) as srv:
        futs = [srv.submit(world["frames16"][i * 200:(i + 1) * 200]) for i in range(5)]
        res = [f.result(timeout=60) for f in futs]
        assert srv.in_use_bytes == 0
        assert srv.stats["frames"] == 1000
    for i in range(5):
        np.testing.assert_array_equal(res[i], _alone(world, i * 200, (i + 1) * 200))


def test_bad_requests_rejected_on_host(world):
    from spinifel_gb300.serving import OrientationServer

    with OrientationServer(world["rs"], slot_frames=128, n_slots=1) as srv:
        with pytest.raises(ValueError):
            srv.submit(torch.zeros(3, 17, dtype=torch.int16))
        with pytest.raises(ValueError):
            srv.submit(torch.zeros(129, 4096, dtype=torch.int16))
        with pytest.raises(TypeError):
            srv.submit(torch.zeros(3, 4096, dtype=torch.float32))
        ok = srv.submit(world["frames16"][:3]).result(timeout=60)
        assert ok.shape == (3,)
    with pytest.raises(RuntimeError):
        srv.submit(world["frames16"][:3])


def test_replayed_poisson_schedule_reports_latency(world):
    from spinifel_gb300.serving import OrientationServer, poisson_schedule, run_schedule

    sched = poisson_schedule(1500, 20000.0, np.random.default_rng(62), max_batch=512)
    with OrientationServer(world["rs"], slot_frames=512, n_slots=3) as srv:
        res = run_schedule(srv, world["frames16"].pin_memory(), sched)
        lat = srv.latency_ms()
    assert sum(r.size for r in res) == 1500
    assert lat.size == len(sched) and np.all(lat > 0)
