"""Host-side serving logic without a GPU: the arrival schedule."""
import numpy as np

from spinifel_gb300.serving import poisson_schedule


def test_poisson_schedule_sizes_and_rate():
    rng = np.random.default_rng(0)
    s = poisson_schedule(200_000, 2000.0, rng, max_batch=512)
    sizes = np.array([n for _, n in s])
    times = np.array([t for t, _ in s])
    assert sizes.sum() == 200_000 and sizes.min() >= 1 and sizes.max() <= 512
    assert np.all(np.diff(times) > 0)
    rate = sizes.sum() / times[-1]
    assert 1700 < rate < 2300
    # log-uniform sizes: the median is near sqrt(512)
    assert 12 < np.median(sizes) < 40
