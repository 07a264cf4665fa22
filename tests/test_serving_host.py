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


def test_mpi_sweep_lambdas_and_choice():
    """The per-rank lambdas and rank 0's L-curve choice of the MPI merge
    (spinifel/mpi/autocorrelation.py:64-67,188-196), host logic only."""
    from spinifel_gb300.mpi.autocorrelation import choose, lambdas

    rl, fl = lambdas(15, 2560, 4)
    np.testing.assert_allclose(rl, 15 ** 3 / 2560 * 2.0 ** (np.arange(4) - 2))
    np.testing.assert_allclose(fl, [1e3, 1e4, 1e5, 1e6])
    v1 = np.array([8.5, 7.8, 6.9, 5.7])
    v2 = np.array([0.1, 0.3, 1.0, 2.5])
    assert choose(0, rl, v1, v2) == 1        # largest lambda among norms >= mean
    assert choose(1, rl, v1, v2) == 2        # smallest v1 + v2 (6.9 + 1.0)
    assert choose(1, rl, v1, v1 * 0) == 3
