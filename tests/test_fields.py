"""The synthetic log-normal conductivity of the batched learned-preconditioner
workload: a Gaussian random field with the requested mean, standard deviation
and squared-exponential correlation, deterministic for a seed."""
import numpy as np

from nonlocal_gb300.fields import gaussian_random_field, lognormal_conductivity, sample_periodic


def test_field_statistics_and_correlation():
    n, ell, std = 256, 0.1, 0.5
    corr = []
    for seed in range(8):
        g = gaussian_random_field(n, ell, std, seed)
        assert abs(g.mean()) < 1e-12 and abs(g.std() - std) < 1e-12
        lag = int(round(ell * n))   # one correlation length along x, periodic
        corr.append(np.mean(g * np.roll(g, lag, axis=1)) / std ** 2)
    # squared-exponential covariance: exp(-1/2) at one correlation length
    assert abs(np.mean(corr) - np.exp(-0.5)) < 0.12, np.mean(corr)


def test_field_is_seeded():
    a = gaussian_random_field(64, 0.1, 0.5, seed=3)
    b = gaussian_random_field(64, 0.1, 0.5, seed=3)
    c = gaussian_random_field(64, 0.1, 0.5, seed=4)
    assert np.array_equal(a, b) and not np.array_equal(a, c)


def test_sampling_at_grid_points_and_lognormal():
    g = gaussian_random_field(32, 0.2, 0.5, seed=1)
    j, i = np.meshgrid(np.arange(32), np.arange(32), indexing="ij")
    xy = np.stack([i / 32.0, j / 32.0], axis=-1)
    np.testing.assert_allclose(sample_periodic(g, xy), g, atol=1e-14)
    lam = lognormal_conductivity(np.random.default_rng(0).random((10, 4, 2)), 0.2, 0.5, seed=1, grid=32)
    assert lam.shape == (40,) and np.all(lam > 0.0)
