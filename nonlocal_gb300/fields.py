"""Random coefficient fields for synthetic workloads.

A stationary Gaussian random field on the unit square with the squared-
exponential covariance C(d) = std^2 exp(-d^2 / (2 l^2)) is drawn on a periodic
n x n grid by spectral synthesis: complex white noise shaped by the square
root of the covariance's spectral density, exp(-2 pi^2 l^2 |k|^2), then the
real part, normalised to zero mean and the requested standard deviation.  The
conductivity of a log-normal field is exp(g) at the quadrature points, g
interpolated bilinearly on the periodic grid.
"""
from __future__ import annotations

import numpy as np


def gaussian_random_field(n: int = 256, correlation_length: float = 0.1, std: float = 0.5,
                          seed: int = 0) -> np.ndarray:
    """An n x n sample (row = y, column = x) of the periodic Gaussian field."""
    if n < 2 or correlation_length <= 0.0 or std < 0.0:
        raise ValueError("n >= 2, correlation_length > 0, std >= 0")
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(n, d=1.0 / n)                       # wave numbers on the unit square
    k2 = k[None, :] ** 2 + k[:, None] ** 2
    amplitude = np.exp(-np.pi ** 2 * correlation_length ** 2 * k2)   # sqrt of exp(-2 pi^2 l^2 |k|^2)
    noise = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    g = np.real(np.fft.ifft2(amplitude * noise))
    g -= g.mean()
    s = g.std()
    return g * (std / s) if s > 0.0 else g


def sample_periodic(field: np.ndarray, xy: np.ndarray) -> np.ndarray:
    """Bilinear interpolation of a periodic grid field (cell-vertex values at
    (j / n, i / n)) at points xy[..., 2] of the unit square."""
    n = field.shape[0]
    x = np.asarray(xy[..., 0]) * n
    y = np.asarray(xy[..., 1]) * n
    i0 = np.floor(x).astype(np.int64)
    j0 = np.floor(y).astype(np.int64)
    fx, fy = x - i0, y - j0
    i0 %= n
    j0 %= n
    i1, j1 = (i0 + 1) % n, (j0 + 1) % n
    return ((1 - fx) * (1 - fy) * field[j0, i0] + fx * (1 - fy) * field[j0, i1] +
            (1 - fx) * fy * field[j1, i0] + fx * fy * field[j1, i1])


def lognormal_conductivity(quadrature_xy: np.ndarray, correlation_length: float = 0.1, std: float = 0.5,
                           seed: int = 0, grid: int = 256) -> np.ndarray:
    """exp(g) at the quadrature points [E][nq][2] (flattened to E * nq values)."""
    g = gaussian_random_field(grid, correlation_length, std, seed)
    return np.exp(sample_periodic(g, quadrature_xy)).reshape(-1)
