"""Seeded smooth Gaussian random fields on structured cell grids (parameter
fields of the adjoint configuration): white noise filtered in Fourier space
with a Gaussian kernel of the given correlation length, scaled to the given
standard deviation."""
from __future__ import annotations

import numpy as np


def gaussian_random_field(shape, h: float, corr_length: float, std: float, seed: int,
                          mean: float = 0.0) -> np.ndarray:
    """Field on cells of spacing h (x fastest when flattened with order C of
    shape[::-1]); covariance exp(-r^2 / (2 l^2)) up to the periodic wrap."""
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(shape)
    k = np.meshgrid(*[np.fft.fftfreq(s, d=h) * 2.0 * np.pi for s in shape], indexing="ij")
    k2 = sum(x * x for x in k)
    f = np.real(np.fft.ifftn(np.fft.fftn(noise) * np.exp(-0.25 * k2 * corr_length ** 2)))
    f -= f.mean()
    f *= std / f.std()
    return f + mean
