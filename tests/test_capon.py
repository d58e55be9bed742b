"""Capon minimum-variance oracle on cases with known answers (CPU)."""
import numpy as np

from oracle import oracle as O
from ustb_gb300 import postprocess


def test_coherent_aperture_gives_uniform_weights():
    N, E, M = 9, 2, 8
    s = (1.5 - 0.5j)
    d = np.full((N, E, M), s)
    z = O.capon_f64(d, np.ones((N, E, M)), L_elements=4, K_samples=1, regCoef=1e-2)
    # w = 1/L, and the reference's w' * x' conjugates: z = M * conj(s)
    assert np.allclose(z, M * np.conj(s))


def test_too_few_active_elements_falls_back_to_the_sum():
    rng = np.random.default_rng(0)
    d = rng.standard_normal((5, 1, 6)) + 1j * rng.standard_normal((5, 1, 6))
    ap = np.zeros((5, 1, 6)); ap[..., 2] = 1  # one active element
    z = O.capon_f64(d, ap, L_elements=3, K_samples=1, regCoef=1e-2)
    assert np.allclose(z[:, 0], d[:, 0, :].sum(1))


def test_k_samples_is_odd():
    z = np.linspace(10e-3, 20e-3, 101)
    k = postprocess.capon_k_samples(z, 0.3e-3, 1.5)
    assert k % 2 == 1
