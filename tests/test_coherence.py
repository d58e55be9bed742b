"""Coherence-factor oracles on cases with known answers (CPU)."""
import numpy as np

from oracle import oracle as O


def test_pcf_of_aligned_phases_is_one():
    d = np.exp(1j * 0.3) * np.arange(1, 9)[None, :]
    fca, fcc, img = O.phase_coherence_factor_f64(d)
    assert np.allclose(fca, 1) and np.allclose(fcc, 1) and np.allclose(img, d.sum(1))


def test_gcf_of_a_constant_aperture_is_one_and_of_an_impulse_is_the_bin_share():
    K = 16
    g, _ = O.generalized_coherence_factor_f64(np.ones((1, K)), M0=4)
    assert np.allclose(g, 1)
    imp = np.zeros((1, K)); imp[0, 3] = 1  # flat spectrum: 9 of 16 bins
    g, _ = O.generalized_coherence_factor_f64(imp, M0=4)
    assert np.allclose(g, 9 / 16)
    g, _ = O.generalized_coherence_factor_f64(imp, M0=1)  # DC only
    assert np.allclose(g, 1 / 16)
