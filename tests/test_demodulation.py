"""RF -> IQ demodulation: filter design and the FP64 oracle (CPU)."""
import math

import numpy as np
import pytest
from scipy.signal import freqz

from oracle import oracle as O
from ustb_gb300 import preprocess


def test_kaiser_lowpass_order_follows_kaiser_formulas():
    n, Wn, beta = preprocess.kaiser_lowpass_order(2.5e6, 5e6, 20e6)
    # A = 60 dB: beta = 0.1102 (A - 8.7); n = ceil((A - 7.95) / (2.285 * 2 pi df / fs))
    assert beta == pytest.approx(0.1102 * (60 - 8.7))
    assert n == math.ceil((60 - 7.95) / (2.285 * 2 * math.pi * 2.5e6 / 20e6))
    assert Wn == pytest.approx(7.5e6 / 20e6)


def test_lowpass_taps_pass_and_stop_bands():
    fs, fc = 20e6, 5e6
    b = preprocess.lowpass_taps(fc, fs)
    assert np.allclose(b, b[::-1])  # linear phase
    w, h = freqz(b, worN=4096, fs=fs)
    g = np.abs(h)
    assert np.all(np.abs(g[w <= 0.5 * fc] - 1) < 2e-3)       # pass band, 1e-3 ripple
    assert np.all(20 * np.log10(g[w >= fc] + 1e-30) < -55)   # stop band


def test_decimation_factor_rounds_like_the_reference():
    assert preprocess.decimation_factor(20e6, 10e6) == (2, 10e6)
    D, fs = preprocess.decimation_factor(20e6, 7e6)  # not a divisor: next higher rate
    assert D == 2 and fs == 10e6


def test_oracle_matches_direct_sum():
    rng = np.random.default_rng(0)
    rf = rng.standard_normal((101, 3))
    b = rng.standard_normal(7)
    fs, t0, fc, D = 20e6, 1.3e-6, 5e6, 3
    got = O.fast_demodulation_f64(rf, fs, t0, fc, b, D)
    t = t0 + np.arange(101) / fs
    mix = rf * np.exp(-2j * np.pi * fc * t)[:, None]
    want = np.zeros((math.ceil(101 / D), 3), complex)
    for mi, m in enumerate(range(0, 101, D)):
        for k in range(7):
            if m - k >= 0:
                want[mi] += b[k] * mix[m - k]
    assert np.allclose(got, want, rtol=1e-12, atol=1e-12)
