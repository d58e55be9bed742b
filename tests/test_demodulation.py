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


# ---- the reference's Python port: firwin + filtfilt + slicing ---------------
GOLDEN = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "python_demod.npz"))
CASES = ["default_dec", "explicit_dec", "no_dec", "int_like"]


def python_port_decimation(fs, fc, fds):
    return max(1, int(np.floor(fs / (4 * fc)))) if fds < 0 else max(1, int(np.floor(fs / fds)))


@pytest.mark.parametrize("name", CASES)
def test_zero_phase_oracle_matches_reference_python_port(name):
    """The oracle restatement against the output of python/src/ustb/preprocess/
    fast_demodulation.py itself (complex64, so agreement to its rounding)."""
    rf = GOLDEN[f"{name}/rf"]
    fs, t0, fc, fds = GOLDEN[f"{name}/params"]
    taps = preprocess.python_port_taps(fc, fs, rf.shape[0])
    assert np.allclose(taps, O.hamming_lowpass_taps(len(taps), 0.5 * fc, fs), rtol=0, atol=1e-15)
    D = python_port_decimation(fs, fc, fds)
    got = O.zero_phase_demodulation_f64(rf, fs, t0, fc, taps, D)
    want = GOLDEN[f"{name}/iq"][..., 0]
    assert got.shape == want.shape
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-7
    assert float(GOLDEN[f"{name}/fs_out"]) == fs / D
    assert float(GOLDEN[f"{name}/t0_out"]) == t0


def test_zero_phase_short_trace_raises_like_the_reference():
    assert int(GOLDEN["short/raises"]) == 1
    L = int(GOLDEN["short/L"])
    taps = preprocess.python_port_taps(4e6, 20e6, L)
    with pytest.raises(ValueError):
        O.zero_phase_demodulation_f64(np.ones((L, 1)), 20e6, 0.0, 4e6, taps, 1)


def test_python_port_taps_lengths():
    assert len(preprocess.python_port_taps(5e6, 40e6, 600)) == 65
    assert len(preprocess.python_port_taps(5e6, 40e6, 30)) == 19   # 2 (30 // 3) - 1
    assert len(preprocess.python_port_taps(5e6, 40e6, 4)) == 3     # at least 3
    assert len(preprocess.python_port_taps(5e6, 40e6, 7)) == 3     # 2 * 2 - 1
