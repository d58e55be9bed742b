"""Depth-direction FIR of the sDMAS band-pass (ustb_fir_depth) against numpy:
out[z] = sum_k b[k] y[z + d - k], y = 0 outside the column
(+postprocess/simplified_delay_multiply_and_sum.m:170-176)."""
import numpy as np
import pytest
import torch

from ustb_gb300 import postprocess

pytestmark = pytest.mark.gpu


def fir_ref(y, b, d):
    nz = y.shape[-1]
    pad = np.concatenate([y.astype(np.float64), np.zeros(y.shape[:-1] + (d,))], axis=-1)
    full = np.apply_along_axis(lambda v: np.convolve(v, b.astype(np.float64))[:nz + d], -1, pad)
    return full[..., d:d + nz]


@pytest.mark.parametrize("nz, ncols, ntaps, delay", [
    (512, 300, 61, None),    # one CTA per column
    (5000, 7, 350, None),    # several runs per column, long filter
    (100, 5, 257, None),     # filter longer than the column
    (333, 9, 12, 0),         # no delay compensation
    (64, 3, 1, 0),           # a single tap
    (4097, 2, 1024, 900),    # the largest filter, uneven delay
])
def test_fir_depth_matches_numpy(cuda_dev, nz, ncols, ntaps, delay):
    rng = np.random.default_rng(nz + ntaps)
    y = rng.standard_normal((ncols, nz)).astype(np.float32)
    b = rng.standard_normal(ntaps).astype(np.float32) / np.sqrt(ntaps)
    got = postprocess.fir_depth(torch.from_numpy(y).to(cuda_dev), b, delay).cpu().numpy()
    d = int(round((ntaps - 1) / 2)) if delay is None else delay
    want = fir_ref(y, b, d)
    assert np.abs(got - want).max() <= 1e-5 * max(1.0, np.abs(want).max())
