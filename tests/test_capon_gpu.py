"""Capon minimum variance on the GPU against the FP64 oracle of capon_minimum_variance.m."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from ustb_gb300 import postprocess

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def cube_case(rng, nz=36, nx=7, M=24):
    """Speckle-like channel data with a plane-wave component and a partial aperture."""
    d = (rng.standard_normal((nz, nx, M)) + 1j * rng.standard_normal((nz, nx, M))) * 0.3
    d += np.exp(1j * 0.2 * np.arange(M))[None, None, :] * rng.standard_normal((nz, nx, 1))
    ap = np.ones((nz, nx, M))
    for iz in range(nz):  # aperture grows with depth, as an F-number would
        half = 4 + iz // 4
        c = M // 2
        ap[iz, :, :max(0, c - half)] = 0
        ap[iz, :, c + half:] = 0
    return d, ap


def run_gpu(d, ap, dev, **kw):
    nz, nx, M = d.shape
    # ABI cube (F, W=1, N=M, P) with P = iz + nz * ix
    cube = torch.from_numpy(np.ascontiguousarray(d.transpose(2, 1, 0).reshape(1, 1, M, nz * nx)).astype(np.complex64))
    apod = torch.from_numpy(np.ascontiguousarray(ap.transpose(2, 1, 0).reshape(M, nz * nx)).astype(np.float32))
    out = postprocess.capon_minimum_variance(cube.to(dev), apod.to(dev), nz, nx, **kw)
    return out[0].cpu().numpy().reshape(nx, nz).T


@pytest.mark.parametrize("fb", [False, True])
@pytest.mark.parametrize("L, K", [(12, 3), (8, 1), (20, 0)])
def test_capon_vs_oracle(cuda_dev, fb, L, K):
    rng = np.random.default_rng(L * 10 + K)
    d, ap = cube_case(rng)
    got = run_gpu(d, ap, cuda_dev, L_elements=L, K_samples=K, regCoef=1e-2, doForwardBackward=fb)
    want = O.capon_f64(d, ap, L, K, 1e-2, fb=fb)
    assert rel(got, want) <= 1e-3


def test_capon_fallbacks(cuda_dev):
    rng = np.random.default_rng(9)
    d, ap = cube_case(rng, nz=12, nx=3, M=16)
    d[3] = 0                      # an all-zero row -> 0
    ap[5, :, :] = 0
    ap[5, :, 7] = 1               # one active element -> plain sum
    got = run_gpu(d, ap, cuda_dev, L_elements=8, K_samples=1, regCoef=1e-2)
    want = O.capon_f64(d, ap, 8, 1, 1e-2)
    assert np.all(got[3] == 0)
    assert np.allclose(got[5], d[5].sum(-1), rtol=1e-5)
    assert rel(got, want) <= 1e-3
