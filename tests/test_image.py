"""Image formation: oracle scan conversion and get_image reshaping (CPU)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from ustb_gb300 import image
from ustb_gb300.uff import BeamformedData, LinearScan, SectorScan


def test_scan_convert_oracle_reproduces_a_linear_field():
    depth = np.linspace(5e-3, 60e-3, 200)
    az = np.deg2rad(np.linspace(-40, 40, 128))
    R, T = np.meshgrid(depth, az, indexing="ij")
    field = 3.0 * R + 2.0 * T + 2.0  # positive, bilinear in (r, theta): interpolated exactly
    xs = np.linspace(-30e-3, 30e-3, 64)
    zs = np.linspace(0, 60e-3, 48)
    out = O.scan_convert_f64(field, depth, az, xs, zs, compression="abs")[0]
    X, Z = np.meshgrid(xs, zs)
    r, th = np.hypot(X, Z), np.arctan2(X, Z)
    inside = (r >= depth[0]) & (r <= depth[-1]) & (np.abs(th) <= np.deg2rad(40))
    assert np.allclose(out[inside], (3.0 * r + 2.0 * th + 2.0)[inside], atol=1e-9)
    assert np.all(np.isneginf(out[~inside]))


def test_get_image_reshapes_like_matlab():
    scan = LinearScan(np.linspace(-1e-3, 1e-3, 3), np.linspace(1e-3, 4e-3, 4))  # Nz = 4, Nx = 3
    data = torch.arange(12, dtype=torch.float32).reshape(12, 1, 1, 1) + 1
    img = image.get_image(BeamformedData(scan, data), "abs")
    assert tuple(img.shape) == (4, 3, 1, 1)
    # MATLAB reshape: pixel p = iz + Nz * ix
    assert img[2, 1, 0, 0].item() == 1 + (2 + 4 * 1)
    lg = image.get_image(BeamformedData(scan, data), "log")
    assert lg.max().item() == pytest.approx(0.0)


def test_cartesian_grid_spans_the_sector():
    s = SectorScan(np.deg2rad(np.linspace(-30, 30, 11)), np.linspace(10e-3, 50e-3, 21))
    xs, zs = image.cartesian_grid(s, 32, 16)
    assert xs[0] == pytest.approx(-50e-3 * np.sin(np.deg2rad(30)))
    assert zs[0] == pytest.approx(10e-3 * np.cos(np.deg2rad(30)))
    assert zs[-1] == pytest.approx(50e-3)
