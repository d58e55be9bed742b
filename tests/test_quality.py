"""Image-quality figures on synthetic images with known answers (CPU)."""
import numpy as np
import pytest

from ustb_gb300 import quality
from ustb_gb300.uff import LinearScan


def flat(a):
    """[Nx, Nz] -> flat [P] in LinearScan order (z fastest)."""
    return np.asarray(a).reshape(-1)


def test_contrast_of_two_level_image():
    scan = LinearScan(np.linspace(-5e-3, 5e-3, 101), np.linspace(10e-3, 20e-3, 101))
    X, Z = np.meshgrid(scan.x_axis, scan.z_axis, indexing="ij")
    img = np.where(np.hypot(X, Z - 15e-3) < 2e-3, 0.1, 1.0)
    c = quality.cyst_contrast_db(flat(img), scan, 0.0, 15e-3, 1.6e-3, 2.5e-3, 4e-3)
    assert c == pytest.approx(-20.0, abs=1e-9)


def test_fwhm_of_gaussian_line():
    scan = LinearScan(np.linspace(-5e-3, 5e-3, 1001), np.linspace(10e-3, 20e-3, 11))
    X, Z = np.meshgrid(scan.x_axis, scan.z_axis, indexing="ij")
    sigma = 0.3e-3
    img = np.exp(-((X - 1e-3) ** 2) / (2 * sigma ** 2)) * np.exp(-((Z - 15e-3) ** 2) / 1e-6)
    # -6.0206 dB is amplitude 1/2: FWHM = 2 sqrt(2 ln 2) sigma; -6 dB is slightly narrower
    want = 2 * sigma * np.sqrt(2 * np.log(10 ** (6 / 20)))
    got = quality.lateral_fwhm(flat(img), scan, 1e-3, 15e-3)
    assert got == pytest.approx(want, rel=1e-3)


def test_isolated_points_rules():
    scan = LinearScan(np.linspace(-10e-3, 10e-3, 11), np.linspace(5e-3, 30e-3, 11))
    pts = np.array([[0, 0, 15e-3], [1e-3, 0, 15.5e-3], [-6e-3, 0, 25e-3], [9.5e-3, 0, 20e-3],
                    [5e-3, 0, 10e-3]])
    keep = quality.isolated_points(pts, scan, cysts=[(5e-3, 12e-3, 1e-3)])
    # 0 and 1 are too close, 3 is at the edge, 4 is next to the cyst
    assert keep.tolist() == [2]


def test_compare_identical_images():
    scan = LinearScan(np.linspace(-5e-3, 5e-3, 201), np.linspace(10e-3, 20e-3, 101))
    rng = np.random.default_rng(0)
    img = rng.rayleigh(size=(201, 101))
    r = quality.compare(flat(img), flat(img), scan, [(0.0, 15e-3, 2e-3)], np.zeros((0, 3)))
    assert r["rel_l2"] == 0 and r["max_contrast_diff_db"] == 0
