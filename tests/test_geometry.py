"""Host geometry precompute (delays, apodization) against the reference.

* delays against the reference Python package's DAS on the same geometry
  (tests/golden/python_das.npz): plane, diverging and focused (hybrid) waves;
* the known answers of python/tests/test_das.py:145-187 (on-axis receive delay
  z/c, photoacoustic transmit delay 0, 0-degree plane wave z/c);
* window values and aperture clamps of +uff/apodization.m:172-223, 452-462.
"""
import math
import os

import numpy as np
import pytest

from ustb_gb300 import geometry
from ustb_gb300.enums import SphericalTransmitDelayModel as STDM
from ustb_gb300.enums import Wavefront, Window
from ustb_gb300.geometry import Apodization
from ustb_gb300.uff import LinearScan, Point, Probe, Scan, SectorScan, Wave


def _golden(golden_dir):
    return np.load(os.path.join(golden_dir, "python_das.npz"))


def _waves(z, name):
    seq = []
    for x, y, zz, az, el, d in z[f"{name}/src"]:
        if name == "plane":
            seq.append(Wave.plane(az))
        else:
            seq.append(Wave(Wavefront.spherical, Point.from_xyz(x, y, zz)))
    return seq


@pytest.mark.parametrize("name", ["plane", "diverging", "focused"])
def test_delays_match_reference_python_das(golden_dir, name):
    z = _golden(golden_dir)
    probe = Probe(z["probe_x"])
    # the golden grid is x-fastest (numpy meshgrid); a LinearScan is z-fastest
    xs, zs = np.unique(z["scan_x"]), np.unique(z["scan_z"])
    scan = LinearScan(xs, zs)
    order = np.array([np.flatnonzero((z["scan_x"] == x) & (z["scan_z"] == zz))[0]
                      for x, zz in zip(scan.x, scan.z)])
    rx = geometry.receive_delay(probe, scan, float(z["c"])).astype(np.float32)
    tx = geometry.transmit_delay(_waves(z, name), scan, STDM.hybrid, 1e-3).astype(np.float32)
    # the reference casts the double result to float32, as this code does
    np.testing.assert_allclose(rx, z[f"{name}/rx_delay"][order], rtol=1e-6, atol=0)
    ref_tx = z[f"{name}/tx_delay"][order]
    if name == "focused":
        # the Python package's hybrid model uses a plane delay from the source
        # angles (das.py:187-198); das.m uses |z - zf| + distance for linear scans
        # (das.m:159-160) — only pixels outside the focal margin are comparable
        keep = np.abs(scan.z - 10e-3) >= 1e-3
        np.testing.assert_allclose(tx[keep], ref_tx[keep], rtol=1e-6, atol=1e-12)
    else:
        np.testing.assert_allclose(tx, ref_tx, rtol=1e-6, atol=1e-12)


def test_known_answers_from_reference_tests():
    probe = Probe(np.zeros(1))
    scan = Scan([0.0], [0.0], [30e-3])
    rx = geometry.receive_delay(probe, scan, 1540.0)
    assert rx[0, 0] == pytest.approx(30e-3 / 1540.0, rel=1e-4)
    pa = Wave(Wavefront.photoacoustic, Point())
    assert geometry.transmit_delay([pa], Scan([0.0], [0.0], [20e-3]))[0, 0] == 0.0
    pw = Wave.plane(0.0)
    assert geometry.transmit_delay([pw], Scan([0.0], [0.0], [20e-3]))[0, 0] == pytest.approx(
        20e-3 / 1540.0, rel=1e-5)


def test_wave_delay_and_sound_speed():
    w = Wave.plane(0.0, c=1500.0, delay=1e-6)
    td = geometry.transmit_delay([w], Scan([0.0], [0.0], [15e-3]))
    assert td[0, 0] == pytest.approx(15e-3 / 1500.0 - 1e-6)


def test_diverging_wave_delay():
    src = Point(-10e-3, 0.3, 0.0)  # negative distance flips the point behind the array
    assert src.z < 0
    w = Wave(Wavefront.spherical, src)
    scan = Scan([0.0, 5e-3], [0.0, 0.0], [20e-3, 30e-3])
    td = geometry.transmit_delay([w], scan) * 1540.0
    d = np.sqrt((scan.x - src.x) ** 2 + (scan.z - src.z) ** 2) - 10e-3
    np.testing.assert_allclose(td[:, 0], d, rtol=1e-12)


def test_point_getters():
    p = Point(10e-3, math.pi / 2, 0.0)
    assert p.z == 0.0 and p.x == pytest.approx(10e-3)
    q = Point.from_xyz(3e-3, 0.0, 4e-3)
    assert q.distance == pytest.approx(5e-3) and q.x == pytest.approx(3e-3) and q.z == pytest.approx(4e-3)


def test_tukey_window_values():
    r = np.array([0.0, 0.3, 0.375, 0.4, 0.45, 0.5, 0.6])
    v = geometry._tukey(r, 0.25)
    assert v[0] == 1 and v[1] == 1 and v[2] == 1
    assert 0 < v[3] < 1 and v[4] < v[3]
    assert v[5] == 0 and v[6] == 0
    assert v[3] == pytest.approx(0.5 * (1 + math.cos(2 * math.pi / 0.25 * (0.4 - 0.125 - 0.5))))


@pytest.mark.parametrize("win", [Window.boxcar, Window.hanning, Window.hamming, Window.tukey25,
                                 Window.tukey50, Window.tukey75, Window.triangle])
def test_windows_vanish_beyond_half(win):
    r = np.array([0.0, 0.51, 1.0])
    v = geometry.apply_window(win, r, np.zeros_like(r))
    assert v[0] == pytest.approx(1.0) and v[1] == 0 and v[2] == 0


def test_receive_apodization_expanding_aperture():
    probe = Probe.linear_array(64, 0.3e-3)
    scan = LinearScan([0.0], [5e-3, 20e-3])
    apo = Apodization(window=Window.boxcar, f_number=1.7)
    a = apo.aperture_apodization(probe, scan)
    width = a.sum(axis=1) * 0.3e-3
    # aperture ~ z / F#
    assert width[0] == pytest.approx(5e-3 / 1.7, abs=0.61e-3)
    assert width[1] == pytest.approx(20e-3 / 1.7, abs=0.61e-3)


def test_minimum_aperture_clamp():
    probe = Probe.linear_array(16, 0.3e-3)
    scan = LinearScan([0.0], [0.1e-3])
    apo = Apodization(window=Window.boxcar, f_number=1.0, minimum_aperture=(2e-3, 2e-3))
    a = apo.aperture_apodization(probe, scan)
    # |x| <= 1 mm pass once z is clamped to the 2 mm minimum aperture
    assert a.sum() == np.sum(np.abs(probe.x) / 2e-3 <= 0.5)


def test_transmit_apodization_plane_waves_constant_per_wave():
    seq = [Wave.plane(a) for a in np.deg2rad([-16, 0, 16])]
    scan = LinearScan(np.linspace(-5e-3, 5e-3, 4), np.linspace(5e-3, 10e-3, 3))
    apo = Apodization(window=Window.tukey25, f_number=1.7)
    a = apo.wave_apodization(seq, scan)
    assert a.shape == (12, 3)
    assert np.all(a[:, 1] == 1.0)
    r = 1.7 * abs(math.tan(math.radians(16)))
    assert np.allclose(a[:, 0], geometry._tukey(np.array([r]), 0.25)[0])


def test_sector_scan_geometry_and_reference_distance():
    s = SectorScan(np.deg2rad([-30, 0, 30]), [10e-3, 20e-3])
    assert s.N_pixels == 6
    np.testing.assert_allclose(np.hypot(s.x, s.z), s.reference_distance)
    assert s.x[0] == pytest.approx(-10e-3 * 0.5)


def test_linear_scan_order_is_z_fastest():
    s = LinearScan([1.0, 2.0], [10.0, 20.0, 30.0])
    np.testing.assert_array_equal(s.z, [10, 20, 30, 10, 20, 30])
    np.testing.assert_array_equal(s.x, [1, 1, 1, 2, 2, 2])


def test_sta_apodization_picks_nearest_element():
    probe = Probe.linear_array(8, 1e-3)
    apo = Apodization(window=Window.sta, origin=Point.from_xyz(probe.x[5] + 1e-4, 0, 0))
    a = apo.aperture_apodization(probe, Scan([0, 1], [0, 0], [1, 2]))
    assert a.shape == (2, 8) and a[:, 5].tolist() == [1, 1] and a.sum() == 2


def test_scanline_apodization_selects_one_wave_per_line():
    scan = LinearScan(np.linspace(-1, 1, 4), [1.0, 2.0])
    seq = [Wave.plane(0.0) for _ in range(4)]
    a = Apodization(window=Window.scanline).wave_apodization(seq, scan)
    assert a.shape == (8, 4)
    np.testing.assert_array_equal(a.sum(axis=1), np.ones(8))
    np.testing.assert_array_equal(np.argmax(a, axis=1), [0, 0, 1, 1, 2, 2, 3, 3])


def test_unified_model_runs_and_matches_spherical_inside_mask():
    probe = Probe.linear_array(32, 0.3e-3)
    scan = LinearScan(np.linspace(-4e-3, 4e-3, 17), np.linspace(5e-3, 30e-3, 26))
    seq = [Wave(Wavefront.spherical, Point.from_xyz(xf, 0, 20e-3)) for xf in (-1e-3, 0.0, 1e-3)]
    tu = geometry.transmit_delay(seq, scan, STDM.unified, unified_f_number=(2.0, 2.0))
    ts = geometry.transmit_delay(seq, scan, STDM.spherical)
    assert tu.shape == ts.shape and np.all(np.isfinite(tu))
    mask = geometry._unified_mask(seq, scan, (2.0, 2.0))[:, :, 1].ravel(order="F") != 0
    mask[scan.z == scan.z.max()] = False
    np.testing.assert_allclose(tu[mask, 1], ts[mask, 1], rtol=1e-12)
