"""Fast path (reduced-precision storage, on-the-fly geometry) against the FP64 oracle.

The oracle gets double-precision tables built by the host geometry code (the
das.m formulas) and the unquantised channel data; the bar is relative L2
<= 1e-3 for FP16 storage (the target of the fast path) and tighter for FP32.
"""
import math

import numpy as np
import pytest
import torch

from oracle import oracle as O
from ustb_gb300 import _lib, fast, geometry
from ustb_gb300.enums import Dimension, Precision, Window
from ustb_gb300.geometry import Apodization
from ustb_gb300.uff import LinearScan, Point, Probe, SectorScan, Wave

pytestmark = pytest.mark.gpu

TOL = {Precision.fp32: 2e-4, Precision.fp16: 1e-3, Precision.bf16: 6e-3}


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def speckle(rng, shape, cplx=True):
    if cplx:
        return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    return rng.standard_normal(shape).astype(np.float32)


def smooth(x):
    """Band-limit along time so that linear interpolation is meaningful."""
    k = np.array([1, 4, 6, 4, 1], np.float32) / 16
    return np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), 0, x).astype(x.dtype)


def oracle_f64(ch, fs, t0, fd, c, probe, scan, seq, dim, rx, tx, model=None):
    txa = tx.wave_apodization(seq, scan)
    rxa = rx.aperture_apodization(probe, scan)
    txd = geometry.transmit_delay(seq, scan) if model is None else geometry.transmit_delay(seq, scan, model)
    rxd = geometry.receive_delay(probe, scan, c)
    out = O.das_f64(ch.astype(np.complex128), fs, t0, txa, rxa, txd, rxd, fd, dim)
    if abs(fd) > 0:
        ph = np.exp(-1j * 2 * (2 * np.pi * fd) * scan.reference_distance / c)
        out = out * ph.reshape((-1,) + (1,) * (out.ndim - 1))
    return out, rxa


def run_fast(ch, prec, geom, dim, F=1, epilogue=False, cube=True):
    dev = geom.device
    L, N, W = ch.shape[:3]
    cplx = np.iscomplexobj(ch)
    abi = np.ascontiguousarray(ch.reshape(L, N, W, F, order="F").transpose(3, 2, 1, 0))
    t = torch.from_numpy(abi).to(dev)
    st = fast.convert_channels(t, prec)
    outs = fast.das_fast(st, prec, cplx, geom, dim, F=F, epilogue=epilogue, cube=cube, L=L)
    torch.cuda.synchronize()
    res = {}
    for k, v in outs.items():
        if k == "flags":
            continue
        a = v.cpu().numpy()
        res[k] = a.transpose(3, 2, 1, 0) if k == "cube" else a.T
    return res


def linear_setup(rng, N=32, W=5, L=512, nx=40, nz=48, F=1, cplx=True):
    probe = Probe.linear_array(N, 0.3e-3)
    fs, f0 = 20e6, 5e6
    seq = [Wave.plane(a) for a in np.deg2rad(np.linspace(-12, 12, W))]
    scan = LinearScan(np.linspace(-4e-3, 4e-3, nx), np.linspace(6e-3, 16e-3, nz))
    ch = smooth(speckle(rng, (L, N, W, F), cplx))
    return probe, scan, seq, fs, f0, ch


@pytest.mark.parametrize("prec", [Precision.fp32, Precision.fp16, Precision.bf16])
@pytest.mark.parametrize("dim", [Dimension.both, Dimension.receive, Dimension.transmit, Dimension.none])
def test_plane_wave_iq_vs_fp64_oracle(cuda_dev, prec, dim):
    rng = np.random.default_rng(3)
    probe, scan, seq, fs, f0, ch = linear_setup(rng)
    t0, c = 2e-6, 1540.0
    rx = Apodization(window=Window.tukey25, f_number=1.7)
    tx = Apodization(window=Window.tukey25, f_number=1.7)
    ref, _ = oracle_f64(ch, fs, t0, f0, c, probe, scan, seq, int(dim), rx, tx)
    ph = np.exp(-1j * 2 * (2 * np.pi * f0) * scan.reference_distance / c)
    g = fast.FastGeometry(probe, scan, seq, fs, t0, f0, c, cuda_dev, rx, tx, pixel_phase=ph)
    out = run_fast(ch, prec, g, dim)["cube"]
    assert out.shape == ref.shape
    assert rel_l2(out, ref) <= TOL[prec]


def test_fp16_storage_error_budget(cuda_dev):
    """FP16 storage error is dominated by the sample quantisation (~3e-4 rel)."""
    rng = np.random.default_rng(4)
    probe, scan, seq, fs, f0, ch = linear_setup(rng, W=7)
    rx = Apodization(window=Window.hanning, f_number=1.5)
    ref, _ = oracle_f64(ch, fs, 1e-6, f0, 1540.0, probe, scan, seq, 3, rx, Apodization())
    ph = np.exp(-1j * 4 * np.pi * f0 * scan.reference_distance / 1540.0)
    g = fast.FastGeometry(probe, scan, seq, fs, 1e-6, f0, 1540.0, cuda_dev, rx, None, pixel_phase=ph)
    e32 = rel_l2(run_fast(ch, Precision.fp32, g, 3)["cube"], ref)
    e16 = rel_l2(run_fast(ch, Precision.fp16, g, 3)["cube"], ref)
    assert e32 < 1e-4 and e16 < 1e-3 and e32 < e16


@pytest.mark.parametrize("dim", [Dimension.both, Dimension.transmit])
def test_rf_real_path(cuda_dev, dim):
    rng = np.random.default_rng(5)
    probe, scan, seq, fs, f0, ch = linear_setup(rng, W=1, cplx=False)
    rx = Apodization(window=Window.tukey25, f_number=1.7)
    ref, _ = oracle_f64(ch.astype(np.complex64), fs, 0.0, 0.0, 1540.0, probe, scan, seq, int(dim), rx,
                        Apodization())
    g = fast.FastGeometry(probe, scan, seq, fs, 0.0, 0.0, 1540.0, cuda_dev, rx, None)
    out = run_fast(ch, Precision.fp32, g, dim)["cube"]
    assert out.dtype == np.float32
    assert rel_l2(out, ref.real) <= 1e-4


def test_multiple_frames(cuda_dev):
    rng = np.random.default_rng(6)
    F = 3
    probe, scan, seq, fs, f0, ch = linear_setup(rng, F=F, W=3)
    rx = Apodization(window=Window.tukey50, f_number=1.2)
    ref, _ = oracle_f64(ch, fs, 1e-6, f0, 1540.0, probe, scan, seq, 3, rx, Apodization())
    ph = np.exp(-1j * 4 * np.pi * f0 * scan.reference_distance / 1540.0)
    g = fast.FastGeometry(probe, scan, seq, fs, 1e-6, f0, 1540.0, cuda_dev, rx, None, pixel_phase=ph)
    out = run_fast(ch, Precision.fp16, g, 3, F=F)["cube"]
    assert out.shape == (scan.N_pixels, 1, 1, F)
    assert rel_l2(out, ref) <= 1e-3


def sector_setup(rng, N=24, W=5, L=768, F=1):
    probe = Probe.linear_array(N, 0.22e-3)
    fs, f0 = 12e6, 3e6
    seq = [Wave(source=Point(-10e-3, a, 0.0)) for a in np.deg2rad(np.linspace(-30, 30, W))]
    scan = SectorScan(np.deg2rad(np.linspace(-40, 40, 33)), np.linspace(5e-3, 40e-3, 64))
    ch = smooth(speckle(rng, (L, N, W, F)))
    return probe, scan, seq, fs, f0, ch


def test_diverging_sector_transmit_with_epilogue(cuda_dev):
    rng = np.random.default_rng(7)
    probe, scan, seq, fs, f0, ch = sector_setup(rng)
    assert all(w.source.z < 0 for w in seq)
    c, t0 = 1540.0, 0.0
    rx = Apodization(window=Window.boxcar, f_number=1.0)
    ref, rxa = oracle_f64(ch, fs, t0, f0, c, probe, scan, seq, 2, rx, Apodization())
    ph = np.exp(-1j * 4 * np.pi * f0 * scan.reference_distance / c)
    g = fast.FastGeometry(probe, scan, seq, fs, t0, f0, c, cuda_dev, rx, None, pixel_phase=ph)
    r = run_fast(ch, Precision.fp16, g, Dimension.transmit, epilogue=True)
    assert rel_l2(r["cube"], ref) <= 1e-3
    cf_ref, img_ref = O.coherence_factor(ref[:, :, 0, :], (rxa > 0.16).sum(axis=1))
    das_ref = ref[:, :, 0, :].sum(axis=1)
    assert rel_l2(r["das"], das_ref) <= 1e-3
    assert rel_l2(r["cf"], cf_ref[:, 0, :]) <= 2e-3
    assert rel_l2(r["cf_image"], img_ref[:, 0, :]) <= 2e-3
    sd_ref = O.sdmas_value(ref[:, :, 0, :].real)[:, 0, :]
    assert rel_l2(r["sdmas"], sd_ref) <= 3e-3
    # epilogue without the channel cube gives the same numbers
    r2 = run_fast(ch, Precision.fp16, g, Dimension.transmit, epilogue=True, cube=False)
    assert np.array_equal(r2["cf"], r["cf"])


def test_sta_spherical_waves_and_hybrid_table(cuda_dev):
    """Single-element transmits (sources on the array, the hybrid model) — no pixel
    lies in the focal margin, so the kernel uses the spherical formula; a focused
    sequence with pixels in the margin falls back to a delay table."""
    rng = np.random.default_rng(8)
    N, L = 16, 640
    probe = Probe.linear_array(N, 0.3e-3)
    fs, f0, c = 20e6, 5e6, 1540.0
    seq = [Wave(source=Point.from_xyz(x, 0, 0), delay=abs(x) / c) for x in probe.x[::3]]
    scan = LinearScan(np.linspace(-3e-3, 3e-3, 24), np.linspace(5e-3, 14e-3, 40))
    ch = smooth(speckle(rng, (L, N, len(seq), 1)))
    rx = Apodization(window=Window.boxcar, f_number=1.0)
    ref, _ = oracle_f64(ch, fs, 0.0, f0, c, probe, scan, seq, 3, rx, Apodization())
    ph = np.exp(-1j * 4 * np.pi * f0 * scan.reference_distance / c)
    g = fast.FastGeometry(probe, scan, seq, fs, 0.0, f0, c, cuda_dev, rx, None, pixel_phase=ph)
    assert g.d_txdelay is None
    assert rel_l2(run_fast(ch, Precision.fp32, g, 3)["cube"], ref) <= 2e-4
    foc = [Wave(source=Point.from_xyz(x, 0, 9e-3)) for x in (-1e-3, 0.0, 1e-3)]
    ch2 = smooth(speckle(rng, (L, N, 3, 1)))
    ref2, _ = oracle_f64(ch2, fs, 0.0, f0, c, probe, scan, foc, 3, rx, Apodization())
    g2 = fast.FastGeometry(probe, scan, foc, fs, 0.0, f0, c, cuda_dev, rx, None, pixel_phase=ph)
    assert g2.d_txdelay is not None
    assert rel_l2(run_fast(ch2, Precision.fp32, g2, 3)["cube"], ref2) <= 2e-4


def test_rx_table_fallback_sta_window(cuda_dev):
    rng = np.random.default_rng(9)
    probe, scan, seq, fs, f0, ch = linear_setup(rng, W=2)
    rx = Apodization(window=Window.sta, origin=Point.from_xyz(probe.x[10], 0, 0))
    ref, _ = oracle_f64(ch, fs, 1e-6, f0, 1540.0, probe, scan, seq, 3, rx, Apodization())
    ph = np.exp(-1j * 4 * np.pi * f0 * scan.reference_distance / 1540.0)
    g = fast.FastGeometry(probe, scan, seq, fs, 1e-6, f0, 1540.0, cuda_dev, rx, None, pixel_phase=ph)
    assert g.d_rxapo is not None
    assert rel_l2(run_fast(ch, Precision.fp32, g, 3)["cube"], ref) <= 2e-4


def test_window_overflow_is_flagged_not_faulted(cuda_dev):
    rng = np.random.default_rng(10)
    probe, scan, seq, fs, f0, ch = linear_setup(rng, W=2)
    # one tile spanning the whole scan: far too long a window
    P = scan.N_pixels
    T = fast.TILE
    tiles = np.full(((P + T - 1) // T, T), -1, np.int32)
    order = np.random.default_rng(0).permutation(P)
    tiles.ravel()[:P] = order
    g = fast.FastGeometry(probe, scan, seq, fs, 1e-6, f0, 1540.0, cuda_dev, Apodization(), None, tiles=tiles)
    with pytest.raises(_lib.UstbError) as e:
        run_fast(ch, Precision.fp16, g, 3)
    assert e.value.code == 7
    # malformed tile maps are refused on the host
    with pytest.raises(ValueError):
        fast.FastGeometry(probe, scan, seq, fs, 1e-6, f0, 1540.0, cuda_dev, Apodization(), None,
                          tiles=np.zeros((1, 256), np.int32))
    # the device is still healthy afterwards
    g_ok = fast.FastGeometry(probe, scan, seq, fs, 1e-6, f0, 1540.0, cuda_dev, Apodization(), None)
    run_fast(ch, Precision.fp16, g_ok, 3)


def test_convert_int16_and_bf16(cuda_dev):
    x = torch.arange(-300, 300, dtype=torch.int16, device=cuda_dev)
    y = fast.convert_channels(x, Precision.fp16, scale=0.5)
    assert torch.equal(y.float().cpu(), (x.float() * 0.5).cpu())
    z = torch.randn(1000, dtype=torch.complex64, device=cuda_dev)
    b = fast.convert_channels(z, Precision.bf16)
    assert b.shape == (1000, 2) and b.dtype == torch.bfloat16
    assert torch.allclose(b.float().cpu(), torch.view_as_real(z).cpu(), rtol=1e-2, atol=1e-2)


def test_tile_planner_bounds_the_window():
    scan = SectorScan(np.deg2rad(np.linspace(-40, 40, 256)), np.linspace(5e-3, 90e-3, 512))
    tiles = fast.plan_tiles(scan, 12e6, 1540.0)
    live = tiles >= 0
    assert np.array_equal(np.sort(tiles[live]), np.arange(scan.N_pixels))
    assert np.all(tiles[:, 0] >= 0)
    lim = fast.SPAN_LIMIT * 1540.0 / 12e6
    for t in tiles[:: max(1, len(tiles) // 200)]:
        xyz = scan.xyz[t[t >= 0]]
        assert np.linalg.norm(xyz.max(0) - xyz.min(0)) <= lim + 1e-12
    # most lanes are busy
    assert live.mean() > 0.6


def test_sdmas_bandpass_and_hilbert_follow_up(cuda_dev):
    """The fused per-pixel sDMAS value, band-passed along depth around 2*f0 and made
    analytic (simplified_delay_multiply_and_sum.m:151-192), against the FP64 chain."""
    from ustb_gb300 import postprocess

    rng = np.random.default_rng(11)
    N, L, W = 24, 768, 3
    probe = Probe.linear_array(N, 0.3e-3)
    fs, f0, c = 20e6, 5e6, 1540.0
    seq = [Wave.plane(a) for a in np.deg2rad([-5.0, 0.0, 5.0])]
    nz, nx = 160, 24
    z = np.linspace(6e-3, 12e-3, nz)
    scan = LinearScan(np.linspace(-2e-3, 2e-3, nx), z)
    ch = smooth(speckle(rng, (L, N, W, 1)))
    rx = Apodization(window=Window.boxcar, f_number=1.0)
    ref, _ = oracle_f64(ch, fs, 0.0, f0, c, probe, scan, seq, 2, rx, Apodization())
    ph = np.exp(-1j * 4 * np.pi * f0 * scan.reference_distance / c)
    g = fast.FastGeometry(probe, scan, seq, fs, 0.0, f0, c, cuda_dev, rx, None, pixel_phase=ph)
    dev_ch = torch.from_numpy(np.ascontiguousarray(ch.transpose(3, 2, 1, 0))).to(cuda_dev)
    st = fast.convert_channels(dev_ch, Precision.fp32)
    outs = fast.das_fast(st, Precision.fp32, True, g, Dimension.transmit, epilogue=True, cube=False, L=L)
    dz = float(np.mean(np.diff(z)))
    img = postprocess.simplified_dmas_image(outs["sdmas"], nz, nx, dz, c, f0=f0 / 4)
    taps = postprocess.bandpass_taps([1.5 * f0 / 4, 1.5 * f0 / 4 + f0 / 16, 2.5 * f0 / 4, 2.5 * f0 / 4 + f0 / 16],
                                     c / dz / 2)
    sd = O.sdmas_value(ref[:, :, 0, :].real)[:, 0, 0].reshape(nx, nz).T
    want = O.sdmas_filtered(sd, taps).T.reshape(-1)
    got = img.cpu().numpy()[0]
    assert rel_l2(got, want) <= 2e-3


def test_kaiser_design_matches_kaiser_formulas():
    from ustb_gb300.postprocess import bandpass_taps, kaiser_order

    n, Wn, beta = kaiser_order([7.5e6, 8.75e6, 12.5e6, 13.75e6], [1e-3] * 3, 1540 / 0.02e-3 / 2)
    assert beta == pytest.approx(0.1102 * (60 - 8.7))
    assert n == math.ceil((60 - 7.95) / (2 * math.pi * 2.285 * (1.25e6 / (1540 / 0.02e-3 / 2))))
    taps = bandpass_taps([7.5e6, 8.75e6, 12.5e6, 13.75e6], 1540 / 0.02e-3 / 2)
    assert taps.size == n + 1 and np.allclose(taps, taps[::-1])
