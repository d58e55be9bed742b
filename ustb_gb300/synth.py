"""Seeded synthetic channel data for the beamformer's workloads.

The reference's public datasets (PICMUS, Verasonics UFF, the legacy ps.zip
set) are not available here, so workloads are synthesised with the shapes and
value distributions of the five benchmark configurations:

* pulse ``cos(2*pi*f0*t) * exp(-1.7886*(t*bw*f0)^2)`` with bw = 0.6, the
  Gaussian pulse of +uff/pulse.m:76-79;
* echoes placed analytically per scatterer with the same transmit-delay model
  das.m uses (plane: z cos(theta) + x sin(theta); diverging: |s - x| - |d|;
  single-element transmit: |e - x|), plus the element-to-scatterer distance;
* IQ data is the analytic baseband signal, amplitude/2 * envelope * exp(-i 2 pi fd tau);
* speckle is many scatterers with complex-Gaussian amplitudes, cysts are
  regions left empty, and noise is white Gaussian at a given level below the peak.

Impulses are placed with linear fractional weights on the sample grid and
convolved with the sampled pulse (FFT), on the torch device given (GPU for the
full-size workloads, CPU for small test cases).  Every draw comes from
``numpy.random.Generator(PCG64(seed))``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import geometry
from .enums import Dimension, Window
from .uff import ChannelData, LinearScan, LinearScan3D, Point, Probe, Scan, SectorScan, Wave

C0 = 1540.0
BW = 0.6


@dataclass
class Workload:
    """A beamforming request: channel data + scan + DAS settings."""
    name: str
    channel_data: ChannelData
    scan: Scan
    dimension: Dimension
    rx_window: Window = Window.tukey25
    rx_f_number: float = 1.7
    tx_window: Window = Window.none
    tx_f_number: float = 1.0
    storage: str = "fp32"          # fp32 | fp16 | bf16 | int16
    epilogue: Optional[str] = None  # None | "cf_sdmas"
    info: Dict = field(default_factory=dict)

    @property
    def units(self) -> int:
        cd = self.channel_data
        return self.scan.N_pixels * cd.N_channels * cd.N_waves * cd.N_frames


def _tx_delay_sim(wave: Wave, xyz: np.ndarray) -> np.ndarray:
    """Transmit path length [S] in metres, same models as das.m:110-204."""
    s = wave.source
    if wave.wavefront == 0 or math.isinf(s.distance):
        ca, sa = math.cos(s.azimuth), math.sin(s.azimuth)
        ce, se = math.cos(s.elevation), math.sin(s.elevation)
        return xyz[:, 2] * ca * ce + xyz[:, 0] * sa * ce + xyz[:, 1] * se
    d = np.sqrt(((xyz - s.xyz[None, :]) ** 2).sum(1))
    sign = np.where(xyz[:, 2] < s.z, -1.0, 1.0)
    if s.z < 0:
        return sign * d - abs(s.distance)
    return sign * d + s.distance


def simulate(probe: Probe, sequence: List[Wave], xyz: np.ndarray, amp: np.ndarray, fs: float,
             t0: float, L: int, f0: float, fd: float, rf: bool, device="cpu", c: float = C0,
             chunk: int = 1 << 22):
    """Channel data for scatterers ``xyz`` [S,3] with complex amplitudes ``amp`` [S].

    Returns a torch tensor shaped (W, N, L) in the ABI layout (one frame):
    complex64 for IQ (``rf=False``) or float32 for RF.
    """
    import torch

    N, W, S = probe.N_elements, len(sequence), xyz.shape[0]
    dev = torch.device(device)
    el = torch.as_tensor(probe.xyz, dtype=torch.float64, device=dev)
    pts = torch.as_tensor(xyz, dtype=torch.float64, device=dev)
    a = torch.as_tensor(amp, dtype=torch.complex128, device=dev)
    # impulses summed in FP64: index_add_ on a GPU adds in no fixed order, and FP64 sums
    # rounded to FP32 make the data the same from run to run
    imp_re = torch.zeros(W * N * (L + 1), dtype=torch.float64, device=dev)
    imp_im = torch.zeros_like(imp_re)
    rx = torch.cdist(pts, el)  # [S, N] metres
    carrier = 0.0 if rf else fd
    for w, wave in enumerate(sequence):
        tx = torch.as_tensor(_tx_delay_sim(wave, xyz) / wave.sound_speed - wave.delay,
                             dtype=torch.float64, device=dev)
        tau = tx[:, None] + rx / c  # [S, N] seconds
        s = (tau - t0) * fs
        k0 = torch.floor(s)
        frac = (s - k0).to(torch.float32)
        ok = (k0 >= 0) & (k0 < L - 1)
        val = a[:, None] * torch.exp(-2j * math.pi * carrier * tau)
        if not rf:
            val = val * 0.5
        base = (w * N + torch.arange(N, device=dev)[None, :]) * (L + 1)
        idx = (base + k0.clamp(0, L - 1).to(torch.int64))
        v = torch.where(ok, val, torch.zeros((), dtype=val.dtype, device=dev))
        vre = v.real.to(torch.float32).double()
        vim = v.imag.to(torch.float32).double()
        frac = frac.double()
        idx, frac, vre, vim = idx.reshape(-1), frac.reshape(-1), vre.reshape(-1), vim.reshape(-1)
        for i in range(0, idx.numel(), chunk):
            sl = slice(i, i + chunk)
            ii, ff = idx[sl], frac[sl]
            imp_re.index_add_(0, ii, vre[sl] * (1 - ff))
            imp_re.index_add_(0, ii + 1, vre[sl] * ff)
            if not rf:
                imp_im.index_add_(0, ii, vim[sl] * (1 - ff))
                imp_im.index_add_(0, ii + 1, vim[sl] * ff)
    imp = imp_re.view(W, N, L + 1)[..., :L].float()
    if not rf:
        imp = torch.complex(imp, imp_im.view(W, N, L + 1)[..., :L].float())
    # pulse (RF) or its envelope (IQ) sampled on the grid
    half = int(math.ceil(3.0 / (BW * f0) * fs))
    tk = torch.arange(-half, half + 1, dtype=torch.float64, device=dev) / fs
    env = torch.exp(-1.7886 * (tk * BW * f0) ** 2)
    pulse = env * torch.cos(2 * math.pi * f0 * tk) if rf else env * torch.exp(
        2j * math.pi * (f0 - fd) * tk)
    nfft = 1 << int(math.ceil(math.log2(L + 2 * half + 1)))
    if rf:
        X = torch.fft.rfft(imp.to(torch.float64), nfft)
        H = torch.fft.rfft(pulse, nfft)
        y = torch.fft.irfft(X * H, nfft)[..., half:half + L]
        return y.to(torch.float32).contiguous()
    X = torch.fft.fft(imp.to(torch.complex128), nfft)
    H = torch.fft.fft(pulse.to(torch.complex128), nfft)
    y = torch.fft.ifft(X * H, nfft)[..., half:half + L]
    return y.to(torch.complex64).contiguous()


def _matlab(abi_wnl):
    """(W, N, L) ABI tensor of one frame -> view with the MATLAB shape [L, N, W, 1]."""
    return abi_wnl.unsqueeze(0).permute(3, 2, 1, 0)


def _add_noise(x, rng, level_db: float):
    import torch

    peak = x.abs().max().item() or 1.0
    sigma = peak * 10 ** (level_db / 20)
    shape = tuple(x.shape)
    if x.is_complex():
        n = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * (sigma / math.sqrt(2))
        return x + torch.as_tensor(n.astype(np.complex64), device=x.device)
    n = rng.standard_normal(shape) * sigma
    return x + torch.as_tensor(n.astype(np.float32), device=x.device)


def _speckle(rng, region, density_per_mm2, cysts=(), ny=None):
    (x0, x1), (z0, z1) = region[0], region[1]
    area = (x1 - x0) * (z1 - z0) * 1e6
    if ny is not None:
        (y0, y1) = ny
        area *= (y1 - y0) * 1e3
    S = int(area * density_per_mm2)
    x = rng.uniform(x0, x1, S)
    z = rng.uniform(z0, z1, S)
    y = rng.uniform(ny[0], ny[1], S) if ny is not None else np.zeros(S)
    keep = np.ones(S, dtype=bool)
    for (cx, cz, r) in cysts:
        keep &= (x - cx) ** 2 + (z - cz) ** 2 > r ** 2
    amp = (rng.standard_normal(S) + 1j * rng.standard_normal(S)) / math.sqrt(2)
    return np.stack([x, y, z], 1)[keep], amp[keep]


def _points(rng, n, xr, zr, yr=None):
    x = rng.uniform(*xr, n)
    z = rng.uniform(*zr, n)
    y = rng.uniform(*yr, n) if yr is not None else np.zeros(n)
    return np.stack([x, y, z], 1), rng.uniform(0.5, 1.0, n).astype(np.complex128)


def cell_density(f0, f_number, c=C0):
    """Scatterers per mm^2 for 10 per resolution cell (lateral lambda*F#, axial c/(2 bw f0))."""
    lam = c / f0
    cell = (lam * f_number) * (c / (2 * BW * f0)) * 1e6
    return 10.0 / cell


def config_rf_plane_wave(seed=1, device="cpu", scale=1.0) -> Workload:
    """128-element linear array, RF, one 0-degree plane wave, 20 point targets."""
    rng = np.random.default_rng(seed)
    N = max(2, int(round(128 * scale)))
    L = max(64, int(round(2048 * scale)))
    nx = max(4, int(round(256 * scale)))
    probe = Probe.linear_array(N, 0.3e-3)
    f0, fs = 5e6, 20e6
    seq = [Wave.plane(0.0)]
    xyz, amp = _points(rng, 20, (-15e-3, 15e-3), (5e-3, 45e-3))
    data = simulate(probe, seq, xyz, amp, fs, 0.0, L, f0, 0.0, rf=True, device=device)
    data = _add_noise(data, rng, -40.0)
    cd = ChannelData(_matlab(data), probe, seq, fs, 0.0, C0, 0.0)
    scan = LinearScan(np.linspace(-19e-3, 19e-3, nx), np.linspace(5e-3, 50e-3, nx))
    return Workload("rf_plane_wave", cd, scan, Dimension.both, storage="fp32",
                    info={"scatterers": xyz, "f0": f0})


def config_iq_cpwc(seed=2, device="cpu", scale=1.0, n_waves=75, density=None) -> Workload:
    """128-element linear array, IQ, 75 plane waves -16..16 deg, speckle + 2 cysts."""
    rng = np.random.default_rng(seed)
    N = max(2, int(round(128 * scale)))
    L = max(64, int(round(1024 * scale)))
    npx = max(4, int(round(400 * scale)))
    W = max(1, int(round(n_waves * scale))) if scale < 1 else n_waves
    probe = Probe.linear_array(N, 0.3e-3)
    f0, fs = 5e6, 20e6
    t0 = 6.5e-6
    ang = np.linspace(-16, 16, W) * math.pi / 180 if W > 1 else np.zeros(1)
    seq = [Wave.plane(float(a)) for a in ang]
    zr = (8e-3, 40e-3)
    cysts = [(0.0, 20e-3, 2e-3), (0.0, 35e-3, 2e-3)]
    dens = cell_density(f0, 1.7) if density is None else density
    sxyz, samp = _speckle(rng, ((-19e-3, 19e-3), zr), dens * (scale if scale < 1 else 1.0), cysts)
    pxyz, pamp = _points(rng, 200, (-19e-3, 19e-3), zr)
    xyz = np.concatenate([sxyz, pxyz])
    amp = np.concatenate([samp * 0.1, pamp])
    data = simulate(probe, seq, xyz, amp, fs, t0, L, f0, f0, rf=False, device=device)
    data = _add_noise(data, rng, -40.0)
    cd = ChannelData(_matlab(data), probe, seq, fs, t0, C0, f0)
    scan = LinearScan(np.linspace(-19e-3, 19e-3, npx), np.linspace(zr[0], zr[1], npx))
    return Workload("iq_cpwc", cd, scan, Dimension.both, storage="fp32",
                    info={"cysts": cysts, "f0": f0, "scatterers": pxyz})


def _with_noise_and_shape(data, rng, level_db):
    return _add_noise(data, rng, level_db)


def config_dw_sector(seed=3, device="cpu", scale=1.0) -> Workload:
    """64-element phased array, 21 diverging waves (-30..30 deg, sources 10 mm behind),
    FP16 IQ storage, 256 x 512 sector scan over +-40 deg, 5-90 mm; dimension.transmit
    with the fused coherence-factor / simplified-DMAS epilogue."""
    rng = np.random.default_rng(seed)
    N = max(4, int(round(64 * scale)))
    L = max(128, int(round(1536 * scale)))
    W = 21 if scale >= 1 else max(3, int(round(21 * scale)))
    naz, nd = max(8, int(round(256 * scale))), max(8, int(round(512 * scale)))
    probe = Probe.linear_array(N, 0.22e-3)
    f0, fs = 3e6, 12e6
    ang = np.deg2rad(np.linspace(-30, 30, W))
    seq = [Wave(source=Point(-10e-3, float(a), 0.0)) for a in ang]
    dmax = 90e-3 if scale >= 1 else 90e-3 * max(scale, 0.25)
    scan = SectorScan(np.deg2rad(np.linspace(-40, 40, naz)), np.linspace(5e-3, dmax, nd))
    # scatterers in polar coordinates over the sector
    area = 0.5 * (dmax ** 2 - 5e-3 ** 2) * np.deg2rad(80) * 1e6
    S = int(area * cell_density(f0, 1.7) * (scale if scale < 1 else 1.0))
    r = np.sqrt(rng.uniform(5e-3 ** 2, dmax ** 2, S))
    th = rng.uniform(-np.deg2rad(40), np.deg2rad(40), S)
    xyz = np.stack([r * np.sin(th), np.zeros(S), r * np.cos(th)], 1)
    cysts = [(0.0, 0.4 * dmax, 2e-3), (0.0, 0.7 * dmax, 2e-3)]
    keep = np.ones(S, bool)
    for cx, cz, cr in cysts:
        keep &= (xyz[:, 0] - cx) ** 2 + (xyz[:, 2] - cz) ** 2 > cr ** 2
    amp = (rng.standard_normal(S) + 1j * rng.standard_normal(S)) / math.sqrt(2) * 0.1
    pr = rng.uniform(10e-3, dmax, 200)
    pth = rng.uniform(-np.deg2rad(35), np.deg2rad(35), 200)
    pxyz = np.stack([pr * np.sin(pth), np.zeros(200), pr * np.cos(pth)], 1)
    xyz = np.concatenate([xyz[keep], pxyz])
    amp = np.concatenate([amp[keep], rng.uniform(0.5, 1.0, 200).astype(np.complex128)])
    data = simulate(probe, seq, xyz, amp, fs, 0.0, L, f0, f0, rf=False, device=device)
    data = _add_noise(data, rng, -40.0)
    cd = ChannelData(_matlab(data), probe, seq, fs, 0.0, C0, f0)
    return Workload("dw_sector", cd, scan, Dimension.transmit, rx_window=Window.tukey25, rx_f_number=1.7,
                    storage="fp16", epilogue="cf_sdmas", info={"cysts": cysts, "f0": f0})


def config_hfr_ensemble(seed=4, device="cpu", frames=200, scale=1.0) -> Workload:
    """200 frames x 11 plane waves (-10..10 deg) x 128 channels x 1536 int16 I/Q samples,
    speckle with a 2 mm-radius vessel whose scatterers move axially 0-0.5 mm/frame
    (sinusoidal profile across the vessel); 256 x 512 linear scan; dimension.both.

    Channel data is returned as int16 (I, Q interleaved): the ABI-layout tensor of
    shape (F, W, N, L, 2) lives in ``info["int16"]`` and ``info["scale"]`` maps it
    back to the simulated amplitude."""
    import torch

    rng = np.random.default_rng(seed)
    N = max(4, int(round(128 * scale)))
    L = max(128, int(round(1536 * scale)))
    nx, nz = max(8, int(round(256 * scale))), max(8, int(round(512 * scale)))
    probe = Probe.linear_array(N, 0.3e-3)
    f0, fs = 5e6, 20e6
    seq = [Wave.plane(float(a)) for a in np.deg2rad(np.linspace(-10, 10, 11))]
    zr = (5e-3, 50e-3)
    scan = LinearScan(np.linspace(-19e-3, 19e-3, nx), np.linspace(zr[0], zr[1], nz))
    dens = cell_density(f0, 1.7) * 0.25 * (scale if scale < 1 else 1.0)
    vc, vr = (0.0, 25e-3), 2e-3
    bxyz, bamp = _speckle(rng, ((-19e-3, 19e-3), zr), dens, cysts=[(vc[0], vc[1], vr)])
    back = simulate(probe, seq, bxyz, bamp * 0.1, fs, 0.0, L, f0, f0, rf=False, device=device)
    Sv = int(np.pi * vr ** 2 * 1e6 * dens)
    vx = rng.uniform(vc[0] - vr, vc[0] + vr, Sv * 2)
    vz = rng.uniform(vc[1] - vr, vc[1] + vr, Sv * 2)
    inside = (vx - vc[0]) ** 2 + (vz - vc[1]) ** 2 < vr ** 2
    vx, vz = vx[inside][:Sv], vz[inside][:Sv]
    vamp = (rng.standard_normal(vx.size) + 1j * rng.standard_normal(vx.size)) / math.sqrt(2) * 0.1
    disp = 0.5e-3 * np.cos(np.pi / 2 * np.abs(vx - vc[0]) / vr)  # per frame, 0..0.5 mm
    out = torch.empty((frames, len(seq), N, L, 2), dtype=torch.int16, device=device)
    peak = float(back.abs().max().item()) * 4 or 1.0
    scale16 = 30000.0 / peak
    for f in range(frames):
        z = vc[1] - vr + np.mod(vz - (vc[1] - vr) + f * disp, 2 * vr)
        ok = (vx - vc[0]) ** 2 + (z - vc[1]) ** 2 < vr ** 2
        xyz = np.stack([vx[ok], np.zeros(ok.sum()), z[ok]], 1)
        fr = back + simulate(probe, seq, xyz, vamp[ok], fs, 0.0, L, f0, f0, rf=False, device=device)
        fr = _add_noise(fr, rng, -40.0)
        ri = torch.view_as_real(fr) * scale16
        out[f] = ri.round().clamp(-32768, 32767).to(torch.int16)
    data_c = None  # int16 is the stored form; ChannelData gets a float view on demand
    cd = ChannelData(_matlab_frames(out, scale16), probe, seq, fs, 0.0, C0, f0)
    return Workload("hfr_ensemble", cd, scan, Dimension.both, storage="int16",
                    info={"int16": out, "scale": 1.0 / scale16, "f0": f0, "frames": frames})


def _matlab_frames(i16, scale16):
    """int16 (F, W, N, L, 2) -> complex64 view with the MATLAB shape [L, N, W, F] (on demand)."""
    import torch

    c = torch.complex(i16[..., 0].float(), i16[..., 1].float()) / scale16
    return c.permute(3, 2, 1, 0)


def config_sta(seed=5, device="cpu", scale=1.0) -> Workload:
    """Synthetic transmit aperture: 128 single-element transmits x 128 channels x 2048
    float32 RF samples, 300 x 300 pixels; dimension.both."""
    rng = np.random.default_rng(seed)
    N = max(4, int(round(128 * scale)))
    L = max(128, int(round(2048 * scale)))
    npx = max(8, int(round(300 * scale)))
    probe = Probe.linear_array(N, 0.3e-3)
    f0, fs = 5e6, 20e6
    seq = [Wave(source=Point.from_xyz(x, 0.0, 0.0), delay=abs(x) / C0) for x in probe.x]
    zr = (5e-3, 50e-3)
    xyz, amp = _points(rng, 20, (-15e-3, 15e-3), (8e-3, 45e-3))
    sxyz, samp = _speckle(rng, ((-19e-3, 19e-3), zr), 2.0 * (scale if scale < 1 else 1.0))
    data = simulate(probe, seq, np.concatenate([xyz, sxyz]), np.concatenate([amp, samp * 0.05]),
                    fs, 0.0, L, f0, 0.0, rf=True, device=device)
    data = _add_noise(data, rng, -40.0)
    cd = ChannelData(_matlab(data), probe, seq, fs, 0.0, C0, 0.0)
    scan = LinearScan(np.linspace(-19e-3, 19e-3, npx), np.linspace(zr[0], zr[1], npx))
    return Workload("sta", cd, scan, Dimension.both, storage="fp32", info={"f0": f0})


def config_matrix_3d(seed=6, device="cpu", scale=1.0) -> Workload:
    """32 x 32 matrix array (0.3 mm pitch), 25 diverging waves, 1024 FP16 IQ samples,
    64 x 64 x 128-voxel volume; dimension.both."""
    rng = np.random.default_rng(seed)
    nxe = max(4, int(round(32 * scale)))
    L = max(128, int(round(1024 * scale)))
    nv = max(8, int(round(64 * scale)))
    nzv = max(8, int(round(128 * scale)))
    probe = Probe.matrix_array(nxe, nxe, 0.3e-3)
    f0, fs = 4e6, 16e6
    ang = np.deg2rad(np.linspace(-15, 15, 5))
    seq = []
    for ay in ang:
        for ax in ang:
            seq.append(Wave(source=Point(-10e-3, float(ax), float(ay))))
    half = 0.3e-3 * nv / 2
    zr = (5e-3, 40e-3)
    scan = LinearScan3D(np.linspace(-half, half, nv), np.linspace(zr[0], zr[1], nzv), np.linspace(-half, half, nv))
    S = int(20000 * (scale if scale < 1 else 1.0))
    xyz = np.stack([rng.uniform(-half, half, S), rng.uniform(-half, half, S), rng.uniform(*zr, S)], 1)
    amp = (rng.standard_normal(S) + 1j * rng.standard_normal(S)) / math.sqrt(2) * 0.1
    pxyz = np.stack([rng.uniform(-half, half, 50), rng.uniform(-half, half, 50), rng.uniform(8e-3, 38e-3, 50)], 1)
    data = simulate(probe, seq, np.concatenate([xyz, pxyz]),
                    np.concatenate([amp, rng.uniform(0.5, 1, 50).astype(np.complex128)]),
                    fs, 0.0, L, f0, f0, rf=False, device=device)
    data = _add_noise(data, rng, -40.0)
    cd = ChannelData(_matlab(data), probe, seq, fs, 0.0, C0, f0)
    return Workload("matrix_3d", cd, scan, Dimension.both, rx_window=Window.tukey25, rx_f_number=1.7,
                    storage="fp16", info={"f0": f0})


CONFIGS = {
    "rf_plane_wave": config_rf_plane_wave,
    "iq_cpwc": config_iq_cpwc,
    "dw_sector": config_dw_sector,
    "hfr_ensemble": config_hfr_ensemble,
    "sta": config_sta,
    "matrix_3d": config_matrix_3d,
}
