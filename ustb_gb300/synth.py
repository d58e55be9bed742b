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
    imp_re = torch.zeros(W * N * (L + 1), dtype=torch.float32, device=dev)
    imp_im = torch.zeros_like(imp_re)
    rx = torch.cdist(pts, el)  # [S, N] metres
    carrier = 0.0 if rf else fd
    for w, wave in enumerate(sequence):
        tx = torch.as_tensor(_tx_delay_sim(wave, xyz), dtype=torch.float64, device=dev)
        tau = (tx[:, None] + rx) / c  # [S, N]
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
        vre = v.real.to(torch.float32)
        vim = v.imag.to(torch.float32)
        idx, frac, vre, vim = idx.reshape(-1), frac.reshape(-1), vre.reshape(-1), vim.reshape(-1)
        for i in range(0, idx.numel(), chunk):
            sl = slice(i, i + chunk)
            ii, ff = idx[sl], frac[sl]
            imp_re.index_add_(0, ii, vre[sl] * (1 - ff))
            imp_re.index_add_(0, ii + 1, vre[sl] * ff)
            if not rf:
                imp_im.index_add_(0, ii, vim[sl] * (1 - ff))
                imp_im.index_add_(0, ii + 1, vim[sl] * ff)
    imp = imp_re.view(W, N, L + 1)[..., :L]
    if not rf:
        imp = torch.complex(imp, imp_im.view(W, N, L + 1)[..., :L])
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
