"""Post-DAS steps: the follow-up of the fused coherence-factor / simplified-DMAS
epilogue, and the coherence, phase-coherence and generalized coherence factors and
Capon's minimum variance on a kept cube.

``simplified_dmas_image`` completes +postprocess/simplified_delay_multiply_and_sum.m
on a linear scan: the per-pixel value ((sum sign(s) sqrt|s|)^2 - sum |s|)/2
comes from the fused epilogue of ``ustb_das_fast`` (dimension.transmit); here it is
band-pass filtered along depth around 2*f0 with the reference's Kaiser design
(:151-176) on the GPU (``ustb_fir_depth``) and made analytic along depth (:192).

The filter design restates MATLAB's ``kaiserord`` (Kaiser's order and beta
formulas) followed by ``fir1(n, Wn, kaiser(n+1, beta), 'noscale')``, which is
scipy's ``firwin(..., scale=False)`` with the same window.  ``estimate_frequency``
restates +tools/estimate_frequency.m / +tools/power_spectrum.m.
"""
from __future__ import annotations

import math
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib


def kaiser_order(f_edges: Sequence[float], devs: Sequence[float], fs: float):
    """(n, Wn, beta) of MATLAB kaiserord(f, [0 1 0], devs, fs) for a band-pass."""
    f = np.asarray(f_edges, np.float64) / fs
    A = -20.0 * math.log10(min(devs))
    if A > 50:
        beta = 0.1102 * (A - 8.7)
    elif A > 21:
        beta = 0.5842 * (A - 21) ** 0.4 + 0.07886 * (A - 21)
    else:
        beta = 0.0
    df = min(f[1] - f[0], f[3] - f[2])
    n = int(math.ceil((A - 7.95) / (2 * math.pi * 2.285 * df))) if A > 21 else int(math.ceil(5.79 / (2 * math.pi * df)))
    Wn = np.array([(f[0] + f[1]), (f[2] + f[3])])  # midpoints, relative to Nyquist
    return n, Wn, beta


def bandpass_taps(f_edges, fs, devs=(1e-3, 1e-3, 1e-3)) -> np.ndarray:
    from scipy.signal import firwin

    n, Wn, beta = kaiser_order(f_edges, devs, fs)
    return firwin(n + 1, Wn, window=("kaiser", beta), pass_zero=False, scale=False)


def estimate_frequency(time: np.ndarray, data: np.ndarray):
    """(fc, bw) from the averaged power spectrum along axis 0 (estimate_frequency.m)."""
    fs = 1.0 / np.mean(np.diff(time))
    d = data.reshape(data.shape[0], -1)
    pw = np.fft.fftshift(np.fft.fft(d, axis=0), axes=0)
    pw = np.mean(np.abs(pw) ** 2, axis=1)
    pw = pw / pw.max()
    fx = np.linspace(-fs / 2, fs / 2, data.shape[0] + 1)[:-1]
    k = np.ones(26) / 26
    fpw = np.convolve(pw, k)[: pw.size]  # filter(ones(1,26)/26, 1, pw)
    fpw = np.concatenate([fpw[12:], np.zeros(12)])
    w = fpw * (fx > 0)
    ic = int(np.argmax(w))
    dc = w[ic]
    fc = fx[ic]
    up = fx[(fx > fc) & (fpw < dc / 2)]
    do = fx[(fx < fc) & (fpw < dc / 2)]
    bw_up = up.min() if up.size else fx[-1]
    bw_do = do.max() if do.size else 0.0
    fc = (bw_up + bw_do) / 2
    return fc, 2 * (bw_up - fc)


def fir_depth(x: torch.Tensor, taps: np.ndarray, delay: Optional[int] = None) -> torch.Tensor:
    """Filter columns of a real (ncols, nz) CUDA tensor along depth with delay compensation."""
    if x.dtype != torch.float32 or not x.is_cuda:
        raise TypeError("x must be a float32 CUDA tensor")
    x = x.contiguous()
    nz = x.shape[-1]
    ncols = x.numel() // max(nz, 1)
    t = torch.as_tensor(np.asarray(taps, np.float32), device=x.device)
    if delay is None:
        delay = int(round((t.numel() - 1) / 2))
    out = torch.empty_like(x)
    with torch.cuda.device(x.device):
        _lib.call("ustb_fir_depth", x.data_ptr(), out.data_ptr(), nz, ncols, t.data_ptr(), t.numel(),
                  delay, torch.cuda.current_stream(x.device).cuda_stream)
    return out


def hilbert_depth(x: torch.Tensor) -> torch.Tensor:
    """Analytic signal along the last (depth) dimension."""
    from .das import hilbert_last

    return hilbert_last(x)


def simplified_dmas_image(sdmas: torch.Tensor, nz: int, nx: int, z_step: float, sound_speed: float,
                          f0: Optional[float] = None, filter_freqs=None,
                          reference_image: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Band-pass + Hilbert of the fused sDMAS value on a linear scan.

    ``sdmas``: (F, P) float32 from ``ustb_das_fast`` (P = nz * nx, depth fastest).
    The pass band is [1.5 f0, 2.5 f0] with f0/4 transitions unless
    ``filter_freqs`` gives the four edges.  Without f0 it is estimated from the
    real part of ``reference_image`` (the channel sum) along depth.  Returns
    complex64 (F, P).
    """
    fs = sound_speed / z_step / 2
    if filter_freqs is None:
        if f0 is None:
            if reference_image is None:
                raise ValueError("give f0, filter_freqs or a reference image")
            img = reference_image.real.reshape(-1, nx, nz).permute(2, 1, 0).cpu().numpy()
            t = 2 * np.arange(nz) * z_step / sound_speed
            f0, _ = estimate_frequency(t, img)
        F_edges = [1.5 * f0, 1.5 * f0 + f0 / 4, 2.5 * f0, 2.5 * f0 + f0 / 4]
    else:
        F_edges = list(filter_freqs)
    if not fs / 2 > F_edges[-1]:
        raise ValueError(f"need {math.ceil(F_edges[-1] * 2 / fs)} times more depth samples for the "
                         "DMAS band-pass around 2*f0")
    taps = bandpass_taps(F_edges, fs)
    y = sdmas.reshape(-1, nx, nz).to(torch.float32)
    filt = fir_depth(y.reshape(-1, nz), taps).reshape(-1, nx, nz)
    return hilbert_depth(filt).reshape(sdmas.shape[0], -1)


def coherence_factor(cube: torch.Tensor, dimension, active_count: Optional[torch.Tensor] = None):
    """Coherence factor (+postprocess/coherence_factor.m:100-135) of an ABI cube
    (F, W, N, P) complex64 over the channels (Dimension.receive), the waves
    (Dimension.transmit) or both (``ustb_coherence_factor``).  ``active_count``: (P,)
    counts M of active units per pixel (the MATLAB rule), or None for M = the number
    summed (the Python port's rule).  Returns dict of 'CF' (float32) and 'image'
    (complex64), each (F, W, 1, P) / (F, 1, N, P) / (F, 1, 1, P) in the ABI layout."""
    from .enums import Dimension

    if cube.dim() != 4 or not cube.is_complex():
        raise TypeError("cube must be a complex (F, W, N, P) tensor")
    c = cube.to(torch.complex64).contiguous()
    F, W, N, P = c.shape
    d = int(dimension)
    shape = {int(Dimension.receive): (F, W, 1, P), int(Dimension.transmit): (F, 1, N, P),
             int(Dimension.both): (F, 1, 1, P)}.get(d)
    if shape is None:
        raise ValueError("dimension must be receive, transmit or both")
    dev = c.device
    m = None if active_count is None else active_count.to(device=dev, dtype=torch.float32).reshape(P).contiguous()
    out = {"CF": torch.empty(shape, dtype=torch.float32, device=dev),
           "image": torch.empty(shape, dtype=torch.complex64, device=dev)}
    with torch.cuda.device(dev):
        _lib.call("ustb_coherence_factor", c.data_ptr(), P, N, W, F, d, 0 if m is None else m.data_ptr(),
                  out["CF"].data_ptr(), out["image"].data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
    return out


class CoherenceFactor:
    """postprocess.coherence_factor: ``input`` is BeamformedData whose ``data`` is the
    channel / wave cube [P, N, W, F] (MATLAB order, complex; a device tensor or an
    array); ``go()`` returns BeamformedData of CF * coherent sum, with the factor in
    ``CF``.  M per pixel follows coherence_factor.m:100-126 when the apodization
    tables are set (``receive_apodization`` [P, N], ``transmit_apodization`` [P, W]:
    units with apodization above ``active_element_criterium``), else the number of
    terms summed, as python/src/ustb/postprocess/coherence_factor.py does."""

    def __init__(self):
        from .enums import Dimension

        self.input = None
        self.dimension = Dimension.both
        self.active_element_criterium = 0.16
        self.receive_apodization = None
        self.transmit_apodization = None
        self.device = torch.device("cuda", 0)
        self.CF = None

    def _active_count(self, P: int):
        from .enums import Dimension

        thr = float(self.active_element_criterium)
        rx, tx = self.receive_apodization, self.transmit_apodization
        t = lambda a: torch.as_tensor(np.asarray(a, np.float32), device=self.device).reshape(P, -1)
        d = int(self.dimension)
        if d == int(Dimension.receive) and rx is not None:
            return (t(rx) > thr).sum(dim=1).float()
        if d == int(Dimension.transmit) and tx is not None:
            return (t(tx) > thr).sum(dim=1).float()
        if d == int(Dimension.both) and rx is not None and tx is not None:
            a, b = t(tx), t(rx)
            m = torch.empty(P, dtype=torch.float32, device=self.device)
            for i in range(0, P, 2048):  # blocks of pixels, as the reference does (:103-114)
                m[i:i + 2048] = ((a[i:i + 2048, None, :] * b[i:i + 2048, :, None]) > thr).sum(dim=(1, 2)).float()
            return m
        return None

    def go(self):
        from .kernels import to_matlab_order
        from .uff import BeamformedData

        data = self.input.data if torch.is_tensor(self.input.data) else torch.as_tensor(np.asarray(self.input.data))
        while data.dim() < 4:
            data = data.unsqueeze(-1)
        cube = data.to(self.device).permute(3, 2, 1, 0).contiguous()  # [P,N,W,F] -> ABI (F, W, N, P)
        out = coherence_factor(cube, self.dimension, self._active_count(cube.shape[-1]))
        self.CF = BeamformedData(self.input.scan, to_matlab_order(out["CF"]))
        return BeamformedData(self.input.scan, to_matlab_order(out["image"]))


def _cube_fkp(cube: torch.Tensor) -> torch.Tensor:
    """ABI cube (F, W|1, N|1, P) with one of W, N equal to 1 -> contiguous (F, K, P)."""
    if cube.dim() != 4 or not cube.is_complex():
        raise TypeError("cube must be a complex (F, W, N, P) tensor")
    F, W, N, P = cube.shape
    if W > 1 and N > 1:
        raise ValueError("the factor runs over one dimension: give a dimension.transmit or .receive cube")
    return cube.reshape(F, W * N, P).to(torch.complex64).contiguous()


def phase_coherence_factor(cube: torch.Tensor, weights: Optional[torch.Tensor] = None, gamma: float = 1.0,
                           sigma_0: float = math.pi / math.sqrt(3)):
    """Phase coherence factor (+postprocess/phase_coherence_factor.m) over the kept
    dimension of ``cube`` (ABI layout (F, W|1, N|1, P) complex).  ``weights``: (K, P)
    apodization of that dimension or None.  Returns dict of (F, P) tensors 'FCA',
    'FCC' and 'image' (= FCC * coherent sum)."""
    c = _cube_fkp(cube)
    F, K, P = c.shape
    dev = c.device
    w = None if weights is None else weights.to(torch.float32).reshape(K, P).contiguous()
    out = {"FCA": torch.empty((F, P), dtype=torch.float32, device=dev),
           "FCC": torch.empty((F, P), dtype=torch.float32, device=dev),
           "image": torch.empty((F, P), dtype=torch.complex64, device=dev)}
    with torch.cuda.device(dev):
        _lib.call("ustb_phase_coherence", c.data_ptr(), P, K, F, 0 if w is None else w.data_ptr(), float(gamma),
                  float(sigma_0), out["FCA"].data_ptr(), out["FCC"].data_ptr(), out["image"].data_ptr(),
                  torch.cuda.current_stream(dev).cuda_stream)
    return out


def generalized_coherence_factor(cube: torch.Tensor, M0: int = 4):
    """Generalized coherence factor (+postprocess/generalized_coherence_factor.m) over
    the kept dimension of ``cube``.  Returns dict of (F, P) tensors 'GCF' and 'image'."""
    c = _cube_fkp(cube)
    F, K, P = c.shape
    dev = c.device
    out = {"GCF": torch.empty((F, P), dtype=torch.float32, device=dev),
           "image": torch.empty((F, P), dtype=torch.complex64, device=dev)}
    with torch.cuda.device(dev):
        _lib.call("ustb_generalized_coherence", c.data_ptr(), P, K, F, int(M0), out["GCF"].data_ptr(),
                  out["image"].data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
    return out


def capon_k_samples(depth_axis: np.ndarray, wavelength: float, K_in_lambda: float) -> int:
    """K_samples of capon_minimum_variance.m:178-197: the depth sample nearest K_in_lambda
    wavelengths below the first, made odd (set.K_in_lambda)."""
    z = np.asarray(depth_axis, np.float64) / wavelength
    z = z - z[0]
    samples = int(np.argmin(np.abs(z - K_in_lambda))) + 1  # MATLAB's 1-based index
    return samples if samples % 2 else samples + 1


def capon_minimum_variance(cube: torch.Tensor, apodization: torch.Tensor, nz: int, nx: int, L_elements: float,
                           K_samples: int, regCoef: float, active_element_criterium: float = 0.16,
                           doForwardBackward: bool = False) -> torch.Tensor:
    """Capon MV (+postprocess/capon_minimum_variance.m) over the kept dimension of
    ``cube`` (ABI (F, W|1, N|1, P) complex, P = nz * nx with depth fastest).
    ``apodization``: (K, P) weights of that dimension (tx x rx apodization), the
    activity test ``|apod| > active_element_criterium``.  Returns (F, P) complex64."""
    c = _cube_fkp(cube)
    F, K, P = c.shape
    if P != nz * nx:
        raise ValueError(f"cube holds {P} pixels, the grid {nz} x {nx}")
    dev = c.device
    ap = apodization.to(torch.float32).reshape(K, P).contiguous()
    out = torch.empty((F, P), dtype=torch.complex64, device=dev)
    with torch.cuda.device(dev):
        _lib.call("ustb_capon", c.data_ptr(), ap.data_ptr(), nz, nx, K, F, float(L_elements), int(K_samples),
                  float(regCoef), float(active_element_criterium), int(bool(doForwardBackward)), out.data_ptr(),
                  torch.cuda.current_stream(dev).cuda_stream)
    return out
