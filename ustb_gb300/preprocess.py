"""RF -> IQ demodulation on the GPU, fused with the conversion into storage type.

``FastDemodulation`` mirrors +preprocess/fast_demodulation.m: down-mix at the
modulation frequency, low-pass FIR (Kaiser window design, :286-293), decimate to
the downsampling frequency (:94-98, :162-167), and shift the initial time by the
filter delay (:170-175).  The three steps are one kernel pass
(``ustb_demodulate``) that reads int16 / single / half RF once and writes IQ in
the storage type the fast beamformer consumes, so the RF -> IQ -> FP16 chain costs
one read of the RF and one write of the IQ.

The filter design restates MATLAB's ``kaiserord`` (Kaiser's order and beta
formulas for a low-pass with pass/stop edges f1 < f2 and ripple ``dev``) and
``fir1(n, Wn, 'low', kaiser(n+1, beta), 'noscale')``, i.e. the windowed ideal
low-pass without gain normalisation: scipy's ``firwin(n+1, Wn, window=('kaiser',
beta), scale=False)``.

The reference's Python port (python/src/ustb/preprocess/fast_demodulation.py)
filters with ``filtfilt`` and keeps t0; this module follows the MATLAB class.
"""
from __future__ import annotations

import math
from typing import Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .enums import Precision
from .uff import ChannelData

SRC = {torch.float32: 0, torch.int16: 1, torch.float16: 2}
STORE = {Precision.fp32: 0, Precision.fp16: 1, Precision.bf16: 2}
TORCH_STORE = {Precision.fp32: torch.float32, Precision.fp16: torch.float16, Precision.bf16: torch.bfloat16}


def kaiser_lowpass_order(f1: float, f2: float, fs: float, dev: Sequence[float] = (1e-3, 1e-3)):
    """(n, Wn, beta) of MATLAB kaiserord([f1 f2], [1 0], dev, fs)."""
    A = -20.0 * math.log10(min(dev))
    if A > 50:
        beta = 0.1102 * (A - 8.7)
    elif A > 21:
        beta = 0.5842 * (A - 21) ** 0.4 + 0.07886 * (A - 21)
    else:
        beta = 0.0
    dw = 2 * math.pi * (f2 - f1) / fs
    n = int(math.ceil((A - 7.95) / (2.285 * dw)))
    Wn = (f1 + f2) / fs  # band-edge midpoint relative to Nyquist
    return n, Wn, beta


def lowpass_taps(fc: float, fs: float, lowpass_frequency_vector=(0.5, 1.0)) -> np.ndarray:
    """Low-pass taps of fast_demodulation.m:286-293 (transition band
    [lowpass_frequency_vector] * |fc|, 1e-3 ripple)."""
    from scipy.signal import firwin

    f1, f2 = (float(v) * abs(fc) for v in lowpass_frequency_vector)
    n, Wn, beta = kaiser_lowpass_order(f1, f2, fs)
    return firwin(n + 1, Wn, window=("kaiser", beta), pass_zero=True, scale=False)


def decimation_factor(fs: float, downsample_frequency: float) -> Tuple[int, float]:
    """(D, fs / D) with D = floor(fs / downsample_frequency) (fast_demodulation.m:94-98)."""
    D = max(1, int(math.floor(fs / downsample_frequency)))
    return D, fs / D


def demodulate(rf: torch.Tensor, fs: float, t0: float, fc: float, taps: np.ndarray, decimation: int,
               precision: Precision = Precision.fp32, scale: float = 1.0, zero_phase: bool = False) -> torch.Tensor:
    """One pass of ``ustb_demodulate`` (causal FIR) or, with ``zero_phase``,
    ``ustb_demodulate_filtfilt`` (forward-backward FIR as scipy's filtfilt): real RF
    (..., L) CUDA tensor (float32, int16 or float16; the last dimension is time) -> IQ
    (..., ceil(L/D), 2) of the storage type (interleaved re, im), where the leading
    dimensions are independent traces."""
    if rf.dtype not in SRC or not rf.is_cuda:
        raise TypeError(f"rf must be a float32 / int16 / float16 CUDA tensor, got {rf.dtype} on {rf.device}")
    rf = rf.contiguous()
    L = rf.shape[-1]
    n_traces = rf.numel() // max(L, 1)
    Ld = (L + decimation - 1) // decimation
    prec = Precision(precision)
    out = torch.empty(tuple(rf.shape[:-1]) + (Ld, 2), dtype=TORCH_STORE[prec], device=rf.device)
    t = torch.as_tensor(np.asarray(taps, np.float32), device=rf.device)
    with torch.cuda.device(rf.device):
        _lib.call("ustb_demodulate_filtfilt" if zero_phase else "ustb_demodulate", rf.data_ptr(), SRC[rf.dtype], out.data_ptr(), STORE[prec], L, n_traces,
                  float(fs), float(t0), float(fc), int(decimation), t.data_ptr(), t.numel(), float(scale),
                  torch.cuda.current_stream(rf.device).cuda_stream)
    return out


class FastDemodulation:
    """preprocess.fast_demodulation on the GPU.  Set ``input`` (RF ChannelData),
    ``modulation_frequency`` (required here: the reference estimates it from the
    power spectrum when empty), optionally ``downsample_frequency`` (default
    2 * modulation_frequency, :87-91) and ``lowpass_frequency_vector``; ``go()``
    returns IQ ChannelData whose ``data`` is a complex64 [L', N, W, F] view of
    device memory.  ``zero_phase = True`` gives the reference's Python port instead
    (``ZeroPhaseDemodulation``: filtfilt, t0 kept, its own default decimation).
    """

    def __init__(self):
        self.input: Optional[ChannelData] = None
        self.modulation_frequency: Optional[float] = None
        self.downsample_frequency: Optional[float] = None
        self.lowpass_frequency_vector = (0.5, 1.0)
        self.precision = Precision.fp32
        self.device = torch.device("cuda", 0)
        self.zero_phase = False

    @property
    def b(self) -> np.ndarray:
        return lowpass_taps(self.modulation_frequency, self.input.sampling_frequency, self.lowpass_frequency_vector)

    def go(self) -> ChannelData:
        if self.zero_phase:
            z = ZeroPhaseDemodulation()
            z.input, z.modulation_frequency = self.input, self.modulation_frequency
            z.downsample_frequency = self.downsample_frequency
            z.lowpass_frequency_vector = list(self.lowpass_frequency_vector)
            z.precision, z.device = self.precision, self.device
            return z.go()
        cd = self.input
        if self.modulation_frequency is None:
            raise ValueError("set modulation_frequency (the centre frequency of the RF data)")
        fs, fc = float(cd.sampling_frequency), float(self.modulation_frequency)
        D, fs_out = decimation_factor(fs, self.downsample_frequency or 2 * fc)
        taps = self.b
        data = cd.data if torch.is_tensor(cd.data) else torch.as_tensor(np.asarray(cd.data))
        data = data.to(self.device)
        if data.is_complex():
            raise ValueError("fast_demodulation takes real RF channel data")
        while data.dim() < 4:
            data = data.unsqueeze(-1)
        rf = data.permute(3, 2, 1, 0).contiguous()  # [L,N,W,F] -> ABI (F, W, N, L)
        if rf.dtype not in SRC:
            rf = rf.to(torch.float32)
        iq = demodulate(rf, fs, float(cd.initial_time), fc, taps, D, self.precision)
        if self.precision != Precision.fp32:
            iq = iq.float()
        iqc = torch.view_as_complex(iq.contiguous()).permute(3, 2, 1, 0)
        delay = (len(taps) - 1) / 2 / fs
        return ChannelData(iqc, cd.probe, cd.sequence, fs_out, float(cd.initial_time) - delay, cd.sound_speed, fc)


def python_port_taps(fc: float, fs: float, L: int, lowpass_frequency_vector=(0.5, 1.0)) -> np.ndarray:
    """Taps of python/src/ustb/preprocess/fast_demodulation.py:57-63: a Hamming-window
    low-pass of min(65, 2 (L // 3) - 1) taps (at least 3, odd) with cut-off
    fc * lowpass_frequency_vector[0], unit gain at DC (scipy ``firwin``)."""
    from scipy.signal import firwin

    numtaps = min(65, L // 3 * 2 - 1)
    if numtaps < 3:
        numtaps = 3
    if numtaps % 2 == 0:
        numtaps += 1
    return firwin(numtaps, fc * float(lowpass_frequency_vector[0]), fs=fs)


class ZeroPhaseDemodulation:
    """The reference's Python ``preprocess.FastDemodulation``
    (python/src/ustb/preprocess/fast_demodulation.py:14-88) on the GPU: down-mix at the
    modulation frequency, zero-phase low-pass (scipy ``filtfilt`` of ``python_port_taps``),
    keep every D-th sample with D = floor(fs / downsample_frequency), or
    floor(fs / (4 fc)) when ``downsample_frequency`` is unset; the initial time is kept.
    The modulation frequency defaults to ``input.pulse.center_frequency`` when the
    input has a pulse, else to ``input.modulation_frequency``.  The whole chain is one
    kernel pass (``ustb_demodulate_filtfilt``); ``go()`` returns IQ ChannelData whose
    ``data`` is a complex64 [L', N, W, F] view of device memory."""

    def __init__(self):
        self.input: Optional[ChannelData] = None
        self.modulation_frequency: Optional[float] = None
        self.downsample_frequency: Optional[float] = None
        self.lowpass_frequency_vector = [0.5, 1.0]
        self.precision = Precision.fp32
        self.device = torch.device("cuda", 0)

    def _fc(self) -> float:
        if self.modulation_frequency is not None:
            return float(self.modulation_frequency)
        pulse = getattr(self.input, "pulse", None)
        if pulse is not None and getattr(pulse, "center_frequency", None) is not None:
            return float(pulse.center_frequency)
        return float(self.input.modulation_frequency)

    def go(self) -> ChannelData:
        cd = self.input
        fs, fc, t0 = float(cd.sampling_frequency), self._fc(), float(cd.initial_time)
        data = cd.data if torch.is_tensor(cd.data) else torch.as_tensor(np.asarray(cd.data))
        data = data.to(self.device)
        if data.is_complex():
            raise ValueError("fast demodulation takes real RF channel data")
        while data.dim() < 4:
            data = data.unsqueeze(-1)
        L = int(data.shape[0])
        taps = python_port_taps(fc, fs, L, self.lowpass_frequency_vector)
        if self.downsample_frequency is not None:
            D = max(1, int(np.floor(fs / float(self.downsample_frequency))))
        else:
            D = max(1, int(np.floor(fs / (4 * fc))))
        rf = data.permute(3, 2, 1, 0).contiguous()  # [L,N,W,F] -> ABI (F, W, N, L)
        if rf.dtype not in SRC:
            rf = rf.to(torch.float32)
        iq = demodulate(rf, fs, t0, fc, taps, D, self.precision, zero_phase=True)
        if self.precision != Precision.fp32:
            iq = iq.float()
        iqc = torch.view_as_complex(iq.contiguous()).permute(3, 2, 1, 0)
        return ChannelData(iqc, cd.probe, cd.sequence, fs / D, t0, cd.sound_speed, fc)
