"""midprocess.das on the GB300 beamformer.

``DAS`` keeps the properties of USTB's ``midprocess.das`` (+midprocess/das.m:49-63)
and of the Python package's ``ustb.midprocess.DAS`` (python/src/ustb/midprocess/das.py:29-41),
and its ``go()`` runs the same steps as das.m:77-317:

1. transmit / receive apodization tables (das.m:91-100),
2. receive and transmit delay tables (das.m:102-206), FP64 on the host, cast
   to single as das.m does,
3. channel data in single precision; RF data is made analytic with a Hilbert
   transform along time (das.m:211-214) unless ``rf_mode = "real"``,
4. the delay-and-sum itself through the C-ABI (``code = Code.gb300``), which
   takes the place of mex.das_c (das.m:251-259),
5. the per-pixel phase epilogue exp(-i 2 w0 r_ref / c) for IQ data (das.m:306-309),
6. a ``BeamformedData`` on the scan (das.m:217-218, 312).

The result tensor lives on the GPU; ``beamformed_data.data`` is a view with the
MATLAB shape [P, N|1, W|1, F] (see ``kernels.to_matlab_order``).
"""
from __future__ import annotations

import hashlib
import math
import time

import numpy as np
import torch

from . import geometry, kernels
from .enums import Code, Dimension, Precision, SphericalTransmitDelayModel, Window
from .geometry import Apodization
from .uff import BeamformedData, ChannelData, Scan


def channel_tensor(data, device) -> torch.Tensor:
    """Channel data with MATLAB shape [L, N, W, F] (numpy or torch) -> ABI-layout tensor."""
    if isinstance(data, np.ndarray):
        a = data
        while a.ndim < 4:
            a = a[..., None]
        dt = np.complex64 if np.iscomplexobj(a) else np.float32
        t = torch.from_numpy(np.ascontiguousarray(a.astype(dt, copy=False).transpose(3, 2, 1, 0)))
        return t.to(device)
    t = data
    while t.dim() < 4:
        t = t.unsqueeze(-1)
    if t.is_complex():
        t = t.to(torch.complex64)
    elif t.dtype not in (torch.float32,):
        t = t.to(torch.float32)
    return kernels.from_matlab_order(t.to(device))


def hilbert_last(x: torch.Tensor) -> torch.Tensor:
    """Analytic signal along the last dimension (the FFT method of MATLAB's hilbert)."""
    L = x.shape[-1]
    X = torch.fft.fft(x.to(torch.float32), dim=-1)
    h = torch.zeros(L, dtype=torch.float32, device=x.device)
    if L % 2 == 0:
        h[0] = h[L // 2] = 1.0
        h[1:L // 2] = 2.0
    else:
        h[0] = 1.0
        h[1:(L + 1) // 2] = 2.0
    return torch.fft.ifft(X * h, dim=-1).to(torch.complex64).contiguous()


class DAS:
    """Generalized delay-and-sum beamformer (midprocess.das) on GB300."""

    def __init__(self):
        self.channel_data: ChannelData = None
        self.scan: Scan = None
        self.dimension = Dimension.both
        self.code = Code.gb300
        self.gpu_id = 0
        self.spherical_transmit_delay_model = SphericalTransmitDelayModel.hybrid
        self.pw_margin = 1e-3
        self.lens_delay = 0.0
        self.blending_power = 0.5
        self.receive_apodization = Apodization()
        self.transmit_apodization = Apodization()
        self.transmit_delay = None
        self.receive_delay = None
        self.elapsed_time = None
        self.beamformed_data = None
        # GB300 additions
        self.precision = Precision.fp32
        # "table": the das_c drop-in on single-precision tables (bit-level das_c semantics);
        # "fast": on-the-fly geometry, channel data stored as `precision`
        self.engine = "table"
        self.rf_mode = "analytic"  # "analytic" (das.m semantics) | "real" (real RF in, real out)
        self.epilogue = False      # fast engine, dimension.transmit: also CF / simplified-DMAS
        self.epilogue_outputs = None
        # the last geometry on the device (tables or fast-path geometry) and the content
        # key it was built from: go() on a new frame of the same acquisition reuses it
        self._geometry = (None, None)
        # True: the caller promises the geometry is unchanged between go() calls, so a
        # cached device geometry is reused without hashing the scan, probe and waves
        # again (call invalidate() after changing any of them)
        self.geometry_fixed = False

    # -- geometry cache ---------------------------------------------------------
    def geometry_key(self, engine: str, dev) -> bytes:
        """Digest of everything the delays, apodizations and phase depend on: probe and
        pixel positions, the waves, acquisition scalars, delay-model settings and both
        apodizations.  Equal keys mean equal tables (das.m:91-209, 306-309)."""
        cd, scan = self.channel_data, self.scan
        h = hashlib.blake2b(digest_size=20)
        add = lambda *v: h.update(repr(v).encode())
        arr = lambda a: h.update(np.ascontiguousarray(np.asarray(a, np.float64)).tobytes())
        add(engine, str(dev), type(scan).__name__, scan.N_pixels, cd.probe.N_elements, len(cd.sequence))
        arr(cd.probe.xyz)
        arr(scan.xyz)
        arr(np.atleast_1d(np.asarray(scan.reference_distance, np.float64)))
        for w in cd.sequence:
            add(int(w.wavefront), w.source.distance, w.source.azimuth, w.source.elevation, w.origin.distance,
                w.origin.azimuth, w.origin.elevation, w.delay, w.sound_speed)
        add(float(cd.sampling_frequency), float(cd.initial_time), float(cd.modulation_frequency),
            float(cd.sound_speed), float(self.lens_delay), int(self.spherical_transmit_delay_model),
            float(self.pw_margin), float(self.blending_power))
        for a in (self.receive_apodization, self.transmit_apodization):
            o = a.origin
            add(int(a.window), a.f_number, a.tilt, a.minimum_aperture, a.maximum_aperture, a.grating_lobe_angle,
                a.MLA, a.MLA_overlap, None if o is None else (o.distance, o.azimuth, o.elevation))
            if a.apodization_vector is not None:
                arr(a.apodization_vector)
        return h.digest()

    def invalidate(self) -> None:
        """Drop the cached device geometry; the next go() rebuilds it."""
        self._geometry = (None, None)

    def _cached(self, engine: str, dev, build):
        if self.geometry_fixed and self._geometry[0] is not None and self._geometry[0][:2] == (engine, str(dev)):
            return self._geometry[1]
        key = (engine, str(dev), self.geometry_key(engine, dev))
        if self._geometry[0] != key:
            self._geometry = (None, None)  # release the old one first
            self._geometry = (key, build())
        return self._geometry[1]

    # -- tables ---------------------------------------------------------------
    def tables(self):
        """Single-precision (tx_apo, rx_apo, tx_delay, rx_delay) as das.m builds them."""
        cd, scan = self.channel_data, self.scan
        tx_apo = self.transmit_apodization.wave_apodization(cd.sequence, scan).astype(np.float32)
        rx_apo = self.receive_apodization.aperture_apodization(cd.probe, scan).astype(np.float32)
        rx_delay = geometry.receive_delay(cd.probe, scan, cd.sound_speed,
                                          self.lens_delay).astype(np.float32)
        tx_delay = geometry.transmit_delay(
            cd.sequence, scan, self.spherical_transmit_delay_model, self.pw_margin,
            self.blending_power, self.transmit_apodization.f_number).astype(np.float32)
        self.receive_delay = rx_delay
        self.transmit_delay = tx_delay
        return tx_apo, rx_apo, tx_delay, rx_delay

    def pixel_phase(self) -> np.ndarray:
        """exp(-1j*2*w0*reference_distance/c) per pixel, in double (das.m:307-309)."""
        cd = self.channel_data
        w0 = 2 * math.pi * float(np.float32(cd.modulation_frequency))
        return np.exp(-1j * 2 * w0 * np.asarray(self.scan.reference_distance, np.float64)
                      * np.ones(self.scan.N_pixels) / cd.sound_speed)

    # -- go -------------------------------------------------------------------
    def go(self) -> BeamformedData:
        if Code(int(self.code)) != Code.gb300:
            raise ValueError("this beamformer implements code.gb300 only")
        if self.engine == "fast" or Precision(int(self.precision)) != Precision.fp32:
            return self._go_fast()
        cd, scan = self.channel_data, self.scan
        dev = torch.device("cuda", int(self.gpu_id))
        fs = float(np.float32(cd.sampling_frequency))
        t0 = float(np.float32(cd.initial_time))
        fd = float(np.float32(cd.modulation_frequency))
        w0 = 2 * math.pi * fd
        T = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).to(dev)

        def build():
            tx_apo, rx_apo, tx_delay, rx_delay = self.tables()
            ph = None
            if abs(w0) > np.finfo(np.float64).eps:
                ph = torch.from_numpy(self.pixel_phase().astype(np.complex64)).to(dev)
            return (T(tx_apo), T(rx_apo), T(tx_delay), T(rx_delay), ph, tx_delay, rx_delay)

        d_txa, d_rxa, d_txd, d_rxd, ph, self.transmit_delay, self.receive_delay = self._cached("table", dev, build)
        ch = self._channels(dev, w0)
        t_start = time.perf_counter()
        out = kernels.das_table_f32(ch, fs, t0, d_txa, d_rxa, d_txd, d_rxd, fd, self.dimension)
        if ph is not None:
            kernels.apply_pixel_phase(out, ph)
        torch.cuda.synchronize(dev)
        self.elapsed_time = time.perf_counter() - t_start
        self.beamformed_data = BeamformedData(scan, kernels.to_matlab_order(out))
        return self.beamformed_data

    def _channels(self, dev, w0):
        ch = channel_tensor(self.channel_data.data, dev)
        if abs(w0) < np.finfo(np.float64).eps:
            if not ch.is_complex() and self.rf_mode == "analytic":
                ch = hilbert_last(ch)
        elif not ch.is_complex():
            raise ValueError("The modulation frequency > 0 but the input data is real. Check inputs.")
        return ch

    def fast_geometry(self, dev, tile_block=None, tile_order: str = "cost",
                      ctas_per_tile: int = 0, stage_shape: int = 0) -> "fast.FastGeometry":
        """Device geometry for the fast engine; ``tile_block`` / ``tile_order`` /
        ``ctas_per_tile`` / ``stage_shape`` as chosen by ``autotune`` (default: the
        library's own)."""
        from . import fast

        cd = self.channel_data
        fd = float(np.float32(cd.modulation_frequency))
        ph = self.pixel_phase() if abs(fd) > 0 else None
        return fast.FastGeometry(cd.probe, self.scan, cd.sequence, float(cd.sampling_frequency),
                                 float(cd.initial_time), fd, float(cd.sound_speed), dev,
                                 self.receive_apodization, self.transmit_apodization,
                                 self.lens_delay, self.spherical_transmit_delay_model,
                                 self.pw_margin, self.blending_power, pixel_phase=ph,
                                 tile_block=tile_block, tile_order=tile_order, ctas_per_tile=ctas_per_tile,
                                 stage_shape=stage_shape)

    def _go_fast(self) -> BeamformedData:
        from . import fast

        cd, scan = self.channel_data, self.scan
        dev = torch.device("cuda", int(self.gpu_id))
        fd = float(np.float32(cd.modulation_frequency))
        ch = self._channels(dev, 2 * math.pi * fd)
        geom = self._cached("fast", dev, lambda: self.fast_geometry(dev))
        prec = Precision(int(self.precision))
        t_start = time.perf_counter()
        st = fast.convert_channels(ch, prec)
        F, W, N, L = ch.shape
        epi = bool(self.epilogue) and int(self.dimension) == int(Dimension.transmit)
        outs = fast.das_fast(st, prec, ch.is_complex(), geom, self.dimension, F=F, epilogue=epi, L=L)
        torch.cuda.synchronize(dev)
        self.elapsed_time = time.perf_counter() - t_start
        self.epilogue_outputs = {k: v for k, v in outs.items() if k not in ("cube", "flags")} if epi else None
        self.beamformed_data = BeamformedData(scan, kernels.to_matlab_order(outs["cube"]))
        return self.beamformed_data
