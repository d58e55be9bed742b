"""Fast path: reduced-precision channel storage and on-the-fly geometry.

``FastGeometry`` turns a probe / scan / sequence / apodization description
(the inputs of midprocess.das) into the device-side ``ustb_das_geometry`` of
the C-ABI: element and pixel positions, one ``ustb_wave`` per transmit event,
and a tile map that groups pixels into compact tiles of 512 so that every
(channel, wave) sample window of a tile stays short (``plan_tiles``).  Anything
the kernel cannot form on the fly (focused waves in the hybrid margin, the
unified and blended models, tilted or vector apodizations) is passed as a
single-precision table computed by ``geometry`` exactly as das.m does.
"""
from __future__ import annotations

import ctypes
import math
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib, geometry
from .enums import Dimension, Precision, SphericalTransmitDelayModel as STDM, Wavefront, Window
from .geometry import Apodization
from .uff import LinearScan, Probe, Scan, SectorScan, Wave

TILE = 512
SLOT_HALF = 79          # kernel: max relative delay (samples) of each component
SPAN_LIMIT = 74.0       # planner: keep tile spans below this many samples
STORE = {Precision.fp32: 0, Precision.fp16: 1, Precision.bf16: 2}
TORCH_STORE = {Precision.fp32: torch.float32, Precision.fp16: torch.float16, Precision.bf16: torch.bfloat16}
FLAG_WINDOW_OVERFLOW = 1


class CWave(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("dir", ctypes.c_float * 3), ("src", ctypes.c_float * 3),
                ("offset", ctypes.c_float), ("sound_speed", ctypes.c_float), ("delay", ctypes.c_float),
                ("apodization", ctypes.c_float), ("reserved", ctypes.c_float)]


class CGeometry(ctypes.Structure):
    _fields_ = [("n_elements", ctypes.c_int64), ("element_xyz", ctypes.c_void_p),
                ("n_pixels", ctypes.c_int64), ("pixel_xyz", ctypes.c_void_p),
                ("n_tiles", ctypes.c_int64), ("tile_pixels", ctypes.c_void_p),
                ("n_waves", ctypes.c_int64), ("waves", ctypes.c_void_p),
                ("tx_delay_table", ctypes.c_void_p), ("tx_apo_table", ctypes.c_void_p),
                ("rx_apo_table", ctypes.c_void_p), ("pixel_phase", ctypes.c_void_p),
                ("fs", ctypes.c_float), ("t0", ctypes.c_float), ("fd", ctypes.c_float),
                ("sound_speed", ctypes.c_float), ("lens_delay", ctypes.c_float),
                ("rx_window", ctypes.c_int32), ("rx_f_number", ctypes.c_float * 2),
                ("rx_min_aperture", ctypes.c_float * 2), ("rx_max_aperture", ctypes.c_float * 2),
                ("rx_use_origin", ctypes.c_int32), ("rx_origin", ctypes.c_float * 3),
                ("cf_threshold", ctypes.c_float), ("ctas_per_tile", ctypes.c_int32),
                ("stage_shape", ctypes.c_int32)]


class COutputs(ctypes.Structure):
    _fields_ = [("cube", ctypes.c_void_p), ("das", ctypes.c_void_p), ("cf", ctypes.c_void_p),
                ("cf_image", ctypes.c_void_p), ("sdmas", ctypes.c_void_p)]


class CRequest(ctypes.Structure):
    _fields_ = [("ch", ctypes.c_void_p), ("storage", ctypes.c_int32), ("is_complex", ctypes.c_int32),
                ("L", ctypes.c_int64), ("N", ctypes.c_int64), ("W", ctypes.c_int64), ("F", ctypes.c_int64),
                ("geometry", ctypes.c_void_p), ("dimension", ctypes.c_int32), ("epilogue", ctypes.c_int32),
                ("out", ctypes.c_void_p)]


assert ctypes.sizeof(CWave) == 48


# ---------------------------------------------------------------------------
# tile planning
# ---------------------------------------------------------------------------

def _diag(xyz: np.ndarray) -> float:
    return float(np.linalg.norm(xyz.max(axis=0) - xyz.min(axis=0)))


def _split_blocks(grid_idx: np.ndarray, xyz: np.ndarray, limit: float, out: list):
    """Recursively split an index block (ndarray of pixel ids, any dims) until its
    bounding-box diagonal is below ``limit`` metres (or it is one pixel)."""
    stack = [grid_idx]
    while stack:
        b = stack.pop()
        flat = b.ravel()
        if flat.size == 0:
            continue
        if flat.size == 1 or _diag(xyz[flat]) <= limit:
            out.append(flat)
            continue
        # split the axis with the largest physical extent
        ext = []
        for ax in range(b.ndim):
            if b.shape[ax] < 2:
                ext.append(-1.0)
                continue
            first = np.take(b, 0, axis=ax).ravel()
            last = np.take(b, b.shape[ax] - 1, axis=ax).ravel()
            ext.append(float(np.linalg.norm(xyz[last].mean(0) - xyz[first].mean(0))))
        ax = int(np.argmax(ext))
        h = b.shape[ax] // 2
        stack.append(np.take(b, range(0, h), axis=ax))
        stack.append(np.take(b, range(h, b.shape[ax]), axis=ax))


def _block_dims(spacing, shape, ndim_target=TILE):
    """Block shape with product <= TILE balancing the physical extents."""
    sp = [max(s, 1e-12) for s in spacing]
    dims = [1] * len(sp)
    while True:
        best, bi = None, None
        for i in range(len(sp)):
            prod = int(np.prod(dims)) * 2
            if prod > ndim_target or dims[i] >= shape[i]:
                continue
            ext = dims[i] * sp[i]
            if best is None or ext < best:
                best, bi = ext, i
        if bi is None:
            return dims
        dims[bi] *= 2


def plan_tiles(scan: Scan, fs: float, sound_speed: float, span_limit: float = SPAN_LIMIT,
               block: Optional[Sequence[int]] = None) -> np.ndarray:
    """Group pixel indices into tiles of 512 lanes (-1 = idle lane).

    A tile's receive and transmit delay spans are bounded by its bounding-box
    diagonal; tiles are shrunk until that diagonal is below
    ``span_limit`` samples of one-way travel.  ``block``: the tile's pixel block
    along the scan's axes (depth, lateral, elevation), product <= 512; default:
    the block whose physical extents are the most even."""
    xyz = scan.xyz
    P = scan.N_pixels
    limit = span_limit * sound_speed / fs
    if isinstance(scan, LinearScan):
        shape = (scan.z_axis.size, scan.x_axis.size, scan.y_axis.size)
        spacing = [np.mean(np.abs(np.diff(a))) if a.size > 1 else 0.0
                   for a in (scan.z_axis, scan.x_axis, scan.y_axis)]
    elif isinstance(scan, SectorScan):
        shape = (scan.depth_axis.size, scan.azimuth_axis.size, scan.elevation_axis.size)
        dr = np.mean(np.abs(np.diff(scan.depth_axis))) if scan.depth_axis.size > 1 else 0.0
        rmax = float(np.max(np.abs(scan.depth_axis)))
        da = rmax * (np.mean(np.abs(np.diff(scan.azimuth_axis))) if scan.azimuth_axis.size > 1 else 0.0)
        de = rmax * (np.mean(np.abs(np.diff(scan.elevation_axis))) if scan.elevation_axis.size > 1 else 0.0)
        spacing = [dr, da, de]
    else:
        # unstructured: order by a coarse spatial grid, then chunk
        cell = limit / 2
        key = np.floor((xyz - xyz.min(0)) / cell).astype(np.int64)
        order = np.lexsort((key[:, 2], key[:, 0], key[:, 1]))
        blocks = []
        for i in range(0, P, TILE):
            _split_blocks(order[i:i + TILE], xyz, limit, blocks)
        return _pack(blocks)
    idx = np.arange(P).reshape(shape, order="F")
    if block is None:
        bd = _block_dims(spacing, shape)
    else:
        bd = [max(1, min(int(b), n)) for b, n in zip(tuple(block) + (1,) * (3 - len(block)), shape)]
        if int(np.prod(bd)) > TILE:
            raise ValueError(f"tile block {tuple(block)} holds more than {TILE} pixels")
    blocks = []
    for i in range(0, shape[0], bd[0]):
        for j in range(0, shape[1], bd[1]):
            for k in range(0, shape[2], bd[2]):
                _split_blocks(idx[i:i + bd[0], j:j + bd[1], k:k + bd[2]], xyz, limit, blocks)
    return _pack(blocks)


def refine_tiles(tiles: np.ndarray, xyz: np.ndarray, tx_samples: np.ndarray,
                 span_limit: float = SPAN_LIMIT) -> np.ndarray:
    """Split tiles whose tabulated transmit delays ([P, W], in samples) span more
    than ``span_limit`` over the tile (e.g. across the discontinuity of the hybrid
    focused-wave model at the edges of its focal band)."""
    out = []
    stack = [t[t >= 0] for t in tiles]
    while stack:
        b = stack.pop()
        if b.size == 0:
            continue
        td = tx_samples[b]
        span = float(np.max(td.max(axis=0) - td.min(axis=0))) if b.size > 1 else 0.0
        if span <= span_limit or b.size == 1:
            out.append(b)
            continue
        ext = xyz[b].max(0) - xyz[b].min(0)
        ax = int(np.argmax(ext))
        order = b[np.argsort(xyz[b, ax], kind="stable")]
        h = order.size // 2
        stack.append(order[:h])
        stack.append(order[h:])
    return _pack(out)


def order_by_cost(tiles: np.ndarray, xyz: np.ndarray, probe_xyz: np.ndarray, rx: "Apodization") -> np.ndarray:
    """Reorder tiles most-expensive first.  A tile's cost is the number of
    channels whose receive window can be nonzero somewhere in the tile (the
    kernel's own bounding-box rule), so the block scheduler hands the long tiles
    out first and the short ones fill the tail."""
    if len(tiles) < 2 or rx is None or rx.window == Window.none or rx.apodization_vector is not None:
        return tiles
    lo = np.empty((len(tiles), 3))
    hi = np.empty((len(tiles), 3))
    for t, row in enumerate(tiles):
        b = xyz[row[row >= 0]]
        lo[t], hi[t] = b.min(0), b.max(0)
    ex, ey, ez = probe_xyz[:, 0][None, :], probe_xyz[:, 1][None, :], probe_xyz[:, 2][None, :]
    xd = np.maximum(0, np.maximum(lo[:, 0:1] - ex, ex - hi[:, 0:1]))
    yd = np.maximum(0, np.maximum(lo[:, 1:2] - ey, ey - hi[:, 1:2]))
    zmax = np.maximum(np.abs(lo[:, 2:3] - ez), np.abs(hi[:, 2:3] - ez))
    zx = np.clip(zmax, rx.minimum_aperture[0] * rx.f_number[0], rx.maximum_aperture[0] * rx.f_number[0])
    zy = np.clip(zmax, rx.minimum_aperture[1] * rx.f_number[1], rx.maximum_aperture[1] * rx.f_number[1])
    with np.errstate(divide="ignore", invalid="ignore"):
        act = ~((rx.f_number[0] * xd / zx > 0.5) | (rx.f_number[1] * yd / zy > 0.5))
    cost = act.sum(axis=1)
    return tiles[np.argsort(-cost, kind="stable")]


def _pack(blocks) -> np.ndarray:
    T = len(blocks)
    tiles = np.full((T, TILE), -1, dtype=np.int32)
    for t, b in enumerate(blocks):
        tiles[t, :b.size] = b
    return tiles


# ---------------------------------------------------------------------------
# geometry
# ---------------------------------------------------------------------------

def _wave_struct(wave: Wave, kind: int, apo: float, offset: float = 0.0) -> CWave:
    s = wave.source
    cw = CWave()
    cw.kind = kind
    if kind == 0:
        ce = math.cos(s.elevation)
        cw.dir[0] = math.sin(s.azimuth) * ce
        cw.dir[1] = math.sin(s.elevation)
        cw.dir[2] = math.cos(s.azimuth) * ce
    elif kind == 1:
        cw.src[0], cw.src[1], cw.src[2] = s.x, s.y, s.z
    cw.offset = offset
    cw.sound_speed = wave.sound_speed
    cw.delay = wave.delay
    cw.apodization = apo
    return cw


class FastGeometry:
    """Device-side geometry of one request for ``ustb_das_fast``."""

    def __init__(self, probe: Probe, scan: Scan, sequence: Sequence[Wave], fs: float, t0: float,
                 fd: float, sound_speed: float, device, rx_apodization: Optional[Apodization] = None,
                 tx_apodization: Optional[Apodization] = None, lens_delay: float = 0.0,
                 model: STDM = STDM.hybrid, pw_margin: float = 1e-3, blending_power: float = 0.5,
                 pixel_phase: Optional[np.ndarray] = None, cf_threshold: float = 0.16,
                 tiles: Optional[np.ndarray] = None, tile_block: Optional[Sequence[int]] = None,
                 tile_order: str = "cost", ctas_per_tile: int = 0, stage_shape: int = 0):
        dev = torch.device(device)
        rx = rx_apodization or Apodization()
        tx = tx_apodization or Apodization()
        self.probe, self.scan, self.sequence = probe, scan, list(sequence)
        P, N, W = scan.N_pixels, probe.N_elements, len(self.sequence)
        self.P, self.N, self.W = P, N, W
        f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)
        self.d_el = f32(probe.xyz)
        self.d_px = f32(scan.xyz)
        self.tile_block, self.tile_order = tile_block, tile_order
        if tiles is None:
            self.tiles = plan_tiles(scan, fs, sound_speed, block=tile_block)
            if tile_order == "cost" and rx.origin is None and not isinstance(scan, SectorScan):
                self.tiles = order_by_cost(self.tiles, scan.xyz, probe.xyz, rx)
        else:
            self.tiles = np.asarray(tiles, np.int32)
        if self.tiles.ndim != 2 or self.tiles.shape[1] != TILE:
            raise ValueError(f"tile map must be [n_tiles, {TILE}], got {self.tiles.shape}")
        if self.tiles.size and (self.tiles.max() >= P or self.tiles.min() < -1):
            raise ValueError("tile map holds pixel indices outside [0, P) other than -1")
        self.d_tiles = torch.from_numpy(np.ascontiguousarray(self.tiles)).to(dev)

        # transmit events
        table_waves = []
        structs = []
        tx_const = self._tx_apodization_constants(tx)
        for w, wave in enumerate(self.sequence):
            wf = Wavefront(int(wave.wavefront))
            s = wave.source
            a = 1.0 if tx_const is None else float(tx_const[w])
            if wf == Wavefront.plane or (wf == Wavefront.spherical and math.isinf(s.distance)):
                structs.append(_wave_struct(wave, 0, a))
            elif wf == Wavefront.photoacoustic:
                structs.append(_wave_struct(wave, 2, a))
            elif s.z < 0:
                structs.append(_wave_struct(wave, 1, a, -abs(s.distance)))
            else:
                m = STDM(int(model))
                band = np.any((scan.z < s.z + pw_margin) & (scan.z > s.z - pw_margin))
                if m == STDM.spherical or (m == STDM.hybrid and not band):
                    structs.append(_wave_struct(wave, 1, a, s.distance))
                else:
                    structs.append(_wave_struct(wave, 3, a))
                    table_waves.append(w)
        arr = (CWave * max(W, 1))(*structs)
        self.d_waves = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(dev)
        self.d_txdelay = None
        if table_waves:
            td = geometry.transmit_delay(self.sequence, scan, model, pw_margin, blending_power,
                                         tx.f_number).astype(np.float32)
            self.d_txdelay = f32(td.T)
            if tiles is None:
                self.tiles = refine_tiles(self.tiles, scan.xyz, td[:, table_waves].astype(np.float64) * fs)
                self.d_tiles = torch.from_numpy(self.tiles).to(dev)
        self.d_txapo = None
        if tx_const is None:
            self.d_txapo = f32(tx.wave_apodization(self.sequence, scan).T)

        # receive apodization
        self.d_rxapo = None
        self.rx_window = int(rx.window)
        on_the_fly = (rx.apodization_vector is None and rx.window not in (Window.sta, Window.scanline)
                      and rx.tilt == (0.0, 0.0))
        if not on_the_fly:
            self.d_rxapo = f32(rx.aperture_apodization(probe, scan).T)
            self.rx_window = 0
        origin = rx.origin
        if origin is None and isinstance(scan, SectorScan):
            origin = scan.origin
        self.d_phase = None
        if pixel_phase is not None:
            self.d_phase = torch.from_numpy(np.asarray(pixel_phase, np.complex64)).to(dev)

        g = CGeometry()
        g.n_elements, g.element_xyz = N, self.d_el.data_ptr()
        g.n_pixels, g.pixel_xyz = P, self.d_px.data_ptr()
        g.n_tiles, g.tile_pixels = self.tiles.shape[0], self.d_tiles.data_ptr()
        g.n_waves, g.waves = W, self.d_waves.data_ptr()
        g.tx_delay_table = self.d_txdelay.data_ptr() if self.d_txdelay is not None else None
        g.tx_apo_table = self.d_txapo.data_ptr() if self.d_txapo is not None else None
        g.rx_apo_table = self.d_rxapo.data_ptr() if self.d_rxapo is not None else None
        g.pixel_phase = self.d_phase.data_ptr() if self.d_phase is not None else None
        g.fs, g.t0, g.fd = fs, t0, fd
        g.sound_speed, g.lens_delay = sound_speed, lens_delay
        g.rx_window = self.rx_window
        g.rx_f_number[0], g.rx_f_number[1] = rx.f_number
        g.rx_min_aperture[0], g.rx_min_aperture[1] = rx.minimum_aperture
        g.rx_max_aperture[0], g.rx_max_aperture[1] = rx.maximum_aperture
        g.rx_use_origin = 1 if origin is not None else 0
        if origin is not None:
            g.rx_origin[0], g.rx_origin[1], g.rx_origin[2] = origin.x, origin.y, origin.z
        g.cf_threshold = cf_threshold
        if ctas_per_tile not in (0, 1, 2, 3, 4):
            raise ValueError("ctas_per_tile must be 0 (library's choice) or 1 to 4")
        g.ctas_per_tile = int(ctas_per_tile)
        self.ctas_per_tile = int(ctas_per_tile)
        if stage_shape not in (0, 1, 2, 3):
            raise ValueError("stage_shape must be 0 (library's choice), 1, 2 or 3")
        g.stage_shape = int(stage_shape)
        self.stage_shape = int(stage_shape)
        self.c = g
        self.device = dev

    def _tx_apodization_constants(self, tx: Apodization):
        """Per-wave constant tx apodization when it does not vary over pixels, else None."""
        W = len(self.sequence)
        if tx.apodization_vector is not None:
            v = np.asarray(tx.apodization_vector, np.float64).ravel()
            return v if v.size == W else None
        if tx.window == Window.none:
            return np.ones(W)
        if tx.window == Window.scanline:
            return None
        planes = all(Wavefront(int(w.wavefront)) == Wavefront.plane or math.isinf(w.source.distance)
                     for w in self.sequence)
        if not planes:
            return None
        one = Scan([0.0], [0.0], [1.0])
        return tx.wave_apodization(self.sequence, one)[0]

    def units(self, F: int = 1) -> int:
        return self.P * self.N * self.W * F


def entry_bytes(L: int, N: int, W: int, F: int, is_complex: bool) -> int:
    """Bytes of the FP32 interpolation entries ``ustb_das_fast`` builds for one request
    (16 per complex sample, 8 per real one)."""
    return L * N * W * F * (16 if is_complex else 8)


def convert_channels(src: torch.Tensor, precision: Precision, scale: float = 1.0) -> torch.Tensor:
    """Channel data -> device storage type through ``ustb_convert_channels``.

    ``src``: complex64 / float32 / int16 / float16 CUDA tensor in the ABI layout (for
    int16 I/Q the last dimension holds interleaved I, Q).  Complex input keeps its
    shape and becomes (..., 2) real pairs of the storage type."""
    if src.is_complex():
        flat = torch.view_as_real(src)
        st = 0
    elif src.dtype == torch.float32:
        flat, st = src, 0
    elif src.dtype == torch.int16:
        flat, st = src, 1
    elif src.dtype == torch.float16:
        flat, st = src, 2
    else:
        raise TypeError(f"unsupported source dtype {src.dtype}")
    dst = torch.empty(flat.shape, dtype=TORCH_STORE[Precision(precision)], device=src.device)
    with torch.cuda.device(src.device):
        _lib.call("ustb_convert_channels", flat.data_ptr(), st, dst.data_ptr(), STORE[Precision(precision)],
                  flat.numel(), float(scale), torch.cuda.current_stream(src.device).cuda_stream)
    return dst


def build_entries(ch: torch.Tensor, precision: Precision, is_complex: bool, N: int, W: int, F: int = 1,
                  L: Optional[int] = None) -> torch.Tensor:
    """``ustb_build_entries``: the FP32 interpolation entries of channel data in its
    storage type, as a uint8 device tensor for ``das_fast(..., entries=...)``."""
    if L is None:
        L = ch.numel() // ((2 if is_complex else 1) * N * W * F)
    nbytes = int(_lib.lib().ustb_entries_bytes(L, N, W, F, int(is_complex)))
    out = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=ch.device)
    with torch.cuda.device(ch.device):
        _lib.call("ustb_build_entries", ch.data_ptr(), STORE[Precision(precision)], int(is_complex), L, N, W, F,
                  out.data_ptr(), torch.cuda.current_stream(ch.device).cuda_stream)
    return out


def das_fast(ch: torch.Tensor, precision: Precision, is_complex: bool, geom: FastGeometry,
             dimension=Dimension.both, F: int = 1, epilogue: bool = False, cube: bool = True,
             flags: Optional[torch.Tensor] = None, check: bool = True, L: Optional[int] = None,
             entries: Optional[torch.Tensor] = None):
    """Run ``ustb_das_fast``.  ``ch`` holds [L,N,W,F] samples of the storage type
    (complex: trailing (re, im) pairs).  Returns a dict of output tensors in the ABI
    layout: 'cube' (F, Wk, Nk, P) and, with the epilogue, 'das', 'cf', 'cf_image',
    'sdmas' of shape (F, P).  With ``entries`` (from ``build_entries`` of the same
    data) only the beamforming kernel runs (``ustb_das_fast_entries``); ``ch`` then
    only supplies the device and, without ``L``, the sample count."""
    dev = ch.device
    P, N, W = geom.P, geom.N, geom.W
    if L is None:
        L = ch.numel() // ((2 if is_complex else 1) * N * W * F)
    outs = {}
    o = COutputs()
    dt = torch.complex64 if is_complex else torch.float32
    if cube:
        from .kernels import out_shape_abi

        outs["cube"] = torch.empty(out_shape_abi(P, N, W, F, dimension), dtype=dt, device=dev)
        o.cube = outs["cube"].data_ptr()
    if epilogue:
        outs["das"] = torch.empty((F, P), dtype=torch.complex64, device=dev)
        outs["cf"] = torch.empty((F, P), dtype=torch.float32, device=dev)
        outs["cf_image"] = torch.empty((F, P), dtype=torch.complex64, device=dev)
        outs["sdmas"] = torch.empty((F, P), dtype=torch.float32, device=dev)
        o.das, o.cf = outs["das"].data_ptr(), outs["cf"].data_ptr()
        o.cf_image, o.sdmas = outs["cf_image"].data_ptr(), outs["sdmas"].data_ptr()
    if flags is None:
        flags = torch.zeros(1, dtype=torch.int32, device=dev)
    with torch.cuda.device(dev):
        if entries is None:
            _lib.call("ustb_das_fast", ch.data_ptr(), STORE[Precision(precision)], int(is_complex), L, N, W, F,
                      ctypes.byref(geom.c), int(dimension), int(epilogue), ctypes.byref(o), flags.data_ptr(),
                      torch.cuda.current_stream(dev).cuda_stream)
        else:
            _lib.call("ustb_das_fast_entries", entries.data_ptr(), int(is_complex), L, N, W, F,
                      ctypes.byref(geom.c), int(dimension), int(epilogue), ctypes.byref(o), flags.data_ptr(),
                      torch.cuda.current_stream(dev).cuda_stream)
    if check:
        fl = int(flags.item())
        if fl & FLAG_WINDOW_OVERFLOW:
            raise _lib.UstbError(7, "a tile's sample window overflowed its slot; plan smaller tiles")
    outs["flags"] = flags
    return outs


class Request:
    """One beamforming request for ``das_fast_batch``: channel data already in the
    storage type on the device, its geometry, and the outputs to fill."""

    def __init__(self, ch: torch.Tensor, precision: Precision, is_complex: bool, geom: FastGeometry,
                 dimension=Dimension.both, F: int = 1, L: Optional[int] = None, epilogue: bool = False,
                 cube: bool = True):
        self.ch, self.precision, self.is_complex, self.geom = ch, Precision(precision), bool(is_complex), geom
        self.dimension, self.F, self.epilogue = int(dimension), int(F), bool(epilogue)
        P, N, W = geom.P, geom.N, geom.W
        self.L = int(L) if L is not None else ch.numel() // ((2 if is_complex else 1) * N * W * F)
        dev = ch.device
        self.outputs = {}
        self.c_out = COutputs()
        if cube:
            from .kernels import out_shape_abi

            dt = torch.complex64 if is_complex else torch.float32
            self.outputs["cube"] = torch.empty(out_shape_abi(P, N, W, F, dimension), dtype=dt, device=dev)
            self.c_out.cube = self.outputs["cube"].data_ptr()
        if epilogue:
            for k, dt in (("das", torch.complex64), ("cf", torch.float32), ("cf_image", torch.complex64),
                          ("sdmas", torch.float32)):
                self.outputs[k] = torch.empty((F, P), dtype=dt, device=dev)
            self.c_out.das, self.c_out.cf = self.outputs["das"].data_ptr(), self.outputs["cf"].data_ptr()
            self.c_out.cf_image = self.outputs["cf_image"].data_ptr()
            self.c_out.sdmas = self.outputs["sdmas"].data_ptr()

    def c_struct(self) -> CRequest:
        q = CRequest()
        q.ch = self.ch.data_ptr()
        q.storage = STORE[self.precision]
        q.is_complex = int(self.is_complex)
        q.L, q.N, q.W, q.F = self.L, self.geom.N, self.geom.W, self.F
        q.geometry = ctypes.addressof(self.geom.c)
        q.dimension = self.dimension
        q.epilogue = int(self.epilogue)
        q.out = ctypes.addressof(self.c_out)
        return q


def workspace_bytes(requests: Sequence[Request]) -> int:
    """Device bytes ``das_fast_batch(..., workspace=...)`` needs for these requests."""
    if not requests:
        return 0
    arr = (CRequest * len(requests))(*[r.c_struct() for r in requests])
    return int(_lib.lib().ustb_das_fast_workspace_bytes(ctypes.addressof(arr), len(requests)))


def das_fast_batch(requests: Sequence[Request], scratch: Optional[torch.Tensor] = None, stream=None,
                   workspace: Optional[torch.Tensor] = None, max_ctas: int = 0):
    """Beamform a batch of requests with the persistent work-queue kernel
    (``ustb_das_fast_batch_ex``).  Returns the int64 scratch tensor (word 0 = flags).

    ``workspace``: optional uint8 device tensor of at least ``workspace_bytes(requests)``
    bytes (256-byte aligned, as torch allocations are) that holds the interpolation
    entries; without it the library allocates them from its own pool.
    ``max_ctas``: at most this many persistent CTAs (0 = one per SM), so that launches
    on other streams can use the remaining SMs meanwhile."""
    if not requests:
        return scratch
    dev = requests[0].ch.device
    n = len(requests)
    if scratch is None or scratch.numel() < n + 1:
        scratch = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    arr = (CRequest * n)(*[r.c_struct() for r in requests])
    st = stream.cuda_stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    with torch.cuda.device(dev):
        if workspace is None:
            _lib.call("ustb_das_fast_batch_ex", ctypes.addressof(arr), n, scratch.data_ptr(), None, 0, int(max_ctas), st)
        else:
            _lib.call("ustb_das_fast_batch_ex", ctypes.addressof(arr), n, scratch.data_ptr(), workspace.data_ptr(),
                      workspace.numel() * workspace.element_size(), int(max_ctas), st)
    return scratch


class FramePipeline:
    """Beamform a stream of frames that live in host memory: frame k+1's copy in and
    frame k-1's copy out overlap frame k's beamforming.

    ``depth`` CUDA streams take frames in turn, each with its own device input
    buffer; a frame's host->device copy, its ``ustb_das_fast`` call and the copy of
    its image back to host memory are ordered on its stream.  ``submit`` returns at
    once; ``synchronize`` waits for every submitted frame."""

    def __init__(self, geom: FastGeometry, ch_shape, ch_dtype, precision: Precision, is_complex: bool,
                 dimension=Dimension.both, L: Optional[int] = None, depth: int = 2):
        dev = geom.device
        self.geom, self.precision, self.is_complex = geom, Precision(precision), bool(is_complex)
        self.dimension, self.L = int(dimension), L
        self.streams = [torch.cuda.Stream(dev) for _ in range(depth)]
        self.inputs = [torch.empty(ch_shape, dtype=ch_dtype, device=dev) for _ in range(depth)]
        self.flags = [torch.zeros(1, dtype=torch.int32, device=dev) for _ in range(depth)]
        self.k = 0

    def start(self) -> None:
        """Order the pipeline after the work already queued on the current stream."""
        cur = torch.cuda.current_stream(self.geom.device)
        for s in self.streams:
            s.wait_stream(cur)

    def submit(self, host_frame: torch.Tensor, host_out: torch.Tensor) -> None:
        """Queue one frame: ``host_frame`` (pinned, the storage type of ``precision``
        or complex64 for FP32) in, its image into ``host_out`` (pinned)."""
        i = self.k % len(self.streams)
        self.k += 1
        s, d_in = self.streams[i], self.inputs[i]
        with torch.cuda.stream(s):
            d_in.copy_(host_frame, non_blocking=True)
            o = das_fast(d_in, self.precision, self.is_complex, self.geom, self.dimension, L=self.L,
                         flags=self.flags[i], check=False)
            host_out.copy_(o["cube"], non_blocking=True)

    def synchronize(self) -> None:
        """Make the current stream wait for every submitted frame (stream-ordered)."""
        cur = torch.cuda.current_stream(self.geom.device)
        for s in self.streams:
            cur.wait_stream(s)

    def overflowed(self) -> bool:
        return any(int(f.item()) & FLAG_WINDOW_OVERFLOW for f in self.flags)
