"""Resident plans and the native continuous-batching server (``ustb_plan_*``,
``ustb_serve_*``).

A ``Plan`` copies one acquisition's geometry to the device once (the library
plans the tiles itself unless given a tile map), so every later frame needs only
its channel data; the reference rebuilds its tables on every ``go()``
(+midprocess/das.m:91-209).  A ``Server`` queues requests on plans and batches
them into persistent launches from a scheduler thread of the library, with a
completion thread marking them done; submitting returns at once with a ticket.
"""
from __future__ import annotations

import ctypes
from typing import Dict, Optional, Tuple

import numpy as np
import torch

from . import _lib
from .enums import Dimension, Precision
from .fast import STORE, COutputs, CGeometry, FastGeometry, TILE
from .uff import LinearScan, SectorScan


class CPlanDesc(ctypes.Structure):
    _fields_ = [("geometry", CGeometry), ("pixel_grid", ctypes.c_int64 * 3), ("L", ctypes.c_int64),
                ("F", ctypes.c_int64), ("storage", ctypes.c_int32), ("is_complex", ctypes.c_int32),
                ("dimension", ctypes.c_int32), ("epilogue", ctypes.c_int32)]


def pixel_grid(scan) -> Tuple[int, int, int]:
    """The scan's pixel grid, first axis fastest, or (0, 0, 0) for a pixel list."""
    if isinstance(scan, LinearScan):
        return scan.z_axis.size, scan.x_axis.size, scan.y_axis.size
    if isinstance(scan, SectorScan):
        return scan.depth_axis.size, scan.azimuth_axis.size, scan.elevation_axis.size
    return 0, 0, 0


def _host(t: Optional[torch.Tensor], keep: list) -> Optional[int]:
    if t is None:
        return None
    h = t.detach().cpu().contiguous()
    keep.append(h)
    return h.data_ptr()


def plan_desc(geom: FastGeometry, L: int, precision: Precision, is_complex: bool, dimension=Dimension.both,
              F: int = 1, epilogue: bool = False, library_tiles: bool = True):
    """(CPlanDesc with host pointers, the host arrays it points into) for a geometry."""
    keep = []
    d = CPlanDesc()
    g = CGeometry()
    ctypes.pointer(g)[0] = geom.c  # copy the scalar fields
    g.element_xyz = _host(geom.d_el, keep)
    g.pixel_xyz = _host(geom.d_px, keep)
    g.waves = _host(geom.d_waves, keep)
    g.tx_delay_table = _host(geom.d_txdelay, keep)
    g.tx_apo_table = _host(geom.d_txapo, keep)
    g.rx_apo_table = _host(geom.d_rxapo, keep)
    g.pixel_phase = _host(geom.d_phase, keep)
    if library_tiles:
        g.tile_pixels, g.n_tiles = None, 0
    else:
        t = np.ascontiguousarray(geom.tiles, np.int32)
        keep.append(t)
        g.tile_pixels, g.n_tiles = t.ctypes.data, t.shape[0]
    d.geometry = g
    d.pixel_grid[0], d.pixel_grid[1], d.pixel_grid[2] = pixel_grid(geom.scan)
    d.L, d.F = int(L), int(F)
    d.storage, d.is_complex = STORE[Precision(precision)], int(bool(is_complex))
    d.dimension, d.epilogue = int(dimension), int(bool(epilogue))
    return d, keep


def library_tiles(geom: FastGeometry, L: int = 1024) -> np.ndarray:
    """The tile map the library plans for a geometry (``ustb_plan_tiles_host``; no GPU
    needed), as an int32 array [n_tiles, TILE] with -1 for idle lanes."""
    d, keep = plan_desc(geom, L, Precision.fp32, True, Dimension.both)
    n = int(_lib.lib().ustb_plan_tiles_host(ctypes.addressof(d), None, 0))
    if n < 0:
        _lib.check(-n)
    out = np.empty((n, TILE), np.int32)
    got = int(_lib.lib().ustb_plan_tiles_host(ctypes.addressof(d), out.ctypes.data, n))
    assert got == n
    return out


class Plan:
    """A resident plan built from a ``FastGeometry`` (its arrays are read back to the
    host and handed to ``ustb_plan_create``, which copies them to the device).
    ``library_tiles``: let the library plan the tiles (default) instead of passing
    the geometry's own tile map."""

    def __init__(self, geom: FastGeometry, L: int, precision: Precision, is_complex: bool,
                 dimension=Dimension.both, F: int = 1, epilogue: bool = False, library_tiles: bool = True):
        d, keep = plan_desc(geom, L, precision, is_complex, dimension, F, epilogue, library_tiles)
        self.precision = Precision(precision)
        self.P, self.N, self.W, self.F, self.L = geom.P, geom.N, geom.W, int(F), int(L)
        self.is_complex, self.dimension, self.epilogue = bool(is_complex), int(dimension), bool(epilogue)
        self.device = geom.device
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("ustb_plan_create", ctypes.addressof(d), ctypes.byref(h))
        self.handle = h

    @property
    def n_tiles(self) -> int:
        n = int(_lib.lib().ustb_plan_tiles(self.handle))
        if n < 0:
            _lib.check(-n)
        return n

    def outputs(self, cube: bool = True) -> Tuple[Dict[str, torch.Tensor], COutputs]:
        """Fresh output tensors for one request on this plan and their C struct."""
        from .kernels import out_shape_abi

        outs, c = {}, COutputs()
        if cube:
            dt = torch.complex64 if self.is_complex else torch.float32
            outs["cube"] = torch.empty(out_shape_abi(self.P, self.N, self.W, self.F, self.dimension), dtype=dt,
                                       device=self.device)
            c.cube = outs["cube"].data_ptr()
        if self.epilogue:
            for k, dt in (("das", torch.complex64), ("cf", torch.float32), ("cf_image", torch.complex64),
                          ("sdmas", torch.float32)):
                outs[k] = torch.empty((self.F, self.P), dtype=dt, device=self.device)
                setattr(c, k, outs[k].data_ptr())
        return outs, c

    def execute(self, ch: torch.Tensor, cube: bool = True) -> Dict[str, torch.Tensor]:
        """``ustb_plan_execute`` on the current stream; ``ch`` in the plan's storage."""
        outs, c = self.outputs(cube)
        flags = torch.zeros(1, dtype=torch.int32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.call("ustb_plan_execute", self.handle, ch.data_ptr(), ctypes.byref(c), flags.data_ptr(),
                      torch.cuda.current_stream(self.device).cuda_stream)
        outs["flags"] = flags
        return outs

    def close(self):
        if self.handle:
            _lib.call("ustb_plan_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """``ustb_serve_*``: queue requests on plans; the library's scheduler thread batches
    small requests (entries within ``workspace_budget`` bytes, at most ``max_batch``)
    into persistent launches on two streams of its own, and launches each request of
    more than ``large_units`` units (0 = 2e9) alone on a third stream with at most
    SMs - ``reserve_sms`` CTAs (0: every SM); its completion threads mark them done.
    Channel data must be ready on the device when submitted (synchronize the
    producing stream first) and stays referenced until ``wait`` returns."""

    def __init__(self, workspace_budget: int = 8 << 30, max_batch: int = 16, device=None, large_units: int = 0,
                 reserve_sms: int = 0):
        self.device = torch.device(device) if device is not None else torch.device("cuda", 0)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("ustb_serve_create_ex", int(workspace_budget), int(max_batch), int(large_units),
                      int(reserve_sms), ctypes.byref(h))
        self.handle = h
        self._pending: Dict[int, tuple] = {}

    def submit(self, plan: Plan, ch: torch.Tensor, cube: bool = True) -> int:
        outs, c = plan.outputs(cube)
        t = ctypes.c_uint64()
        _lib.call("ustb_serve_submit", self.handle, plan.handle, ch.data_ptr(), ctypes.byref(c), ctypes.byref(t))
        self._pending[t.value] = (plan, ch, outs, c)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> Dict[str, torch.Tensor]:
        """Outputs of a finished request (with its flag bits under 'flags'); raises
        UstbError (USTB_E_TIMEOUT) when it is not done within ``timeout_ms``."""
        flags = ctypes.c_uint32()
        _lib.call("ustb_serve_wait", self.handle, ctypes.c_uint64(ticket), int(timeout_ms), ctypes.byref(flags))
        outs = self._pending.pop(ticket)[2]
        outs["flags"] = int(flags.value)
        return outs

    def close(self):
        if self.handle:
            _lib.call("ustb_serve_destroy", self.handle)
            self.handle = None
            self._pending.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
