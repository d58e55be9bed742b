"""Per-shape tuning of the fast path's tile plan, cached in a JSON file.

What is tuned: the pixel block of a 512-pixel tile along the scan's (depth,
lateral, elevation) axes, the order in which tiles are handed to the SMs (most
receive channels first, or scan order), the stage shape (which (channel, wave)
pairs share a shared-memory stage and the loop order: waves outer 2 x 16, channels
outer 8 x 4 or 16 x 2), and for dimension.both the number of CTAs per tile (1 to 4,
each taking an equal part of the tile's stages and adding its partial sum; tried on
the fastest plan after the other knobs, it shortens the launch's tail at the cost of
one tile setup per CTA).  The block
sets each tile's delay spans, hence the length of every staged sample window, how
many receive channels are active somewhere in the tile, and how the 32 pixels of a
warp spread over shared-memory banks; the order sets the tail of the launch; the
stage shape sets how often the receive geometry (per pixel and channel) and the
transmit geometry (per pixel and wave) are formed, and how many of a stage's slots
a short wave sequence fills (11 waves fill 11 of 16 slots of a waves-outer chunk,
11 of 12 of channels-outer chunks).  Fixed by the kernel, because measurement showed
no gain from changing them: the samples per slot (160; 104- and 80-entry slots with
3- and 4-deep buffer rings ran at the same speed) and one 512-thread CTA per SM (the
register file's limit); the persistent launches use one CTA per SM unless a caller
bounds them to share the GPU with other streams (``fast.das_fast_batch(max_ctas=)``).

Each candidate is timed with CUDA events on the caller's data; the fastest is
stored under a key made of the device name and the request's shape, so later
processes with the same shape skip the search.  The cache file is
``$USTB_GB300_TUNE_CACHE`` or ``~/.cache/ustb_gb300/tune.json``.

The reference has no tuning step: das_c's work split is fixed per pixel
(+mex/source/das_c.cpp:355-409) and das_cuda's block size is a constant
(+mex/source/das_cuda.cu:128-306).
"""
from __future__ import annotations

import json
import os
import threading
from dataclasses import dataclass, asdict
from typing import Callable, List, Optional, Sequence, Tuple

import torch

from . import fast
from .uff import LinearScan, Scan, SectorScan

_lock = threading.Lock()


@dataclass
class Choice:
    block: Optional[Tuple[int, ...]]  # None: the planner's default
    order: str                        # "cost" | "scan"
    ms: float = float("nan")          # measured time of one call (CUDA events)
    ctas_per_tile: int = 0            # dimension.both: 1 to 4 CTAs per tile, 0 = library's choice
    stage_shape: int = 0              # 1 waves outer 2x16, 2 channels outer 8x4, 3 channels outer 16x2, 0 library's


def cache_path() -> str:
    return os.environ.get("USTB_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "ustb_gb300", "tune.json"))


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key: str, choice: Choice) -> None:
    path = cache_path()
    with _lock:
        data = _load()
        data[key] = asdict(choice)
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        tmp = path + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def _grid_shape(scan: Scan) -> Optional[Tuple[int, int, int]]:
    if isinstance(scan, LinearScan):
        return scan.z_axis.size, scan.x_axis.size, scan.y_axis.size
    if isinstance(scan, SectorScan):
        return scan.depth_axis.size, scan.azimuth_axis.size, scan.elevation_axis.size
    return None


def shape_key(scan: Scan, n_elements: int, n_waves: int, L: int, F: int, precision, dimension,
              is_complex: bool, device) -> str:
    dev = torch.device(device)
    name = torch.cuda.get_device_name(dev) if dev.type == "cuda" else "cpu"
    g = _grid_shape(scan)
    return "|".join(str(v) for v in (name, type(scan).__name__, g if g else scan.N_pixels, n_elements, n_waves,
                                     L, F, int(precision), int(dimension), int(bool(is_complex))))


def shapes_for(dimension) -> List[int]:
    """Stage shapes a dimension mode runs with (ustb_das_geometry.stage_shape values)."""
    d = int(dimension)
    if d == 1:
        return [1]
    if d in (0, 2):
        return [2, 3]
    return [1, 2, 3]


def candidates(scan: Scan, both: bool = False, dimension: Optional[int] = None) -> List[Choice]:
    """The planner's default block plus power-of-two blocks of 512 pixels over the
    scan's two largest axes, each in both orders; for dimension.both also the default
    block with 1 and with 2 CTAs per tile; with ``dimension`` given, the default block
    with every stage shape that mode runs with."""
    out = [Choice(None, "cost"), Choice(None, "scan")]
    if both:
        out += [Choice(None, "cost", ctas_per_tile=1), Choice(None, "cost", ctas_per_tile=2)]
    if dimension is not None:
        out += [Choice(None, "cost", stage_shape=sh) for sh in shapes_for(dimension)]
    g = _grid_shape(scan)
    if g is None:
        return out
    nz, nx, ny = g
    if ny > 1:
        for bz, bx, by in ((8, 8, 8), (16, 8, 4), (32, 4, 4), (8, 16, 4), (4, 16, 8), (16, 16, 2)):
            out.append(Choice((bz, bx, by), "cost"))
        return out
    bz = 4
    while bz <= 256:
        bx = fast.TILE // bz
        if bz <= 2 * nz and bx <= 2 * nx:
            out.append(Choice((bz, bx, 1), "cost"))
        bz *= 2
    return out


def tune(make_geometry: Callable[..., "fast.FastGeometry"],
         run: Callable[["fast.FastGeometry"], None], key: str, reps: int = 3, refresh: bool = False,
         cands: Optional[List[Choice]] = None, scan: Optional[Scan] = None, both: bool = False,
         dimension: Optional[int] = None) -> Choice:
    """Return the cached choice for ``key``, or time every candidate and cache the fastest.

    ``make_geometry(block, order, ctas_per_tile, stage_shape)`` builds a ``FastGeometry``
    with that plan; ``run(geometry)`` launches the work to time on the current stream.
    Candidates whose plan overflows a sample window (the kernel flags it) are skipped.
    For dimension.both (``both``) the fastest candidate is then tried with 1 to 4 CTAs
    per tile."""
    if not refresh:
        hit = _load().get(key)
        if hit is not None:
            b = hit.get("block")
            return Choice(tuple(b) if b is not None else None, hit.get("order", "cost"), hit.get("ms", float("nan")),
                          int(hit.get("ctas_per_tile", 0)), int(hit.get("stage_shape", 0)))
    if cands is None:
        cands = candidates(scan, both, dimension) if scan is not None else [Choice(None, "cost")]

    def time_of(c: Choice) -> Optional[float]:
        try:
            geom = make_geometry(c.block, c.order, c.ctas_per_tile, c.stage_shape)
        except ValueError:
            return None
        try:
            run(geom)  # warm-up; raises on a window overflow
        except _lib_error() as e:
            if getattr(e, "code", None) == 7:
                return None
            raise
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            run(geom)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    best: Optional[Choice] = None
    for c in cands:
        ms = time_of(c)
        if ms is not None and (best is None or ms < best.ms):
            best = Choice(c.block, c.order, ms, c.ctas_per_tile, c.stage_shape)
    if best is None:
        raise RuntimeError("no tile plan candidate ran")
    if both:
        for cpt in range(1, 5):
            if cpt == best.ctas_per_tile:
                continue
            c = Choice(best.block, best.order, ctas_per_tile=cpt, stage_shape=best.stage_shape)
            ms = time_of(c)
            if ms is not None and ms < best.ms:
                best = Choice(c.block, c.order, ms, cpt, c.stage_shape)
    _store(key, best)
    return best


def _lib_error():
    from ._lib import UstbError

    return UstbError
