"""Headless image formation after the beamformer.

``get_image`` mirrors +uff/beamformed_data.m:300-325 (envelope and compression,
reshaped onto the scan's grid) on device tensors; ``scan_convert`` mirrors
+tools/scan_convert.m for a sector scan: the compressed image is interpolated
bilinearly in (azimuth, depth) onto a uniform Cartesian (x, z) grid spanning the
sector, -inf outside it.  The display itself is out of scope: the result is a
device buffer.  Compression and conversion of a sector image run in one kernel
pass (``ustb_scan_convert``) after a max reduction.
"""
from __future__ import annotations

import math
from typing import Tuple

import numpy as np
import torch

from . import _lib
from .uff import BeamformedData, LinearScan, SectorScan

COMPRESSION = {"log": 0, "sqrt": 1, "abs": 2}


def get_image(bd: BeamformedData, compression: str = "log") -> torch.Tensor:
    """Envelope/compression of ``bd.data`` ([P, N|1, W|1, F] device tensor), reshaped to
    [N_z, N_x, ...] (linear scan) or [N_depth, N_azimuth, ...] (sector scan)."""
    d = bd.data if torch.is_tensor(bd.data) else torch.as_tensor(np.asarray(bd.data))
    if compression == "log":
        env = d.abs()
        env = 20 * torch.log10(env / env.max())
    elif compression == "sqrt":
        env = d.abs().sqrt()
    elif compression == "abs":
        env = d.abs()
    elif compression in ("none", "none-complex"):
        env = d
    else:
        raise ValueError(f"unknown compression {compression!r}")
    rest = tuple(env.shape[2:]) if env.dim() > 2 else ()
    if isinstance(bd.scan, LinearScan):
        shape = (bd.scan.N_z_axis, bd.scan.N_x_axis) + rest
    elif isinstance(bd.scan, SectorScan):
        shape = (bd.scan.depth_axis.size, bd.scan.azimuth_axis.size) + rest
    else:
        raise ValueError(f"don't know how to form an image on a {type(bd.scan).__name__}")
    # MATLAB reshape (column-major) of a [P, ...] array
    return env.permute(*reversed(range(env.dim()))).reshape(tuple(reversed(shape))).permute(
        *reversed(range(len(shape))))


def cartesian_grid(scan: SectorScan, size_x: int = 512, size_z: int = 512) -> Tuple[np.ndarray, np.ndarray]:
    """(Xs, Zs) axes of tools.scan_convert: the bounding box of the sector's (x, z)
    pixel positions sampled uniformly."""
    th, r = np.meshgrid(scan.azimuth_axis, scan.depth_axis)
    z, x = r * np.cos(th), r * np.sin(th)
    return np.linspace(x.min(), x.max(), size_x), np.linspace(z.min(), z.max(), size_z)


def scan_convert(data: torch.Tensor, scan: SectorScan, size_x: int = 512, size_z: int = 512,
                 compression: str = "log") -> Tuple[torch.Tensor, np.ndarray, np.ndarray]:
    """Compressed, scan-converted image of sector-scan data.

    ``data``: [P, F] or [P] device tensor (complex64 or float32), P = depth fastest.
    Returns (image (F, size_z, size_x) float32 on the device, Xs, Zs)."""
    if not isinstance(scan, SectorScan):
        raise TypeError("scan conversion takes a sector scan")
    if not data.is_cuda:
        raise TypeError("data must be a CUDA tensor")
    nd, na = scan.depth_axis.size, scan.azimuth_axis.size
    cplx = data.is_complex()
    d = data.to(torch.complex64 if cplx else torch.float32).reshape(nd * na, -1)
    F = d.shape[1]
    d = d.t().contiguous()  # (F, P): frame-major, depth fastest
    dev = data.device
    key = (str(dev), size_x, size_z)
    cache = scan.__dict__.setdefault("_scan_convert_cache", {})
    if key not in cache:  # axes on the device and the Cartesian grid, once per scan
        if not (np.all(np.diff(scan.depth_axis) > 0) and np.all(np.diff(scan.azimuth_axis) > 0)):
            raise ValueError("depth and azimuth axes must increase")
        f32 = lambda a: torch.as_tensor(np.asarray(a, np.float32), device=dev)
        xs, zs = cartesian_grid(scan, size_x, size_z)
        cache[key] = (f32(scan.depth_axis), f32(scan.azimuth_axis), xs, zs,
                      torch.zeros(1, dtype=torch.float32, device=dev))
    depth, azim, xs, zs, peak = cache[key]
    out = torch.empty((F, size_x, size_z), dtype=torch.float32, device=dev)
    dx = (xs[-1] - xs[0]) / max(size_x - 1, 1)
    dz = (zs[-1] - zs[0]) / max(size_z - 1, 1)
    with torch.cuda.device(dev):
        _lib.call("ustb_scan_convert", d.data_ptr(), int(cplx), COMPRESSION[compression], nd, na, F,
                  depth.data_ptr(), azim.data_ptr(), peak.data_ptr(), out.data_ptr(), size_x, size_z,
                  float(xs[0]), float(dx), float(zs[0]), float(dz), torch.cuda.current_stream(dev).cuda_stream)
    return out.transpose(1, 2), xs, zs
