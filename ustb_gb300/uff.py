"""Minimal UFF data model: the inputs and output of midprocess.das.

Mirrors the properties of USTB's MATLAB classes that the delay-and-sum path
reads (the Python package's duck-typed fakes, python/tests/test_das.py:13-117,
show the same surface):

* ``Point``      +uff/point.m — stored as (distance, azimuth, elevation) with
                 derived x, y, z (getters at point.m:87-110, set.xyz :36-49).
* ``Wave``       +uff/wave.m — wavefront, source, origin, delay, sound_speed.
* ``Probe``      element positions; ``linear_array`` (+uff/linear_array.m:21-35)
                 and ``matrix_array`` (+uff/matrix_array.m:24-42) builders.
* ``Scan``       pixel positions; ``LinearScan`` (ndgrid(z, x, y), z fastest,
                 +uff/linear_scan.m:27-39, reference_distance = z),
                 ``SectorScan`` (ndgrid(depth, az, el), +uff/sector_scan.m:34-67,
                 reference_distance = rho) and ``LinearScan3D``
                 (+uff/linear_scan_3D.m, reference_distance = 0).
* ``ChannelData`` +uff/channel_data.m — data [L, N, W, F], fs, t0, c, fd.
* ``BeamformedData`` +uff/beamformed_data.m:41-63 — data [P, N|1, W|1, F].
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from .enums import Wavefront


def _cosd(deg: float) -> float:
    r = math.fmod(deg, 360.0)
    if abs(math.fmod(abs(r) - 90.0, 180.0)) == 0.0:
        return 0.0
    return math.cos(math.radians(deg))


class Point:
    """A point in spherical coordinates (distance, azimuth, elevation)."""

    def __init__(self, distance: float = 0.0, azimuth: float = 0.0, elevation: float = 0.0):
        self.distance = float(distance)
        self.azimuth = float(azimuth)
        self.elevation = float(elevation)
        if self.distance < 0:  # point.m:19-26: negative distance mirrors the point
            x, y, z = self.x, self.y, self.z  # the getters already give the mirrored point
            self.set_xyz(x, y, z)

    @classmethod
    def from_xyz(cls, x: float, y: float, z: float) -> "Point":
        p = cls()
        p.set_xyz(x, y, z)
        return p

    def set_xyz(self, x: float, y: float, z: float) -> None:
        d = math.sqrt(x * x + y * y + z * z)
        self.distance = d
        self.azimuth = math.atan2(x, z)
        if d > 0:
            self.elevation = math.copysign(math.pi / 2, y) if math.isinf(y) else math.asin(y / d)
        else:
            self.elevation = 0.0

    @property
    def x(self) -> float:
        if self.azimuth == math.pi or self.azimuth == 0:
            return 0.0
        return self.distance * math.sin(self.azimuth) * math.cos(self.elevation)

    @property
    def y(self) -> float:
        if self.elevation == 0:
            return 0.0
        return self.distance * math.sin(self.elevation)

    @property
    def z(self) -> float:
        if abs(self.azimuth) == math.pi / 2 or abs(self.elevation) == math.pi / 2:
            return 0.0
        return self.distance * _cosd(self.azimuth * 180 / math.pi) * _cosd(self.elevation * 180 / math.pi)

    @property
    def xyz(self) -> np.ndarray:
        return np.array([self.x, self.y, self.z])


@dataclass
class Wave:
    wavefront: Wavefront = Wavefront.spherical
    source: Point = field(default_factory=Point)
    origin: Point = field(default_factory=Point)
    delay: float = 0.0
    sound_speed: float = 1540.0

    @classmethod
    def plane(cls, azimuth: float, elevation: float = 0.0, c: float = 1540.0, delay: float = 0.0):
        return cls(Wavefront.plane, Point(math.inf, azimuth, elevation), Point(), delay, c)

    @classmethod
    def diverging(cls, source_xyz, c: float = 1540.0, delay: float = 0.0):
        """Spherical wave from a virtual source (behind the array: z < 0)."""
        return cls(Wavefront.spherical, Point.from_xyz(*source_xyz), Point(), delay, c)


class Probe:
    """Element positions [N] (x, y, z) in metres."""

    def __init__(self, x, y=None, z=None):
        self.x = np.asarray(x, dtype=np.float64).ravel()
        self.y = np.zeros_like(self.x) if y is None else np.asarray(y, np.float64).ravel()
        self.z = np.zeros_like(self.x) if z is None else np.asarray(z, np.float64).ravel()

    @property
    def N_elements(self) -> int:
        return self.x.size

    @property
    def xyz(self) -> np.ndarray:
        return np.stack([self.x, self.y, self.z], axis=1)

    @classmethod
    def linear_array(cls, N: int, pitch: float) -> "Probe":
        x0 = np.arange(1, N + 1) * pitch
        return cls(x0 - x0.mean())

    @classmethod
    def matrix_array(cls, N_x: int, N_y: int, pitch_x: float, pitch_y: Optional[float] = None):
        pitch_y = pitch_x if pitch_y is None else pitch_y
        x0 = np.arange(1, N_x + 1) * pitch_x
        y0 = np.arange(1, N_y + 1) * pitch_y
        X, Y = np.meshgrid(x0 - x0.mean(), y0 - y0.mean(), indexing="ij")
        return cls(X.ravel(order="F"), Y.ravel(order="F"))


class Scan:
    """Arbitrary pixel positions [P]."""

    kind = "scan"

    def __init__(self, x, y, z):
        self.x = np.asarray(x, np.float64).ravel()
        self.y = np.asarray(y, np.float64).ravel()
        self.z = np.asarray(z, np.float64).ravel()

    @property
    def N_pixels(self) -> int:
        return self.x.size

    @property
    def xyz(self) -> np.ndarray:
        return np.stack([self.x, self.y, self.z], axis=1)

    @property
    def reference_distance(self):
        return np.zeros(self.N_pixels)


class LinearScan(Scan):
    kind = "linear"

    def __init__(self, x_axis, z_axis, y_axis=(0.0,)):
        self.x_axis = np.asarray(x_axis, np.float64).ravel()
        self.z_axis = np.asarray(z_axis, np.float64).ravel()
        self.y_axis = np.asarray(y_axis, np.float64).ravel()
        Z, X, Y = np.meshgrid(self.z_axis, self.x_axis, self.y_axis, indexing="ij")
        super().__init__(X.ravel(order="F"), Y.ravel(order="F"), Z.ravel(order="F"))

    @property
    def N_x_axis(self):
        return self.x_axis.size

    @property
    def N_z_axis(self):
        return self.z_axis.size

    @property
    def reference_distance(self):
        return self.z


class LinearScan3D(LinearScan):
    kind = "linear3d"

    @property
    def reference_distance(self):
        return np.zeros(self.N_pixels)


class SectorScan(Scan):
    kind = "sector"

    def __init__(self, azimuth_axis, depth_axis, elevation_axis=(0.0,), origin: Optional[Point] = None):
        self.azimuth_axis = np.asarray(azimuth_axis, np.float64).ravel()
        self.depth_axis = np.asarray(depth_axis, np.float64).ravel()
        self.elevation_axis = np.asarray(elevation_axis, np.float64).ravel()
        self.origin = origin if origin is not None else Point()
        rho, th, ph = np.meshgrid(self.depth_axis, self.azimuth_axis, self.elevation_axis, indexing="ij")
        self.rho = rho.ravel(order="F")
        # MATLAB sph2cart(phi, theta, rho) -> [Z, Y, X] (sector_scan.m:49)
        Zc = rho * np.cos(th) * np.cos(ph)
        Yc = rho * np.cos(th) * np.sin(ph)
        Xc = rho * np.sin(th)
        o = self.origin
        super().__init__((Xc + o.x).ravel(order="F"), (Yc + o.y).ravel(order="F"),
                         (Zc + o.z).ravel(order="F"))

    @property
    def N_azimuth_axis(self):
        return self.azimuth_axis.size

    @property
    def N_depth_axis(self):
        return self.depth_axis.size

    @property
    def reference_distance(self):
        return self.rho


class ChannelData:
    """Channel data [L, N, W, F] with its acquisition parameters."""

    def __init__(self, data, probe: Probe, sequence: Sequence[Wave], sampling_frequency: float,
                 initial_time: float = 0.0, sound_speed: float = 1540.0,
                 modulation_frequency: float = 0.0):
        self.data = data
        self.probe = probe
        self.sequence: List[Wave] = list(sequence)
        self.sampling_frequency = float(sampling_frequency)
        self.initial_time = float(initial_time)
        self.sound_speed = float(sound_speed)
        self.modulation_frequency = float(modulation_frequency)

    def _shape(self):
        s = tuple(self.data.shape) + (1,) * (4 - self.data.ndim)
        return s[:4]

    @property
    def N_samples(self):
        return self._shape()[0]

    @property
    def N_channels(self):
        return self.probe.N_elements

    @property
    def N_waves(self):
        return self._shape()[2]

    @property
    def N_frames(self):
        return self._shape()[3]

    def time(self):
        return self.initial_time + np.arange(self.N_samples) / self.sampling_frequency


class BeamformedData:
    """Beamformed data [P, N|1, W|1, F] on its scan (+uff/beamformed_data.m:41-63)."""

    def __init__(self, scan: Scan, data):
        self.scan = scan
        self.data = data

    def _size(self, i):
        return int(self.data.shape[i]) if self.data.ndim > i else 1

    @property
    def N_pixels(self):
        return self._size(0)

    @property
    def N_channels(self):
        return self._size(1)

    @property
    def N_waves(self):
        return self._size(2)

    @property
    def N_frames(self):
        return self._size(3)
