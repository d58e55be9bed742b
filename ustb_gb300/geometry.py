"""Host FP64 geometry precompute of midprocess.das: delays and apodization.

Everything here follows the reference's MATLAB, in double precision, so that
the single-precision tables handed to the GPU are the ones das.m would hand to
das_c:

* ``receive_delay``   +midprocess/das.m:102-107
* ``transmit_delay``  +midprocess/das.m:110-206 (plane, spherical at infinity,
                      diverging, focused with the spherical / unified / hybrid /
                      blended models, photoacoustic), with the unified model of
                      +tools/calculate_unified_delay_model.m:1-100
* ``Apodization``     +uff/apodization.m: windows (:172-223), aperture
                      apodization (:323-367) with incidence (:370-468) and tilt
                      (+tools/rotate_points.m), wave apodization (:249-320) with
                      incidence (:472-555), scanline/MLA (:266-304), STA
                      (:345-349), apodization_vector overrides.
"""
from __future__ import annotations

import math
from typing import Optional, Sequence

import numpy as np

from .enums import SphericalTransmitDelayModel as STDM
from .enums import Wavefront, Window
from .uff import LinearScan, Point, Probe, Scan, SectorScan, Wave

EPS = np.finfo(np.float64).eps  # MATLAB eps


# ---------------------------------------------------------------------------
# delays
# ---------------------------------------------------------------------------

def receive_delay(probe: Probe, scan: Scan, sound_speed: float, lens_delay: float = 0.0):
    """[P, N] receive delay in seconds (double), das.m:103-106."""
    xm = probe.x[None, :] - scan.x[:, None]
    ym = probe.y[None, :] - scan.y[:, None]
    zm = probe.z[None, :] - scan.z[:, None]
    return np.sqrt(xm ** 2 + ym ** 2 + zm ** 2) / sound_speed + lens_delay


def _plane_distance(scan: Scan, src: Point):
    ca, sa = math.cos(src.azimuth), math.sin(src.azimuth)
    ce, se = math.cos(src.elevation), math.sin(src.elevation)
    return scan.z * ca * ce + scan.x * sa * ce + scan.y * se


def transmit_delay(sequence: Sequence[Wave], scan: Scan,
                   model: STDM = STDM.hybrid, pw_margin: float = 1e-3,
                   blending_power: float = 0.5, unified_f_number=(1.0, 1.0)):
    """[P, W] transmit delay in seconds (double), das.m:110-204."""
    P, W = scan.N_pixels, len(sequence)
    td = np.zeros((P, W))
    mask_all = None
    for w, wave in enumerate(sequence):
        src = wave.source
        wf = Wavefront(int(wave.wavefront))
        if wf == Wavefront.spherical:
            if math.isinf(src.distance):
                td[:, w] = _plane_distance(scan, src)
            else:
                sx, sy, sz = src.x, src.y, src.z
                dist = np.where(scan.z < sz, -1.0, 1.0) * np.sqrt(
                    (sx - scan.x) ** 2 + (sy - scan.y) ** 2 + (sz - scan.z) ** 2)
                if sz < 0:  # diverging wave
                    td[:, w] = dist - abs(src.distance)
                else:
                    m = STDM(int(model))
                    if m == STDM.spherical:
                        td[:, w] = dist + src.distance
                    elif m == STDM.unified:
                        if mask_all is None:
                            mask_all = _unified_mask(sequence, scan, unified_f_number)
                        mk = mask_all[:, :, w].copy()
                        mk[np.isnan(mk)] = 0
                        td[:, w] = unified_delay_model(dist, mk != 0, scan, src)
                    elif m in (STDM.hybrid, STDM.blended):
                        if isinstance(scan, LinearScan):
                            plane = np.where(scan.z < sz, -1.0, 1.0) * np.sqrt((sz - scan.z) ** 2) + src.distance
                        elif isinstance(scan, SectorScan):
                            plane = _plane_distance(scan, src)
                        else:
                            raise ValueError("Only linear scan and sector scan in 2D is supported "
                                             "for the hybrid spherical transmit delay model.")
                        if m == STDM.hybrid:
                            zmask = (scan.z < sz + pw_margin) & (scan.z > sz - pw_margin)
                            t = dist + src.distance
                            t[zmask] = plane[zmask]
                            td[:, w] = t
                        else:
                            r = np.sqrt(scan.x ** 2 + scan.y ** 2 + scan.z ** 2)
                            nd = np.minimum(np.abs(src.distance - r) / src.distance, 1.0)
                            t = dist + src.distance
                            td[:, w] = t * nd ** blending_power + plane * (1 - nd ** blending_power)
                    else:
                        raise ValueError(f"unknown spherical transmit delay model {model}")
        elif wf == Wavefront.plane:
            td[:, w] = _plane_distance(scan, src)
        elif wf == Wavefront.photoacoustic:
            td[:, w] = 0.0
        else:
            raise ValueError("Unknown wavefront. Check available options at uff.wavefront")
        td[:, w] = td[:, w] / wave.sound_speed - wave.delay
    return td


def _unified_mask(sequence, scan, f_number):
    apo = Apodization(window=Window.boxcar, minimum_aperture=(0.0, 0.0), f_number=f_number)
    data = apo.wave_apodization(sequence, scan)
    if isinstance(scan, SectorScan):
        return data.reshape(scan.N_depth_axis, scan.N_azimuth_axis, len(sequence), order="F")
    if isinstance(scan, LinearScan):
        return data.reshape(scan.N_z_axis, scan.N_x_axis, len(sequence), order="F")
    raise ValueError("Only linear scan and sector scan in 2D is supported for the unified "
                     "spherical transmit delay model.")


def unified_delay_model(delay_dist, mask, scan, source: Point):
    """Nguyen-Prager unified delay (+tools/calculate_unified_delay_model.m:1-100).

    ``delay_dist`` is the signed source distance [P], ``mask`` a boolean [Nz, Nx]
    of the region inside the transmit aperture.  Returns distance + source
    distance, in metres, like the reference.
    """
    if isinstance(scan, SectorScan):
        nz, nx = scan.N_depth_axis, scan.N_azimuth_axis
        dirtest = scan.azimuth_axis[-1] - scan.azimuth_axis[0]
    else:
        nz, nx = scan.N_z_axis, scan.N_x_axis
        dirtest = scan.x_axis[-1] - scan.x_axis[0]
    tx = np.asarray(delay_dist, np.float64).reshape(nz, nx, order="F")
    xm = scan.x.reshape(nz, nx, order="F")
    zm = scan.z.reshape(nz, nx, order="F")
    mask = np.array(mask, dtype=bool).reshape(nz, nx, order="F")
    botinds = ~mask[-1, :]
    maxval = np.max(tx[-1, :] * mask[-1, :])
    masked = mask * tx
    mask[-1, :] = True
    masked[-1, botinds] = maxval
    interp = np.zeros_like(tx)
    mask_before = np.zeros(tx.shape, dtype=bool)
    mask_after = np.zeros(tx.shape, dtype=bool)
    last_before = None
    first_after = None
    for x in range(nx):
        zf = int(np.argmin(np.abs(zm[:, x] - source.z)))
        if np.sum(mask[zf:, x] > 0):
            ray = masked[:, x]
            pos = ray.copy()
            pos[ray > 0] = 0
            pos[pos == 0] = -np.inf
            neg = ray.copy()
            neg[ray < 0] = 0
            neg[neg == 0] = np.inf
            ia = int(np.argmax(pos))
            ib = int(np.argmin(neg))
            pa = np.array([xm[ia, x], zm[ia, x]])
            pb = np.array([xm[ib, x], zm[ib, x]])
            nrm = np.linalg.norm(pb - pa)
            with np.errstate(divide="ignore", invalid="ignore"):
                w1 = np.sqrt((zm[ia, x] - zm[:, x]) ** 2) / nrm
                w1 = w1 / w1[ib]
                w2 = np.sqrt((zm[ib, x] - zm[:, x]) ** 2) / nrm
                w2 = w2 / w2[ia]
            interp[:, x] = w1 * tx[ib, x] + w2 * tx[ia, x]
        elif np.sum(masked[zf:, x] == 0) and (xm[zf, x] - source.x) * dirtest < 0:
            last_before = x
            mask_before[:, x] = True
        elif np.sum(masked[zf:, x] == 0) and (xm[zf, x] - source.x) * dirtest > 0:
            if first_after is None:
                first_after = x
            mask_after[:, x] = True
    if mask_before.any():
        interp[mask_before] = np.repeat(interp[:, last_before + 1][:, None],
                                        int(mask_before[0, :].sum()), axis=1).ravel(order="F")
    if mask_after.any():
        interp[mask_after] = np.repeat(interp[:, first_after - 1][:, None],
                                       int(mask_after[0, :].sum()), axis=1).ravel(order="F")
    interp[mask] = tx[mask]
    interp[np.isinf(interp)] = 0
    return interp.ravel(order="F") + source.distance


# ---------------------------------------------------------------------------
# apodization
# ---------------------------------------------------------------------------

def _rect(r):
    return (r <= 0.5).astype(np.float64)


def _hann(r):
    return (r <= 0.5) * (0.5 + 0.5 * np.cos(2 * np.pi * r))


def _hamm(r):
    return (r <= 0.5) * (0.53836 + 0.46164 * np.cos(2 * np.pi * r))


def _tukey(r, roll):
    return ((r <= 0.5 * (1 - roll)).astype(np.float64)
            + (r > 0.5 * (1 - roll)) * (r < 0.5) * 0.5 * (1 + np.cos(2 * np.pi / roll * (r - roll / 2 - 0.5))))


def _tri(r):
    return (r <= 0.5) * (1 - 2 * r)


def apply_window(window: Window, rt, rp):
    """apodization.m:189-223."""
    w = Window(int(window))
    if w == Window.boxcar:
        return _rect(rt) * _rect(rp)
    if w == Window.hanning:
        return _hann(rt) * _hann(rp)
    if w == Window.hamming:
        return _hamm(rt) * _hamm(rp)
    if w in (Window.tukey25, Window.tukey50, Window.tukey75):
        roll = {Window.tukey25: 0.25, Window.tukey50: 0.5, Window.tukey75: 0.75}[w]
        return _tukey(rt, roll) * _tukey(rp, roll)
    if w == Window.triangle:
        return _tri(rt) * _tri(rp)
    raise ValueError("Unknown apodization type!")


def rotate_points(x, y, z, theta, phi):
    """+tools/rotate_points.m."""
    if abs(theta) > 0:
        x, z = x * math.cos(theta) - z * math.sin(theta), x * math.sin(theta) + z * math.cos(theta)
    if abs(phi) > 0:
        y, z = y * math.cos(phi) - z * math.sin(phi), y * math.sin(phi) + z * math.cos(phi)
    return x, y, z


def _clamp_apertures(z_dist, f_number, minimum_aperture, maximum_aperture):
    zx = z_dist.copy()
    zy = z_dist.copy()
    a = np.abs(z_dist)
    for zz, i in ((zx, 0), (zy, 1)):
        lo = minimum_aperture[i] * f_number[i]
        m = a <= lo
        zz[m] = np.sign(zz[m]) * lo
        hi = maximum_aperture[i] * f_number[i]
        m = a >= hi
        zz[m] = np.sign(zz[m]) * hi
    return zx, zy


def _pair(v):
    v = np.atleast_1d(np.asarray(v, np.float64)).ravel()
    return (float(v[0]), float(v[0])) if v.size == 1 else (float(v[0]), float(v[1]))


class Apodization:
    """uff.apodization: receive (aperture) or transmit (wave) apodization."""

    def __init__(self, window: Window = Window.none, f_number=(1.0, 1.0), tilt=(0.0, 0.0),
                 minimum_aperture=(1e-3, 1e-3), maximum_aperture=(10.0, 10.0),
                 grating_lobe_angle=(math.pi, math.pi), MLA=(1, 1), MLA_overlap=(0, 0),
                 apodization_vector=None, origin: Optional[Point] = None):
        self.window = Window(int(window))
        self.f_number = _pair(f_number)
        t = np.atleast_1d(np.asarray(tilt, np.float64)).ravel()
        self.tilt = (float(t[0]), 0.0) if t.size == 1 else (float(t[0]), float(t[1]))
        self.minimum_aperture = _pair(minimum_aperture)
        self.maximum_aperture = _pair(maximum_aperture)
        self.grating_lobe_angle = _pair(grating_lobe_angle)
        self.MLA = tuple(int(v) for v in np.broadcast_to(MLA, 2))
        self.MLA_overlap = tuple(int(v) for v in np.broadcast_to(MLA_overlap, 2))
        self.apodization_vector = apodization_vector
        self.origin = origin

    # -- receive -------------------------------------------------------------
    def aperture_apodization(self, probe: Probe, scan: Scan):
        """[P, N] receive apodization, apodization.m:323-367."""
        P, N = scan.N_pixels, probe.N_elements
        if self.apodization_vector is not None:
            v = np.asarray(self.apodization_vector, np.float64)
            if v.size == N:
                return np.ones((P, 1)) * v.ravel()[None, :]
            return v.reshape(P, N)
        if self.window == Window.none:
            return np.ones((P, N))
        if self.window == Window.sta:
            if self.origin is None:
                raise ValueError("origin must be set to use STA apodization")
            o = self.origin
            d = np.sqrt((probe.x - o.x) ** 2 + (probe.y - o.y) ** 2 + (probe.z - o.z) ** 2)
            return np.ones((P, 1)) * (d == d.min()).astype(np.float64)[None, :]
        tan_t, tan_p = self.incidence_aperture(probe, scan)
        return apply_window(self.window, np.abs(self.f_number[0] * tan_t), np.abs(self.f_number[1] * tan_p))

    def incidence_aperture(self, probe: Probe, scan: Scan):
        """apodization.m:370-468 (flat probes; curvilinear probes are not modelled)."""
        P, N = scan.N_pixels, probe.N_elements
        x = np.ones((P, 1)) * probe.x[None, :]
        y = np.ones((P, 1)) * probe.y[None, :]
        z = np.ones((P, 1)) * probe.z[None, :]
        origin = self.origin
        if origin is None and isinstance(scan, SectorScan):
            origin = scan.origin
        if isinstance(scan, SectorScan) or origin is not None:
            x0, y0, z0 = origin.x, origin.y, origin.z
            pd = np.sqrt((scan.x - x0) ** 2 + (scan.y - y0) ** 2 + (scan.z - z0) ** 2)
            x_dist = x - x0
            y_dist = y - y0
            z_dist = pd[:, None] * np.ones((1, N))
        else:
            x_dist = scan.x[:, None] - x
            y_dist = scan.y[:, None] - y
            z_dist = scan.z[:, None] - z
        x_dist, y_dist, z_dist = rotate_points(x_dist, y_dist, z_dist, self.tilt[0], self.tilt[1])
        zx, zy = _clamp_apertures(z_dist, self.f_number, self.minimum_aperture, self.maximum_aperture)
        with np.errstate(divide="ignore", invalid="ignore"):
            return x_dist / zx, y_dist / zy

    # -- transmit ------------------------------------------------------------
    def wave_apodization(self, sequence: Sequence[Wave], scan: Scan):
        """[P, W] transmit apodization, apodization.m:249-320."""
        P, W = scan.N_pixels, len(sequence)
        if self.apodization_vector is not None:
            v = np.asarray(self.apodization_vector, np.float64).ravel()
            if v.size != W:
                raise ValueError("If an apodization_vector is given its size must match the "
                                 "number of events in the sequence.")
            return np.ones((P, 1)) * v[None, :]
        if self.window == Window.none:
            return np.ones((P, W))
        if self.window == Window.scanline:
            return self._scanline(scan, W)
        tan_t, tan_p = self.incidence_wave(sequence, scan)
        return apply_window(self.window, np.abs(self.f_number[0] * tan_t), np.abs(self.f_number[1] * tan_p))

    def incidence_wave(self, sequence: Sequence[Wave], scan: Scan):
        """apodization.m:472-555 (flat probes)."""
        P, W = scan.N_pixels, len(sequence)
        tan_t = np.zeros((P, W))
        tan_p = np.zeros((P, W))
        for n, wave in enumerate(sequence):
            src, org = wave.source, wave.origin
            if Wavefront(int(wave.wavefront)) == Wavefront.plane or math.isinf(src.distance):
                tan_t[:, n] = math.tan(src.azimuth - self.tilt[0])
                tan_p[:, n] = math.tan(src.elevation - self.tilt[1])
                continue
            SP = np.stack([scan.x - src.x, scan.y - src.y, scan.z - src.z], axis=1)
            OP = np.stack([scan.x - org.x, scan.y - org.y, scan.z - org.z], axis=1)
            OS = np.array([src.x - org.x, src.y - org.y, src.z - org.z])
            if np.linalg.norm(src.xyz - org.xyz) <= EPS:
                OS = np.array([0.0, 0.0, 1.0])
            zu = OS / math.sqrt(float(np.sum(OS ** 2)))
            yu = np.cross(zu, [1.0, 0.0, 0.0])
            xu = np.cross(zu, yu)
            z_dist = SP @ zu
            x_dist = SP @ xu
            y_dist = SP @ yu
            zx, zy = _clamp_apertures(z_dist, self.f_number, self.minimum_aperture, self.maximum_aperture)
            zx[np.abs(np.arctan2(OP[:, 0], OP[:, 2]) - math.atan2(OS[0], OS[2])) > 0.5 * self.grating_lobe_angle[0]] = EPS
            zy[np.abs(np.arctan2(OP[:, 1], OP[:, 2]) - math.atan2(OS[1], OS[2])) > 0.5 * self.grating_lobe_angle[1]] = EPS
            with np.errstate(divide="ignore", invalid="ignore"):
                tan_t[:, n] = x_dist / zx
                tan_p[:, n] = y_dist / zy
        return tan_t, tan_p

    def _scanline(self, scan: Scan, W: int):
        """Scanline/MLA apodization, apodization.m:266-304 (y direction singleton)."""
        from scipy.signal import correlate2d

        if isinstance(scan, LinearScan):
            nl, ny, nd = scan.N_x_axis, scan.y_axis.size, scan.N_z_axis
        elif isinstance(scan, SectorScan):
            nl, ny, nd = scan.N_azimuth_axis, scan.elevation_axis.size, scan.N_depth_axis
        else:
            raise ValueError("The scan class does not support scanline based beamforming.")
        mla = self.MLA
        if W != nl * ny // (mla[0] * mla[1]):
            raise ValueError("The number of waves in the sequence does not match with the number "
                             "of scanlines and set MLA.")
        A = np.zeros((nl, ny))
        A[:mla[0], :mla[1]] = 1.0
        k = np.ones((self.MLA_overlap[0] + 1, self.MLA_overlap[1] + 1))
        k /= k.size
        B = np.zeros((W, nl, ny))
        for i in range(nl // mla[0]):
            for j in range(ny // mla[1]):
                sh = np.roll(A, (i * mla[0], j * mla[1]), axis=(0, 1))
                B[i + j * (nl // mla[0])] = correlate2d(sh, k, mode="same")
        out = np.broadcast_to(B.transpose(1, 2, 0)[None], (nd, nl, ny, W))
        return out.reshape(nd * nl * ny, W, order="F").copy()


# ---------------------------------------------------------------------------
# the same receive tables built on the GPU (large scans)
# ---------------------------------------------------------------------------

def _window_torch(window: Window, r):
    import torch

    w = Window(int(window))
    if w == Window.boxcar:
        return (r <= 0.5).to(r.dtype)
    if w == Window.hanning:
        return (r <= 0.5) * (0.5 + 0.5 * torch.cos(2 * math.pi * r))
    if w == Window.hamming:
        return (r <= 0.5) * (0.53836 + 0.46164 * torch.cos(2 * math.pi * r))
    if w in (Window.tukey25, Window.tukey50, Window.tukey75):
        roll = {Window.tukey25: 0.25, Window.tukey50: 0.5, Window.tukey75: 0.75}[w]
        return ((r <= 0.5 * (1 - roll)).to(r.dtype)
                + (r > 0.5 * (1 - roll)) * (r < 0.5) * 0.5 * (1 + torch.cos(2 * math.pi / roll * (r - roll / 2 - 0.5))))
    if w == Window.triangle:
        return (r <= 0.5) * (1 - 2 * r)
    raise ValueError("Unknown apodization type!")


def receive_tables_device(probe: Probe, scan: Scan, sound_speed: float, apo: "Apodization",
                          lens_delay: float = 0.0, device="cuda", chunk: int = 64):
    """Single-precision receive delay and apodization tables in the ABI layout
    (N, P), computed on ``device`` in double precision with the formulas of
    ``receive_delay`` and ``Apodization.aperture_apodization`` (windows, flat
    probes, no tilt, optional origin)."""
    import torch

    dev = torch.device(device)
    P, N = scan.N_pixels, probe.N_elements
    px = torch.as_tensor(scan.xyz, dtype=torch.float64, device=dev)
    el = torch.as_tensor(probe.xyz, dtype=torch.float64, device=dev)
    dly = torch.empty((N, P), dtype=torch.float32, device=dev)
    ap = torch.empty((N, P), dtype=torch.float32, device=dev)
    origin = apo.origin
    if origin is None and isinstance(scan, SectorScan):
        origin = scan.origin
    for n0 in range(0, N, chunk):
        e = el[n0:n0 + chunk]  # [c, 3]
        d = px[None, :, :] - e[:, None, :]  # pixel - element, [c, P, 3]
        dly[n0:n0 + chunk] = (torch.linalg.norm(d, dim=2) / sound_speed + lens_delay).float()
        if apo.apodization_vector is not None or apo.window in (Window.sta, Window.scanline) or apo.tilt != (0.0, 0.0):
            raise ValueError("device tables cover windowed apodization without tilt")
        if apo.window == Window.none:
            ap[n0:n0 + chunk] = 1.0
            continue
        if origin is not None:
            o = torch.tensor([origin.x, origin.y, origin.z], dtype=torch.float64, device=dev)
            xd = (e[:, 0] - o[0])[:, None].expand(-1, P)
            yd = (e[:, 1] - o[1])[:, None].expand(-1, P)
            zd = torch.linalg.norm(px - o, dim=1)[None, :].expand(e.shape[0], -1)
        else:
            xd, yd, zd = d[..., 0], d[..., 1], d[..., 2]
        a = zd.abs()
        zz = []
        for i in range(2):
            z = zd.clone()
            lo = apo.minimum_aperture[i] * apo.f_number[i]
            hi = apo.maximum_aperture[i] * apo.f_number[i]
            z = torch.where(a <= lo, torch.sign(zd) * lo, z)
            z = torch.where(a >= hi, torch.sign(zd) * hi, z)
            zz.append(z)
        rt = (apo.f_number[0] * xd / zz[0]).abs()
        rp = (apo.f_number[1] * yd / zz[1]).abs()
        ap[n0:n0 + chunk] = (_window_torch(apo.window, rt) * _window_torch(apo.window, rp)).float()
    return dly, ap
