"""Image-quality figures of a beamformed linear-scan image.

Used to state the error of the reduced-precision paths against the FP64 oracle
in imaging terms, beside the relative L2 error:

* ``cyst_contrast_db``: ``20 log10(mean|b| inside / mean|b| in a speckle ring)``,
  the contrast ``C`` of +tools/measure_contrast_ratio.m:28-33,58-61 (cyst mask
  ``r < r_cyst``, speckle ring ``r_inner <= r < r_outer``, both centred on the cyst);
* ``lateral_fwhm``: the -6 dB width of a point target's lateral line, the
  measurement of publications/DynamicRange/functions/measureFWHM.m:4-14 (the
  depth row nearest the target, dB relative to the line's maximum), with the
  two crossings found by linear interpolation in dB.

Images are flat ``[P]`` arrays in the scan's pixel order; for ``LinearScan``
the pixel index is ``iz + Nz * ix``.
"""
from __future__ import annotations

from typing import Dict, List, Sequence, Tuple

import numpy as np

from .uff import LinearScan


def _grid(img: np.ndarray, scan: LinearScan) -> np.ndarray:
    """[P] -> |img| as [Nx, Nz]."""
    a = np.abs(np.asarray(img).reshape(-1))
    if a.size != scan.N_x_axis * scan.N_z_axis:
        raise ValueError("image does not match the scan")
    return a.reshape(scan.N_x_axis, scan.N_z_axis)


def cyst_contrast_db(img: np.ndarray, scan: LinearScan, xc: float, zc: float, r_cyst: float,
                     r_inner: float, r_outer: float) -> float:
    """Contrast in dB of a cyst centred at (xc, zc) (metres) against its speckle ring."""
    a = _grid(img, scan)
    X, Z = np.meshgrid(scan.x_axis, scan.z_axis, indexing="ij")
    d2 = (X - xc) ** 2 + (Z - zc) ** 2
    inside = d2 < r_cyst ** 2
    ring = (d2 < r_outer ** 2) & ~(d2 < r_inner ** 2)
    if not inside.any() or not ring.any():
        raise ValueError("cyst or speckle ring holds no pixel")
    return float(20.0 * np.log10(a[inside].mean() / a[ring].mean()))


def lateral_fwhm(img: np.ndarray, scan: LinearScan, x: float, z: float, half_width: float = 1.5e-3) -> float:
    """-6 dB lateral width (metres) of the point target nearest (x, z), on the depth row
    nearest z, within ``x +- half_width``.  NaN when the line never falls 6 dB below its
    peak on both sides."""
    a = _grid(img, scan)
    iz = int(np.argmin(np.abs(scan.z_axis - z)))
    sel = np.nonzero(np.abs(scan.x_axis - x) <= half_width)[0]
    if sel.size < 3:
        raise ValueError("lateral line holds fewer than 3 pixels")
    line = a[sel, iz]
    xs = scan.x_axis[sel]
    with np.errstate(divide="ignore"):
        db = 20.0 * np.log10(line / line.max())
    k = int(np.argmax(line))

    def crossing(step: int) -> float:
        i = k
        while 0 <= i + step < db.size:
            j = i + step
            if db[j] < -6.0:
                t = (-6.0 - db[i]) / (db[j] - db[i])
                return float(xs[i] + t * (xs[j] - xs[i]))
            i = j
        return float("nan")

    return abs(crossing(1) - crossing(-1))


def isolated_points(points: np.ndarray, scan: LinearScan, cysts: Sequence[Tuple[float, float, float]] = (),
                    min_separation: float = 3e-3, margin: float = 2e-3) -> np.ndarray:
    """Indices of point targets ([S, 3] xyz) with no other target within
    ``min_separation``, away from every cyst and at least ``margin`` inside the scan."""
    p = np.asarray(points)
    keep = []
    for i, (x, _, z) in enumerate(p):
        d = np.hypot(p[:, 0] - x, p[:, 2] - z)
        d[i] = np.inf
        if d.min() < min_separation:
            continue
        if any(np.hypot(x - cx, z - cz) < r + min_separation for cx, cz, r in cysts):
            continue
        if not (scan.x_axis[0] + margin <= x <= scan.x_axis[-1] - margin
                and scan.z_axis[0] + margin <= z <= scan.z_axis[-1] - margin):
            continue
        keep.append(i)
    return np.asarray(keep, dtype=np.int64)


def compare(img: np.ndarray, ref: np.ndarray, scan: LinearScan, cysts: Sequence[Tuple[float, float, float]],
            points: np.ndarray, max_points: int = 10, min_separation: float = 2e-3) -> Dict[str, object]:
    """Relative L2 error, per-cyst contrast and per-point FWHM of ``img`` against ``ref``
    (point targets with no neighbour within ``min_separation``)."""
    img = np.asarray(img).reshape(-1)
    ref = np.asarray(ref).reshape(-1)
    out: Dict[str, object] = {"rel_l2": float(np.linalg.norm(img - ref) / np.linalg.norm(ref))}
    cr: List[Tuple[float, float]] = []
    for cx, cz, r in cysts:
        args = (cx, cz, 0.8 * r, 1.25 * r, 2.0 * r)
        cr.append((cyst_contrast_db(img, scan, *args), cyst_contrast_db(ref, scan, *args)))
    out["contrast_db"] = cr
    out["max_contrast_diff_db"] = max((abs(a - b) for a, b in cr), default=0.0)
    fw: List[Tuple[float, float]] = []
    for i in isolated_points(points, scan, cysts, min_separation)[:max_points]:
        x, _, z = points[i]
        fw.append((lateral_fwhm(img, scan, x, z), lateral_fwhm(ref, scan, x, z)))
    fw = [(a, b) for a, b in fw if np.isfinite(a) and np.isfinite(b)]
    out["fwhm_m"] = fw
    out["max_fwhm_diff_m"] = max((abs(a - b) for a, b in fw), default=0.0)
    return out
