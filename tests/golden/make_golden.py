"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a container where the reference checkout is present (it is not needed
afterwards; the fixtures are committed):

    make -C oracle ref                       # builds the reference das_c from source
    python tests/golden/make_golden.py --reference <reference checkout>

Fixtures written:

* ``das_c_cases.npz``   seeded small inputs and the output of the reference's
                        own das_c (+mex/source/das_c.cpp, compiled unmodified by
                        oracle/Makefile), all four sum modes, with edge cases
                        (delays on exact sample positions, first/last samples,
                        out-of-window delays, zero and negative apodization).
* ``python_das.npz``    tables and outputs of the reference's Python
                        ``ustb.midprocess.DAS`` (python/src/ustb/midprocess/das.py)
                        for plane-wave, diverging-wave and focused (hybrid)
                        sequences: receive/transmit delays and the beamformed
                        output under its interp1 edge rule.
* ``python_demod.npz``  RF inputs and the IQ output of the reference's Python
                        ``ustb.preprocess.FastDemodulation``
                        (python/src/ustb/preprocess/fast_demodulation.py): default
                        and explicit decimation, 65-tap and short-trace filters,
                        and a trace too short for filtfilt's padding (the
                        reference raises there).
* ``python_cf.npz``     a seeded channel/wave cube (with an all-zero pixel) and
                        the coherence factor and CF image of the reference's
                        Python ``ustb.postprocess.CoherenceFactor``
                        (python/src/ustb/postprocess/coherence_factor.py) for
                        dimension receive, transmit and both.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def _rand_case(rng, L, N, W, F, P, t0, fs, fd, span):
    ch = (rng.standard_normal((L, N, W, F)) + 1j * rng.standard_normal((L, N, W, F))).astype(np.complex64)
    dtx = rng.uniform(-0.1 * span, 0.55 * span, (P, W)).astype(np.float32)
    drx = rng.uniform(0.0, 0.55 * span, (P, N)).astype(np.float32)
    atx = rng.uniform(0.0, 1.0, (P, W)).astype(np.float32)
    arx = rng.uniform(-0.25, 1.0, (P, N)).astype(np.float32)
    atx[rng.random((P, W)) < 0.15] = 0
    arx[rng.random((P, N)) < 0.15] = 0
    return dict(ch=ch, fs=np.float32(fs), t0=np.float32(t0), fd=np.float32(fd), atx=atx, arx=arx,
                dtx=dtx, drx=drx)


def _edge_case(rng, L, fs, t0):
    """Delays that land exactly on samples 0, 1, L-2, L-1, just inside/outside."""
    N, W, F = 4, 2, 1
    ch = (rng.standard_normal((L, N, W, F)) + 1j * rng.standard_normal((L, N, W, F))).astype(np.complex64)
    targets = np.array([-1.5, -0.25, 0.0, 0.5, 0.999, 1.0, 1.25, L - 2.5, L - 2.0, L - 1.75,
                        L - 1.0, L - 0.5, L + 3.0, 17.0, 17.5, 3.0], dtype=np.float64)
    P = targets.size
    dt = np.float32(1.0 / fs)
    drx = np.zeros((P, N), np.float32)
    dtx = np.zeros((P, W), np.float32)
    for p, s in enumerate(targets):
        d = np.float32(t0 + s / fs)
        drx[p, :] = d * np.float32(0.5)
        dtx[p, :] = d - drx[p, 0]
    atx = np.ones((P, W), np.float32)
    arx = np.ones((P, N), np.float32)
    arx[3, 1] = 0.0
    arx[4, 2] = -0.5
    atx[5, 1] = 0.0
    return dict(ch=ch, fs=np.float32(fs), t0=np.float32(t0), fd=np.float32(0.0), atx=atx, arx=arx,
                dtx=dtx, drx=drx)


def make_das_c_cases(out_path):
    if not O.have_reference():
        raise SystemExit("oracle/_ref/libdas_c_ref.so missing: run `make -C oracle ref` first")
    rng = np.random.default_rng(20261203)
    cases = {}
    specs = [
        ("iq_small", dict(L=96, N=8, W=3, F=2, P=120, t0=2e-6, fs=20e6, fd=5e6, span=96 / 20e6)),
        ("iq_long_delay", dict(L=256, N=6, W=2, F=1, P=80, t0=40e-6, fs=20e6, fd=5e6, span=256 / 20e6)),
        ("rf_analytic", dict(L=80, N=5, W=2, F=3, P=60, t0=0.0, fs=40e6, fd=0.0, span=80 / 40e6)),
    ]
    for name, s in specs:
        c = _rand_case(rng, **s)
        # shift the delays so that most land inside [t0, t0 + L/fs)
        c["dtx"] = (c["dtx"] + np.float32(s["t0"])).astype(np.float32)
        for dim in range(4):
            out = O.das_c_ref(c["ch"], c["fs"], c["t0"], c["atx"], c["arx"], c["dtx"], c["drx"],
                              c["fd"], dim)
            c[f"out_dim{dim}"] = np.ascontiguousarray(out)
        cases[name] = c
    e = _edge_case(rng, 40, 10e6, 1e-6)
    for dim in range(4):
        e[f"out_dim{dim}"] = np.ascontiguousarray(
            O.das_c_ref(e["ch"], e["fs"], e["t0"], e["atx"], e["arx"], e["dtx"], e["drx"], e["fd"], dim))
    cases["edges"] = e
    flat = {}
    for cname, c in cases.items():
        for k, v in c.items():
            flat[f"{cname}/{k}"] = np.asarray(v)
    np.savez_compressed(out_path, **flat)


# ---------------------------------------------------------------------------
# reference Python package
# ---------------------------------------------------------------------------

class _Pt:
    def __init__(self, x=0.0, y=0.0, z=0.0, azimuth=0.0, elevation=0.0, distance=0.0):
        self.x, self.y, self.z = x, y, z
        self.azimuth, self.elevation, self.distance = azimuth, elevation, distance


class _Wave:
    def __init__(self, wavefront, source, c=1540.0, delay=0.0):
        self.wavefront, self.source, self.sound_speed, self.delay = wavefront, source, c, delay


class _Probe:
    def __init__(self, x):
        self.x = np.asarray(x, float)
        self.y = np.zeros_like(self.x)
        self.z = np.zeros_like(self.x)

    @property
    def N_elements(self):
        return self.x.size


class _Scan:
    def __init__(self, x, z):
        self.x = np.asarray(x, float).ravel()
        self.z = np.asarray(z, float).ravel()
        self.y = np.zeros_like(self.x)

    @property
    def reference_distance(self):
        return self.z


class _CD:
    def __init__(self, data, probe, seq, fs, t0, c, fd):
        self.data, self.probe, self.sequence = data, probe, seq
        self.sampling_frequency, self.initial_time, self.sound_speed = fs, t0, c
        self.modulation_frequency = fd

    @property
    def N_channels(self):
        return self.data.shape[1]

    @property
    def N_waves(self):
        return self.data.shape[2]

    @property
    def N_frames(self):
        return self.data.shape[3]


def make_python_das(out_path, reference_root):
    sys.path.insert(0, os.path.join(reference_root, "python", "src"))
    from ustb.enums import Dimension, Wavefront, Window  # reference package
    from ustb.midprocess.das import DAS

    rng = np.random.default_rng(7)
    N, L, fs, c = 16, 400, 20e6, 1540.0
    x_el = (np.arange(1, N + 1) * 0.3e-3)
    x_el = x_el - x_el.mean()
    probe = _Probe(x_el)
    X, Z = np.meshgrid(np.linspace(-3e-3, 3e-3, 7), np.linspace(6e-3, 14e-3, 9))
    scan = _Scan(X.ravel(), Z.ravel())
    res = {"probe_x": x_el, "scan_x": scan.x, "scan_z": scan.z, "fs": fs, "c": c}
    seqs = {
        "plane": [_Wave(Wavefront.plane, _Pt(azimuth=a, distance=np.inf)) for a in (-0.2, 0.0, 0.15)],
        "diverging": [_Wave(Wavefront.spherical, _Pt(x=-2e-3 * s, z=-8e-3, azimuth=0.0,
                                                     distance=np.hypot(2e-3 * s, 8e-3)))
                      for s in (-1.0, 0.0, 1.0)],
        "focused": [_Wave(Wavefront.spherical, _Pt(x=xf, z=10e-3, distance=np.hypot(xf, 10e-3)))
                    for xf in (-1e-3, 0.0, 1e-3)],
    }
    for name, seq in seqs.items():
        W = len(seq)
        data = (rng.standard_normal((L, N, W, 1)) + 1j * rng.standard_normal((L, N, W, 1))).astype(np.complex64)
        fd = 5e6
        t0 = 1e-6
        mid = DAS()
        mid.channel_data = _CD(data, probe, seq, fs, t0, c, fd)
        mid.scan = scan
        mid.receive_apodization.window = Window.none
        mid.transmit_apodization.window = Window.none
        mid.dimension = Dimension.both
        b = mid.go()
        res[f"{name}/data"] = data
        res[f"{name}/t0"] = t0
        res[f"{name}/fd"] = fd
        res[f"{name}/rx_delay"] = np.asarray(mid.receive_delay)
        res[f"{name}/tx_delay"] = np.asarray(mid.transmit_delay)
        res[f"{name}/bf"] = np.asarray(b.data)
        res[f"{name}/src"] = np.array([[w.source.x, w.source.y, w.source.z, w.source.azimuth,
                                        w.source.elevation, w.source.distance] for w in seq])
    np.savez_compressed(out_path, **res)


def make_python_demod(out_path, reference_root):
    """Run the reference's Python FastDemodulation on seeded RF and keep its output."""
    import types

    sys.path.insert(0, os.path.join(reference_root, "python", "src"))
    # go() imports pyuff_ustb.objects.uff.Uff (unused); a stub module satisfies it
    for name in ("pyuff_ustb", "pyuff_ustb.objects", "pyuff_ustb.objects.uff"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["pyuff_ustb.objects.uff"].Uff = object
    from ustb.preprocess.fast_demodulation import FastDemodulation  # reference package

    rng = np.random.default_rng(17)
    cases = {
        # name: (L, N, W, fs, t0, fc, downsample_frequency)
        "default_dec": (600, 3, 2, 40e6, 2e-6, 5e6, None),
        "explicit_dec": (517, 2, 1, 50e6, 0.0, 3.5e6, 12e6),
        "no_dec": (400, 2, 2, 20e6, 1e-6, 4e6, 25e6),
        "int_like": (300, 4, 1, 31.25e6, 5e-7, 5.2e6, None),
    }
    res = {}
    for name, (L, N, W, fs, t0, fc, fds) in cases.items():
        t = t0 + np.arange(L) / fs
        env = np.exp(-((t[:, None, None] - rng.uniform(t[L // 4], t[3 * L // 4], (1, N, W))) * fc / 2) ** 2)
        rf = env * np.cos(2 * np.pi * fc * t[:, None, None] + rng.uniform(0, 2 * np.pi, (1, N, W)))
        rf += 0.05 * rng.standard_normal((L, N, W))
        if name == "int_like":
            rf = np.round(rf * 2000.0)
        cd = _CD(rf, _Probe(np.arange(N) * 3e-4), [None] * W, fs, t0, 1540.0, 0.0)
        cd.pulse = None
        dm = FastDemodulation()
        dm.input = cd
        dm.modulation_frequency = fc
        dm.downsample_frequency = fds
        out = dm.go()
        res[f"{name}/rf"] = rf
        res[f"{name}/params"] = np.array([fs, t0, fc, -1.0 if fds is None else fds])
        res[f"{name}/iq"] = np.asarray(out.data)
        res[f"{name}/fs_out"] = np.float64(out.sampling_frequency)
        res[f"{name}/t0_out"] = np.float64(out.initial_time)
    # too short for filtfilt's padding: the reference raises ValueError
    L = 150
    cd = _CD(rng.standard_normal((L, 1, 1)), _Probe(np.zeros(1)), [None], 20e6, 0.0, 1540.0, 0.0)
    cd.pulse = None
    dm = FastDemodulation()
    dm.input = cd
    dm.modulation_frequency = 4e6
    try:
        dm.go()
        raised = 0
    except ValueError:
        raised = 1
    res["short/L"] = np.int64(L)
    res["short/raises"] = np.int64(raised)
    np.savez_compressed(out_path, **res)


def make_python_cf(out_path, reference_root):
    """Run the reference's Python CoherenceFactor on a seeded cube."""
    sys.path.insert(0, os.path.join(reference_root, "python", "src"))
    from ustb.beamformed_data import BeamformedData  # reference package
    from ustb.enums import Dimension
    from ustb.postprocess.coherence_factor import CoherenceFactor

    rng = np.random.default_rng(23)
    P, N, W, F = 37, 6, 5, 2
    cube = (rng.standard_normal((P, N, W, F)) + 1j * rng.standard_normal((P, N, W, F))).astype(np.complex64)
    cube[:, :, :, 0] += (0.8 * np.exp(1j * rng.uniform(0, 2 * np.pi, (P, 1, 1)))).astype(np.complex64)
    cube[5] = 0  # a pixel with no signal: CF 0
    res = {"cube": cube}
    for name in ("receive", "transmit", "both"):
        cf = CoherenceFactor()
        cf.input = BeamformedData(scan=None, data=cube)
        cf.dimension = getattr(Dimension, name)
        out = cf.go()
        res[f"{name}/image"] = np.asarray(out.data)
    np.savez_compressed(out_path, **res)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("USTB_REFERENCE_ROOT"),
                    help="the reference checkout (default: $USTB_REFERENCE_ROOT)")
    a = ap.parse_args()
    if not a.reference:
        ap.error("give --reference <reference checkout> or set USTB_REFERENCE_ROOT")
    make_das_c_cases(os.path.join(HERE, "das_c_cases.npz"))
    make_python_das(os.path.join(HERE, "python_das.npz"), a.reference)
    make_python_demod(os.path.join(HERE, "python_demod.npz"), a.reference)
    make_python_cf(os.path.join(HERE, "python_cf.npz"), a.reference)
    for f in ("das_c_cases.npz", "python_das.npz", "python_demod.npz", "python_cf.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
