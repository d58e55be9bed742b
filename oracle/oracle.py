"""ORACLE — CPU checker for the delay-and-sum path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module.  The product package ``ustb_gb300`` never does.

What is here:

* ``das_f32``      — ctypes front end of ``das_port.c:oracle_das_f32``, the
                     operation-for-operation single-precision restatement of the
                     reference's das_c loop (+mex/source/das_c.cpp:355-409).
* ``das_f64``      — the same formula in double precision ("FP64 oracle").
* ``das_c_ref``    — the reference's own das_c (+mex/source/das_c.cpp) compiled
                     unmodified by ``make -C oracle ref`` into oracle/_ref/.
                     Available only where the reference sources were present at
                     build time (the checkout, or the copy ``make -C oracle stage``
                     puts into the git-ignored oracle/_ref/src/ so that it travels to
                     the GPU machine); returns None otherwise.
* ``das_cuda_ref`` — the reference's own das_cuda (+mex/source/das_cuda.cu,
                     dimension both only) compiled unmodified for sm_103a by
                     ``make -C oracle ref_cuda``; None where it was not built.
* ``coherence_factor`` / ``sdmas_value`` — FP64 numpy restatements of
                     +postprocess/coherence_factor.m:100-135 and of the per-pixel
                     term of +postprocess/simplified_delay_multiply_and_sum.m:140-148.
                     The CF is pinned to the output of the reference's Python
                     CoherenceFactor (tests/golden/python_cf.npz).
* ``phase_coherence_factor_f64`` / ``generalized_coherence_factor_f64`` — FP64
                     numpy restatements of +postprocess/phase_coherence_factor.m:64-129
                     (with tools/weigthed_std.m, weigthed_var.m, weigthed_mean.m) and
                     +postprocess/generalized_coherence_factor.m:66-97 over one
                     dimension.  Parity unpinned (no golden vectors in the reference).
* ``capon_f64``     — FP64 numpy restatement of capon_minimum_variance_implementation
                     (+postprocess/capon_minimum_variance.m:117-177).  Parity unpinned.
* ``scan_convert_f64`` — FP64 numpy restatement of get_image's compression
                     (+uff/beamformed_data.m:300-316) and +tools/scan_convert.m
                     (bilinear interp2 in (azimuth, depth), -inf outside).  Parity
                     unpinned: no golden vectors in the reference.
* ``fast_demodulation_f64`` — FP64 numpy restatement of the down-mix, causal FIR
                     and decimation of +preprocess/fast_demodulation.m:121-167.
                     Parity unpinned: the reference ships no golden vectors for
                     this step and MATLAB is not available to run it.
* ``hamming_lowpass_taps`` / ``zero_phase_demodulation_f64`` — FP64 numpy
                     restatement of the reference's Python port,
                     python/src/ustb/preprocess/fast_demodulation.py:42-88: Hamming
                     windowed-sinc low-pass (scipy firwin's method), down-mix,
                     forward-backward filtering with odd extension and steady-state
                     initial conditions (scipy filtfilt's method), decimation by
                     slicing.  Pinned to that code's own outputs
                     (tests/golden/python_demod.npz).

Array convention: every array is given with its MATLAB logical shape
(channel data [L, N, W, F], tables [P, W] / [P, N]) and is passed to C in
column-major (Fortran) order, as MATLAB stores it.  Outputs come back as
Fortran-ordered arrays of shape [P, N|1, W|1, F].
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PORT_SO = os.path.join(_HERE, "_build", "liboracle.so")
_REF_SO = os.path.join(_HERE, "_ref", "libdas_c_ref.so")
_CUDA_SO = os.path.join(_HERE, "_ref", "libdas_cuda_ref.so")
_STAGED = os.path.join(_HERE, "_ref", "src")

_port = None
_ref = None
_cuda_ref = None

_i64 = ctypes.c_int64
_f32 = ctypes.c_float
_f64 = ctypes.c_double
_ptr = ctypes.c_void_p


def build(reference: Optional[str] = None) -> None:
    """Compile the C restatement; and the reference's own das_c and das_cuda, from the
    checkout at ``reference`` (or ``$USTB_REFERENCE_ROOT``), whose two sources are then
    also staged into oracle/_ref/src/, or else from an earlier staged copy."""
    import shutil
    import subprocess

    subprocess.check_call(["make", "-s", "-C", _HERE, "all"])
    ref = reference or os.environ.get("USTB_REFERENCE_ROOT")
    args = []
    if ref and os.path.isfile(os.path.join(ref, "+mex", "source", "das_c.cpp")):
        subprocess.check_call(["make", "-s", "-C", _HERE, "stage", f"REF={ref}"])
    elif not os.path.isfile(os.path.join(_STAGED, "das_c.cpp")):
        return
    subprocess.check_call(["make", "-s", "-C", _HERE, "ref"] + args)
    if shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc"):
        env = dict(os.environ)
        if not shutil.which("nvcc"):
            env["NVCC"] = "/usr/local/cuda/bin/nvcc"
        # the reference GPU point is optional: a failed build leaves it unavailable
        subprocess.call(["make", "-s", "-C", _HERE, "ref_cuda"] + args, env=env)


def _load_port():
    global _port
    if _port is None:
        if not os.path.isfile(_PORT_SO):
            build()
        lib = ctypes.CDLL(_PORT_SO)
        lib.oracle_das_f32.restype = ctypes.c_int
        lib.oracle_das_f32.argtypes = [_ptr, _i64, _i64, _i64, _i64, _f32, _f32, _ptr, _ptr, _ptr,
                                       _ptr, _i64, _f32, ctypes.c_int32, _ptr, ctypes.c_int]
        lib.oracle_das_f64.restype = ctypes.c_int
        lib.oracle_das_f64.argtypes = [_ptr, _i64, _i64, _i64, _i64, _f64, _f64, _ptr, _ptr, _ptr,
                                       _ptr, _i64, _f64, ctypes.c_int32, ctypes.c_int32, _ptr,
                                       ctypes.c_int]
        _port = lib
    return _port


def _load_ref():
    global _ref
    if _ref is None:
        if not os.path.isfile(_REF_SO):
            return None
        lib = ctypes.CDLL(_REF_SO)
        lib.das_c_ref_run.restype = ctypes.c_int
        lib.das_c_ref_run.argtypes = [_ptr, _i64, _i64, _i64, _i64, _f32, _f32, _ptr, _ptr, _ptr,
                                      _ptr, _i64, _f32, ctypes.c_int32, _ptr, ctypes.c_char_p,
                                      ctypes.c_int]
        _ref = lib
    return _ref


def have_reference() -> bool:
    return _load_ref() is not None


def _load_cuda_ref():
    global _cuda_ref
    if _cuda_ref is None:
        if not os.path.isfile(_CUDA_SO):
            return None
        try:
            lib = ctypes.CDLL(_CUDA_SO)
        except OSError:
            return None
        lib.das_cuda_ref_run.restype = ctypes.c_int
        lib.das_cuda_ref_run.argtypes = [_ptr, _i64, _i64, _i64, _i64, _f32, _f32, _ptr, _ptr, _ptr,
                                         _ptr, _i64, _f32, ctypes.c_int32, _ptr, ctypes.c_char_p,
                                         ctypes.c_int, ctypes.c_int32]
        _cuda_ref = lib
    return _cuda_ref


def have_cuda_reference() -> bool:
    return _load_cuda_ref() is not None


def _dims(ch):
    s = list(ch.shape) + [1] * (4 - ch.ndim)
    return tuple(int(v) for v in s[:4])


def out_shape(P, N, W, F, dim):
    return {0: (P, N, W, F), 1: (P, 1, W, F), 2: (P, N, 1, F), 3: (P, 1, 1, F)}[int(dim)]


def _f(a, dtype):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


def _threads(threads):
    return int(threads) if threads else (os.cpu_count() or 1)


def das_f32(ch, fs, t0, apo_tx, apo_rx, delay_tx, delay_rx, fd, dim, threads=None):
    """Single-precision das_c restatement. ``ch`` complex64 [L,N,W,F]."""
    L, N, W, F = _dims(ch)
    c = _f(ch, np.complex64).reshape((L, N, W, F), order="F")
    atx, arx = _f(apo_tx, np.float32), _f(apo_rx, np.float32)
    dtx, drx = _f(delay_tx, np.float32), _f(delay_rx, np.float32)
    P = atx.shape[0]
    out = np.zeros(out_shape(P, N, W, F, dim), dtype=np.complex64, order="F")
    rc = _load_port().oracle_das_f32(c.ctypes.data, L, N, W, F, float(np.float32(fs)),
                                     float(np.float32(t0)), atx.ctypes.data, arx.ctypes.data,
                                     dtx.ctypes.data, drx.ctypes.data, P, float(np.float32(fd)),
                                     int(dim), out.ctypes.data, _threads(threads))
    if rc != 0:
        raise ValueError(f"oracle_das_f32 rejected its arguments (rc={rc})")
    return out


def das_f64(ch, fs, t0, apo_tx, apo_rx, delay_tx, delay_rx, fd, dim, edge_rule=0, threads=None):
    """Double-precision restatement of the same formula. ``ch`` complex128 [L,N,W,F]."""
    L, N, W, F = _dims(ch)
    c = _f(ch, np.complex128).reshape((L, N, W, F), order="F")
    atx, arx = _f(apo_tx, np.float64), _f(apo_rx, np.float64)
    dtx, drx = _f(delay_tx, np.float64), _f(delay_rx, np.float64)
    P = atx.shape[0]
    out = np.zeros(out_shape(P, N, W, F, dim), dtype=np.complex128, order="F")
    rc = _load_port().oracle_das_f64(c.ctypes.data, L, N, W, F, float(fs), float(t0),
                                     atx.ctypes.data, arx.ctypes.data, dtx.ctypes.data,
                                     drx.ctypes.data, P, float(fd), int(dim), int(edge_rule),
                                     out.ctypes.data, _threads(threads))
    if rc != 0:
        raise ValueError(f"oracle_das_f64 rejected its arguments (rc={rc})")
    return out


def das_c_ref(ch, fs, t0, apo_tx, apo_rx, delay_tx, delay_rx, fd, dim) -> Optional[np.ndarray]:
    """The reference's das_c itself (None when it was not built on this machine)."""
    lib = _load_ref()
    if lib is None:
        return None
    L, N, W, F = _dims(ch)
    c = _f(ch, np.complex64).reshape((L, N, W, F), order="F")
    atx, arx = _f(apo_tx, np.float32), _f(apo_rx, np.float32)
    dtx, drx = _f(delay_tx, np.float32), _f(delay_rx, np.float32)
    P = atx.shape[0]
    out = np.zeros(out_shape(P, N, W, F, dim), dtype=np.complex64, order="F")
    err = ctypes.create_string_buffer(512)
    rc = lib.das_c_ref_run(c.ctypes.data, L, N, W, F, float(np.float32(fs)), float(np.float32(t0)),
                           atx.ctypes.data, arx.ctypes.data, dtx.ctypes.data, drx.ctypes.data, P,
                           float(np.float32(fd)), int(dim), out.ctypes.data, err, 512)
    if rc != 0:
        raise ValueError(err.value.decode())
    return out


def das_cuda_ref(ch, fs, t0, apo_tx, apo_rx, delay_tx, delay_rx, fd, gpu=0) -> Optional[np.ndarray]:
    """The reference's das_cuda itself on GPU ``gpu`` (dimension both; host buffers in
    and out, as its MEX call takes them).  None when it was not built here."""
    lib = _load_cuda_ref()
    if lib is None:
        return None
    L, N, W, F = _dims(ch)
    c = _f(ch, np.complex64).reshape((L, N, W, F), order="F")
    atx, arx = _f(apo_tx, np.float32), _f(apo_rx, np.float32)
    dtx, drx = _f(delay_tx, np.float32), _f(delay_rx, np.float32)
    P = atx.shape[0]
    out = np.zeros(out_shape(P, N, W, F, 3), dtype=np.complex64, order="F")
    err = ctypes.create_string_buffer(512)
    rc = lib.das_cuda_ref_run(c.ctypes.data, L, N, W, F, float(np.float32(fs)), float(np.float32(t0)),
                              atx.ctypes.data, arx.ctypes.data, dtx.ctypes.data, drx.ctypes.data, P,
                              float(np.float32(fd)), 3, out.ctypes.data, err, 512, int(gpu))
    if rc != 0:
        raise ValueError(err.value.decode())
    return out


def coherence_factor(s, active_count):
    """CF per +postprocess/coherence_factor.m:122-135 over axis 1 (channels).

    ``s`` complex [P, N, ...]; ``active_count`` M per pixel.  Returns (CF, CF*sum).
    """
    s = np.asarray(s, dtype=np.complex128)
    coh = s.sum(axis=1, keepdims=True)
    inc = (np.abs(s) ** 2).sum(axis=1, keepdims=True)
    M = np.asarray(active_count, dtype=np.float64).reshape((-1,) + (1,) * (s.ndim - 1))
    with np.errstate(divide="ignore", invalid="ignore"):
        cf = (np.abs(coh) ** 2 / inc) * (1.0 / M)
    cf[np.isnan(cf)] = 0.0
    return cf, cf * coh


def sdmas_value(s_real):
    """Per-pixel simplified-DMAS term, simplified_delay_multiply_and_sum.m:143-146,
    over axis 1 of a real array [P, N, ...]: ((sum sign*sqrt|s|)^2 - sum|s|)/2."""
    s = np.asarray(s_real, dtype=np.float64)
    root = (np.sign(s) * np.sqrt(np.abs(s))).sum(axis=1, keepdims=True)
    absum = np.abs(s).sum(axis=1, keepdims=True)
    return (root ** 2 - absum) / 2.0


def sdmas_filtered(y, taps):
    """Band-pass along axis 0 with delay compensation and Hilbert transform
    (simplified_delay_multiply_and_sum.m:170-192): y real [Nz, ...]."""
    from scipy.signal import hilbert, lfilter

    y = np.asarray(y, np.float64)
    d = int(round((len(taps) - 1) / 2))
    pad = np.concatenate([y, np.zeros((d,) + y.shape[1:])], axis=0)
    f = lfilter(taps, 1.0, pad, axis=0)[d:]
    return hilbert(f, axis=0)


def fast_demodulation_f64(rf, fs, t0, fc, taps, decimation):
    """IQ of real RF ``rf`` [L, ...] (time first, as MATLAB stores channel data):
    data .* exp(-1j*2*pi*fc*time) (fast_demodulation.m:121), filter(b, 1, data, [], 1)
    (:140), data(1:D:end, ...) (:162), all in double precision."""
    from scipy.signal import lfilter

    x = np.asarray(rf, np.float64)
    t = float(t0) + np.arange(x.shape[0]) / float(fs)
    mix = np.exp(-1j * 2 * np.pi * float(fc) * t).reshape((-1,) + (1,) * (x.ndim - 1))
    y = lfilter(np.asarray(taps, np.float64), [1.0], x * mix, axis=0)
    return y[::int(decimation)]


def hamming_lowpass_taps(numtaps, cutoff, fs):
    """Windowed-sinc low-pass with a Hamming window, scaled to unit gain at DC: the
    design scipy's firwin(numtaps, cutoff, fs=fs) makes for the reference's Python
    port (fast_demodulation.py:57-63)."""
    n = np.arange(int(numtaps), dtype=np.float64) - (int(numtaps) - 1) / 2.0
    wc = 2.0 * float(cutoff) / float(fs)  # relative to Nyquist
    h = wc * np.sinc(wc * n)
    h *= 0.54 - 0.46 * np.cos(2.0 * np.pi * np.arange(int(numtaps)) / (int(numtaps) - 1))
    return h / h.sum()


def _steady_fir(b, x):
    """y[n] = sum_k b[k] x[max(n - k, 0)] along axis 0: FIR whose input is held at
    x[0] before the start (lfilter with zi = lfilter_zi(b, 1) * x[0])."""
    M = len(b)
    pad = np.concatenate([np.repeat(x[:1], M - 1, axis=0), x], axis=0)
    y = np.zeros_like(x)
    for k in range(M):
        y += b[k] * pad[M - 1 - k:M - 1 - k + x.shape[0]]
    return y


def zero_phase_demodulation_f64(rf, fs, t0, fc, taps, decimation):
    """IQ of real RF ``rf`` [L, ...] as the reference's Python port makes it
    (fast_demodulation.py:47-76): data * exp(-1j 2 pi fc t), then filtfilt(b, 1, .)
    along time — odd extension by P = 3 len(b) samples at both ends, the FIR run
    forward and backward, each with the input held at its first value before the
    start, P samples stripped from both ends — then iq[::D].  Raises ValueError
    when L <= P, as filtfilt does."""
    b = np.asarray(taps, np.float64)
    x = np.asarray(rf, np.float64)
    L = x.shape[0]
    P = 3 * len(b)
    if L <= P:
        raise ValueError(f"trace of {L} samples is not longer than the padding {P}")
    t = float(t0) + np.arange(L) / float(fs)
    mix = x * np.exp(-1j * 2 * np.pi * float(fc) * t).reshape((-1,) + (1,) * (x.ndim - 1))
    ext = np.concatenate([2 * mix[:1] - mix[P:0:-1], mix, 2 * mix[-1:] - mix[-2:-(P + 2):-1]], axis=0)
    f = _steady_fir(b, ext)
    g = _steady_fir(b, f[::-1])[::-1]
    return g[P:P + L][::int(decimation)]


def scan_convert_f64(img, depth_axis, azimuth_axis, xs, zs, compression="log"):
    """Compressed image [n_depth, n_azimuth, F] (|.| of complex or real data) on the
    Cartesian grid (xs, zs): returns [F, len(zs), len(xs)], -inf outside the sector.
    Follows scan_convert.m: cart2pol(Zs, Xs) -> theta = atan2(x, z), r = hypot(x, z);
    interp2(thetaGrid, rangeGrid, image, theta, r, 'linear', -inf)."""
    a = np.abs(np.asarray(img)).astype(np.float64)
    if a.ndim == 2:
        a = a[:, :, None]
    if compression == "log":
        v = 20 * np.log10(a / a.max())
    elif compression == "sqrt":
        v = np.sqrt(a)
    else:
        v = a
    d = np.asarray(depth_axis, np.float64)
    t = np.asarray(azimuth_axis, np.float64)
    X, Z = np.meshgrid(np.asarray(xs, np.float64), np.asarray(zs, np.float64))
    th, r = np.arctan2(X, Z), np.hypot(X, Z)
    out = np.full((v.shape[2],) + X.shape, -np.inf)
    ok = (r >= d[0]) & (r <= d[-1]) & (th >= t[0]) & (th <= t[-1])
    i = np.clip(np.searchsorted(d, r[ok], side="right") - 1, 0, d.size - 2)
    j = np.clip(np.searchsorted(t, th[ok], side="right") - 1, 0, t.size - 2)
    u = (r[ok] - d[i]) / (d[i + 1] - d[i])
    w = (th[ok] - t[j]) / (t[j + 1] - t[j])
    for f in range(v.shape[2]):
        vf = v[:, :, f]
        out[f][ok] = ((1 - u) * ((1 - w) * vf[i, j] + w * vf[i, j + 1])
                      + u * ((1 - w) * vf[i + 1, j] + w * vf[i + 1, j + 1]))
    return out


def _wmean(D, W, axis):
    return (W * D).sum(axis) / W.sum(axis)


def _wvar(D, W, axis):
    m = np.expand_dims(_wmean(D, W, axis), axis)
    return (W * (D - m) ** 2).sum(axis) / W.sum(axis)


def phase_coherence_factor_f64(data, weights=None, gamma=1.0, sigma_0=np.pi / np.sqrt(3), axis=1):
    """FCA, FCC and FCC * coherent sum over ``axis`` of complex ``data`` (e.g. [P, K])."""
    d = np.asarray(data, np.complex128)
    W = np.ones(d.shape) if weights is None else np.broadcast_to(np.asarray(weights, np.float64), d.shape)
    phase = np.angle(d)
    aux = np.where(phase <= 0, phase + np.pi, phase - np.pi)
    sf = np.minimum(np.sqrt(_wvar(phase, W, axis)), np.sqrt(_wvar(aux, W, axis)))
    fca = 1 - (gamma / sigma_0) * sf
    fca[fca < 0] = 0
    fca[np.isnan(fca)] = 0
    fcc = 1 - np.sqrt(_wvar(np.cos(phase), W, axis) + _wvar(np.sin(phase), W, axis))
    return fca, fcc, fcc * d.sum(axis)


def generalized_coherence_factor_f64(data, M0=4, axis=1):
    """GCF and GCF * coherent sum over ``axis`` of complex ``data``."""
    d = np.asarray(data, np.complex128)
    K = d.shape[axis]
    idx = np.r_[0:M0 + 1, K - M0:K] if M0 > 1 else np.array([0])
    X = np.abs(np.fft.fft(d, axis=axis)) ** 2
    g = np.take(X, idx, axis=axis).sum(axis) / X.sum(axis)
    g[np.isnan(g)] = 0
    return g, g * d.sum(axis)


def capon_f64(data_cube, apod, L_elements, K_samples, regCoef, crit=0.16, fb=False):
    """z [N, E] from data_cube [N (depth), E (lateral), M] and apod [N, E, M], following
    capon_minimum_variance_implementation line by line (0-based indices)."""
    d = np.asarray(data_cube, np.complex128)
    ap = np.asarray(apod, np.float64)
    N, E, M = d.shape
    z = np.zeros((N, E), np.complex128)
    eps = np.finfo(np.float64).eps
    for e in range(E):
        rf = d[:, e, :]
        for k in range(N):
            if np.sum(np.abs(rf[k]) > eps) == 0:
                continue
            idx = np.nonzero(np.abs(ap[k, e]) > crit)[0]
            Mn = idx.size
            if Mn < 2:
                z[k, e] = rf[k].sum()
                continue
            Ln = int(np.floor(L_elements / M * Mn))
            Ln = 1 if Ln < 1 else (Mn - 1 if Ln >= Mn else Ln)
            if idx[-1] - Ln + 1 < idx[0]:
                z[k, e] = rf[k].sum()
                continue
            if k - K_samples < 0:
                rows = rf[:k + K_samples + 1]
            elif k + K_samples > N - 1:
                rows = rf[k - K_samples:]
            else:
                rows = rf[k - K_samples:k + K_samples + 1]
            R = np.zeros((Ln, Ln), np.complex128)
            for l in range(idx[0], idx[-1] - Ln + 2):
                A = rows[:, l:l + Ln]
                R += A.conj().T @ A
            R /= (2 * K_samples + 1) * (Mn - Ln + 1)
            if fb:
                R = 0.5 * (R + np.rot90(R.conj(), 2))
            a = np.ones(Ln)
            Ria = np.linalg.solve(R + np.eye(Ln) * (regCoef / Ln) * np.trace(R), a)
            w = Ria / (a.conj() @ Ria)
            acc = 0
            for j in range(idx[0], idx[-1] - Ln + 2):
                acc += w.conj() @ rf[k, j:j + Ln].conj()
            z[k, e] = acc / (Mn - Ln + 1) * Mn
    return z
