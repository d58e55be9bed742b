"""Pins the oracle (oracle/das_port.c) before anything is checked against it.

* bit-exact against the golden outputs of the reference's own das_c
  (+mex/source/das_c.cpp, compiled unmodified; tests/golden/make_golden.py),
  all four sum modes, edge cases included;
* bit-exact against the reference das_c on fresh seeded inputs when it is
  built on this machine (oracle/_ref);
* the FP64 restatement under the interp1 edge rule against the reference
  Python package's DAS output (python/src/ustb/midprocess/das.py:203-261).
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

CASES = ("iq_small", "iq_long_delay", "rf_analytic", "edges")


def _load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def _case(z, name):
    return {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("dim", [0, 1, 2, 3])
def test_port_matches_reference_golden_bit_exact(golden_dir, case, dim):
    c = _case(_load(golden_dir, "das_c_cases.npz"), case)
    out = O.das_f32(c["ch"], c["fs"], c["t0"], c["atx"], c["arx"], c["dtx"], c["drx"], c["fd"], dim,
                    threads=3)
    ref = c[f"out_dim{dim}"]
    assert out.shape == ref.shape
    assert np.array_equal(_bits(out), _bits(ref))


def test_edge_golden_has_the_das_c_rule(golden_dir):
    """das_c never uses sample 0 nor n0 = L-1 (das_c.cpp:377,381)."""
    c = _case(_load(golden_dir, "das_c_cases.npz"), "edges")
    out = c["out_dim0"]  # [P, N, W, F]
    L = c["ch"].shape[0]
    f32 = np.float32
    live_units = 0
    for p in range(out.shape[0]):
        for n in range(out.shape[1]):
            for w in range(out.shape[2]):
                if c["atx"][p, w] == 0 or c["arx"][p, n] == 0:
                    assert np.all(out[p, n, w] == 0)
                    continue
                delay = f32(c["dtx"][p, w] + c["drx"][p, n])
                denay = f32(f32(delay - c["t0"]) * c["fs"])
                n0 = int(denay) if abs(denay) < 2 ** 31 else -1
                if 0 < n0 < L - 1:
                    live_units += 1
                    assert np.any(out[p, n, w] != 0)
                else:
                    assert np.all(out[p, n, w] == 0), (p, n, w, denay)
    assert live_units > 0


@pytest.mark.skipif(not O.have_reference(), reason="reference das_c not built here")
@pytest.mark.parametrize("seed", [11, 12])
def test_port_matches_reference_das_c_fresh(seed):
    rng = np.random.default_rng(seed)
    L, N, W, F, P = 128, 12, 5, 2, 300
    ch = (rng.standard_normal((L, N, W, F)) + 1j * rng.standard_normal((L, N, W, F))).astype(np.complex64)
    t0, fs, fd = np.float32(3e-6), np.float32(25e6), np.float32(6.25e6)
    dtx = (rng.uniform(0, 3e-6, (P, W)) + 3e-6).astype(np.float32)
    drx = rng.uniform(0, 3e-6, (P, N)).astype(np.float32)
    atx = rng.uniform(0, 1, (P, W)).astype(np.float32)
    arx = rng.uniform(-0.1, 1, (P, N)).astype(np.float32)
    arx[rng.random((P, N)) < 0.3] = 0
    for dim in range(4):
        a = O.das_c_ref(ch, fs, t0, atx, arx, dtx, drx, fd, dim)
        b = O.das_f32(ch, fs, t0, atx, arx, dtx, drx, fd, dim, threads=4)
        assert np.array_equal(_bits(a), _bits(b))


def test_port_thread_count_invariant(golden_dir):
    c = _case(_load(golden_dir, "das_c_cases.npz"), "iq_small")
    a = O.das_f32(c["ch"], c["fs"], c["t0"], c["atx"], c["arx"], c["dtx"], c["drx"], c["fd"], 3, threads=1)
    b = O.das_f32(c["ch"], c["fs"], c["t0"], c["atx"], c["arx"], c["dtx"], c["drx"], c["fd"], 3, threads=7)
    assert np.array_equal(_bits(a), _bits(b))


@pytest.mark.parametrize("case", ["iq_small", "iq_long_delay"])
def test_f64_oracle_close_to_das_c(golden_dir, case):
    c = _case(_load(golden_dir, "das_c_cases.npz"), case)
    for dim in range(4):
        o64 = O.das_f64(c["ch"].astype(np.complex128), float(c["fs"]), float(c["t0"]), c["atx"],
                        c["arx"], c["dtx"], c["drx"], float(c["fd"]), dim)
        ref = c[f"out_dim{dim}"]
        rel = np.linalg.norm(o64 - ref) / np.linalg.norm(o64)
        # das_c's own single-precision rounding of delay and phase (1e-4 rad at 40 us)
        assert rel < 3e-4, rel


@pytest.mark.parametrize("seq", ["plane", "diverging", "focused"])
def test_f64_interp1_rule_matches_reference_python_das(golden_dir, seq):
    z = np.load(os.path.join(golden_dir, "python_das.npz"))
    data = z[f"{seq}/data"]
    rxd, txd = z[f"{seq}/rx_delay"], z[f"{seq}/tx_delay"]
    P, N = rxd.shape
    W = txd.shape[1]
    fs, t0, fd, c = float(z["fs"]), float(z[f"{seq}/t0"]), float(z[f"{seq}/fd"]), float(z["c"])
    # the Python package forms its sample index from float32 time-axis values
    fs32 = 1.0 / (float(np.float32(t0) + np.float32(1) / np.float32(fs)) - float(np.float32(t0)))
    out = O.das_f64(data.astype(np.complex128), fs32, float(np.float32(t0)),
                    np.ones((P, W)), np.ones((P, N)), txd.astype(np.float64), rxd.astype(np.float64),
                    float(np.float32(fd)), 3, edge_rule=1)
    w0 = 2 * np.pi * np.float32(fd)
    out = out[:, 0, 0, 0] * np.exp(-1j * 2 * w0 * z["scan_z"] / c)
    ref = z[f"{seq}/bf"][:, 0, 0, 0]
    rel = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert rel < 2e-4, rel


def test_cf_and_sdmas_restatements():
    s = np.array([[1 + 0j, 1 + 0j, 1 + 0j, 1 + 0j]])  # fully coherent, M = 4
    cf, img = O.coherence_factor(s[:, :, None], [4])
    assert np.allclose(cf, 1.0) and np.allclose(img, 4.0)
    s2 = np.array([[1 + 0j, -1 + 0j]])
    cf2, _ = O.coherence_factor(s2[:, :, None], [2])
    assert np.allclose(cf2, 0.0)
    v = O.sdmas_value(np.array([[4.0, 1.0, -9.0]])[:, :, None])
    # ((2 + 1 - 3)^2 - 14) / 2 = -7
    assert np.allclose(v, -7.0)


@pytest.mark.parametrize("dim", ["receive", "transmit", "both"])
def test_cf_restatement_matches_reference_python_coherence_factor(golden_dir, dim):
    """oracle.coherence_factor against the image of the reference's Python
    CoherenceFactor (python/src/ustb/postprocess/coherence_factor.py), whose M is the
    number of summed channels / waves: the restatement with every unit active."""
    d = np.load(os.path.join(golden_dir, "python_cf.npz"))
    cube = d["cube"].astype(np.complex128)
    P, N, W, F = cube.shape
    if dim == "receive":
        s, M = cube, N                                           # sum over channels
    elif dim == "transmit":
        s, M = np.swapaxes(cube, 1, 2), W                        # sum over waves
    else:
        s, M = cube.reshape((P, N * W, 1, F), order="F"), N * W  # both
    cf, img = O.coherence_factor(s, np.full(P, M))
    want = d[f"{dim}/image"]
    got = img if dim != "transmit" else np.swapaxes(img, 1, 2)
    got = got.reshape(want.shape, order="F")
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-6
    assert np.all(got[5] == 0) and np.all(want[5] == 0)  # the silent pixel
