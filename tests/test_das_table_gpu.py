"""Parity of the single-precision table kernel (the das_c drop-in) on the GPU.

Bar: relative L2 <= 1e-5 against the reference's das_c (golden fixtures made
by the reference itself) and against the oracle port on fresh inputs.  Calls go
through the C-ABI (ustb_das_table_f32 / _host).
"""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def _case(golden_dir, name):
    z = np.load(os.path.join(golden_dir, "das_c_cases.npz"))
    return {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}


def to_dev_ch(ch, dev):
    """MATLAB [L,N,W,F] numpy -> ABI (F,W,N,L) tensor."""
    return torch.from_numpy(np.ascontiguousarray(ch.transpose(3, 2, 1, 0))).to(dev)


def to_dev_tab(t, dev):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(t, np.float32).T)).to(dev)


def from_dev_out(t):
    """ABI (F,Wk,Nk,P) -> MATLAB [P,Nk,Wk,F] numpy."""
    return t.cpu().numpy().transpose(3, 2, 1, 0)


def run_table(c, dim, dev, real=False):
    from ustb_gb300 import kernels

    ch = c["ch"].real.astype(np.float32) if real else c["ch"]
    out = kernels.das_table_f32(to_dev_ch(ch, dev), float(c["fs"]), float(c["t0"]),
                                to_dev_tab(c["atx"], dev), to_dev_tab(c["arx"], dev),
                                to_dev_tab(c["dtx"], dev), to_dev_tab(c["drx"], dev),
                                float(c["fd"]), dim)
    torch.cuda.synchronize()
    return from_dev_out(out)


@pytest.mark.parametrize("case", ["iq_small", "iq_long_delay", "rf_analytic", "edges"])
@pytest.mark.parametrize("dim", [0, 1, 2, 3])
def test_table_kernel_vs_reference_das_c_golden(golden_dir, cuda_dev, case, dim):
    c = _case(golden_dir, case)
    out = run_table(c, dim, cuda_dev)
    ref = c[f"out_dim{dim}"]
    assert out.shape == ref.shape
    assert rel_l2(out, ref) <= TOL
    # units das_c leaves at zero stay exactly zero
    assert np.all(out[ref == 0] == 0)


@pytest.mark.parametrize("F", [1, 2, 3, 5])
@pytest.mark.parametrize("dim", [0, 1, 2, 3])
def test_table_kernel_vs_oracle_frames(cuda_dev, F, dim):
    rng = np.random.default_rng(100 + F)
    L, N, W, P = 200, 9, 4, 333
    ch = (rng.standard_normal((L, N, W, F)) + 1j * rng.standard_normal((L, N, W, F))).astype(np.complex64)
    c = dict(ch=ch, fs=np.float32(20e6), t0=np.float32(1e-6), fd=np.float32(5e6),
             dtx=(rng.uniform(0, 4.5e-6, (P, W)) + 1e-6).astype(np.float32),
             drx=rng.uniform(0, 4.5e-6, (P, N)).astype(np.float32),
             atx=rng.uniform(0, 1, (P, W)).astype(np.float32),
             arx=rng.uniform(-0.2, 1, (P, N)).astype(np.float32))
    c["arx"][rng.random((P, N)) < 0.25] = 0
    out = run_table(c, dim, cuda_dev)
    ref = O.das_f32(c["ch"], c["fs"], c["t0"], c["atx"], c["arx"], c["dtx"], c["drx"], c["fd"], dim)
    assert rel_l2(out, ref) <= TOL


@pytest.mark.parametrize("dim", [0, 1, 2, 3])
def test_table_kernel_rf_real_path(golden_dir, cuda_dev, dim):
    """Real RF in, real out == real(das_c(x + 0j)) with fd = 0."""
    c = _case(golden_dir, "rf_analytic")
    out = run_table(c, dim, cuda_dev, real=True)
    ch0 = c["ch"].real.astype(np.float32).astype(np.complex64)
    ref = O.das_f32(ch0, c["fs"], c["t0"], c["atx"], c["arx"], c["dtx"], c["drx"], 0.0, dim).real
    assert out.dtype == np.float32
    assert rel_l2(out, ref) <= TOL


def test_table_kernel_deterministic(golden_dir, cuda_dev):
    c = _case(golden_dir, "iq_small")
    a = run_table(c, 3, cuda_dev)
    b = run_table(c, 3, cuda_dev)
    assert np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32))


def test_host_entry_point(golden_dir, cuda_dev):
    from ustb_gb300 import _lib

    c = _case(golden_dir, "iq_small")
    for dim in range(4):
        ref = c[f"out_dim{dim}"]
        out = np.zeros(ref.shape, np.complex64, order="F")
        f = lambda a: np.asfortranarray(a)
        ch, atx, arx, dtx, drx = f(c["ch"]), f(c["atx"]), f(c["arx"]), f(c["dtx"]), f(c["drx"])
        L, N, W, F = ch.shape
        _lib.call("ustb_das_table_f32_host", ch.ctypes.data, 1, L, N, W, F, float(c["fs"]),
                  float(c["t0"]), atx.ctypes.data, arx.ctypes.data, dtx.ctypes.data, drx.ctypes.data,
                  atx.shape[0], float(c["fd"]), dim, out.ctypes.data, 0)
        assert rel_l2(out, ref) <= TOL


def test_empty_and_degenerate_sizes(cuda_dev):
    from ustb_gb300 import kernels

    dev = cuda_dev
    # P = 0: nothing to do
    ch = torch.zeros((1, 1, 2, 8), dtype=torch.complex64, device=dev)
    e = torch.zeros((1, 0), dtype=torch.float32, device=dev)
    e2 = torch.zeros((2, 0), dtype=torch.float32, device=dev)
    out = kernels.das_table_f32(ch, 1.0, 0.0, e, e2, e, e2, 0.0, 3)
    assert out.numel() == 0
    # L = 2: no valid n0 exists (0 < n0 < 1) -> zeros, like das_c
    ch = torch.ones((1, 1, 2, 2), dtype=torch.complex64, device=dev)
    t = torch.full((1, 5), 1.0, dtype=torch.float32, device=dev)
    t2 = torch.full((2, 5), 1.0, dtype=torch.float32, device=dev)
    out = kernels.das_table_f32(ch, 1.0, 0.0, t, t2, t * 0.5, t2 * 0.25, 0.0, 0)
    torch.cuda.synchronize()
    assert torch.count_nonzero(out).item() == 0
    # L = 1 and 2, real and complex, sample positions well past the trace: no valid unit
    for L in (1, 2):
        for cplx in (True, False):
            ch = torch.ones((1, 2, 3, L), dtype=torch.complex64 if cplx else torch.float32, device=dev)
            ta = torch.ones((2, 7), dtype=torch.float32, device=dev)
            ra = torch.ones((3, 7), dtype=torch.float32, device=dev)
            for dim in range(4):
                out = kernels.das_table_f32(ch, 1.0, 0.0, ta, ra, ta * 3.0, ra * 2.0, 0.0, dim)
                torch.cuda.synchronize()
                assert torch.count_nonzero(out).item() == 0, (L, cplx, dim)


def test_error_codes(cuda_dev):
    from ustb_gb300 import _lib, kernels

    ch = torch.zeros((1, 1, 2, 8), dtype=torch.float32, device=cuda_dev)
    t = torch.zeros((1, 4), dtype=torch.float32, device=cuda_dev)
    t2 = torch.zeros((2, 4), dtype=torch.float32, device=cuda_dev)
    with pytest.raises(_lib.UstbError) as e:
        kernels.das_table_f32(ch, 1.0, 0.0, t, t2, t, t2, 5e6, 3)
    assert e.value.code == 3
    with pytest.raises(ValueError):
        kernels.das_table_f32(ch, 1.0, 0.0, t, t, t, t, 0.0, 3)
