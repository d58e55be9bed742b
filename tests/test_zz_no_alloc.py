"""The allocation-free host entry point against the regular one.

ustb_das_table_f32_host_noalloc serves callers that cannot allocate device
memory while they run (latency-bound acquisition loops, processes whose GPU
memory is owned by another allocator): it stages through a fixed static device
array instead of cudaMalloc.  Its output must equal that of
ustb_das_table_f32_host, call after call, since every call reuses the same array.
This file is collected last on purpose.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the table kernel's parity bar


def _case(golden_dir, name):
    z = np.load(os.path.join(golden_dir, "das_c_cases.npz"))
    return {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}


def _run(entry, c, dim):
    from ustb_gb300 import _lib

    f = lambda a: np.asfortranarray(a)
    ch, atx, arx, dtx, drx = f(c["ch"]), f(c["atx"]), f(c["arx"]), f(c["dtx"]), f(c["drx"])
    L, N, W, F = ch.shape
    P = atx.shape[0]
    nk = N if dim in (0, 2) else 1
    wk = W if dim in (0, 1) else 1
    out = np.full((P, nk, wk, F), np.nan + 1j * np.nan, np.complex64, order="F")
    _lib.call(entry, ch.ctypes.data, 1, L, N, W, F, float(c["fs"]), float(c["t0"]), atx.ctypes.data,
              arx.ctypes.data, dtx.ctypes.data, drx.ctypes.data, P, float(c["fd"]), dim,
              out.ctypes.data, 0)
    return out


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("dim", [0, 1, 2, 3])
def test_noalloc_matches_regular_entry_two_calls_in_a_row(golden_dir, cuda_dev, dim):
    a = _case(golden_dir, "iq_small")
    b = _case(golden_dir, "iq_long_delay")
    ref_a = _run("ustb_das_table_f32_host", a, dim)
    ref_b = _run("ustb_das_table_f32_host", b, dim)
    first = _run("ustb_das_table_f32_host_noalloc", a, dim)
    second = _run("ustb_das_table_f32_host_noalloc", a, dim)
    assert _rel(first, ref_a) <= TOL
    assert _rel(second, ref_a) <= TOL
    # a different request in between leaves nothing behind in the shared array
    other = _run("ustb_das_table_f32_host_noalloc", b, dim)
    again = _run("ustb_das_table_f32_host_noalloc", a, dim)
    assert _rel(other, ref_b) <= TOL
    assert _rel(again, ref_a) <= TOL


def test_noalloc_rejects_requests_beyond_its_scratch(cuda_dev):
    from ustb_gb300 import _lib

    h = _lib.lib()
    tiny = np.zeros(16, np.float32)
    out = np.zeros(16, np.complex64)
    # 2048 x 128 x 128 complex samples alone need 256 MiB: rejected before any copy
    rc = h.ustb_das_table_f32_host_noalloc(tiny.ctypes.data, 1, 2048, 128, 128, 1, 20e6, 0.0,
                                           tiny.ctypes.data, tiny.ctypes.data, tiny.ctypes.data,
                                           tiny.ctypes.data, 4, 0.0, 3, out.ctypes.data, 0)
    assert rc == 2
    assert b"scratch" in h.ustb_last_error()
