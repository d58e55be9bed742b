"""The allocation-free host entry point against the regular one.

ustb_das_table_f32_host_noalloc serves callers that cannot allocate device
memory while they run.  Examples are acquisition loops with a hard latency
budget, where cudaMalloc may block or synchronise the device, and processes
whose GPU memory belongs to another allocator.  It stages through a fixed static
device array instead of calling cudaMalloc.  Its output must be bit-for-bit that
of ustb_das_table_f32_host, call after call, because every call reuses the same
array.  It must also match the reference das_c's own golden output, take no
device memory, and leave the caller's current device as it was.
This file is collected last on purpose.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the table kernel's parity bar against das_c


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


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("dim", [0, 1, 2, 3])
def test_noalloc_matches_regular_entry_two_calls_in_a_row(golden_dir, cuda_dev, dim):
    a = _case(golden_dir, "iq_small")
    b = _case(golden_dir, "iq_long_delay")
    ref_a = _run("ustb_das_table_f32_host", a, dim)
    ref_b = _run("ustb_das_table_f32_host", b, dim)
    first = _run("ustb_das_table_f32_host_noalloc", a, dim)
    second = _run("ustb_das_table_f32_host_noalloc", a, dim)
    # the same kernel on the same inputs: bit-for-bit the regular entry's result
    assert np.array_equal(_bits(first), _bits(ref_a))
    assert np.array_equal(_bits(second), _bits(ref_a))
    # and within the parity bar of the reference das_c's own output
    assert _rel(first, a[f"out_dim{dim}"]) <= TOL
    # a different request in between leaves nothing behind in the shared array
    other = _run("ustb_das_table_f32_host_noalloc", b, dim)
    again = _run("ustb_das_table_f32_host_noalloc", a, dim)
    assert np.array_equal(_bits(other), _bits(ref_b))
    assert _rel(other, b[f"out_dim{dim}"]) <= TOL
    assert np.array_equal(_bits(again), _bits(ref_a))


def test_noalloc_takes_no_device_memory_and_keeps_the_current_device(golden_dir, cuda_dev):
    import torch

    a = _case(golden_dir, "iq_small")
    b = _case(golden_dir, "iq_long_delay")
    for dim in range(4):  # warm-up: every kernel variant used below is loaded
        _run("ustb_das_table_f32_host_noalloc", a, dim)
        _run("ustb_das_table_f32_host_noalloc", b, dim)
    torch.cuda.synchronize()
    before = torch.cuda.mem_get_info(cuda_dev)[0]
    cur = torch.cuda.current_device()
    for _ in range(5):
        for dim in range(4):
            _run("ustb_das_table_f32_host_noalloc", a, dim)
            _run("ustb_das_table_f32_host_noalloc", b, dim)
        assert torch.cuda.current_device() == cur
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(cuda_dev)[0] == before


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
    # sizes whose byte counts wrap 64 bits are rejected too, not under-counted
    big = 1 << 31
    rc = h.ustb_das_table_f32_host_noalloc(tiny.ctypes.data, 1, big - 1, big, 1 << 20, 1, 20e6, 0.0,
                                           tiny.ctypes.data, tiny.ctypes.data, tiny.ctypes.data,
                                           tiny.ctypes.data, 4, 0.0, 3, out.ctypes.data, 0)
    assert rc == 2
    assert b"overflow" in h.ustb_last_error()
