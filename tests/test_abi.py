"""The C-ABI library builds, loads and exports every symbol include/*.h declares.

No compute calls here: this runs on machines without a GPU.
"""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def _declared():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^[A-Za-z_][\w\s\*]*?\b(ustb_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib_path():
    from ustb_gb300 import build

    return build.build()


def test_header_declares_entry_points():
    names = _declared()
    assert "ustb_das_table_f32" in names and "ustb_last_error" in names


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_every_symbol(lib_path):
    from ustb_gb300 import _lib

    assert set(_declared()) == set(_lib.SIGNATURES)


def test_abi_version_and_error_string(lib_path):
    from ustb_gb300 import _lib

    h = _lib.lib()
    assert h.ustb_abi_version() >= 10000
    # every entry point clears the thread's message first: an empty call succeeds
    # (no work, no CUDA call) and leaves no message behind
    assert h.ustb_demodulate(None, 0, None, 0, 16, 0, 1.0, 0.0, 0.0, 1, None, 1, 1.0, None) == 0
    assert h.ustb_last_error() == b""


def test_argument_errors_without_gpu(lib_path):
    """Argument checks run before any CUDA call, so they work without a GPU."""
    from ustb_gb300 import _lib

    h = _lib.lib()
    rc = h.ustb_das_table_f32(None, 1, 4, 2, 1, 1, 1.0, 0.0, None, None, None, None, 3, 0.0, 7,
                              None, None)
    assert rc == 1 and b"sum mode" in h.ustb_last_error()
    rc = h.ustb_das_table_f32(None, 0, 4, 2, 1, 1, 1.0, 0.0, None, None, None, None, 3, 5e6, 3,
                              None, None)
    assert rc == 3 and b"real" in h.ustb_last_error()


def test_plan_and_server_argument_errors_without_gpu(lib_path):
    """NULL handles and descriptors are rejected before any CUDA call."""
    import ctypes

    from ustb_gb300 import _lib

    h = _lib.lib()
    assert h.ustb_plan_create(None, None) == 1
    assert h.ustb_plan_destroy(None) == 1
    assert h.ustb_plan_tiles(None) == -1
    assert h.ustb_plan_execute(None, None, None, None, None) == 1
    assert h.ustb_serve_create(0, 1, 0, None) == 1
    out = ctypes.c_void_p()
    assert h.ustb_serve_create(0, 1, 0, ctypes.byref(out)) == 1 and b"budget" in h.ustb_last_error()
    assert h.ustb_serve_create(1 << 20, 41, 0, ctypes.byref(out)) == 1 and b"max_batch" in h.ustb_last_error()
    assert h.ustb_serve_create_ex(1 << 20, 1, 0, -1, ctypes.byref(out)) == 1 and b"reserve_sms" in h.ustb_last_error()
    assert h.ustb_serve_submit(None, None, None, None, None) == 1
    assert h.ustb_serve_wait(None, 1, 0, None) == 1
    assert h.ustb_serve_destroy(None) == 1


def test_plan_descriptor_checks_without_gpu(lib_path):
    import ctypes

    import numpy as np

    from ustb_gb300 import _lib
    from ustb_gb300.fast import CWave
    from ustb_gb300.plan import CPlanDesc

    h = _lib.lib()
    el = np.zeros((4, 3), np.float32)
    px = np.zeros((6, 3), np.float32)
    waves = (CWave * 1)()
    d = CPlanDesc()
    d.geometry.n_elements, d.geometry.element_xyz = 4, el.ctypes.data
    d.geometry.n_pixels, d.geometry.pixel_xyz = 6, px.ctypes.data
    d.geometry.n_waves, d.geometry.waves = 1, ctypes.addressof(waves)
    d.geometry.fs, d.geometry.sound_speed = 20e6, 1540.0
    d.L, d.F, d.dimension, d.is_complex = 64, 1, 3, 1
    out = ctypes.c_void_p()
    d.pixel_grid[0], d.pixel_grid[1], d.pixel_grid[2] = 2, 2, 2  # 8 != 6 pixels
    assert h.ustb_plan_create(ctypes.byref(d), ctypes.byref(out)) == 2 and b"pixel_grid" in h.ustb_last_error()
    d.pixel_grid[0], d.pixel_grid[1], d.pixel_grid[2] = 3, 2, 1
    d.L = 1
    assert h.ustb_plan_create(ctypes.byref(d), ctypes.byref(out)) == 2
    d.L, d.is_complex, d.geometry.fd = 64, 0, 5e6  # real data with a modulation frequency
    assert h.ustb_plan_create(ctypes.byref(d), ctypes.byref(out)) == 3
    d.geometry.fd, d.epilogue, d.dimension = 0.0, 1, 3  # epilogue needs complex transmit mode
    assert h.ustb_plan_create(ctypes.byref(d), ctypes.byref(out)) == 1
    d.epilogue = 0
    waves[0].kind = 3  # table wave without a table
    assert h.ustb_plan_create(ctypes.byref(d), ctypes.byref(out)) == 1 and b"tx_delay_table" in h.ustb_last_error()


def test_kernel_entry_argument_errors_without_gpu(lib_path):
    """Argument checks of the kernels around the beamformer, before any CUDA call."""
    from ustb_gb300 import _lib

    h = _lib.lib()
    # coherence factor: only receive / transmit / both; empty input is a no-op
    assert h.ustb_coherence_factor(None, 4, 2, 2, 1, 0, None, None, None, None) == 1
    assert b"dimension" in h.ustb_last_error()
    assert h.ustb_coherence_factor(None, 0, 2, 2, 1, 3, None, None, None, None) == 0
    assert h.ustb_coherence_factor(None, 4, 2, 2, 1, 3, None, None, None, None) == 1  # NULL cube
    # zero-phase demodulation: the trace must outlast filtfilt's padding of 3 * ntaps
    assert h.ustb_demodulate_filtfilt(None, 0, None, 0, 150, 1, 20e6, 0.0, 4e6, 1, None, 65, 1.0, None) == 2
    assert b"padding" in h.ustb_last_error()
    assert h.ustb_demodulate_filtfilt(None, 0, None, 0, 300, 0, 20e6, 0.0, 4e6, 1, None, 65, 1.0, None) == 0
    assert h.ustb_demodulate_filtfilt(None, 0, None, 0, 300, 1, 20e6, 0.0, 4e6, 0, None, 65, 1.0, None) == 1
    # depth FIR
    assert h.ustb_fir_depth(None, None, 16, 2, None, 0, 0, None) == 1
    assert h.ustb_fir_depth(None, None, 16, 2, None, 5, -1, None) == 1
