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
