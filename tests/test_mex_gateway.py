"""The MATLAB MEX gateway (ustb_gb300/mex/das_gb300.cpp) without MATLAB.

The gateway is compiled against the mex.h stand-in of the oracle and driven
through the same mxArray harness the reference das_c runs in, so the test sees
exactly the prhs layout das.m passes (+midprocess/das.m:251-259).
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

BUILD = os.path.join(ROOT, "tests", "_build")
SO = os.path.join(BUILD, "libmex_gateway.so")


@pytest.fixture(scope="module")
def gateway():
    from ustb_gb300 import build

    lib = build.build()
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-DMEX_RUN_NAME=das_gb300_mex_run",
           "-I" + os.path.join(ROOT, "oracle", "shim"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "ustb_gb300", "mex", "das_gb300.cpp"),
           os.path.join(ROOT, "oracle", "ref_driver.cpp"),
           lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", SO]
    subprocess.check_call(cmd)
    h = ctypes.CDLL(SO)
    f = h.das_gb300_mex_run
    i64, f32, vp = ctypes.c_int64, ctypes.c_float, ctypes.c_void_p
    f.argtypes = [vp, i64, i64, i64, i64, f32, f32, vp, vp, vp, vp, i64, f32, ctypes.c_int32, vp,
                  ctypes.c_char_p, ctypes.c_int]
    f.restype = ctypes.c_int
    return f


def call(gw, c, dim, P_override=None):
    F = lambda a: np.asfortranarray(a)
    ch, atx, arx, dtx, drx = F(c["ch"]), F(c["atx"]), F(c["arx"]), F(c["dtx"]), F(c["drx"])
    L, N, W, Fr = ch.shape
    P = atx.shape[0] if P_override is None else P_override
    nk = N if dim in (0, 2) else 1
    wk = W if dim in (0, 1) else 1
    out = np.zeros((atx.shape[0], nk, wk, Fr), np.complex64, order="F")
    err = ctypes.create_string_buffer(512)
    rc = gw(ch.ctypes.data, L, N, W, Fr, float(c["fs"]), float(c["t0"]), atx.ctypes.data,
            arx.ctypes.data, dtx.ctypes.data, drx.ctypes.data, P, float(c["fd"]), dim,
            out.ctypes.data, err, 512)
    return rc, err.value.decode(), out


def _case(golden_dir, name):
    z = np.load(os.path.join(golden_dir, "das_c_cases.npz"))
    return {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}


def test_gateway_rejects_bad_arguments_like_das_c(gateway, golden_dir):
    c = dict(_case(golden_dir, "iq_small"))
    rc, msg, _ = call(gateway, c, 7)
    assert rc == 1 and "sum mode" in msg


def test_gateway_maps_library_failures_to_mex_errors(gateway, golden_dir):
    import torch

    if torch.cuda.is_available():
        pytest.skip("needs a machine without a usable GPU")
    rc, msg, _ = call(gateway, _case(golden_dir, "iq_small"), 3)
    assert rc == 1 and msg.startswith("Toolbox:SRP_SRC:GPU") and "CUDA" in msg


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [0, 1, 2, 3])
def test_gateway_matches_reference_das_c(gateway, golden_dir, cuda_dev, dim):
    c = _case(golden_dir, "iq_small")
    rc, msg, out = call(gateway, c, dim)
    assert rc == 0, msg
    ref = c[f"out_dim{dim}"]
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) <= 1e-5
