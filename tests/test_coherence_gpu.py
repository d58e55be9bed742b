"""Phase and generalized coherence factors on a kept channel cube vs the FP64 oracle."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from ustb_gb300 import fast, postprocess, synth
from ustb_gb300.das import DAS, channel_tensor
from ustb_gb300.enums import Precision
from ustb_gb300.geometry import Apodization

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.fixture(scope="module")
def sector_cube(cuda_dev):
    wl = synth.config_dw_sector(device=cuda_dev, scale=0.3)
    das = DAS()
    das.channel_data, das.scan, das.dimension = wl.channel_data, wl.scan, wl.dimension
    das.receive_apodization = Apodization(window=wl.rx_window, f_number=wl.rx_f_number)
    geom = das.fast_geometry(cuda_dev)
    ch = channel_tensor(wl.channel_data.data, cuda_dev)
    st = fast.convert_channels(ch, Precision.fp32)
    cube = fast.das_fast(st, Precision.fp32, True, geom, int(wl.dimension), L=ch.shape[-1])["cube"]  # (1,1,N,P)
    torch.cuda.synchronize()
    rxa = das.receive_apodization.aperture_apodization(wl.channel_data.probe, wl.scan)  # [P, N]
    return cube, rxa


def test_phase_coherence_factor(sector_cube, cuda_dev):
    cube, rxa = sector_cube
    w = torch.from_numpy(np.ascontiguousarray(rxa.T).astype(np.float32)).to(cuda_dev)
    got = postprocess.phase_coherence_factor(cube, w)
    d = cube[0, 0].cpu().numpy().T  # [P, N]
    live = rxa.sum(1) > 0  # pixels with any weight (elsewhere both sides are NaN -> 0 / undefined)
    fca, fcc, img = O.phase_coherence_factor_f64(d, rxa)
    g_fca, g_fcc, g_img = (got[k][0].cpu().numpy() for k in ("FCA", "FCC", "image"))
    assert np.max(np.abs(g_fca[live] - fca[live])) <= 1e-4
    assert np.max(np.abs(g_fcc[live] - fcc[live])) <= 1e-4
    assert rel(g_img[live], img[live]) <= 1e-4
    # unweighted (apodization none)
    got1 = postprocess.phase_coherence_factor(cube)
    fca1, fcc1, _ = O.phase_coherence_factor_f64(d)
    assert np.max(np.abs(got1["FCC"][0].cpu().numpy() - fcc1)) <= 1e-4


@pytest.mark.parametrize("M0", [4, 1, 2])
def test_generalized_coherence_factor(sector_cube, M0):
    cube, _ = sector_cube
    got = postprocess.generalized_coherence_factor(cube, M0)
    d = cube[0, 0].cpu().numpy().T
    g, img = O.generalized_coherence_factor_f64(d, M0)
    assert np.max(np.abs(got["GCF"][0].cpu().numpy() - g)) <= 1e-5
    assert rel(got["image"][0].cpu().numpy(), img) <= 1e-5


# ---- coherence factor on a kept cube (ustb_coherence_factor) -----------------------
import os as _os

from ustb_gb300.enums import Dimension as _Dim


@pytest.mark.parametrize("dim", ["receive", "transmit", "both"])
def test_coherence_factor_matches_reference_python_port(cuda_dev, dim):
    """Against the output of python/src/ustb/postprocess/coherence_factor.py itself
    (M = number summed)."""
    g = np.load(_os.path.join(_os.path.dirname(__file__), "golden", "python_cf.npz"))
    cube = g["cube"]  # [P, N, W, F]
    abi = torch.from_numpy(np.ascontiguousarray(cube.transpose(3, 2, 1, 0))).to(cuda_dev)
    out = postprocess.coherence_factor(abi, getattr(_Dim, dim))
    got = out["image"].cpu().numpy().transpose(3, 2, 1, 0)
    want = g[f"{dim}/image"]
    assert got.shape == want.shape
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-6
    assert np.all(got[5] == 0)  # the silent pixel


@pytest.mark.parametrize("dim", [_Dim.receive, _Dim.transmit, _Dim.both])
def test_coherence_factor_class_with_active_counts(cuda_dev, dim):
    """The MATLAB rule: M = units whose apodization exceeds the criterium."""
    from ustb_gb300.uff import BeamformedData

    rng = np.random.default_rng(int(dim))
    P, N, W, F = 300, 12, 7, 2
    cube = (rng.standard_normal((P, N, W, F)) + 1j * rng.standard_normal((P, N, W, F))).astype(np.complex64)
    rx = rng.uniform(0, 1, (P, N)).astype(np.float32)
    tx = rng.uniform(0, 1, (P, W)).astype(np.float32)
    cf = postprocess.CoherenceFactor()
    cf.input = BeamformedData(None, torch.from_numpy(cube))
    cf.dimension, cf.receive_apodization, cf.transmit_apodization = dim, rx, tx
    cf.device = cuda_dev
    img = cf.go().data.cpu().numpy()
    thr = 0.16
    if dim == _Dim.receive:
        s, M = cube, (rx > thr).sum(1)
    elif dim == _Dim.transmit:
        s, M = np.swapaxes(cube, 1, 2), (tx > thr).sum(1)
    else:
        s = cube.reshape((P, N * W, 1, F), order="F")
        M = ((tx[:, None, :] * rx[:, :, None]) > thr).sum((1, 2))
    _, want = O.coherence_factor(s, M)
    if dim == _Dim.transmit:
        want = np.swapaxes(want, 1, 2)
    want = want.reshape(img.shape, order="F")
    assert np.linalg.norm(img - want) / np.linalg.norm(want) <= 1e-5
