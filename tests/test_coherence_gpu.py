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
