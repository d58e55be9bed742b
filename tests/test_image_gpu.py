"""Headless scan conversion on the GPU against the FP64 oracle of scan_convert.m."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from ustb_gb300 import fast, image, synth
from ustb_gb300.das import DAS, channel_tensor
from ustb_gb300.enums import Precision
from ustb_gb300.geometry import Apodization

pytestmark = pytest.mark.gpu


def compare(got, want, tol):
    g, w = got.cpu().numpy(), want
    fin = np.isfinite(w) & np.isfinite(g)
    # pixels on the sector's edge may fall either side in single vs double precision
    assert np.mean(np.isfinite(w) != np.isfinite(g)) < 2e-3
    assert np.max(np.abs(g[fin] - w[fin])) <= tol


@pytest.mark.parametrize("compression, tol", [("log", 1e-3), ("sqrt", 1e-4), ("abs", 1e-4)])
def test_random_sector_image(cuda_dev, compression, tol):
    """Uncorrelated pixels: single-precision pixel positions move the bilinear weights by
    ~1e-7, which moves the interpolated values by up to ~1e-5 of the maximum."""
    rng = np.random.default_rng(3)
    s = synth.config_dw_sector(device="cpu", scale=0.25).scan
    nd, na = s.depth_axis.size, s.azimuth_axis.size
    data = (rng.standard_normal((nd * na, 2)) + 1j * rng.standard_normal((nd * na, 2))).astype(np.complex64)
    got, xs, zs = image.scan_convert(torch.from_numpy(data).to(cuda_dev), s, 200, 150, compression)
    want = O.scan_convert_f64(data.reshape(na, nd, 2).transpose(1, 0, 2), s.depth_axis, s.azimuth_axis, xs, zs,
                              compression)
    got = got.float()
    scale = 1.0 if compression == "log" else float(np.abs(want[np.isfinite(want)]).max())
    compare(got / scale, want / scale, tol)


def test_sector_beamformed_image_to_cartesian(cuda_dev):
    wl = synth.config_dw_sector(device=cuda_dev, scale=0.5)
    das = DAS()
    das.channel_data, das.scan, das.dimension = wl.channel_data, wl.scan, wl.dimension
    das.receive_apodization = Apodization(window=wl.rx_window, f_number=wl.rx_f_number)
    geom = das.fast_geometry(cuda_dev)
    ch = channel_tensor(wl.channel_data.data, cuda_dev)
    st = fast.convert_channels(ch, Precision.fp16)
    o = fast.das_fast(st, Precision.fp16, True, geom, int(wl.dimension), L=ch.shape[-1], epilogue=True, cube=False)
    img = o["das"][0]  # channel sum, [P]
    got, xs, zs = image.scan_convert(img, wl.scan)
    s = wl.scan
    want = O.scan_convert_f64(img.cpu().numpy().reshape(s.azimuth_axis.size, s.depth_axis.size).T,
                              s.depth_axis, s.azimuth_axis, xs, zs)
    assert tuple(got.shape) == (1, 512, 512)
    compare(got, want, 1e-2)  # dB; the deepest pixels sit 80 dB down, where 1e-7 relative is ~1e-3 dB
