"""Frame pipeline: host frames through two streams give the single-call results."""
import numpy as np
import pytest
import torch

from ustb_gb300 import fast, synth
from ustb_gb300.das import DAS, channel_tensor
from ustb_gb300.enums import Precision
from ustb_gb300.geometry import Apodization

pytestmark = pytest.mark.gpu


def test_pipeline_matches_single_calls(cuda_dev):
    wl = synth.config_iq_cpwc(device=cuda_dev, scale=0.25)
    das = DAS()
    das.channel_data, das.scan, das.dimension = wl.channel_data, wl.scan, wl.dimension
    das.receive_apodization = Apodization(window=wl.rx_window, f_number=wl.rx_f_number)
    geom = das.fast_geometry(cuda_dev)
    ch = channel_tensor(wl.channel_data.data, cuda_dev)
    frames = [ch * (1.0 + 0.5 * k) + 0.1j * k for k in range(5)]  # distinct frames
    hosts = [f.cpu().pin_memory() for f in frames]
    L = ch.shape[-1]
    refs = [fast.das_fast(f, Precision.fp32, True, geom, 3, L=L)["cube"].cpu() for f in frames]
    outs = [torch.empty(refs[0].shape, dtype=torch.complex64).pin_memory() for _ in frames]
    pipe = fast.FramePipeline(geom, ch.shape, ch.dtype, Precision.fp32, True, 3, L=L, depth=2)
    pipe.start()
    for h, o in zip(hosts, outs):
        pipe.submit(h, o)
    pipe.synchronize()
    torch.cuda.synchronize()
    assert not pipe.overflowed()
    for o, r in zip(outs, refs):
        assert torch.equal(o, r)


def test_prebuilt_entries_give_the_single_call_result(cuda_dev):
    wl = synth.config_dw_sector(device=cuda_dev, scale=0.25)
    das = DAS()
    das.channel_data, das.scan, das.dimension = wl.channel_data, wl.scan, wl.dimension
    das.receive_apodization = Apodization(window=wl.rx_window, f_number=wl.rx_f_number)
    geom = das.fast_geometry(cuda_dev)
    ch = channel_tensor(wl.channel_data.data, cuda_dev)
    st = fast.convert_channels(ch, Precision.fp16)
    L, N, W = ch.shape[-1], geom.N, geom.W
    ref = fast.das_fast(st, Precision.fp16, True, geom, int(wl.dimension), L=L, epilogue=True)
    ent = fast.build_entries(st, Precision.fp16, True, N, W, L=L)
    for _ in range(2):  # the entries serve any number of calls
        got = fast.das_fast(st, Precision.fp16, True, geom, int(wl.dimension), L=L, epilogue=True, entries=ent)
        for k in ("cube", "das", "cf", "sdmas"):
            assert torch.equal(got[k], ref[k]), k


@pytest.mark.parametrize("cplx", [True, False])
def test_two_ctas_per_tile_match_one(cuda_dev, cplx):
    """dimension.both with 1 to 4 CTAs per tile: the same sums, added in parts."""
    wl = synth.config_iq_cpwc(device=cuda_dev, scale=0.25) if cplx else synth.config_rf_plane_wave(device=cuda_dev,
                                                                                                   scale=0.5)
    das = DAS()
    das.channel_data, das.scan, das.dimension = wl.channel_data, wl.scan, wl.dimension
    das.receive_apodization = Apodization(window=wl.rx_window, f_number=wl.rx_f_number)
    ch = channel_tensor(wl.channel_data.data, cuda_dev)
    st = fast.convert_channels(ch, Precision.fp32)
    L = ch.shape[-1]
    outs = {}
    for c in (1, 2, 3, 4):
        g = das.fast_geometry(cuda_dev, ctas_per_tile=c)
        outs[c] = fast.das_fast(st, Precision.fp32, cplx, g, 3, L=L)["cube"]
    torch.cuda.synchronize()
    for c in (2, 3, 4):
        rel = float((outs[1] - outs[c]).abs().norm() / outs[1].abs().norm())
        assert rel <= 1e-6, c
    again = fast.das_fast(st, Precision.fp32, cplx, das.fast_geometry(cuda_dev, ctas_per_tile=2), 3, L=L)["cube"]
    assert torch.equal(again, outs[2])  # two partial sums: fl(a + b) in either order
