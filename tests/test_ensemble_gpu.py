"""High-frame-rate ensembles: graph replay, tuning, and agreement with single launches.

An int16 I/Q ensemble goes through ``Ensemble`` (conversion + one persistent
launch, replayed from a CUDA graph) and must give what ``das_fast`` gives on the
same converted data; each new ensemble copied into the resident buffer must give
its own result; and FP16 storage stays within 1e-3 relative L2 of the FP64 oracle.
"""
import math

import numpy as np
import pytest
import torch

from oracle import oracle as O
from ustb_gb300 import autotune, fast, geometry, synth
from ustb_gb300.das import DAS
from ustb_gb300.ensemble import Ensemble
from ustb_gb300.enums import Precision
from ustb_gb300.geometry import Apodization

pytestmark = pytest.mark.gpu

TOL = 1e-6


def rel(a, b):
    return float((a - b).abs().norm() / b.abs().norm())


@pytest.fixture(scope="module")
def hfr(cuda_dev):
    wl = synth.config_hfr_ensemble(device=cuda_dev, frames=4, scale=0.25)
    das = DAS()
    das.channel_data, das.scan, das.dimension = wl.channel_data, wl.scan, wl.dimension
    das.receive_apodization = Apodization(window=wl.rx_window, f_number=wl.rx_f_number)
    return wl, das


def single(wl, geom, i16):
    st = fast.convert_channels(i16, Precision.fp16, wl.info["scale"])
    F, W, N, L, _ = i16.shape
    o = fast.das_fast(st, Precision.fp16, True, geom, int(wl.dimension), F=F, L=L)
    torch.cuda.synchronize()
    return o["cube"]


@pytest.mark.parametrize("graph", [True, False])
def test_ensemble_matches_single_launch_and_takes_new_data(hfr, cuda_dev, graph):
    wl, das = hfr
    geom = das.fast_geometry(cuda_dev)
    x = wl.info["int16"]
    F, W, N, L, _ = x.shape
    ens = Ensemble(geom, F, L, wl.dimension, Precision.fp16, wl.info["scale"], graph=graph)
    out = ens.run(x)["cube"].clone()  # the output buffer is reused by the next run
    torch.cuda.synchronize()
    assert ens.flags() == 0
    assert rel(out, single(wl, geom, x)) <= TOL
    y = torch.flip(x, dims=[0]).contiguous()  # a different ensemble, same shape
    out2 = ens.run(y)["cube"].clone()
    torch.cuda.synchronize()
    assert rel(out2, single(wl, geom, y)) <= TOL
    assert rel(out2[0], out[-1]) <= TOL


def test_ensemble_frame_vs_fp64_oracle(hfr, cuda_dev):
    wl, das = hfr
    geom = das.fast_geometry(cuda_dev)
    x = wl.info["int16"]
    F, W, N, L, _ = x.shape
    ens = Ensemble(geom, F, L, wl.dimension, Precision.fp16, wl.info["scale"])
    got = ens.run(x)["cube"][1, 0, 0].cpu().numpy()
    cd, scan = wl.channel_data, wl.scan
    ch = (x[1].double()[..., 0] + 1j * x[1].double()[..., 1]).cpu().numpy() * wl.info["scale"]  # (W, N, L)
    chm = np.ascontiguousarray(ch.transpose(2, 1, 0))[..., None]
    txa = das.transmit_apodization.wave_apodization(cd.sequence, scan)
    rxa = das.receive_apodization.aperture_apodization(cd.probe, scan)
    txd = geometry.transmit_delay(cd.sequence, scan)
    rxd = geometry.receive_delay(cd.probe, scan, cd.sound_speed)
    ref = O.das_f64(chm, cd.sampling_frequency, cd.initial_time, txa, rxa, txd, rxd,
                    cd.modulation_frequency, int(wl.dimension))[:, 0, 0, 0]
    ref = ref * np.exp(-1j * 4 * math.pi * cd.modulation_frequency * scan.reference_distance / cd.sound_speed)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-3


def test_autotuned_plan_gives_the_same_image(hfr, cuda_dev, tmp_path, monkeypatch):
    monkeypatch.setenv("USTB_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    wl, das = hfr
    x = wl.info["int16"]
    F, W, N, L, _ = x.shape
    st = fast.convert_channels(x, Precision.fp16, wl.info["scale"])
    run = lambda g: fast.das_fast(st, Precision.fp16, True, g, int(wl.dimension), F=F, L=L)
    key = autotune.shape_key(wl.scan, N, W, L, F, Precision.fp16, wl.dimension, True, cuda_dev)
    choice = autotune.tune(lambda b, o, c, sh: das.fast_geometry(cuda_dev, b, o, c, sh), run, key, scan=wl.scan,
                           both=True, dimension=int(wl.dimension))
    assert choice.ms > 0
    again = autotune.tune(lambda *a: 1 / 0, run, key)  # served from the cache
    assert (again.block, again.order, again.ctas_per_tile) == (choice.block, choice.order, choice.ctas_per_tile)
    tuned = run(das.fast_geometry(cuda_dev, choice.block, choice.order, choice.ctas_per_tile,
                                  choice.stage_shape))["cube"]
    default = run(das.fast_geometry(cuda_dev))["cube"]
    torch.cuda.synchronize()
    assert rel(tuned, default) <= 1e-5
