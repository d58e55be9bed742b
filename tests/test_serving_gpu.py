"""Batched persistent launches and the continuous-batching server on the GPU.

Each request's result must be the same alone and in the mix: beamformed by its
own ustb_das_fast launch, and as one request among several of different shapes
in a persistent ustb_das_fast_batch launch driven by the server.
"""
import numpy as np
import pytest
import torch

from ustb_gb300 import fast, serving, synth
from ustb_gb300.das import DAS, channel_tensor
from ustb_gb300.enums import Precision
from ustb_gb300.geometry import Apodization

pytestmark = pytest.mark.gpu

TOL = 1e-6  # same kernel code per tile: only launch order may differ


def rel(a, b):
    return float((a - b).abs().norm() / b.abs().norm())


@pytest.fixture(scope="module")
def workloads(cuda_dev):
    out = {}
    for name, fn in (("iq", synth.config_iq_cpwc), ("sector", synth.config_dw_sector),
                     ("rf", synth.config_rf_plane_wave), ("sta", synth.config_sta),
                     ("m3d", synth.config_matrix_3d)):
        wl = fn(device=cuda_dev, scale=0.15)
        das = DAS()
        das.channel_data, das.scan, das.dimension = wl.channel_data, wl.scan, wl.dimension
        das.receive_apodization = Apodization(window=wl.rx_window, f_number=wl.rx_f_number)
        das.transmit_apodization = Apodization(window=wl.tx_window, f_number=wl.tx_f_number)
        geom = das.fast_geometry(cuda_dev)
        ch = channel_tensor(wl.channel_data.data, cuda_dev)
        prec = Precision.fp16
        out[name] = (wl, geom, fast.convert_channels(ch, prec), prec, ch.is_complex(), ch.shape[-1])
    return out


def alone(wl, geom, st, prec, cplx, L):
    epi = wl.epilogue is not None
    o = fast.das_fast(st, prec, cplx, geom, wl.dimension, L=L, epilogue=epi, cube=True)
    torch.cuda.synchronize()
    return o


def test_persistent_batch_matches_single_launches(workloads):
    reqs, refs = [], []
    for name, (wl, geom, st, prec, cplx, L) in workloads.items():
        epi = wl.epilogue is not None
        refs.append(alone(wl, geom, st, prec, cplx, L))
        reqs.append(fast.Request(st, prec, cplx, geom, wl.dimension, L=L, epilogue=epi, cube=True))
    scratch = fast.das_fast_batch(reqs)
    torch.cuda.synchronize()
    assert int(scratch[0].item()) == 0
    for r, ref in zip(reqs, refs):
        for k, v in r.outputs.items():
            assert rel(v, ref[k]) <= TOL, k


def test_server_results_same_alone_and_in_mix(workloads, cuda_dev):
    refs = {name: alone(*w) for name, w in workloads.items()}
    srv = serving.Server(cuda_dev, hbm_budget_bytes=150e9, max_batch=8)
    for name, (wl, geom, *_rest) in workloads.items():
        srv.add_plan(name, geom)
    names = list(workloads)
    order = [names[i % len(names)] for i in range(12)]
    # a burst: everything arrives while the first launch is still on the GPU
    arrivals = serving.poisson_arrivals(len(order), 1e7, seed=3)

    def make(i):
        wl, geom, st, prec, cplx, L = workloads[order[i]]
        return serving.Job(order[i], st, prec, cplx, 1, L, int(wl.dimension), epilogue=wl.epilogue is not None)

    jobs = srv.run(list(arrivals), make)
    assert len(srv.completed) == len(order)
    assert srv.launches < len(order)  # requests were merged into shared launches
    for j in jobs:
        ref = refs[j.key]
        for k, v in j.outputs.items():
            assert rel(v, ref[k]) <= TOL, (j.key, k)
    st = serving.latency_stats(jobs)
    assert st["p99_ms"] >= st["p50_ms"] > 0
