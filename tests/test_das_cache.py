"""DAS.go() keeps the last geometry on the device (tables, or the fast path's
geometry) and reuses it while the acquisition's geometry is unchanged."""
import numpy as np
import pytest
import torch

import bench
from ustb_gb300 import synth
from ustb_gb300.enums import Precision
from ustb_gb300.uff import LinearScan


@pytest.fixture()
def das():
    return bench.build_das(synth.config_iq_cpwc(device="cpu", scale=0.15))


def test_geometry_key_tracks_what_the_tables_depend_on(das):
    k = das.geometry_key("fast", "cuda:0")
    assert das.geometry_key("fast", "cuda:0") == k
    assert das.geometry_key("table", "cuda:0") != k
    assert das.geometry_key("fast", "cuda:1") != k
    cd = das.channel_data
    changes = [
        lambda: setattr(das.receive_apodization, "f_number", (2.5, 2.5)),
        lambda: setattr(das.transmit_apodization, "f_number", (0.5, 0.5)),
        lambda: setattr(cd.sequence[3], "delay", 1e-7),
        lambda: setattr(cd, "initial_time", cd.initial_time + 1e-8),
        lambda: setattr(das, "lens_delay", 1e-8),
        lambda: setattr(das, "scan", LinearScan(das.scan.x_axis, das.scan.z_axis * 1.01)),
    ]
    seen = {k}
    for change in changes:
        change()
        k2 = das.geometry_key("fast", "cuda:0")
        assert k2 not in seen
        seen.add(k2)


@pytest.mark.gpu
@pytest.mark.parametrize("engine, prec", [("table", Precision.fp32), ("fast", Precision.fp16)])
def test_go_reuses_device_geometry(cuda_dev, engine, prec):
    wl = synth.config_iq_cpwc(device=cuda_dev, scale=0.15)
    d = bench.build_das(wl)
    d.engine, d.precision, d.gpu_id = engine, prec, cuda_dev.index or 0
    a = d.go().data.clone()
    geom = d._geometry[1]
    b = d.go().data
    assert d._geometry[1] is geom  # reused
    assert torch.equal(a, b)
    d.scan = LinearScan(d.scan.x_axis, d.scan.z_axis + 1e-3)
    c = d.go().data
    assert d._geometry[1] is not geom  # rebuilt for the new scan
    assert not torch.equal(a, c)


@pytest.mark.gpu
def test_fixed_geometry_skips_the_key_until_invalidated(cuda_dev, monkeypatch):
    wl = synth.config_iq_cpwc(device=cuda_dev, scale=0.15)
    d = bench.build_das(wl)
    d.engine, d.precision, d.gpu_id = "fast", Precision.fp16, cuda_dev.index or 0
    a = d.go().data.clone()
    geom = d._geometry[1]
    d.geometry_fixed = True
    calls = []
    orig = type(d).geometry_key
    monkeypatch.setattr(type(d), "geometry_key", lambda self, *a_: calls.append(1) or orig(self, *a_))
    b = d.go().data
    assert not calls and d._geometry[1] is geom and torch.equal(a, b)
    d.invalidate()
    d.go()
    assert calls and d._geometry[1] is not geom
