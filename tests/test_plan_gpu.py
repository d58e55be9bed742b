"""Resident plans (ustb_plan_*) and the native continuous-batching server
(ustb_serve_*) on the GPU.

A plan's results must be those of ustb_das_fast on the same geometry, whether the
library plans the tiles itself or is given the Python planner's tile map, and a
request served in a batch by the library's scheduler thread must give what it gives
alone.
"""
import threading

import numpy as np
import pytest
import torch

from ustb_gb300 import fast, synth
from ustb_gb300._lib import UstbError
from ustb_gb300.das import DAS, channel_tensor
from ustb_gb300.enums import Precision
from ustb_gb300.geometry import Apodization
from ustb_gb300.plan import Plan, Server

pytestmark = [pytest.mark.gpu, pytest.mark.timeout(300)]  # a stuck server thread fails the test

TOL = 1e-6  # same kernel; tiles may differ, which only moves the two-CTA split point


def rel(a, b):
    return float((a - b).abs().norm() / b.abs().norm())


@pytest.fixture(scope="module")
def workloads(cuda_dev):
    out = {}
    for name, fn in (("iq", synth.config_iq_cpwc), ("sector", synth.config_dw_sector),
                     ("rf", synth.config_rf_plane_wave), ("sta", synth.config_sta)):
        wl = fn(device=cuda_dev, scale=0.15)
        das = DAS()
        das.channel_data, das.scan, das.dimension = wl.channel_data, wl.scan, wl.dimension
        das.receive_apodization = Apodization(window=wl.rx_window, f_number=wl.rx_f_number)
        das.transmit_apodization = Apodization(window=wl.tx_window, f_number=wl.tx_f_number)
        geom = das.fast_geometry(cuda_dev)
        ch = channel_tensor(wl.channel_data.data, cuda_dev)
        prec = Precision.fp16
        st = fast.convert_channels(ch, prec)
        epi = wl.epilogue is not None
        ref = fast.das_fast(st, prec, ch.is_complex(), geom, wl.dimension, L=ch.shape[-1], epilogue=epi, cube=True)
        out[name] = dict(wl=wl, geom=geom, st=st, prec=prec, cplx=ch.is_complex(), L=ch.shape[-1], epi=epi, ref=ref)
    torch.cuda.synchronize()
    return out


def make_plan(w, library_tiles=True):
    return Plan(w["geom"], w["L"], w["prec"], w["cplx"], w["wl"].dimension, epilogue=w["epi"],
                library_tiles=library_tiles)


def check(outs, ref):
    for k in ("cube", "das", "cf", "cf_image", "sdmas"):
        if k in ref and k in outs:
            assert rel(outs[k], ref[k]) <= TOL, k


@pytest.mark.parametrize("name", ["iq", "sector", "rf", "sta"])
@pytest.mark.parametrize("library_tiles", [True, False])
def test_plan_execute_matches_das_fast(workloads, name, library_tiles):
    w = workloads[name]
    p = make_plan(w, library_tiles)
    if not library_tiles:
        assert p.n_tiles == len(w["geom"].tiles)
    else:  # the library's planner follows the same rules as the Python one
        assert 0.5 * len(w["geom"].tiles) <= p.n_tiles <= 2 * len(w["geom"].tiles)
    outs = p.execute(w["st"])
    torch.cuda.synchronize()
    assert int(outs["flags"].item()) == 0
    check(outs, w["ref"])
    p.close()


@pytest.mark.parametrize("budget", [8 << 30, 1])  # one batch of everything / a batch per request
def test_server_batches_match_single_launches(workloads, budget):
    plans = {k: make_plan(w) for k, w in workloads.items()}
    srv = Server(workspace_budget=budget, max_batch=16)
    tickets = []
    for rep in range(3):
        for k, w in workloads.items():
            tickets.append((k, srv.submit(plans[k], w["st"])))
    for k, t in tickets:
        outs = srv.wait(t)
        assert outs["flags"] == 0
        check(outs, workloads[k]["ref"])
    srv.close()


@pytest.mark.parametrize("reserve_sms", [0, 24])
def test_server_large_stream_matches_single_launches(workloads, reserve_sms):
    """Requests above large_units launch alone on the large stream (capped at
    SMs - reserve_sms CTAs) while the others batch on the small streams; each result
    is what the request gives alone."""
    plans = {k: make_plan(w) for k, w in workloads.items()}
    units = {k: w["geom"].P * w["geom"].N * w["geom"].W for k, w in workloads.items()}
    cut = sorted(units.values())[1]  # two kinds large, two small
    srv = Server(max_batch=16, large_units=cut, reserve_sms=reserve_sms)
    tickets = []
    for rep in range(4):
        for k, w in workloads.items():
            tickets.append((k, srv.submit(plans[k], w["st"])))
    for k, t in tickets:
        outs = srv.wait(t)
        assert outs["flags"] == 0
        check(outs, workloads[k]["ref"])
    srv.close()


def test_server_reserve_must_leave_sms(cuda_dev):
    sms = torch.cuda.get_device_properties(cuda_dev).multi_processor_count
    with pytest.raises(UstbError) as e:
        Server(reserve_sms=sms)
    assert e.value.code == 1


def test_server_from_several_threads(workloads):
    plans = {k: make_plan(w) for k, w in workloads.items()}
    srv = Server(max_batch=8)
    errors = []

    def client(k, n):
        try:
            w = workloads[k]
            ts = [srv.submit(plans[k], w["st"]) for _ in range(n)]
            for t in ts:
                check(srv.wait(t), w["ref"])
        except Exception as e:  # collected and raised in the main thread
            errors.append(e)

    threads = [threading.Thread(target=client, args=(k, 4)) for k in workloads]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    srv.close()
    assert not errors, errors


def test_server_ticket_rules(workloads):
    w = workloads["iq"]
    p = make_plan(w)
    srv = Server()
    t = srv.submit(p, w["st"])
    try:
        srv.wait(t, timeout_ms=0)  # may or may not be done yet
    except UstbError as e:
        assert e.code == 6  # USTB_E_TIMEOUT: the ticket stays valid
        srv.wait(t)
    with pytest.raises(UstbError) as e:  # released by the wait above
        srv.wait(t)
    assert e.value.code == 1
    srv.close()


def test_destroy_finishes_queued_requests(workloads):
    """Requests still queued when the server is destroyed are beamformed first."""
    w = workloads["sta"]
    p = make_plan(w)
    srv = Server(workspace_budget=1, max_batch=1)
    outs = []
    for _ in range(6):
        o, c = p.outputs()
        o["cube"].zero_()
        outs.append((o, c))
    torch.cuda.synchronize()
    import ctypes
    from ustb_gb300 import _lib

    for o, c in outs:
        t = ctypes.c_uint64()
        _lib.call("ustb_serve_submit", srv.handle, p.handle, w["st"].data_ptr(), ctypes.byref(c), ctypes.byref(t))
    srv.close()
    torch.cuda.synchronize()
    for o, _ in outs:
        assert rel(o["cube"], w["ref"]["cube"]) <= TOL


# ---- plans on geometry the library tiles by other rules --------------------------

def _case(cuda_dev, seq, scan, rx, seed):
    from ustb_gb300.uff import Probe

    rng = np.random.default_rng(seed)
    N, L = 16, 640
    probe = Probe.linear_array(N, 0.3e-3)
    fs, f0, c = 20e6, 5e6, 1540.0
    x = (rng.standard_normal((L, N, len(seq))) + 1j * rng.standard_normal((L, N, len(seq)))).astype(np.complex64)
    k = np.array([1, 4, 6, 4, 1], np.float32) / 16
    x = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), 0, x).astype(np.complex64)
    ph = np.exp(-1j * 4 * np.pi * f0 * scan.reference_distance / c)
    g = fast.FastGeometry(probe, scan, seq, fs, 0.0, f0, c, cuda_dev, rx, None, pixel_phase=ph)
    t = torch.from_numpy(np.ascontiguousarray(x[..., None].transpose(3, 2, 1, 0))).to(cuda_dev)
    st = fast.convert_channels(t, Precision.fp32)
    ref = fast.das_fast(st, Precision.fp32, True, g, 3, L=L)["cube"]
    p = Plan(g, L, Precision.fp32, True, 3)
    got = p.execute(st)
    torch.cuda.synchronize()
    return g, p, got, ref


def test_plan_with_table_waves_and_receive_table(cuda_dev):
    """Focused waves whose focal band crosses the scan take their delays from the
    table (the library re-splits tiles by the tabulated span), and a receive window
    without a closed form (sta) comes from the receive table."""
    from ustb_gb300.enums import Window
    from ustb_gb300.uff import LinearScan, Point, Wave

    scan = LinearScan(np.linspace(-3e-3, 3e-3, 24), np.linspace(5e-3, 14e-3, 40))
    seq = [Wave(source=Point.from_xyz(x, 0, 9e-3)) for x in (-1e-3, 0.0, 1e-3)]
    rx = Apodization(window=Window.sta, origin=Point.from_xyz(0.0, 0, 0))
    g, p, got, ref = _case(cuda_dev, seq, scan, rx, 21)
    assert g.d_txdelay is not None and g.d_rxapo is not None
    assert int(got["flags"].item()) == 0
    assert rel(got["cube"], ref) <= TOL
    p.close()


def test_plan_on_a_pixel_list(cuda_dev):
    """Pixels given as a list (no grid): the library orders them on a coarse spatial
    grid and cuts runs of 512."""
    from ustb_gb300.enums import Window
    from ustb_gb300.uff import Scan, Wave

    rng = np.random.default_rng(22)
    P = 3000
    scan = Scan(rng.uniform(-3e-3, 3e-3, P), np.zeros(P), rng.uniform(5e-3, 14e-3, P))
    seq = [Wave.plane(a) for a in np.deg2rad([-8.0, 0.0, 8.0])]
    g, p, got, ref = _case(cuda_dev, seq, scan, Apodization(window=Window.tukey25, f_number=1.5), 22)
    assert int(got["flags"].item()) == 0
    assert p.n_tiles >= 6  # 3000 pixels in tiles of at most 512
    assert rel(got["cube"], ref) <= TOL
    p.close()
