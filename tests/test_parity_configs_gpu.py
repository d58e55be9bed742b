"""Parity at the benchmark configurations' full sizes.

* The das_c-exact table kernel (``ustb_das_table_f32``) beamforms the whole
  RF plane-wave frame (2048 x 128 x 1, 256 x 256 pixels) and the whole IQ
  compounding frame (1024 x 128 x 75, 400 x 400 pixels) on das.m's
  single-precision tables.  The oracle port of das_c (+mex/source/das_c.cpp:
  355-409) beamforms a seeded subset of 2000 pixels from the same tables and
  channel data.  Bar: relative L2 <= 1e-5 on the subset, and every output the
  port leaves at zero is exactly zero.
* The fast path with FP16 storage beamforms the whole 3D matrix-array volume
  (1024 elements, 25 diverging waves, 64 x 64 x 128 voxels) and is compared with
  the FP64 oracle on a seeded subset of 1000 voxels.  Bar: relative L2 <= 1e-3.
"""
import math

import numpy as np
import pytest
import torch

from oracle import oracle as O
from ustb_gb300 import fast, geometry, kernels, synth
from ustb_gb300.das import DAS, channel_tensor, hilbert_last
from ustb_gb300.enums import Precision, Window
from ustb_gb300.geometry import Apodization
from ustb_gb300.uff import Scan

pytestmark = pytest.mark.gpu

TOL_DAS_C = 1e-5
TOL_FP16 = 1e-3


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def make_das(wl):
    das = DAS()
    das.channel_data, das.scan, das.dimension = wl.channel_data, wl.scan, wl.dimension
    das.receive_apodization = Apodization(window=wl.rx_window, f_number=wl.rx_f_number)
    das.transmit_apodization = Apodization(window=wl.tx_window, f_number=wl.tx_f_number)
    return das


def workload(name, dev):
    wl = synth.CONFIGS[name](device=dev)
    if name == "iq_cpwc":  # transmit apodization from the plane-wave angle
        wl.tx_window, wl.tx_f_number = Window.tukey25, 1.7
    return wl


@pytest.mark.parametrize("name", ["rf_plane_wave", "iq_cpwc"])
def test_table_kernel_vs_das_c_port_full_config(cuda_dev, name):
    wl = workload(name, cuda_dev)
    das = make_das(wl)
    cd = wl.channel_data
    fs = float(np.float32(cd.sampling_frequency))
    t0 = float(np.float32(cd.initial_time))
    fd = float(np.float32(cd.modulation_frequency))
    tx_apo, rx_apo, tx_delay, rx_delay = das.tables()
    ch = channel_tensor(cd.data, cuda_dev)
    if not ch.is_complex():  # das.m:211-214: RF is made analytic before das_c
        ch = hilbert_last(ch)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).to(cuda_dev)
    out = kernels.das_table_f32(ch, fs, t0, T(tx_apo), T(rx_apo), T(tx_delay), T(rx_delay), fd,
                                int(wl.dimension))
    torch.cuda.synchronize()
    got_all = kernels.to_matlab_order(out).cpu().numpy()
    P = wl.scan.N_pixels
    sel = np.sort(np.random.default_rng(11).choice(P, 2000, replace=False))
    ch_np = kernels.to_matlab_order(ch).cpu().numpy()
    ref = O.das_f32(ch_np, fs, t0, tx_apo[sel], rx_apo[sel], tx_delay[sel], rx_delay[sel], fd,
                    int(wl.dimension))
    got = got_all[sel]
    assert got.shape == ref.shape
    assert np.abs(ref).max() > 0
    assert rel_l2(got, ref) <= TOL_DAS_C
    assert np.all(got[ref == 0] == 0)
    assert np.all(np.isfinite(got_all))


def test_table_kernel_real_rf_full_config(cuda_dev):
    """Real RF in, real out: real(das_c(x + 0j)) on the whole RF plane-wave frame."""
    wl = workload("rf_plane_wave", cuda_dev)
    das = make_das(wl)
    cd = wl.channel_data
    fs = float(np.float32(cd.sampling_frequency))
    t0 = float(np.float32(cd.initial_time))
    tx_apo, rx_apo, tx_delay, rx_delay = das.tables()
    ch = channel_tensor(cd.data, cuda_dev)
    assert not ch.is_complex()
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).to(cuda_dev)
    out = kernels.das_table_f32(ch, fs, t0, T(tx_apo), T(rx_apo), T(tx_delay), T(rx_delay), 0.0, 3)
    torch.cuda.synchronize()
    sel = np.sort(np.random.default_rng(12).choice(wl.scan.N_pixels, 2000, replace=False))
    ch0 = kernels.to_matlab_order(ch).cpu().numpy().astype(np.complex64)
    ref = O.das_f32(ch0, fs, t0, tx_apo[sel], rx_apo[sel], tx_delay[sel], rx_delay[sel], 0.0, 3).real
    got = kernels.to_matlab_order(out).cpu().numpy()[sel]
    assert rel_l2(got, ref) <= TOL_DAS_C
    assert np.all(got[ref == 0] == 0)


def fp64_subset(wl, das, ch_matlab, sel):
    """The FP64 oracle (das_c's formula in double) on a pixel subset, with double
    tables from the host geometry code and the das.m phase epilogue."""
    cd = wl.channel_data
    sub = Scan(wl.scan.x[sel], wl.scan.y[sel], wl.scan.z[sel])
    txa = das.transmit_apodization.wave_apodization(cd.sequence, wl.scan)[sel]
    rxa = das.receive_apodization.aperture_apodization(cd.probe, sub)
    txd = geometry.transmit_delay(cd.sequence, wl.scan)[sel]
    rxd = geometry.receive_delay(cd.probe, sub, cd.sound_speed)
    ref = O.das_f64(ch_matlab.astype(np.complex128), cd.sampling_frequency, cd.initial_time, txa, rxa, txd, rxd,
                    cd.modulation_frequency, int(wl.dimension))
    if abs(cd.modulation_frequency) > 0:
        ph = np.exp(-1j * 4 * math.pi * cd.modulation_frequency * np.asarray(wl.scan.reference_distance)[sel]
                    / cd.sound_speed)
        ref = ref * ph.reshape((-1,) + (1,) * (ref.ndim - 1))
    return ref


def test_fast_fp16_matrix_3d_full_volume(cuda_dev):
    wl = synth.config_matrix_3d(device=cuda_dev)
    das = make_das(wl)
    geom = das.fast_geometry(cuda_dev)
    ch = channel_tensor(wl.channel_data.data, cuda_dev)
    st = fast.convert_channels(ch, Precision.fp16)
    outs = fast.das_fast(st, Precision.fp16, True, geom, wl.dimension, L=ch.shape[-1])
    torch.cuda.synchronize()
    assert int(outs["flags"].item()) == 0
    got_all = kernels.to_matlab_order(outs["cube"]).cpu().numpy()
    assert got_all.shape == (64 * 64 * 128, 1, 1, 1)
    assert np.all(np.isfinite(got_all))
    sel = np.sort(np.random.default_rng(13).choice(wl.scan.N_pixels, 1000, replace=False))
    ref = fp64_subset(wl, das, kernels.to_matlab_order(ch).cpu().numpy(), sel)
    assert rel_l2(got_all[sel], ref) <= TOL_FP16
