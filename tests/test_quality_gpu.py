"""Reduced-precision storage against the FP64 oracle in imaging terms.

Full-size IQ plane-wave compounding (1024 samples x 128 channels x 75 waves,
400 x 400 pixels) through ``DAS.go()`` with FP16 and BF16 channel storage.  The
bars: relative L2 <= 1e-3 (FP16) / 6e-3 (BF16), cyst contrast within 0.1 dB and
the -6 dB lateral width of isolated point targets within 1 % of the oracle's image.
"""
import math

import numpy as np
import pytest
import torch

from oracle import oracle as O
from ustb_gb300 import geometry, quality, synth
from ustb_gb300.das import DAS
from ustb_gb300.enums import Precision, Window
from ustb_gb300.geometry import Apodization

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def compounding(cuda_dev):
    wl = synth.config_iq_cpwc(seed=2, device=cuda_dev)
    cd, scan = wl.channel_data, wl.scan
    das = DAS()
    das.channel_data, das.scan, das.dimension = cd, scan, wl.dimension
    das.receive_apodization = Apodization(window=wl.rx_window, f_number=wl.rx_f_number)
    das.transmit_apodization = Apodization(window=Window.tukey25, f_number=1.7)
    txa = das.transmit_apodization.wave_apodization(cd.sequence, scan)
    rxa = das.receive_apodization.aperture_apodization(cd.probe, scan)
    txd = geometry.transmit_delay(cd.sequence, scan)
    rxd = geometry.receive_delay(cd.probe, scan, cd.sound_speed)
    ch = np.asarray(cd.data.cpu().numpy() if torch.is_tensor(cd.data) else cd.data).astype(np.complex128)
    ref = O.das_f64(ch, cd.sampling_frequency, cd.initial_time, txa, rxa, txd, rxd,
                    cd.modulation_frequency, int(wl.dimension))[:, 0, 0, 0]
    ref = ref * np.exp(-1j * 4 * math.pi * cd.modulation_frequency * scan.reference_distance / cd.sound_speed)
    return wl, das, ref


@pytest.mark.parametrize("prec, l2", [(Precision.fp16, 1e-3), (Precision.bf16, 6e-3)])
def test_contrast_and_resolution_vs_fp64_oracle(compounding, prec, l2):
    wl, das, ref = compounding
    das.engine, das.precision = "fast", prec
    img = das.go().data.cpu().numpy().reshape(-1)
    r = quality.compare(img, ref, wl.scan, wl.info["cysts"], wl.info["scatterers"])
    assert r["rel_l2"] <= l2
    assert len(r["contrast_db"]) == 2 and r["max_contrast_diff_db"] <= 0.1, r["contrast_db"]
    assert len(r["fwhm_m"]) >= 3
    for a, b in r["fwhm_m"]:
        assert abs(a - b) <= 0.01 * b, (a, b)
