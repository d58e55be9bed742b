"""RF -> IQ demodulation kernel against the FP64 oracle of fast_demodulation.m."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from ustb_gb300 import preprocess, synth
from ustb_gb300.enums import Precision

pytestmark = pytest.mark.gpu

TOL = {Precision.fp32: 1e-5, Precision.fp16: 1e-3, Precision.bf16: 6e-3}


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def band_rf(rng, shape, fs, fc):
    """RF traces (..., L): noise band-passed around fc (time last)."""
    x = rng.standard_normal(shape)
    X = np.fft.rfft(x, axis=-1)
    f = np.fft.rfftfreq(shape[-1], 1 / fs)
    X *= np.exp(-0.5 * ((f - fc) / (0.3 * fc)) ** 2)
    return np.fft.irfft(X, n=shape[-1], axis=-1)


@pytest.mark.parametrize("prec", [Precision.fp32, Precision.fp16, Precision.bf16])
@pytest.mark.parametrize("D, L", [(2, 777), (3, 1024), (1, 300)])
def test_kernel_vs_oracle(cuda_dev, prec, D, L):
    rng = np.random.default_rng(D * 1000 + L)
    fs, t0, fc = 20e6, 1.7e-6, 5e6
    rf = band_rf(rng, (2, 3, 5, L), fs, fc).astype(np.float32)
    b = preprocess.lowpass_taps(fc, fs)
    got = preprocess.demodulate(torch.from_numpy(rf).to(cuda_dev), fs, t0, fc, b, D, prec)
    got = got.float().cpu().numpy()
    got = got[..., 0] + 1j * got[..., 1]
    want = O.fast_demodulation_f64(np.moveaxis(rf, -1, 0), fs, t0, fc, b.astype(np.float32), D)
    want = np.moveaxis(want, 0, -1)
    assert got.shape == want.shape
    assert rel(got, want) <= TOL[prec]


def test_int16_input_with_scale(cuda_dev):
    rng = np.random.default_rng(5)
    fs, t0, fc = 20e6, 0.0, 5e6
    rf = band_rf(rng, (4, 2048), fs, fc)
    i16 = np.round(rf / np.abs(rf).max() * 30000).astype(np.int16)
    b = preprocess.lowpass_taps(fc, fs)
    got = preprocess.demodulate(torch.from_numpy(i16).to(cuda_dev), fs, t0, fc, b, 2, Precision.fp32, 1 / 30000)
    got = got.cpu().numpy()
    got = got[..., 0] + 1j * got[..., 1]
    want = np.moveaxis(O.fast_demodulation_f64(i16.T.astype(np.float64) / 30000, fs, t0, fc,
                                               b.astype(np.float32), 2), 0, -1)
    assert rel(got, want) <= 1e-5


def test_fast_demodulation_class_on_the_rf_workload(cuda_dev):
    wl = synth.config_rf_plane_wave(device=cuda_dev)
    cd = wl.channel_data
    d = preprocess.FastDemodulation()
    d.input, d.modulation_frequency, d.device = cd, wl.info["f0"], cuda_dev
    iq = d.go()
    b = d.b
    assert iq.sampling_frequency == pytest.approx(cd.sampling_frequency / 2)
    assert iq.initial_time == pytest.approx(cd.initial_time - (len(b) - 1) / 2 / cd.sampling_frequency)
    assert iq.modulation_frequency == wl.info["f0"]
    rf = cd.data.cpu().numpy() if torch.is_tensor(cd.data) else np.asarray(cd.data)
    want = O.fast_demodulation_f64(rf, cd.sampling_frequency, cd.initial_time, wl.info["f0"],
                                   b.astype(np.float32), 2)
    got = iq.data.cpu().numpy()
    assert rel(got.reshape(want.shape), want) <= 1e-5


# ---- zero-phase variant (the reference's Python port) -----------------------
GOLDEN = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "python_demod.npz"))


class _CD:
    def __init__(self, data, fs, t0):
        from ustb_gb300.uff import ChannelData, Probe, Wave
        self.cd = ChannelData(data, Probe.linear_array(data.shape[1], 3e-4), [Wave()] * data.shape[2], fs, t0)


@pytest.mark.parametrize("name", ["default_dec", "explicit_dec", "no_dec", "int_like"])
@pytest.mark.parametrize("prec", [Precision.fp32, Precision.fp16])
def test_zero_phase_class_matches_reference_python_port(cuda_dev, name, prec):
    rf = GOLDEN[f"{name}/rf"]
    fs, t0, fc, fds = GOLDEN[f"{name}/params"]
    dm = preprocess.ZeroPhaseDemodulation()
    dm.input = _CD(rf.astype(np.float32), fs, t0).cd
    dm.modulation_frequency = fc
    dm.downsample_frequency = None if fds < 0 else fds
    dm.precision = prec
    dm.device = cuda_dev
    out = dm.go()
    got = out.data.cpu().numpy()[..., 0]
    want = GOLDEN[f"{name}/iq"][..., 0]
    assert got.shape == want.shape
    assert rel(got, want) <= TOL[prec]
    assert out.sampling_frequency == float(GOLDEN[f"{name}/fs_out"])
    assert out.initial_time == float(GOLDEN[f"{name}/t0_out"])


@pytest.mark.parametrize("D, L, src", [(4, 4096, "f32"), (1, 700, "f32"), (3, 2000, "i16"), (7, 9001, "f16")])
def test_zero_phase_kernel_vs_oracle(cuda_dev, D, L, src):
    """Long traces (several output chunks per trace) and every source type."""
    rng = np.random.default_rng(D * 7 + L)
    fs, t0, fc = 40e6, 0.8e-6, 5e6
    rf = band_rf(rng, (3, 5, L), fs, fc)
    if src == "i16":
        rf = np.round(rf / np.abs(rf).max() * 20000)
        x = torch.from_numpy(rf.astype(np.int16))
    elif src == "f16":
        rf = rf.astype(np.float16).astype(np.float64)
        x = torch.from_numpy(rf.astype(np.float16))
    else:
        rf = rf.astype(np.float32).astype(np.float64)
        x = torch.from_numpy(rf.astype(np.float32))
    b = preprocess.python_port_taps(fc, fs, L)
    got = preprocess.demodulate(x.to(cuda_dev), fs, t0, fc, b, D, Precision.fp32, zero_phase=True)
    got = got.cpu().numpy()
    got = got[..., 0] + 1j * got[..., 1]
    want = np.moveaxis(O.zero_phase_demodulation_f64(np.moveaxis(rf, -1, 0), fs, t0, fc, b.astype(np.float32), D),
                       0, -1)
    assert got.shape == want.shape
    assert rel(got, want) <= 1e-5


def test_zero_phase_short_trace_is_a_shape_error(cuda_dev):
    from ustb_gb300._lib import UstbError

    L = int(GOLDEN["short/L"])
    b = preprocess.python_port_taps(4e6, 20e6, L)
    x = torch.zeros((1, L), dtype=torch.float32, device=cuda_dev)
    with pytest.raises(UstbError) as e:
        preprocess.demodulate(x, 20e6, 0.0, 4e6, b, 1, zero_phase=True)
    assert e.value.code == 2  # USTB_E_SHAPE


def test_fast_demodulation_zero_phase_switch(cuda_dev):
    """FastDemodulation(zero_phase=True) is the Python port's variant."""
    rf = GOLDEN["default_dec/rf"]
    fs, t0, fc, fds = GOLDEN["default_dec/params"]
    a = preprocess.FastDemodulation()
    a.input, a.modulation_frequency, a.zero_phase, a.device = _CD(rf.astype(np.float32), fs, t0).cd, fc, True, cuda_dev
    b = preprocess.ZeroPhaseDemodulation()
    b.input, b.modulation_frequency, b.device = _CD(rf.astype(np.float32), fs, t0).cd, fc, cuda_dev
    oa, ob = a.go(), b.go()
    assert torch.equal(oa.data, ob.data)
    assert oa.sampling_frequency == ob.sampling_frequency and oa.initial_time == ob.initial_time
