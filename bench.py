"""Benchmark: delay-and-sum throughput and serving on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--no-serving] [--no-cpu-baseline]

Headline workload (one "step" = one beamformed frame): IQ coherent plane-wave
compounding — 128-element linear array (pitch 0.3 mm, f0 = 5 MHz, fs = 20 MHz),
1024 complex64 samples x 128 channels x 75 plane waves (-16..16 deg),
400 x 400 pixels, Tukey-25% receive apodization at F# 1.7, transmit
apodization from the plane-wave angle, dimension 'both'.  Seeded synthetic
channel data (speckle, two cysts, point targets) stands in for the reference's
datasets.

``value``  G pixel.channel.wave/s of the fast path with FP32 channel storage
           (geometry formed on the fly), inputs resident in HBM, L2 flushed
           between steps.  The das_c-exact table kernel and FP16 storage are
           reported beside it in ``config``.
``e2e``    the same metric through the C-ABI with host buffers: complex64
           channel data copied in, the image copied out, every step.
``serving`` a seeded Poisson stream of requests drawn uniformly from five
           workloads (RF plane wave, IQ compounding, diverging-wave sector with
           the CF/DMAS epilogue, synthetic transmit aperture, 3D matrix array),
           served with FP16 storage by continuous batching into persistent
           launches, against the same requests beamformed one at a time by the
           plain FP32 das_c-exact kernel and by the fast path.
``--impl reference`` times the reference's CPU implementation of the path on
           the host cores: its own das_c, compiled from the staged source on this
           machine (the bit-identical oracle port where it was not built), and
           beside it its own das_cuda on the GPU (``reference_gpu_das_cuda``).
Multi-GPU runs are replicas: every rank beamforms its own frames.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "beamformed G pixel·channel·wave/s; serving frames/s + p50/p99 ms vs plain DAS"
UNIT = "G pixel·channel·wave/s"
FLOP_PER_UNIT_IQ = 22  # algorithmic FP32 FLOP per IQ unit (+2 MUFU sincos)
FLOP_PER_UNIT_RF = 10
FP32_LANES_PER_SM = 128
# DRAM bytes (read + write) of one das_fast_kernel<both, complex, f32> launch on the
# headline workload, from an ncu capture of `bench.py --profile headline`
TRAFFIC_FAST_F32_HEADLINE = 210_949_376


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.proc, self.path = index, None, None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path:
            return None
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = float(parts[2])
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        finally:
            os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def build_das(wl):
    from ustb_gb300.das import DAS
    from ustb_gb300.geometry import Apodization

    das = DAS()
    das.channel_data, das.scan, das.dimension = wl.channel_data, wl.scan, wl.dimension
    das.receive_apodization = Apodization(window=wl.rx_window, f_number=wl.rx_f_number)
    das.transmit_apodization = Apodization(window=wl.tx_window, f_number=wl.tx_f_number)
    return das


def make_headline(device):
    from ustb_gb300 import synth
    from ustb_gb300.das import channel_tensor
    from ustb_gb300.enums import Window

    wl = synth.config_iq_cpwc(seed=2, device=device)
    wl.tx_window, wl.tx_f_number = Window.tukey25, 1.7
    das = build_das(wl)
    ch = channel_tensor(wl.channel_data.data, device)
    return wl, das, ch


def tuned_geometry(das, wl, st, prec, cplx, L, device, F=1, epilogue=False):
    """The request's FastGeometry with the tile plan and stage shape the autotuner picks
    (cached per device and shape), timed on this request's own data."""
    from ustb_gb300 import autotune, fast

    dim = int(wl.dimension)
    cd = wl.channel_data
    run = lambda g: fast.das_fast(st, prec, cplx, g, dim, F=F, L=L, epilogue=epilogue, cube=not epilogue)
    key = autotune.shape_key(wl.scan, cd.N_channels, cd.N_waves, L, F, prec, dim, cplx, device)
    choice = autotune.tune(lambda b, o, c, sh: das.fast_geometry(device, b, o, c, sh), run,
                           key + ("|epi" if epilogue else ""), scan=wl.scan, both=dim == 3, dimension=dim)
    return das.fast_geometry(device, choice.block, choice.order, choice.ctas_per_tile, choice.stage_shape), choice


def active_units(tx_apo, rx_apo, F=1):
    """Units with nonzero tx and rx apodization: the ones das_c evaluates."""
    ntx = (tx_apo != 0).sum(axis=1).astype(np.int64)
    nrx = (rx_apo != 0).sum(axis=1).astype(np.int64)
    return int((ntx * nrx).sum()) * F


def cuda_time(fn, steps, flush, stream, torch):
    """Per-step CUDA-event time (ms) of fn(), L2 flushed outside the events."""
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for i in range(steps):
        flush.zero_()
        evs[i][0].record(stream)
        fn()
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in evs]


# ---------------------------------------------------------------------------
def cpu_reference(ch_np, fs, t0, fd, tabs, dim, target_s=12.0, steps=1):
    """The reference's own das_c (built from its source into oracle/_ref, on all host
    cores through its std::thread parallel_for) over a strided pixel sample; the
    bit-identical port where das_c was not built on this machine."""
    from oracle import oracle as O

    tx_apo, rx_apo, tx_delay, rx_delay = tabs
    P = tx_apo.shape[0]
    threads = os.cpu_count() or 1
    use_ref = O.have_reference()

    def run(stride):
        sel = np.arange(0, P, stride)
        t = time.perf_counter()
        if use_ref:
            O.das_c_ref(ch_np, fs, t0, tx_apo[sel], rx_apo[sel], tx_delay[sel], rx_delay[sel], fd, dim)
        else:
            O.das_f32(ch_np, fs, t0, tx_apo[sel], rx_apo[sel], tx_delay[sel], rx_delay[sel], fd, dim,
                      threads=threads)
        return time.perf_counter() - t, sel.size

    dt, n = run(200)
    stride = max(1, int(math.ceil(P * dt / max(n, 1) / target_s)))
    times = []
    for _ in range(max(1, steps)):
        dt, n = run(stride)
        times.append(dt)
    L, N, W, F = ch_np.shape
    t = statistics.median(times)
    what = ("the reference's +mex/source/das_c.cpp compiled unmodified (oracle/_ref/libdas_c_ref.so), "
            f"parallel_for over {threads} threads" if use_ref else
            f"oracle/das_port.c oracle_das_f32 (bit-identical to das_c) on {threads} threads")
    return {"value": n * N * W * F / t / 1e9, "unit": UNIT, "cores": threads,
            "kind": "reference" if use_ref else "port",
            "sample": f"every {stride}-th pixel ({n} of {P} pixels, all channels/waves), {t:.1f} s per pass, {what}"}


def das_cuda_reference(ch_np, fs, t0, fd, tabs, steps=3):
    """The reference's das_cuda (+mex/source/das_cuda.cu compiled unmodified for sm_103a)
    on the whole frame, timed as its MEX call is used: host buffers in, host image out
    (tables and channel data copied every call).  None where it was not built."""
    from oracle import oracle as O

    if not O.have_cuda_reference():
        return None
    tx_apo, rx_apo, tx_delay, rx_delay = tabs
    O.das_cuda_ref(ch_np, fs, t0, tx_apo, rx_apo, tx_delay, rx_delay, fd)  # warm-up
    times = []
    for _ in range(max(1, steps)):
        t = time.perf_counter()
        out = O.das_cuda_ref(ch_np, fs, t0, tx_apo, rx_apo, tx_delay, rx_delay, fd)
        times.append(time.perf_counter() - t)
    L, N, W, F = ch_np.shape
    P = tx_apo.shape[0]
    ms = statistics.median(times) * 1e3
    return {"ms_per_frame": round(ms, 3), "value": round(P * N * W * F / (ms * 1e-3) / 1e9, 3), "unit": UNIT,
            "call": "mex.das_cuda argument layout (das.m:262-271), host buffers, dimension both, median of "
                    f"{len(times)} calls", "output": out}


def fp64_subset_reference(wl, das, ch_matlab, sel):
    """The FP64 oracle (das_c's formula in double) on a pixel subset, with double tables
    from the host geometry code, and the das.m phase epilogue."""
    from oracle import oracle as O
    from ustb_gb300 import geometry
    from ustb_gb300.uff import Scan, SectorScan

    cd = wl.channel_data
    sub = Scan(wl.scan.x[sel], wl.scan.y[sel], wl.scan.z[sel])
    txa = das.transmit_apodization.wave_apodization(cd.sequence, wl.scan)[sel]
    if isinstance(wl.scan, SectorScan):  # aperture centred on the sector origin: full-scan table
        rxa = das.receive_apodization.aperture_apodization(cd.probe, wl.scan)[sel]
    else:
        rxa = das.receive_apodization.aperture_apodization(cd.probe, sub)
    txd = geometry.transmit_delay(cd.sequence, wl.scan)[sel]
    rxd = geometry.receive_delay(cd.probe, sub, cd.sound_speed)
    ref = O.das_f64(ch_matlab.astype(np.complex128), cd.sampling_frequency, cd.initial_time, txa, rxa, txd, rxd,
                    cd.modulation_frequency, int(wl.dimension))
    if abs(cd.modulation_frequency) > 0:
        ph = np.exp(-1j * 4 * np.pi * cd.modulation_frequency * np.asarray(wl.scan.reference_distance)[sel]
                    / cd.sound_speed)
        ref = ref * ph.reshape((-1,) + (1,) * (ref.ndim - 1))
    return ref


def headline_parity(wl, das, ch, tabs, phase, fast_step, st32, st16, table_step, out_t, torch, n_pix=2000):
    """Measured relative L2 of the headline outputs on a seeded pixel subset: the table
    kernel and the FP32 fast path against the das_c port (das.m's single-precision
    tables, then the per-pixel phase), and both storages of the fast path against the
    FP64 oracle."""
    from oracle import oracle as O
    from ustb_gb300 import kernels
    from ustb_gb300.enums import Precision

    cd = wl.channel_data
    fs, t0, fd = (float(np.float32(cd.sampling_frequency)), float(np.float32(cd.initial_time)),
                  float(np.float32(cd.modulation_frequency)))
    sel = np.sort(np.random.default_rng(11).choice(wl.scan.N_pixels, n_pix, replace=False))
    ch_np = kernels.to_matlab_order(ch).cpu().numpy()
    ph = phase.cpu().numpy()[sel].reshape(-1, 1, 1, 1)
    port = O.das_f32(ch_np, fs, t0, tabs[0][sel], tabs[1][sel], tabs[2][sel], tabs[3][sel], fd, 3,
                     threads=os.cpu_count() or 1) * ph
    f64 = fp64_subset_reference(wl, das, ch_np, sel)
    table_step()
    got_t = kernels.to_matlab_order(out_t).cpu().numpy()[sel]
    got32 = kernels.to_matlab_order(fast_step(st32, Precision.fp32)()["cube"]).cpu().numpy()[sel]
    got16 = kernels.to_matlab_order(fast_step(st16, Precision.fp16)()["cube"]).cpu().numpy()[sel]
    rel = lambda a, b: float(f"{np.linalg.norm(a - b) / np.linalg.norm(b):.3g}")
    return {"pixels": int(n_pix), "seed": 11,
            "table_vs_das_c_port": rel(got_t, port),
            "fast_fp32_vs_das_c_port": rel(got32, port),
            "fast_fp32_vs_fp64_oracle": rel(got32, f64),
            "fast_fp16_vs_fp64_oracle": rel(got16, f64),
            "table_vs_fp64_oracle": rel(got_t, f64)}


# ---------------------------------------------------------------------------
def serving_mix(device, n_requests, seed, torch):
    """Served FP16 continuous batching vs plain single-request FP32 DAS on a seeded
    Poisson stream over five workloads.  Returns a summary dict."""
    from oracle import oracle as O
    from ustb_gb300 import fast, geometry, kernels, serving, synth
    from ustb_gb300.das import channel_tensor
    from ustb_gb300.enums import Precision

    kinds = ["rf_plane_wave", "iq_cpwc", "dw_sector", "sta", "matrix_3d"]
    srv = serving.Server(device, hbm_budget_bytes=150e9, max_batch=32, max_inflight=2)
    prep = {}
    plain = {}
    tuned = {}
    for k in kinds:
        wl = synth.CONFIGS[k](device=device)
        das = build_das(wl)
        ch = channel_tensor(wl.channel_data.data, device)
        cplx = ch.is_complex()
        st = fast.convert_channels(ch, Precision.fp16)
        geom, choice = tuned_geometry(das, wl, st, Precision.fp16, cplx, ch.shape[-1], device,
                                      epilogue=wl.epilogue is not None)
        tuned[k] = {"block": choice.block, "order": choice.order, "stage_shape": choice.stage_shape,
                    "ctas_per_tile": choice.ctas_per_tile}
        srv.add_plan(k, geom)
        prep[k] = (wl, das, ch, st, cplx)
        # plain path: das_c-exact FP32 kernel on resident single-precision tables
        cd = wl.channel_data
        T = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).to(device)
        txa = das.transmit_apodization.wave_apodization(cd.sequence, wl.scan).astype(np.float32)
        txd = geometry.transmit_delay(cd.sequence, wl.scan).astype(np.float32)
        rxd, rxa = geometry.receive_tables_device(cd.probe, wl.scan, cd.sound_speed, das.receive_apodization,
                                                  device=device)
        chp = ch if cplx else ch  # real RF stays real in the plain path
        plain[k] = (chp, float(np.float32(cd.sampling_frequency)), float(np.float32(cd.initial_time)),
                    T(txa), rxa, T(txd), rxd, float(np.float32(cd.modulation_frequency)), int(wl.dimension))
    rng = np.random.default_rng(seed)
    order = [kinds[i] for i in rng.integers(0, len(kinds), n_requests)]

    def run_plain(k):
        a = plain[k]
        kernels.das_table_f32(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8])

    def ev_ms(fn, n=3):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    per_kind = {}
    for k in kinds:
        wl, das, ch, st, cplx = prep[k]
        epi = wl.epilogue is not None
        per_kind[k] = {
            "plain_fp32_ms": round(ev_ms(lambda: run_plain(k)), 3),
            "fast_fp16_ms": round(ev_ms(lambda: fast.das_fast(st, Precision.fp16, cplx, srv.plans[k], wl.dimension,
                                                               L=ch.shape[-1], epilogue=epi, cube=not epi,
                                                               check=False)), 3),
            "units": wl.units}
    # plain single-request FP32 DAS: the requests one after another
    torch.cuda.synchronize()
    t = time.perf_counter()
    for k in order:
        run_plain(k)
        torch.cuda.synchronize()
    plain_s = time.perf_counter() - t

    # the same requests on the fast path (FP16 storage), one launch per request and one
    # request at a time: what continuous batching is measured against
    def run_fast(k):
        wl, das, ch, st, cplx = prep[k]
        epi = wl.epilogue is not None
        fast.das_fast(st, Precision.fp16, cplx, srv.plans[k], wl.dimension, L=ch.shape[-1], epilogue=epi,
                      cube=not epi, check=False)

    for k in kinds:
        run_fast(k)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for k in order:
        run_fast(k)
        torch.cuda.synchronize()
    serial_fast_s = time.perf_counter() - t

    def make(i, order=order):
        k = order[i]
        wl, das, ch, st, cplx = prep[k]
        return serving.Job(k, st, Precision.fp16, cplx, 1, ch.shape[-1], int(wl.dimension),
                           epilogue=wl.epilogue is not None)

    srv.run([0.0] * 8, make)  # warm-up
    # saturated throughput: the whole stream arrives at once
    srv.completed.clear()
    launches0 = srv.launches
    burst = srv.run([0.0] * n_requests, make)
    sat = serving.latency_stats(burst)
    launches = srv.launches - launches0
    # latency: Poisson arrivals at 70 % of the saturated request rate
    rate = 0.7 * n_requests / sat["seconds"]
    srv.completed.clear()
    jobs = srv.run(list(serving.poisson_arrivals(n_requests, rate, seed)), make)
    stats = serving.latency_stats(jobs, per_key=True)
    # the same arrivals with a sixth of the SMs kept from the large requests for the small ones
    lsrv = serving.Server(device, hbm_budget_bytes=150e9, max_batch=32,
                          reserve_sms=torch.cuda.get_device_properties(device).multi_processor_count // 6)
    for k in kinds:
        lsrv.add_plan(k, srv.plans[k])
    lsrv.run([0.0] * 8, make)
    lsrv.completed.clear()
    lburst = serving.latency_stats(lsrv.run([0.0] * n_requests, make))
    lsrv.completed.clear()
    lstats = serving.latency_stats(lsrv.run(list(serving.poisson_arrivals(n_requests, rate, seed)), make), per_key=True)
    # the same burst through the library's own server (ustb_serve_*: resident plans,
    # scheduler and completion threads in C++)
    from ustb_gb300 import plan as native

    nplans = {}
    for k in kinds:
        wl, das, ch, st, cplx = prep[k]
        nplans[k] = native.Plan(srv.plans[k], ch.shape[-1], Precision.fp16, cplx, wl.dimension,
                                epilogue=wl.epilogue is not None, library_tiles=False)
    nsrv = native.Server(workspace_budget=16 << 30, max_batch=32, device=device)
    for t in [nsrv.submit(nplans[k], prep[k][3], cube=prep[k][0].epilogue is None) for k in order[:8]]:
        nsrv.wait(t)  # warm-up
    torch.cuda.synchronize()
    t = time.perf_counter()
    tickets = [nsrv.submit(nplans[k], prep[k][3], cube=prep[k][0].epilogue is None) for k in order]
    nflags = 0
    for tk in tickets:
        nflags |= nsrv.wait(tk)["flags"]
    native_s = time.perf_counter() - t
    nsrv.close()
    for p_ in nplans.values():
        p_.close()
    # accuracy of each kind against the FP64 oracle on a pixel subset
    errs = {}
    for k in kinds:
        wl, das, ch, st, cplx = prep[k]
        job = next(j for j in jobs if j.key == k)
        cd = wl.channel_data
        sel = np.random.default_rng(0).choice(wl.scan.N_pixels, min(1500, wl.scan.N_pixels), replace=False)
        ref = fp64_subset_reference(wl, das, kernels.to_matlab_order(ch).cpu().numpy(), sel)
        if job.epilogue:
            got = job.outputs["das"].cpu().numpy()[0][sel]
            want = ref[:, :, 0, 0].sum(axis=1)
        else:
            got = kernels.to_matlab_order(job.outputs["cube"]).cpu().numpy()[sel]
            want = ref if cplx else ref.real
        errs[k] = float(np.linalg.norm(got - want) / np.linalg.norm(want))
    return {
        "requests": n_requests, "kinds": kinds, "seed": seed,
        "served_frames_per_s": round(sat["frames_per_s"], 1),
        "plain_fp32_frames_per_s": round(n_requests / plain_s, 1),
        "speedup_vs_plain": round(sat["frames_per_s"] / (n_requests / plain_s), 2),
        "serial_fast_frames_per_s": round(n_requests / serial_fast_s, 1),
        "speedup_vs_serial_fast": round(sat["frames_per_s"] / (n_requests / serial_fast_s), 3),
        "policy": f"small requests batched per kernel variant (<= 32 per launch, {srv.max_inflight} streams); "
                  f"requests above {srv.large_units:.0e} units alone on another stream, queued back to back, "
                  f"with all {srv.large_ctas} SMs",
        "latency_policy": {"reserve_sms": lsrv.reserve_sms, "large_ctas": lsrv.large_ctas,
                           "served_frames_per_s": round(lburst["frames_per_s"], 1),
                           "latency_at_same_arrivals": {"p50_ms": round(lstats["p50_ms"], 3),
                                                        "p99_ms": round(lstats["p99_ms"], 3),
                                                        "per_kind": lstats["per_kind"]}},
        "launches_for_stream": launches,
        "native_server": {"frames_per_s": round(n_requests / native_s, 1),
                          "speedup_vs_plain": round(plain_s / native_s, 2),
                          "speedup_vs_serial_fast": round(serial_fast_s / native_s, 3), "flags": int(nflags),
                          "api": "ustb_plan_create (the tuned tile maps) + ustb_serve_submit/wait (C++ "
                                 "scheduler and completion threads, persistent batches within a 16 GB entries "
                                 "budget; requests above 2e9 units alone on a third stream)"},
        "latency_at_70pct_load": {"arrival_rate_hz": round(rate, 1), "p50_ms": round(stats["p50_ms"], 3),
                                  "p99_ms": round(stats["p99_ms"], 3), "frames_per_s": round(stats["frames_per_s"], 1),
                                  "per_kind": stats["per_kind"]},
        "per_kind": per_kind,
        "hbm_budget_gb": 150, "storage": "fp16",
        "rel_l2_vs_fp64_oracle": {k: float(f"{v:.3g}") for k, v in errs.items()},
        "tile_plans": tuned,
        "plain_path": "ustb_das_table_f32 (das_c-exact FP32 tables resident), one request at a time",
    }


# ---------------------------------------------------------------------------
def hfr_ensemble(device, torch, reps=5, plain_frames=20):
    """High-frame-rate ensemble: 200 frames x 11 plane waves x 128 channels x 1536 int16
    I/Q samples, 256 x 512 pixels, dimension both.  The tile plan is chosen by the
    autotuner; the int16 -> FP16 conversion, the entries pass and ONE persistent launch
    over all (frame, tile) items are replayed from a CUDA graph.  Against it: the plain
    FP32 das_c-exact kernel looped per frame on resident tables."""
    from oracle import oracle as O
    from ustb_gb300 import autotune, fast, geometry, kernels, synth
    from ustb_gb300.ensemble import Ensemble
    from ustb_gb300.enums import Precision

    wl = synth.config_hfr_ensemble(device=device)
    das = build_das(wl)
    x = wl.info["int16"]
    F, W, N, L, _ = x.shape
    P = wl.scan.N_pixels
    scale = wl.info["scale"]
    # tile plan: tuned on the first 8 frames, cached per shape
    sub = fast.convert_channels(x[:8].contiguous(), Precision.fp16, scale)
    run = lambda g: fast.das_fast(sub, Precision.fp16, True, g, int(wl.dimension), F=8, L=L)
    key = autotune.shape_key(wl.scan, N, W, L, 8, Precision.fp16, wl.dimension, True, device)
    choice = autotune.tune(lambda b, o, c, sh: das.fast_geometry(device, b, o, c, sh), run, key, scan=wl.scan,
                           dimension=int(wl.dimension))
    del sub
    geom = das.fast_geometry(device, choice.block, choice.order, 0, choice.stage_shape)
    ens = Ensemble(geom, F, L, wl.dimension, Precision.fp16, scale, graph=True)
    ens.run(x)
    torch.cuda.synchronize()
    if ens.flags():
        raise RuntimeError("the ensemble's tile plan overflowed a sample window")
    for _ in range(2):
        ens.run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        ens.run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    # end to end: the int16 ensemble copied in from pinned host memory every time
    h = torch.empty(x.shape, dtype=torch.int16, pin_memory=True)
    h.copy_(x)
    h_out = torch.empty(ens.outputs["cube"].shape, dtype=torch.complex64, pin_memory=True)
    e0.record()
    for _ in range(reps):
        o = ens.run(h)
        h_out.copy_(o["cube"], non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / reps
    # plain FP32 per frame
    cd = wl.channel_data
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).to(device)
    txa = T(das.transmit_apodization.wave_apodization(cd.sequence, wl.scan).astype(np.float32))
    txd = T(geometry.transmit_delay(cd.sequence, wl.scan).astype(np.float32))
    rxd, rxa = geometry.receive_tables_device(cd.probe, wl.scan, cd.sound_speed, das.receive_apodization,
                                              device=device)
    fs, t0, fd = (float(np.float32(cd.sampling_frequency)), float(np.float32(cd.initial_time)),
                  float(np.float32(cd.modulation_frequency)))
    frames = [torch.complex(x[f, ..., 0].float(), x[f, ..., 1].float()) * scale for f in range(plain_frames)]
    out = torch.empty(kernels.out_shape_abi(P, N, W, 1, 3), dtype=torch.complex64, device=device)
    for f in range(2):
        kernels.das_table_f32(frames[f].unsqueeze(0), fs, t0, txa, rxa, txd, rxd, fd, 3, out=out)
    torch.cuda.synchronize()
    e0.record()
    for f in range(plain_frames):
        kernels.das_table_f32(frames[f].unsqueeze(0), fs, t0, txa, rxa, txd, rxd, fd, 3, out=out)
    e1.record()
    torch.cuda.synchronize()
    plain_ms_frame = e0.elapsed_time(e1) / plain_frames
    # accuracy of frame 0 against the FP64 oracle on a pixel subset
    sel = np.random.default_rng(0).choice(P, 2000, replace=False)
    from ustb_gb300.uff import Scan

    subscan = Scan(wl.scan.x[sel], wl.scan.y[sel], wl.scan.z[sel])
    ch0 = (x[0].double()[..., 0] + 1j * x[0].double()[..., 1]).cpu().numpy() * scale
    chm = np.ascontiguousarray(ch0.transpose(2, 1, 0))[..., None]
    ref = O.das_f64(chm, cd.sampling_frequency, cd.initial_time,
                    das.transmit_apodization.wave_apodization(cd.sequence, subscan),
                    das.receive_apodization.aperture_apodization(cd.probe, subscan),
                    geometry.transmit_delay(cd.sequence, subscan),
                    geometry.receive_delay(cd.probe, subscan, cd.sound_speed), cd.modulation_frequency, 3)[:, 0, 0, 0]
    ref = ref * np.exp(-1j * 4 * math.pi * cd.modulation_frequency * subscan.z / cd.sound_speed)
    got = ens.outputs["cube"][0, 0, 0].cpu().numpy()[sel]
    err = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    units = P * N * W * F
    return {
        "workload": f"{F} frames x {W} plane waves x {N} channels x {L} int16 I/Q samples, "
                    f"{wl.scan.N_x_axis}x{wl.scan.N_z_axis} pixels, dimension both",
        "ms_per_ensemble": round(ms, 3), "frames_per_s": round(F / (ms * 1e-3), 1),
        "value": round(units / (ms * 1e-3) / 1e9, 2), "unit": UNIT,
        "e2e_ms_per_ensemble": round(e2e_ms, 3), "e2e_frames_per_s": round(F / (e2e_ms * 1e-3), 1),
        "e2e_h2d_bytes": int(h.numel() * 2), "e2e_d2h_bytes": int(h_out.numel() * 8),
        "plain_fp32_ms_per_frame": round(plain_ms_frame, 4),
        "plain_fp32_frames_per_s": round(1e3 / plain_ms_frame, 1),
        "speedup_vs_plain": round(plain_ms_frame * F / ms, 2),
        "launch": "one CUDA graph replay per ensemble: int16->FP16 conversion, entries pass, "
                  "one persistent launch over all (frame, tile) items",
        "tile_plan": {"block": list(choice.block) if choice.block else "planner default",
                      "stage_shape": choice.stage_shape,
                      "order": choice.order, "tuned_ms_8_frames": round(choice.ms, 3)},
        "rel_l2_vs_fp64_oracle_frame0": float(f"{err:.3g}"),
        "storage": "fp16",
    }


# ---------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-hfr", action="store_true", help="skip the high-frame-rate ensemble section")
    ap.add_argument("--serving-requests", type=int, default=200)
    ap.add_argument("--profile", default=None, metavar="WORKLOAD",
                    help="launch only the kernels of one workload (headline, a synth.CONFIGS name, or "
                         "demod / image / coherence for the kernels around the beamformer) "
                         "--steps times each, for ncu; prints their CUDA-event times")
    ap.add_argument("--stage-shape", type=int, default=0, choices=[0, 1, 2, 3],
                    help="stage shape of the fast kernel under --profile (0: the library's choice)")
    ap.add_argument("--storage", default="fp32", choices=["fp32", "fp16", "bf16"],
                    help="channel storage of the fast kernel under --profile")
    args = ap.parse_args()
    if args.profile:
        return main_profile(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.impl == "reference":
        return main_reference(args, rank, world)

    from ustb_gb300 import _lib, fast, kernels
    from ustb_gb300.enums import Precision

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    warm = max(args.warmup, 3)
    wl, das, ch = make_headline(dev)
    cd = wl.channel_data
    P, N, W, F, L = wl.scan.N_pixels, cd.N_channels, cd.N_waves, cd.N_frames, cd.N_samples
    units = P * N * W * F
    tabs = das.tables()
    act = active_units(tabs[0], tabs[1], F)
    fs, t0, fd = (float(np.float32(cd.sampling_frequency)), float(np.float32(cd.initial_time)),
                  float(np.float32(cd.modulation_frequency)))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    flags = torch.zeros(1, dtype=torch.int32, device=dev)
    st32 = fast.convert_channels(ch, Precision.fp32)
    st16 = fast.convert_channels(ch, Precision.fp16)
    # the tile plan and stage shape the autotuner picks for this shape (cached per device)
    geom, plan = tuned_geometry(das, wl, st32, Precision.fp32, True, L, dev)

    def fast_step(st, prec):
        return lambda: fast.das_fast(st, prec, True, geom, 3, L=L, flags=flags, check=False)

    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).to(dev)
    d_tab = [T(a) for a in tabs]
    out_t = torch.empty(kernels.out_shape_abi(P, N, W, F, 3), dtype=torch.complex64, device=dev)
    phase = torch.from_numpy(das.pixel_phase().astype(np.complex64)).to(dev)

    def table_step():
        kernels.das_table_f32(ch, fs, t0, d_tab[0], d_tab[1], d_tab[2], d_tab[3], fd, 3, out=out_t)
        kernels.apply_pixel_phase(out_t, phase)

    for fn in (fast_step(st32, Precision.fp32), fast_step(st16, Precision.fp16), table_step):
        for _ in range(warm):
            fn()
    torch.cuda.synchronize()
    if int(flags.item()):
        raise RuntimeError("fast path flagged a window overflow on the headline workload")
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms32 = cuda_time(fast_step(st32, Precision.fp32), args.steps, flush, stream, torch)
    ms16 = cuda_time(fast_step(st16, Precision.fp16), args.steps, flush, stream, torch)
    mst = cuda_time(table_step, args.steps, flush, stream, torch)
    # the two halves of a fast-path step, each timed alone: the entries pass and the
    # beamforming kernel on prebuilt entries
    ent = fast.build_entries(st32, Precision.fp32, True, N, W, L=L)
    kern_step = lambda: fast.das_fast(st32, Precision.fp32, True, geom, 3, L=L, flags=flags, check=False,
                                      entries=ent)
    entries_step = lambda: fast.build_entries(st32, Precision.fp32, True, N, W, L=L)
    for fn in (kern_step, entries_step):
        for _ in range(warm):
            fn()
    msk = cuda_time(kern_step, args.steps, flush, stream, torch)
    mse = cuda_time(entries_step, args.steps, flush, stream, torch)
    if world > 1:
        torch.distributed.barrier()
    from ustb_gb300 import replicas

    ms = replicas.max_over_ranks(statistics.mean(ms32), dev)  # replicas: the slowest rank's step
    value = units * world / (ms * 1e-3) / 1e9

    # end to end through the C-ABI: pinned host channel data in, image out, every step;
    # a two-stream frame pipeline overlaps frame k's beamforming with the copies of its
    # neighbours
    h_ch = torch.empty(ch.shape, dtype=ch.dtype, pin_memory=True)
    h_ch.copy_(ch)
    h_out = [torch.empty(kernels.out_shape_abi(P, N, W, F, 3), dtype=torch.complex64, pin_memory=True)
             for _ in range(2)]
    pipe = fast.FramePipeline(geom, ch.shape, ch.dtype, Precision.fp32, True, 3, L=L, depth=2)
    pipe.start()
    for k in range(warm):
        pipe.submit(h_ch, h_out[k % 2])
    pipe.synchronize()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    pipe.start()
    for k in range(args.steps):
        pipe.submit(h_ch, h_out[k % 2])
    pipe.synchronize()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    if pipe.overflowed():
        raise RuntimeError("fast path flagged a window overflow in the end-to-end run")

    parity = headline_parity(wl, das, ch, tabs, phase, fast_step, st32, st16, table_step, out_t, torch)

    serving = None
    if world == 1 and not args.no_serving:
        serving = serving_mix(dev, args.serving_requests, 11, torch)
    hfr = None
    if world == 1 and not args.no_hfr:
        hfr = hfr_ensemble(dev, torch)

    if rank != 0:
        return
    peaks = measured_peaks()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = sms * FP32_LANES_PER_SM * 2 * sm_max * 1e6 / 1e12
    ms_kernel, ms_entries = statistics.mean(msk), statistics.mean(mse)
    achieved = FLOP_PER_UNIT_IQ * act / (ms_kernel * 1e-3) / 1e12
    entry_bytes = ch.numel() * ch.element_size() + fast.entry_bytes(L, N, W, F, True)
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    # compulsory bytes of the fast path: channel data, image, pixel xyz, tile map
    h_bytes_alg = (ch.numel() * ch.element_size() + P * F * 8 + P * 12 + geom.tiles.size * 4)
    res = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": warm, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded speckle + cysts + point targets)",
        "config": {
            "workload": "iq_cpwc: 1024 complex64 samples x 128 channels x 75 plane waves, 400x400 pixels, "
                        "dimension both; fast path, FP32 channel storage, geometry on the fly",
            "units_per_step": units, "das_c_active_units_per_step": act,
            "frames_per_s": round(1e3 / ms * world, 1),
            "fp16_storage": {"ms_per_step": round(statistics.mean(ms16), 4),
                             "value": round(units / statistics.mean(ms16) / 1e6, 2)},
            "das_c_exact_table_kernel": {"ms_per_step": round(statistics.mean(mst), 4),
                                         "value": round(units / statistics.mean(mst) / 1e6, 2),
                                         "rel_l2_vs_das_c_port": parity["table_vs_das_c_port"]},
            "parity": parity,
            "l2": "flushed between steps (256 MB write)", "parallelism": f"replicas x{world}",
            "tile_plan": {"block": list(plan.block) if plan.block else "planner default", "order": plan.order,
                          "stage_shape": plan.stage_shape, "ctas_per_tile": plan.ctas_per_tile,
                          "tuned_ms": round(plan.ms, 4)},
        },
        "roofline": {
            "bound": "fp32", "achieved": round(achieved, 3), "peak": round(fp32_peak, 2), "unit": "TFLOP/s",
            "frac": round(achieved / fp32_peak, 4), "traffic": TRAFFIC_FAST_F32_HEADLINE,
            "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch)",
            "algorithmic_bytes": int(h_bytes_alg),
            "kernel": "das_fast_kernel<both, complex, f32>", "kernel_ms": round(ms_kernel, 4),
            "timing": "CUDA events around the beamforming kernel alone (ustb_das_fast_entries on prebuilt entries)",
            "flop_per_unit": FLOP_PER_UNIT_IQ, "units_counted": "das_c_active_units (nonzero tx x rx apodization)",
            "step_frac": round(FLOP_PER_UNIT_IQ * act / (ms * 1e-3) / 1e12 / fp32_peak, 4),
            "entries_pass": {"ms": round(ms_entries, 4), "bound": "hbm", "algorithmic_bytes": int(entry_bytes),
                             "achieved_gbs": round(entry_bytes / (ms_entries * 1e-3) / 1e9, 1),
                             "peak_gbs": hbm_peak,
                             "frac": round(entry_bytes / (ms_entries * 1e-3) / 1e9 / hbm_peak, 4)},
            "peak_source": f"nominal {sms} SMs x 128 FP32 lanes x 2 x sm_max_mhz {sm_max:.0f} "
                           "(MEASURED_PEAKS.json has no FP32 figure)",
        },
        "e2e": {"value": round(units / (e2e_ms * 1e-3) / 1e9, 2), "unit": UNIT, "ms_per_step": round(e2e_ms, 4),
                "h2d_bytes_per_step": int(h_ch.numel() * h_ch.element_size()),
                "d2h_bytes_per_step": int(h_out[0].numel() * h_out[0].element_size()),
                "call": "per frame: cudaMemcpyAsync in + ustb_das_fast + cudaMemcpyAsync out (geometry resident), "
                        "two streams so neighbouring frames' copies overlap the beamforming (fast.FramePipeline)"},
        "gpu_launches": 2 * args.steps,  # per step: build_entries_kernel + das_fast_kernel
        "clocks": clk.summary(),
    }
    if serving is not None:
        res["serving"] = serving
    if hfr is not None:
        res["hfr_ensemble"] = hfr
    if world == 1 and not args.no_cpu_baseline:
        ch_np = kernels.to_matlab_order(ch).cpu().numpy()
        res["cpu_baseline"] = cpu_reference(ch_np, fs, t0, fd, tabs, 3)
    print(json.dumps(res), flush=True)


def profile_post(args, torch):
    """--profile demod | image | coherence: the kernels around the beamformer.

    demod:     20 frames x 11 waves x 128 channels x 3072 int16 RF samples (fs 40 MHz,
               f0 5 MHz) -> IQ at fs/4 in FP16 (ustb_demodulate);
    demod_zero_phase: the same RF through the Python port's zero-phase demodulation
               (65 Hamming taps forward and backward, D = floor(fs / 4 f0) = 2;
               ustb_demodulate_filtfilt);
    image:     the diverging-wave sector image (256 azimuths x 512 depths) -> 512 x 512
               log-compressed Cartesian image (ustb_scan_convert);
    coherence: its 64-channel cube (dimension.transmit) -> phase, generalized and
               plain coherence factors over the channels;
    capon:     the same cube -> Capon minimum variance (32-element subarrays, +-1.5
               wavelengths of depth averaging, 1 % diagonal loading)."""
    from ustb_gb300 import fast, image, postprocess, preprocess, synth
    from ustb_gb300.das import channel_tensor
    from ustb_gb300.enums import Precision

    dev = torch.device("cuda", 0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    out = {"profile": args.profile}
    if args.profile in ("demod", "demod_zero_phase"):
        g = torch.Generator(device=dev).manual_seed(7)
        rf = (torch.randn((20, 11, 128, 3072), generator=g, device=dev) * 3000).to(torch.int16)
        fs, fc = 40e6, 5e6
        if args.profile == "demod":
            taps = preprocess.lowpass_taps(fc, fs)
            D, _ = preprocess.decimation_factor(fs, 2 * fc)
            fn = lambda: preprocess.demodulate(rf, fs, 0.0, fc, taps, D, Precision.fp16, 1 / 3000)
        else:
            taps = preprocess.python_port_taps(fc, fs, rf.shape[-1])
            D = max(1, int(np.floor(fs / (4 * fc))))
            fn = lambda: preprocess.demodulate(rf, fs, 0.0, fc, taps, D, Precision.fp16, 1 / 3000, zero_phase=True)
            L, M, n_tr = rf.shape[-1], len(taps), rf.numel() // rf.shape[-1]
            # filtfilt at the kept samples is one FIR with the 2M - 1 taps of b's
            # autocorrelation: 4 FLOP per tap and kept sample (real tap, complex sample)
            out.update(flop=int(n_tr * (-(-L // D)) * (2 * M - 1) * 4))
        out.update(samples=int(rf.numel()), ntaps=int(len(taps)), decimation=D,
                   bytes=int(rf.numel() * 2 + (rf.numel() // D) * 4))
    else:
        wl = synth.config_dw_sector(device=dev)
        das = build_das(wl)
        geom = das.fast_geometry(dev)
        ch = channel_tensor(wl.channel_data.data, dev)
        st = fast.convert_channels(ch, Precision.fp16)
        o = fast.das_fast(st, Precision.fp16, True, geom, int(wl.dimension), L=ch.shape[-1], epilogue=True)
        torch.cuda.synchronize()
        if args.profile == "image":
            img = o["das"][0]
            fn = lambda: image.scan_convert(img, wl.scan)
            out.update(pixels_in=int(img.numel()), pixels_out=512 * 512)
        elif args.profile == "capon":
            cube = o["cube"]
            cd = wl.channel_data
            rxa = das.receive_apodization.aperture_apodization(cd.probe, wl.scan)
            apod = torch.from_numpy(np.ascontiguousarray(rxa.T).astype(np.float32)).to(dev)
            lam = cd.sound_speed / wl.info["f0"]
            K = postprocess.capon_k_samples(wl.scan.depth_axis, lam, 1.5)
            nz, nx = wl.scan.depth_axis.size, wl.scan.azimuth_axis.size
            fn = lambda: postprocess.capon_minimum_variance(cube, apod, nz, nx, L_elements=32, K_samples=K,
                                                            regCoef=1e-2)
            out.update(pixels=nz * nx, channels=int(cube.shape[2]), L_elements=32, K_samples=K)
        else:
            cube = o["cube"]
            from ustb_gb300.enums import Dimension

            fn = lambda: (postprocess.phase_coherence_factor(cube), postprocess.generalized_coherence_factor(cube),
                          postprocess.coherence_factor(cube, Dimension.receive))
            out.update(cube_bytes=int(cube.numel() * 8))
    for _ in range(args.warmup):
        fn()
    out["ms"] = [round(t, 4) for t in cuda_time(fn, args.steps, flush, stream, torch)]
    print(json.dumps(out), flush=True)


def profile_small(args, torch):
    """--profile small: the HBM-bound helper kernels at sizes above L2.
    convert:  the headline channel data, complex64 -> FP16 (78.6 MB in, 39.3 MB out);
    phase:    the per-pixel phase on 200 frames of a 131,072-pixel complex image (210 MB);
    fir:      the sDMAS band-pass along depth of 200 frames x 256 columns x 512 depths
              (105 MB), Kaiser band-pass 3-5 MHz (0.5 MHz transitions) at 48 MHz."""
    from ustb_gb300 import fast, kernels, postprocess
    from ustb_gb300.enums import Precision

    dev = torch.device("cuda", 0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    _, _, ch = make_headline(dev)
    g = torch.Generator(device=dev).manual_seed(3)
    img = torch.randn((200, 131072), dtype=torch.complex64, device=dev, generator=g)  # (F, P)
    ph = torch.exp(1j * torch.rand(131072, device=dev, generator=g) * 6.28).to(torch.complex64)
    col = torch.randn((200 * 256, 512), device=dev, generator=g)
    taps = postprocess.bandpass_taps([2.5e6, 3e6, 5e6, 5.5e6], 48e6)
    steps = {"convert": lambda: fast.convert_channels(ch, Precision.fp16),
             "phase": lambda: kernels.apply_pixel_phase(img, ph),
             "fir": lambda: postprocess.fir_depth(col, taps)}
    out = {"profile": "small", "bytes": {"convert": int(ch.numel() * 8 + ch.numel() * 4),
                                         "phase": int(img.numel() * 16 + ph.numel() * 8),
                                         "fir": int(col.numel() * 8)}, "fir_taps": int(len(taps))}
    for name, fn in steps.items():
        for _ in range(args.warmup):
            fn()
        out[name + "_ms"] = [round(t, 4) for t in cuda_time(fn, args.steps, flush, stream, torch)]
    print(json.dumps(out), flush=True)


def profile_ensemble(args, torch):
    """--profile ensemble: the persistent batch kernel on a 20-frame slice of the
    high-frame-rate ensemble (20 frames x 11 plane waves x 128 channels x 1536 int16 I/Q
    samples, 256 x 512 pixels, dimension both): per run the int16 -> FP16 conversion,
    the entries pass and one persistent launch over all (frame, tile) items."""
    from ustb_gb300 import synth
    from ustb_gb300.ensemble import Ensemble
    from ustb_gb300.enums import Precision

    dev = torch.device("cuda", 0)
    wl = synth.config_hfr_ensemble(device=dev, frames=20)
    das = build_das(wl)
    x = wl.info["int16"]
    F, W, N, L, _ = x.shape
    ens = Ensemble(das.fast_geometry(dev), F, L, wl.dimension, Precision.fp16, wl.info["scale"], graph=False)
    ens.run(x)
    fn = lambda: ens.run()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        fn()
    out = {"profile": "ensemble", "frames": F, "units": int(wl.scan.N_pixels) * N * W * F,
           "ms": [round(t, 4) for t in cuda_time(fn, args.steps, flush, torch.cuda.current_stream(dev), torch)]}
    torch.cuda.synchronize()
    out["window_overflow"] = int(ens.flags())
    print(json.dumps(out), flush=True)


def main_profile(args):
    """A short run for ncu: the fast kernel, then the das_c-exact table kernel, on one
    workload, ``--steps`` launches each after ``--warmup`` warm-up launches each."""
    import torch

    if args.profile in ("demod", "demod_zero_phase", "image", "coherence", "capon"):
        return profile_post(args, torch)
    if args.profile == "ensemble":
        return profile_ensemble(args, torch)
    if args.profile == "small":
        return profile_small(args, torch)

    from ustb_gb300 import fast, geometry, kernels, synth
    from ustb_gb300.enums import Precision

    dev = torch.device("cuda", 0)
    if args.profile == "headline":
        wl, das, ch = make_headline(dev)
    else:
        from ustb_gb300.das import channel_tensor

        wl = synth.CONFIGS[args.profile](device=dev)
        das = build_das(wl)
        ch = channel_tensor(wl.channel_data.data, dev)
    cd = wl.channel_data
    prec = Precision[args.storage]
    cplx = ch.is_complex()
    epi = wl.epilogue is not None
    geom = das.fast_geometry(dev, stage_shape=args.stage_shape)
    st = fast.convert_channels(ch, prec)
    flags = torch.zeros(1, dtype=torch.int32, device=dev)
    L = ch.shape[-1]

    def fast_step():
        fast.das_fast(st, prec, cplx, geom, int(wl.dimension), L=L, epilogue=epi, cube=not epi, flags=flags,
                      check=False)

    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).to(dev)
    txa = das.transmit_apodization.wave_apodization(cd.sequence, wl.scan).astype(np.float32)
    txd = geometry.transmit_delay(cd.sequence, wl.scan).astype(np.float32)
    rxd, rxa = geometry.receive_tables_device(cd.probe, wl.scan, cd.sound_speed, das.receive_apodization,
                                              device=dev)
    fs, t0, fd = (float(np.float32(cd.sampling_frequency)), float(np.float32(cd.initial_time)),
                  float(np.float32(cd.modulation_frequency)))
    d_txa, d_txd = T(txa), T(txd)

    def table_step():
        kernels.das_table_f32(ch, fs, t0, d_txa, rxa, d_txd, rxd, fd, int(wl.dimension))

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    out = {"profile": args.profile, "storage": args.storage, "units": wl.units}
    for name, fn in (("fast", fast_step), ("table", table_step)):
        for _ in range(args.warmup):
            fn()
        out[name + "_ms"] = [round(t, 4) for t in cuda_time(fn, args.steps, flush, stream, torch)]
    torch.cuda.synchronize()
    out["window_overflow"] = int(flags.item())
    print(json.dumps(out), flush=True)


def main_reference(args, rank, world):
    import torch

    if rank != 0:
        return
    device = torch.device("cuda", 0) if torch.cuda.is_available() else torch.device("cpu")
    from ustb_gb300 import kernels

    wl, das, ch = make_headline(device)  # inputs are generated on the GPU when there is one
    cd = wl.channel_data
    tabs = das.tables()
    ch_np = kernels.to_matlab_order(ch).cpu().numpy()
    fs, t0, fd = (float(np.float32(cd.sampling_frequency)), float(np.float32(cd.initial_time)),
                  float(np.float32(cd.modulation_frequency)))
    for _ in range(min(args.warmup, 1)):
        cpu_reference(ch_np, fs, t0, fd, tabs, 3, target_s=2.0)
    cb = cpu_reference(ch_np, fs, t0, fd, tabs, 3, target_s=max(2.0, 60.0 / max(args.steps, 1)),
                       steps=args.steps)
    val = cb["value"]
    units = wl.units
    res = {"metric": METRIC, "value": round(val, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(units / (val * 1e9) * 1e3, 2), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
           "config": {"workload": "iq_cpwc: 1024 complex64 samples x 128 channels x 75 plane waves, "
                                  "400x400 pixels, dimension both", "units_per_step": units},
           "cpu_baseline": cb,
           "e2e": {"value": round(val, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if device.type == "cuda":
        # the reference's own GPU point beside it: das_cuda on the same frame
        dc = das_cuda_reference(ch_np, fs, t0, fd, tabs)
        if dc is not None:
            from oracle import oracle as O

            out = dc.pop("output")
            sel = np.arange(0, tabs[0].shape[0], 97)
            ref = O.das_f32(ch_np, fs, t0, tabs[0][sel], tabs[1][sel], tabs[2][sel], tabs[3][sel], fd, 3)
            dc["rel_l2_vs_das_c_port"] = float(f"{np.linalg.norm(out[sel] - ref) / np.linalg.norm(ref):.3g}")
            res["reference_gpu_das_cuda"] = dc
        else:
            res["reference_gpu_das_cuda"] = {"unavailable": "das_cuda was not built on this machine"}
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
