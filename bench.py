"""Benchmark: delay-and-sum throughput on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step" = one beamformed frame of it): plain DAS, IQ coherent
plane-wave compounding, FP32 — 128-element linear array (pitch 0.3 mm,
f0 = 5 MHz, fs = 20 MHz), 1024 complex64 samples x 128 channels x 75 plane
waves (-16..16 deg), 400 x 400 pixels, Tukey-25% receive apodization at F# 1.7,
transmit apodization from the plane-wave angle, dimension 'both'.  Seeded
synthetic channel data (point targets + speckle with two cysts) stands in for
the reference's datasets.

Prints one JSON line (rank 0).  ``value`` is G pixel.channel.wave/s with the
inputs resident in HBM; ``e2e`` is the same metric through the host-pointer
C-ABI call (copies in and out inside the timed region).  ``--impl reference``
times the reference's CPU implementation of the same path (the oracle port of
das_c; the reference's own das_c build is x86-only) on the host cores.
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
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "beamformed G pixel·channel·wave/s; serving frames/s + p50/p99 ms vs plain DAS"
UNIT = "G pixel·channel·wave/s"
FLOP_PER_UNIT_IQ = 22  # algorithmic FP32 FLOP per IQ unit (+2 MUFU sincos)
FP32_LANES_PER_SM = 128


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

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
# workload
# ---------------------------------------------------------------------------
def make_workload(device):
    from ustb_gb300 import synth
    from ustb_gb300.das import DAS, channel_tensor
    from ustb_gb300.enums import Window
    from ustb_gb300.geometry import Apodization

    wl = synth.config_iq_cpwc(seed=2, device=device)
    das = DAS()
    das.channel_data = wl.channel_data
    das.scan = wl.scan
    das.receive_apodization = Apodization(window=Window.tukey25, f_number=1.7)
    das.transmit_apodization = Apodization(window=Window.tukey25, f_number=1.7)
    tx_apo, rx_apo, tx_delay, rx_delay = das.tables()
    ch = channel_tensor(wl.channel_data.data, device)
    return wl, das, ch, (tx_apo, rx_apo, tx_delay, rx_delay)


def active_units(tx_apo, rx_apo, F):
    ntx = (tx_apo != 0).sum(axis=1).astype(np.int64)
    nrx = (rx_apo != 0).sum(axis=1).astype(np.int64)
    return int((ntx * nrx).sum()) * F


# ---------------------------------------------------------------------------
# CPU (reference) timing: the das_c port on the host cores
# ---------------------------------------------------------------------------
def cpu_reference(ch_np, fs, t0, fd, tabs, dim, target_s=12.0, steps=1):
    from oracle import oracle as O

    tx_apo, rx_apo, tx_delay, rx_delay = tabs
    P = tx_apo.shape[0]
    threads = os.cpu_count() or 1

    def run(stride):
        sel = np.arange(0, P, stride)
        t = time.perf_counter()
        O.das_f32(ch_np, fs, t0, tx_apo[sel], rx_apo[sel], tx_delay[sel], rx_delay[sel], fd, dim,
                  threads=threads)
        return time.perf_counter() - t, sel.size

    dt, n = run(200)  # calibration on 0.5 % of the pixels
    per_px = dt / max(n, 1)
    stride = max(1, int(math.ceil(P * per_px / target_s)))
    times = []
    for _ in range(max(1, steps)):
        dt, n = run(stride)
        times.append(dt)
    L, N, W, F = ch_np.shape
    units = n * N * W * F
    t = statistics.median(times)
    return {"value": units / t / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"every {stride}-th pixel ({n} of {P} pixels, all channels/waves), "
                      f"{t:.1f} s per pass, oracle/das_port.c oracle_das_f32 on {threads} threads"}


# ---------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.impl == "reference":
        return main_reference(args, rank, world)

    from ustb_gb300 import _lib, kernels

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    wl, das, ch, tabs = make_workload(dev)
    tx_apo, rx_apo, tx_delay, rx_delay = tabs
    cd = wl.channel_data
    P, N, W, F = wl.scan.N_pixels, cd.N_channels, cd.N_waves, cd.N_frames
    L = cd.N_samples
    units = P * N * W * F
    act = active_units(tx_apo, rx_apo, F)
    fs, t0, fd = float(np.float32(cd.sampling_frequency)), float(np.float32(cd.initial_time)), float(
        np.float32(cd.modulation_frequency))
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).to(dev)
    d_atx, d_arx, d_dtx, d_drx = T(tx_apo), T(rx_apo), T(tx_delay), T(rx_delay)
    phase = torch.from_numpy(das.pixel_phase().astype(np.complex64)).to(dev)
    out = torch.empty(kernels.out_shape_abi(P, N, W, F, 3), dtype=torch.complex64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        kernels.das_table_f32(ch, fs, t0, d_atx, d_arx, d_dtx, d_drx, fd, 3, out=out)
        if ev is not None:
            ev[1].record(stream)
        kernels.apply_pixel_phase(out, phase)
        if ev is not None:
            ev[2].record(stream)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize(dev)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            flush.zero_()  # L2 flush between steps, outside the timed events
            step(evs[i])
        torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    step_ms = [e[0].elapsed_time(e[2]) for e in evs]
    kern_ms = [e[0].elapsed_time(e[1]) for e in evs]
    ms = sum(step_ms) / len(step_ms)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = units * world / (ms * 1e-3) / 1e9

    # end to end through the host-pointer C-ABI (pinned host buffers)
    h_ch = torch.empty(ch.shape, dtype=ch.dtype, pin_memory=True)
    h_ch.copy_(ch)
    h_tab = [torch.from_numpy(np.ascontiguousarray(a.T)).pin_memory() for a in tabs]
    h_out = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)

    def e2e_step():
        _lib.call("ustb_das_table_f32_host", h_ch.data_ptr(), 1, L, N, W, F, fs, t0,
                  h_tab[0].data_ptr(), h_tab[1].data_ptr(), h_tab[2].data_ptr(), h_tab[3].data_ptr(),
                  P, fd, 3, h_out.data_ptr(), local)

    for _ in range(2):
        e2e_step()
    e2e_steps = max(3, min(args.steps, 10))
    t_e = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_ms = (time.perf_counter() - t_e) * 1e3 / e2e_steps
    h2d = h_ch.numel() * h_ch.element_size() + sum(t.numel() * 4 for t in h_tab)
    d2h = h_out.numel() * h_out.element_size()

    if rank != 0:
        return
    peaks = measured_peaks()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = sms * FP32_LANES_PER_SM * 2 * sm_max * 1e6 / 1e12  # TFLOP/s
    kms = sum(kern_ms) / len(kern_ms)
    achieved = FLOP_PER_UNIT_IQ * act / (kms * 1e-3) / 1e12
    alg_bytes = (ch.numel() * 8 + 4 * 4 * P * 0 + (2 * P * W + 2 * P * N) * 4 + P * F * 8)
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    res = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "iq_cpwc_fp32: 1024 samples x 128 ch x 75 plane waves, 400x400 px, "
                               "dimension both, das_c-exact table kernel",
                   "units_per_step": units, "active_units_per_step": act,
                   "frames_per_s": round(1e3 / ms * world, 2), "l2": "flushed between steps (256 MB)",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "fp32", "achieved": round(achieved, 3), "peak": round(fp32_peak, 2),
                     "unit": "TFLOP/s", "frac": round(achieved / fp32_peak, 4), "traffic": None,
                     "kernel": "das_table_kernel<both, complex, FC=1>",
                     "kernel_ms": round(kms, 4),
                     "peak_source": f"nominal {sms} SMs x 128 FP32 lanes x 2 x sm_max_mhz {sm_max:.0f} "
                                    "(MEASURED_PEAKS.json has no FP32 figure)",
                     "flop_per_unit": FLOP_PER_UNIT_IQ, "mufu_per_unit": 2,
                     "algorithmic_bytes": alg_bytes,
                     "hbm_frac_of_measured": round(alg_bytes / (kms * 1e-3) / 1e9 / hbm, 4)},
        "e2e": {"value": round(units / (e2e_ms * 1e-3) / 1e9, 3), "unit": UNIT,
                "ms_per_step": round(e2e_ms, 3), "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "call": "ustb_das_table_f32_host"},
        "gpu_launches": 2 * args.steps,
        "clocks": clk.summary(),
    }
    if world == 1 and not args.no_cpu_baseline:
        ch_np = kernels.to_matlab_order(ch).cpu().numpy()
        res["cpu_baseline"] = cpu_reference(ch_np, fs, t0, fd, tabs, 3)
    print(json.dumps(res), flush=True)


def main_reference(args, rank, world):
    import torch

    if rank != 0:
        return
    wl, das, ch, tabs = make_workload("cpu")
    from ustb_gb300 import kernels

    cd = wl.channel_data
    ch_np = kernels.to_matlab_order(ch).numpy()
    fs, t0, fd = float(np.float32(cd.sampling_frequency)), float(np.float32(cd.initial_time)), float(
        np.float32(cd.modulation_frequency))
    for _ in range(min(args.warmup, 1)):
        cpu_reference(ch_np, fs, t0, fd, tabs, 3, target_s=2.0)
    cb = cpu_reference(ch_np, fs, t0, fd, tabs, 3, target_s=max(2.0, 60.0 / max(args.steps, 1)),
                       steps=args.steps)
    val = cb["value"]
    units = wl.units
    res = {"metric": METRIC, "value": round(val, 4), "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(units / (val * 1e9) * 1e3, 2), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "impl": "reference",
           "config": {"workload": "iq_cpwc_fp32: 1024 samples x 128 ch x 75 plane waves, 400x400 px, "
                                  "dimension both", "units_per_step": units},
           "cpu_baseline": cb,
           "e2e": {"value": round(val, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
