"""Continuous-batching beamforming server on one GPU.

Requests of different probes, scans and sizes arrive over time.  The server
keeps each shape's geometry (``FastGeometry``: element and pixel positions,
transmit events, tile map) resident on the device, admits arrived requests
while their buffers fit an HBM budget, and merges everything admitted into the
next persistent launch (``ustb_das_fast_batch_ex``).  Up to ``max_inflight``
launches overlap on the device: requests that arrive while a batch runs join
the next one instead of waiting for the GPU to drain.  A request above
``large_units`` runs in a launch of its own on a separate stream with at most
``SMs - reserve_sms`` persistent CTAs, so small requests keep being served on
the reserved SMs while it runs instead of queueing behind it.  Latency is
measured from arrival to the completion event of the request's batch.

The reference has no serving layer: midprocess.das beamforms one dataset per
call (+midprocess/das.m:77-317).
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional

import numpy as np
import torch

from . import fast
from .enums import Precision


@dataclass
class Job:
    """A request in flight: channel data (device, storage type), its shape key and frames."""
    key: str
    ch: torch.Tensor
    precision: Precision
    is_complex: bool
    F: int
    L: int
    dimension: int
    epilogue: bool = False
    arrival: float = 0.0
    admitted: float = 0.0
    done: float = 0.0
    outputs: Dict[str, torch.Tensor] = field(default_factory=dict)
    reserved: int = 0
    callback: Optional[Callable[["Job"], None]] = None

    @property
    def latency(self) -> float:
        return self.done - self.arrival


class Server:
    """Event-loop server: ``submit`` jobs, call ``poll`` (or ``run``) to make progress."""

    def __init__(self, device, hbm_budget_bytes: float = 150e9, max_batch: int = 32, max_inflight: int = 3,
                 large_units: float = 2e9, reserve_sms: Optional[int] = None, large_queue: int = 2):
        self.device = torch.device(device)
        # requests with more pixel-channel-wave units than this launch on their own, on
        # their own stream and with SMs left over for the small requests
        self.large_units = large_units
        sms = (torch.cuda.get_device_properties(self.device).multi_processor_count
               if self.device.type == "cuda" else 152)
        # SMs kept free of large launches for small requests: 0 favours throughput (the
        # large launch uses every SM), a sixth of the SMs cuts small requests' latency
        self.reserve_sms = 0 if reserve_sms is None else max(0, int(reserve_sms))
        self.large_ctas = max(1, sms - self.reserve_sms)
        self.pending_large: collections.deque = collections.deque()
        self.large_stream = torch.cuda.Stream(self.device)
        # large launches queued back to back on their stream (no host gap between them)
        self.large_queue = max(1, int(large_queue))
        self.large_inflight: List = []
        self.budget = int(hbm_budget_bytes)
        self.used = 0
        self.max_batch = max_batch
        self.max_inflight = max_inflight
        self.plans: Dict[str, fast.FastGeometry] = {}
        self.pending: collections.deque = collections.deque()
        self.inflight: List = []  # (event, jobs, requests, scratch)
        self.completed: List[Job] = []
        self.streams = [torch.cuda.Stream(self.device) for _ in range(max_inflight)]
        self._next_stream = 0
        self.launches = 0

    # -- plans -------------------------------------------------------------------
    def add_plan(self, key: str, geom: fast.FastGeometry) -> None:
        self.plans[key] = geom

    # -- requests ----------------------------------------------------------------
    def _bytes(self, job: Job) -> int:
        """Device bytes a job holds while in flight: channel data, outputs and the
        interpolation entries its launch builds."""
        g = self.plans[job.key]
        out = g.P * job.F * (8 if job.is_complex else 4)
        if job.dimension in (0, 2):
            out *= g.N
        if job.dimension in (0, 1):
            out *= g.W
        ent = fast.entry_bytes(job.L, g.N, g.W, job.F, job.is_complex)
        return int(job.ch.numel() * job.ch.element_size() + out + ent)

    def submit(self, job: Job, now: Optional[float] = None) -> Job:
        if job.key not in self.plans:
            raise KeyError(f"no plan for shape {job.key!r}: add_plan first")
        job.arrival = time.perf_counter() if now is None else now
        job.reserved = self._bytes(job)
        if job.reserved > self.budget:
            raise MemoryError(f"request needs {job.reserved} bytes, budget is {self.budget}")
        (self.pending_large if self._units(job) > self.large_units else self.pending).append(job)
        return job

    def _units(self, job: Job) -> int:
        g = self.plans[job.key]
        return g.P * g.N * g.W * job.F

    def _start(self, batch: List[Job], stream, max_ctas: int):
        t = time.perf_counter()
        reqs = []
        with torch.cuda.stream(stream):
            for job in batch:
                job.admitted = t
                cube = not job.epilogue
                r = fast.Request(job.ch, job.precision, job.is_complex, self.plans[job.key], job.dimension,
                                 F=job.F, L=job.L, epilogue=job.epilogue, cube=cube)
                job.outputs = r.outputs
                reqs.append(r)
            scratch = fast.das_fast_batch(reqs, stream=stream, max_ctas=max_ctas)
            ev = torch.cuda.Event()
            ev.record(stream)
        self.launches += 1
        return (ev, batch, reqs, scratch)

    @staticmethod
    def _variant(job: Job):
        """Jobs of one kernel variant share a persistent launch."""
        return (int(job.dimension), bool(job.is_complex), bool(job.epilogue))

    def _launch(self) -> None:
        """Admit pending small jobs in arrival order, as many as fit the budget and the
        batch size, into one launch of the first job's kernel variant (other variants
        keep their place and go to the next stream)."""
        batch: List[Job] = []
        skipped = collections.deque()
        want = self._variant(self.pending[0]) if self.pending else None
        while self.pending and len(batch) < self.max_batch:
            job = self.pending.popleft()
            if self._variant(job) != want:
                skipped.append(job)
                continue
            if self.used + job.reserved > self.budget:
                skipped.append(job)
                break
            self.used += job.reserved
            batch.append(job)
        while skipped:
            self.pending.appendleft(skipped.pop())
        if not batch:
            return
        stream = self.streams[self._next_stream]
        self._next_stream = (self._next_stream + 1) % len(self.streams)
        self.inflight.append(self._start(batch, stream, 0))

    def _launch_large(self) -> None:
        job = self.pending_large[0]
        if self.used + job.reserved > self.budget:
            return
        self.pending_large.popleft()
        self.used += job.reserved
        self.large_inflight.append(self._start([job], self.large_stream, self.large_ctas))

    def _retire(self, entry) -> int:
        ev, batch, reqs, scratch = entry
        t = time.perf_counter()
        flags = int(scratch[0].item()) & 0xFFFFFFFF
        for job in batch:
            job.done = t
            self.used -= job.reserved
            if flags & fast.FLAG_WINDOW_OVERFLOW:
                job.outputs["error"] = "window overflow"
            self.completed.append(job)
            if job.callback:
                job.callback(job)
        return len(batch)

    def poll(self) -> int:
        """Retire finished batches and launch new ones.  Returns jobs completed now."""
        n = 0
        still = []
        for entry in self.inflight:
            if entry[0].query():
                n += self._retire(entry)
            else:
                still.append(entry)
        self.inflight = still
        while self.large_inflight and self.large_inflight[0][0].query():
            n += self._retire(self.large_inflight.pop(0))
        while self.pending_large and len(self.large_inflight) < self.large_queue:
            before = len(self.pending_large)
            self._launch_large()
            if len(self.pending_large) == before:
                break
        while self.pending and len(self.inflight) < self.max_inflight:
            before = len(self.pending)
            self._launch()
            if len(self.pending) == before:
                break
        return n

    def busy(self) -> bool:
        return bool(self.pending or self.pending_large or self.inflight or self.large_inflight)

    def drain(self) -> None:
        while self.busy():
            self.poll()

    # -- replay a timed arrival stream -------------------------------------------
    def run(self, arrivals: List[float], make_job: Callable[[int], Job]) -> List[Job]:
        """Submit job i at time start + arrivals[i] (seconds) and serve until all are done."""
        jobs = [make_job(i) for i in range(len(arrivals))]
        start = time.perf_counter()
        i = 0
        while i < len(jobs) or self.busy():
            now = time.perf_counter() - start
            while i < len(jobs) and arrivals[i] <= now:
                self.submit(jobs[i], start + arrivals[i])
                i += 1
            self.poll()
        return jobs


def poisson_arrivals(n: int, rate_hz: float, seed: int) -> np.ndarray:
    """Arrival times (s) of a Poisson stream of ``n`` requests."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_hz, n))


def latency_stats(jobs: List[Job], per_key: bool = False) -> Dict[str, float]:
    lat = np.array([j.latency for j in jobs]) * 1e3
    frames = sum(j.F for j in jobs)
    span = max(j.done for j in jobs) - min(j.arrival for j in jobs)
    out = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "mean_ms": float(lat.mean()), "frames": int(frames), "seconds": float(span),
           "frames_per_s": float(frames / span)}
    if per_key:
        keys = sorted({j.key for j in jobs})
        out["per_kind"] = {k: {"p50_ms": round(float(np.percentile([j.latency * 1e3 for j in jobs if j.key == k], 50)), 3),
                               "p99_ms": round(float(np.percentile([j.latency * 1e3 for j in jobs if j.key == k], 99)), 3)}
                           for k in keys}
    return out
