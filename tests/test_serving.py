"""Serving logic on the host: arrivals, admission against the HBM budget,
batching, latency accounting (the device launch is faked; no GPU needed)."""
import numpy as np
import pytest

from ustb_gb300 import serving


class FakeEvent:
    def __init__(self):
        self.done = False

    def record(self, stream=None):
        pass

    def query(self):
        return self.done


class FakeTensor:
    def __init__(self, nbytes):
        self._n = nbytes

    def numel(self):
        return self._n

    def element_size(self):
        return 1

    def __getitem__(self, i):
        class V:
            def item(self):
                return 0
        return V()


class FakeGeom:
    P, N, W = 100, 4, 2


@pytest.fixture
def fake_server(monkeypatch):
    events = []

    class FakeRequest:
        def __init__(self, *a, **k):
            self.outputs = {"cube": None}

    launched = []

    def fake_batch(reqs, scratch=None, stream=None, max_ctas=0):
        launched.append((len(reqs), max_ctas))
        return FakeTensor(8)

    def fake_event():
        e = FakeEvent()
        events.append(e)
        return e

    monkeypatch.setattr(serving.fast, "Request", FakeRequest)
    monkeypatch.setattr(serving.fast, "das_fast_batch", fake_batch)
    monkeypatch.setattr(serving.torch.cuda, "Event", fake_event)
    monkeypatch.setattr(serving.torch.cuda, "Stream", lambda dev: None)

    class Ctx:
        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

    monkeypatch.setattr(serving.torch.cuda, "stream", lambda s: Ctx())
    srv = serving.Server("cpu", hbm_budget_bytes=10_000, max_batch=3, max_inflight=2, large_queue=2)
    srv.add_plan("a", FakeGeom())
    srv.launched = launched
    return srv, events


def job(nbytes, F=1):
    return serving.Job("a", FakeTensor(nbytes), 1, True, F, 16, 3)


def test_poisson_arrivals_seeded():
    a = serving.poisson_arrivals(1000, 50.0, seed=7)
    b = serving.poisson_arrivals(1000, 50.0, seed=7)
    assert np.array_equal(a, b) and np.all(np.diff(a) > 0)
    assert abs(len(a) / a[-1] - 50.0) < 5.0


def test_batches_merge_arrived_requests_and_respect_inflight_limit(fake_server):
    srv, events = fake_server
    srv.budget = 30_000  # 7 jobs x (1000 B channels + 800 B output + 2048 B entries) fit
    for _ in range(7):
        srv.submit(job(1000))
    srv.poll()
    # two launches in flight of at most 3 requests each; one request waits
    assert srv.launches == 2 and len(srv.pending) == 1
    events[0].done = True
    assert srv.poll() == 3
    assert srv.launches == 3 and not srv.pending
    for e in events:
        e.done = True
    srv.drain()
    assert len(srv.completed) == 7 and srv.used == 0


def test_admission_waits_for_budget(fake_server):
    srv, events = fake_server
    srv.budget = 10_000  # one 6800-byte job at a time
    big = job(6000)
    srv.submit(big)
    srv.submit(job(6000))  # fits alone, not together with the first
    srv.poll()
    assert srv.launches == 1 and len(srv.pending) == 1
    events[0].done = True
    srv.poll()
    assert srv.launches == 2
    with pytest.raises(MemoryError):
        srv.submit(job(20_000))


def test_latency_stats():
    js = []
    for i in range(10):
        j = serving.Job("a", None, 1, True, 2, 16, 3)
        j.arrival, j.done = float(i), float(i) + 0.001 * (i + 1)
        js.append(j)
    st = serving.latency_stats(js)
    assert st["frames"] == 20
    assert st["p50_ms"] == pytest.approx(5.5)
    assert st["frames_per_s"] == pytest.approx(20 / 9.01)


def test_one_launch_per_kernel_variant(fake_server):
    srv, events = fake_server
    srv.budget = 1e9
    srv.max_inflight = 3
    kinds = [3, 2, 3, 3, 2]  # dimension both / transmit interleaved
    for d in kinds:
        srv.submit(serving.Job("a", FakeTensor(100), 1, True, 1, 16, d))
    srv.poll()
    # the three dimension.both jobs share one launch, the two transmit jobs another
    assert sorted(n for n, _ in srv.launched) == [2, 3] and not srv.pending


def test_large_requests_launch_alone(fake_server):
    srv, events = fake_server
    srv.budget = 1e9
    srv.large_units = 500  # FakeGeom: 100 px x 4 ch x 2 waves = 800 units per frame
    srv.submit(serving.Job("a", FakeTensor(100), 1, True, 1, 16, 3))  # large (800)
    small = FakeGeom()
    small.P = 10
    srv.add_plan("s", small)
    for _ in range(3):
        srv.submit(serving.Job("s", FakeTensor(100), 1, True, 1, 16, 3))  # 80 units each
    srv.poll()
    # the large job went alone, the three small ones together in the second launch
    assert srv.launches == 2 and not srv.pending and not srv.pending_large
    # the large launch runs with SMs - reserve CTAs (every SM by default)
    assert srv.launched[0] == (1, srv.large_ctas) and srv.launched[1] == (3, 0)
    assert srv.large_ctas == 152
    lat = serving.Server("cpu", reserve_sms=25)
    assert lat.large_ctas == 127


def test_small_requests_flow_past_a_running_large_one(fake_server):
    srv, events = fake_server
    srv.budget = 1e9
    srv.large_units = 500
    small = FakeGeom()
    small.P = 10
    srv.add_plan("s", small)
    srv.large_queue = 1
    srv.submit(serving.Job("a", FakeTensor(100), 1, True, 1, 16, 3))  # large, in flight below
    srv.submit(serving.Job("a", FakeTensor(100), 1, True, 1, 16, 3))  # a second large one waits
    srv.poll()
    assert len(srv.large_inflight) == 1 and len(srv.pending_large) == 1
    # small requests arriving while the large launch runs are served without waiting for it
    for _ in range(5):
        srv.submit(serving.Job("s", FakeTensor(100), 1, True, 1, 16, 3))
    srv.poll()
    assert srv.launches == 3 and len(srv.pending) == 0  # 3 + 2 small jobs in two launches
    events[1].done = events[2].done = True
    assert srv.poll() == 5
    assert len(srv.pending_large) == 1  # the first large one has not finished
    events[0].done = True
    assert srv.poll() == 1 and not srv.pending_large  # its successor starts at once
    for e in events:
        e.done = True
    srv.drain()
    assert len(srv.completed) == 7 and srv.used == 0
