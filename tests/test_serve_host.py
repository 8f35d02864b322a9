"""Scheduling of the propagation service on the host (no GPU): admission against
the memory budget, first fit, arrivals, concurrency limit, rejection of requests
above the budget, latency and throughput bookkeeping."""
import threading
import time

import numpy as np

from richmol_gb300 import serve


class FakeJob:
    """A job that holds ``nbytes`` for ``seconds`` and records the concurrency."""
    lock = threading.Lock()
    active = 0
    peak = 0
    held = 0
    peak_held = 0

    def __init__(self, req):
        self.req = req
        self.nbytes = int(req.abc[0])
        self.seconds = float(req.abc[1])
        self.state_steps = 0

    def device_bytes(self):
        return self.nbytes

    def run(self):
        with FakeJob.lock:
            FakeJob.active += 1
            FakeJob.held += self.nbytes
            FakeJob.peak = max(FakeJob.peak, FakeJob.active)
            FakeJob.peak_held = max(FakeJob.peak_held, FakeJob.held)
        time.sleep(self.seconds)
        with FakeJob.lock:
            FakeJob.active -= 1
            FakeJob.held -= self.nbytes
        self.state_steps = 10
        return ("done", self.req.rid)


def reset():
    FakeJob.active = FakeJob.peak = FakeJob.held = FakeJob.peak_held = 0


def req(rid, arrival, nbytes, seconds):
    return serve.Request(rid, arrival, (nbytes, seconds, 0.0), 10, np.eye(3), (0, 0, 0, np.array([0, 0, 1.0])), 1.0)


def test_budget_is_never_exceeded_and_all_requests_finish():
    reset()
    reqs = [req(i, 0.0, 40, 0.05) for i in range(10)]
    srv = serve.Server(budget_bytes=100, max_active=8, make_job=FakeJob, device=None)
    results, stats = srv.serve(reqs, realtime=False)
    assert sorted(results) == list(range(10))
    assert all(results[i] == ("done", i) for i in range(10))
    assert FakeJob.peak_held <= 100 and stats.peak_bytes <= 100
    assert FakeJob.peak == 2  # two 40-byte jobs fit in 100 bytes
    assert stats.state_steps == 100


def test_first_fit_admits_a_smaller_later_request():
    reset()
    # a large job holds 70 bytes; the next 60-byte request must wait, the 20-byte one runs at once
    reqs = [req(0, 0.0, 70, 0.3), req(1, 0.0, 60, 0.05), req(2, 0.0, 20, 0.05)]
    srv = serve.Server(budget_bytes=100, max_active=8, make_job=FakeJob, device=None)
    results, stats = srv.serve(reqs, realtime=False)
    assert stats.latencies[2] < stats.latencies[1]
    assert stats.latencies[1] >= 0.3 - 0.02  # admitted once the large job released its memory


def test_concurrency_limit():
    reset()
    reqs = [req(i, 0.0, 1, 0.05) for i in range(12)]
    srv = serve.Server(budget_bytes=1000, max_active=3, make_job=FakeJob, device=None)
    results, stats = srv.serve(reqs, realtime=False)
    assert len(results) == 12 and FakeJob.peak <= 3 and stats.max_active <= 3


def test_arrivals_are_waited_for_and_latency_counts_from_arrival():
    reset()
    reqs = [req(0, 0.0, 1, 0.02), req(1, 0.25, 1, 0.02)]
    srv = serve.Server(budget_bytes=10, max_active=4, make_job=FakeJob, device=None)
    t0 = time.perf_counter()
    results, stats = srv.serve(reqs, realtime=True)
    assert time.perf_counter() - t0 >= 0.25
    assert stats.latencies[1] < 0.2  # measured from its own arrival, not from the start
    s = stats.summary()
    assert s["requests"] == 2 and s["p50_ms"] is not None and s["p99_ms"] >= s["p50_ms"]


def test_request_above_the_budget_is_rejected_not_run():
    reset()
    reqs = [req(0, 0.0, 500, 0.01), req(1, 0.0, 5, 0.01)]
    srv = serve.Server(budget_bytes=100, max_active=4, make_job=FakeJob, device=None)
    results, stats = srv.serve(reqs, realtime=False)
    assert isinstance(results[0], MemoryError)
    assert results[1] == ("done", 1)


def test_a_failing_job_is_reported_and_the_others_finish():
    reset()

    class Boom(FakeJob):
        def run(self):
            if self.req.rid == 1:
                raise RuntimeError("boom")
            return super().run()

    reqs = [req(i, 0.0, 1, 0.01) for i in range(4)]
    results, stats = serve.Server(budget_bytes=10, make_job=Boom, device=None).serve(reqs, realtime=False)
    assert isinstance(results[1], RuntimeError)
    assert all(results[i] == ("done", i) for i in (0, 2, 3))


def test_poisson_stream_and_request_distributions():
    rs = serve.poisson_requests(7, rate=200.0, duration=1.0, jmax_range=(10, 50))
    assert 150 < len(rs) < 250
    arr = np.array([r.arrival for r in rs])
    assert np.all(np.diff(arr) > 0) and arr[-1] < 1.0
    for r in rs:
        a, b, c = r.abc
        assert 0.05 <= c <= b <= a <= 5.0
        assert 10 <= r.jmax <= 50
        ev = np.linalg.eigvalsh(r.pol)
        assert np.allclose(r.pol, r.pol.T) and 5.0 - 1e-9 <= ev.min() and ev.max() <= 100.0 + 1e-9
        t0, fwhm, inten, d = r.pulse
        assert 0.05 <= fwhm <= 1.0 and 1e10 <= inten <= 1e13 and abs(np.linalg.norm(d) - 1) < 1e-12
        assert 0.5 <= r.temp <= 10.0


def test_device_bytes_bound_the_batch_allocation():
    r = serve.draw_request(np.random.default_rng(0), 0, 0.0, jmax_range=(12, 12))
    dim = serve.c1_dim(12)
    assert dim == sum((2 * J + 1) ** 2 for J in range(13))
    nvec = min(512, dim)
    assert serve.Job(r).device_bytes() > serve.batch_device_bytes(dim, nvec, 20)


class BuildJob(FakeJob):
    """A job with a host set-up (build) of ``abc[2]`` seconds; records when its
    build ran and when it was admitted (run started)."""
    events = []

    def build(self):
        t0 = time.perf_counter()
        time.sleep(float(self.req.abc[2]))
        BuildJob.events.append(("built", self.req.rid, t0, time.perf_counter()))

    def run(self):
        BuildJob.events.append(("run", self.req.rid, time.perf_counter(), None))
        return super().run()


def test_builds_start_at_arrival_and_overlap_running_jobs():
    """Host set-up off the latency path: the builder thread starts each build
    as its request arrives, while earlier jobs run; a job is admitted only
    once built."""
    reset()
    BuildJob.events = []
    reqs = [serve.Request(i, 0.05 * i, (10, 0.3, 0.1), 10, np.eye(3), (0, 0, 0, np.array([0, 0, 1.0])), 1.0)
            for i in range(4)]
    srv = serve.Server(budget_bytes=100, max_active=8, make_job=BuildJob, device=None)
    results, stats = srv.serve(reqs, realtime=True)
    assert all(results[i] == ("done", i) for i in range(4))
    built = {rid: (t0, t1) for kind, rid, t0, t1 in BuildJob.events if kind == "built"}
    run = {rid: t0 for kind, rid, t0, _ in BuildJob.events if kind == "run"}
    for rid in range(4):
        assert run[rid] >= built[rid][1]          # admitted once built
    # the second build ran while the first job was running (not after it)
    assert built[1][0] < run[0] + 0.3
