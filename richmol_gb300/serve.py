"""Propagation service: continuous batching of propagation requests on one GPU.

A request is a molecule, a pulse and a temperature; the answer is the
Boltzmann-weighted <cos^2 theta>(t) trace of its thermal ensemble (at most
``max_vectors`` eigenstates of H0), propagated with the batched path
(richmol_gb300.batch.Ensemble: complex64 mat-vec, FP64 Lanczos scalars and
state). This is the loop a user of the reference writes around
``TDSE.update`` (richmol/tdse.py:265-414, examples/ocs_alignment.py:70-100),
run for many requests at once:

* requests arrive over time (a Poisson stream in ``poisson_requests``);
* a job's host set-up (its molecule's factors) starts when its request
  arrives, on a builder thread, while admitted jobs run (``prebuild``);
* a request is admitted as soon as it has arrived, is built, and its device memory
  (``Job.device_bytes``: state, Krylov basis, operator) fits the HBM budget
  beside the jobs already running, first fit in arrival order;
* every admitted job owns its operator plans (private factor sources, so no
  two jobs share a field buffer), its CUDA stream and a host thread, so the
  kernels of different jobs overlap on the device while each thread waits on
  its own stream;
* memory returns to the budget when a job finishes, and waiting requests are
  admitted then.

A job's arithmetic is independent of the others' (its own buffers, its own
stream, deterministic reductions), so a result is the same alone and in the
mix. ``ServeStats`` reports p50/p99 latency (arrival to completion) and the
aggregate state-steps/s.
"""
import math
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import rot, workloads


@dataclass
class Request:
    """One propagation request: molecule (rotational constants A >= B >= C in
    cm^-1, Jmax, polarizability in au), pulse (centre ps, FWHM ps, intensity
    W/cm^2, unit polarisation vector), temperature K, time grid (ps)."""
    rid: int
    arrival: float
    abc: tuple
    jmax: int
    pol: np.ndarray
    pulse: tuple
    temp: float
    t_end: float = 5.0
    dt: float = 0.01
    max_vectors: int = 512


def draw_request(rng, rid, arrival, jmax_range=(10, 50), t_end=5.0, dt=0.01, max_vectors=512):
    """A request from the uneven-size distributions: A >= B >= C log-uniform in
    0.05-5 cm^-1, Jmax uniform in ``jmax_range``, polarizability Q diag(U(5, 100)) Q^T
    with Q a random rotation, pulse intensity log-uniform in 1e10-1e13 W/cm^2,
    FWHM uniform in 50-1000 fs, polarisation uniform on the sphere, centred at
    t_end / 2; temperature uniform in 0.5-10 K."""
    abc = tuple(sorted(np.exp(rng.uniform(math.log(0.05), math.log(5.0), 3)), reverse=True))
    jmax = int(rng.integers(jmax_range[0], jmax_range[1] + 1))
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    pol = q @ np.diag(rng.uniform(5.0, 100.0, 3)) @ q.T
    pol = 0.5 * (pol + pol.T)
    inten = float(np.exp(rng.uniform(math.log(1e10), math.log(1e13))))
    fwhm = float(rng.uniform(0.05, 1.0))
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    temp = float(rng.uniform(0.5, 10.0))
    return Request(rid, float(arrival), abc, jmax, pol, (0.5 * t_end, fwhm, inten, d), temp, t_end, dt, max_vectors)


def poisson_requests(seed, rate, duration, **kw):
    """Requests of a Poisson stream: arrivals at ``rate`` per second over
    ``duration`` seconds, each drawn with ``draw_request``."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        out.append(draw_request(rng, len(out), t, **kw))


def batch_device_bytes(dim, nvec, mmax, nslab=0):
    """Device bytes of one kr_batch (kr_batch_create): double-float state,
    complex64 Krylov basis and H V, per-vector scalars, reduction partials."""
    nb = (nvec + 127) // 128 * 128
    m1 = mmax + 1
    return (dim * nb * 16 + dim * 16 + m1 * dim * nb * 8 + dim * nb * 8 + (5 * m1 + 8) * nb * 8
            + 256 * (m1 + 1) * nb * 16 + nslab * nb * 8)


def c1_dim(jmax):
    """Basis size of an asymmetric top without symmetry, J = 0..jmax."""
    return sum((2 * J + 1) ** 2 for J in range(jmax + 1))


class Job:
    """An admitted request: operators, thermal ensemble, batched propagation.
    Admission uses ``device_bytes``, an upper bound from the request alone (the
    C1 basis size and ``max_vectors``); ``run`` builds the molecule's factors on
    the host, then propagates."""

    def __init__(self, req, mmax=20, tol=1e-8, matvec="tensor_tmem"):
        # a fixed kernel kind: a timed choice (matvec="auto") could differ between a
        # job alone and the same job among others, and so could its last digits
        self.req = req
        self.mmax, self.tol, self.matvec = mmax, tol, matvec
        self.state_steps = 0

    def device_bytes(self):
        dim = c1_dim(self.req.jmax)
        nvec = min(self.req.max_vectors, dim)
        # batch buffers, the loaded vectors (complex128) and the H0 phase, plus
        # the operators (factors in FP64 and FP32, MF buffers, the tensor-core
        # tiles' prebuilt B blocks): a margin
        return batch_device_bytes(dim, nvec, self.mmax, 2 * (self.req.jmax + 1)) + 16 * dim * (nvec + 1) + (256 << 20)

    def build(self):
        if hasattr(self, "wl"):
            return
        req = self.req
        mol = rot.Molecule(B=req.abc, sym="C1", pol=req.pol)
        self.wl = workloads.Workload("request_%d" % req.rid, mol, req.jmax, 0.0, req.t_end, req.dt, None, req.pulse)
        self.dim = self.wl.dim
        ens = workloads.Ensemble(self.wl, min(req.max_vectors, self.dim), req.temp)
        self.nvec = max(1, min(req.max_vectors, ens.n_natural))
        self.index = ens.index[: self.nvec]
        self.weights = ens.weights[: self.nvec]

    def run(self):
        """Builds the request's operators and propagates its ensemble through the
        time grid; returns the <cos^2 theta> trace."""
        from . import TDSE
        from .batch import Ensemble
        if not hasattr(self, "wl"):
            self.build()
        td = TDSE(t_start=0.0, t_end=self.req.t_end, dt=self.req.dt)
        tc = td.time_grid()
        ens = Ensemble(td, self.wl.h0, self.nvec, tol=self.tol, mmax=self.mmax, matvec=self.matvec)
        v = np.zeros((self.nvec, self.dim), np.complex128)
        v[np.arange(self.nvec), self.index] = 1.0
        ens.load(v)
        # the trace stays on the device: every step and its observable are queued
        # whole (the Krylov loop runs on the device), with no host synchronisation
        # until the end, so the steps of different jobs overlap on the GPU
        import torch
        w = torch.from_numpy(np.ascontiguousarray(self.weights, np.float64)).cuda()
        trace_d = torch.zeros(len(tc), dtype=torch.float64, device="cuda")
        for i, t in enumerate(tc):
            ens.step(self.wl.hamiltonian(t), sync=False)
            ens.expect_into(self.wl.cos2, trace_d[i:i + 1], w)
        ens.sync()  # a step error (Krylov order above mmax, observable mat-vec) is raised here
        trace = trace_d.cpu().numpy() + 1.0 / 3.0
        self.state_steps = self.nvec * len(tc)
        del ens
        return trace


@dataclass
class ServeStats:
    latencies: dict = field(default_factory=dict)   # rid -> seconds (arrival to completion)
    state_steps: int = 0
    wall: float = 0.0
    peak_bytes: int = 0
    max_active: int = 0

    def summary(self):
        lat = np.array(sorted(self.latencies.values())) * 1e3
        return {"requests": len(lat), "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
                "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
                "state_steps_per_s": self.state_steps / self.wall if self.wall > 0 else None,
                "wall_s": self.wall, "peak_admitted_bytes": self.peak_bytes, "max_concurrent": self.max_active}


class Server:
    """Admits requests against an HBM budget and runs each admitted job on its
    own stream and host thread.

    Args:
        budget_bytes : device memory the admitted jobs may hold together
        max_active : at most this many jobs at once (host threads)
        make_job : request -> job (default ``Job``); the job has
                   ``device_bytes()``, ``run() -> result`` and ``state_steps``
        device : CUDA device index; None runs jobs without CUDA streams (tests
                 of the scheduling on the host)
    """

    def __init__(self, budget_bytes=150e9, max_active=16, make_job=None, device=0, prebuild=True):
        self.budget = int(budget_bytes)
        self.max_active = int(max_active)
        self.make_job = make_job if make_job is not None else Job
        self.device = device
        self.prebuild = bool(prebuild)

    def serve(self, requests, realtime=True):
        """Serves ``requests`` (their ``arrival`` seconds after the start; with
        ``realtime`` False all have arrived at the start). Returns ({rid: result},
        ServeStats); a job that raised has its exception as result."""
        pending = sorted(requests, key=lambda r: r.arrival)
        stats = ServeStats()
        results = {}
        lock = threading.Condition()
        state = {"used": 0, "active": 0}
        threads = []
        t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        def worker(req, job):
            try:
                if self.device is not None:
                    import torch
                    torch.cuda.set_device(self.device)
                    with torch.cuda.stream(torch.cuda.Stream()):
                        res = job.run()
                        torch.cuda.current_stream().synchronize()
                else:
                    res = job.run()
                steps = int(getattr(job, "state_steps", 0))
            except Exception as e:  # reported per request, the service goes on
                res, steps = e, 0
            with lock:
                results[req.rid] = res
                stats.latencies[req.rid] = now() - (req.arrival if realtime else 0.0)
                stats.state_steps += steps
                state["used"] -= job.device_bytes()
                state["active"] -= 1
                lock.notify_all()

        jobs = {}
        built = {}  # rid -> True once the job's host set-up (factor build) is done
        if self.prebuild:
            # host set-up off the latency path: one builder thread prepares the
            # jobs in arrival order as they arrive, while admitted jobs run
            for req in pending:
                jobs[req.rid] = self.make_job(req)

            def builder():
                for req in list(pending):
                    if realtime:
                        wait = req.arrival - now()
                        if wait > 0:
                            time.sleep(wait)
                    job = jobs[req.rid]
                    try:
                        if hasattr(job, "build"):
                            job.build()
                    except Exception:
                        pass  # run() repeats the build and reports the error
                    with lock:
                        built[req.rid] = True
                        lock.notify_all()
            bth = threading.Thread(target=builder, daemon=True)
            bth.start()
        with lock:
            while pending or state["active"] > 0:
                t = now()
                admitted = False
                for req in list(pending):
                    if realtime and req.arrival > t:
                        break
                    if state["active"] >= self.max_active:
                        break
                    if self.prebuild and not built.get(req.rid):
                        continue  # its build is still running
                    job = jobs.get(req.rid)
                    if job is None:
                        job = jobs[req.rid] = self.make_job(req)
                    need = job.device_bytes()
                    if need > self.budget:
                        results[req.rid] = MemoryError(
                            f"request {req.rid} needs {need} bytes, above the budget of {self.budget}")
                        stats.latencies[req.rid] = t - (req.arrival if realtime else 0.0)
                        pending.remove(req)
                        continue
                    if state["used"] + need > self.budget:
                        continue  # first fit: a later, smaller request may still fit
                    pending.remove(req)
                    state["used"] += need
                    state["active"] += 1
                    stats.peak_bytes = max(stats.peak_bytes, state["used"])
                    stats.max_active = max(stats.max_active, state["active"])
                    th = threading.Thread(target=worker, args=(req, job), daemon=True)
                    threads.append(th)
                    th.start()
                    admitted = True
                if admitted:
                    continue
                # wait for a job to finish, a build to end or the next arrival
                timeout = None
                if realtime and pending and pending[0].arrival > t:
                    timeout = pending[0].arrival - t
                waiting_build = self.prebuild and any(not built.get(r.rid) for r in pending)
                if state["active"] > 0 or timeout is not None or waiting_build:
                    lock.wait(timeout=timeout if timeout is not None else 1.0)
        for th in threads:
            th.join()
        stats.wall = now()
        return results, stats
