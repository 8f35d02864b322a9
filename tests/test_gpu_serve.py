"""Propagation service on the GPU: a request's result is the same alone and in
the mix (jobs overlapping on their own streams), and a served trace agrees with
the plain FP64 propagation of the same ensemble within 1e-6."""
import numpy as np
import pytest
import torch

from richmol_gb300 import TDSE, serve

pytestmark = pytest.mark.gpu

# results of one request alone and among others: same buffers, same reductions
MIX_TOL = 1e-12
# served (complex64 mat-vec, FP64 Lanczos) against the plain FP64 path
FP64_TOL = 1e-6


def small_requests(n, seed=11):
    rng = np.random.default_rng(seed)
    return [serve.draw_request(rng, i, 0.0, jmax_range=(10, 13), t_end=0.12, max_vectors=96) for i in range(n)]


def test_result_same_alone_and_in_the_mix():
    reqs = small_requests(5)
    alone = {}
    for r in reqs[:2]:
        res, _ = serve.Server(budget_bytes=40e9, max_active=1).serve([r], realtime=False)
        assert not isinstance(res[r.rid], Exception), res[r.rid]
        alone[r.rid] = res[r.rid]
    mix, stats = serve.Server(budget_bytes=40e9, max_active=5).serve(reqs, realtime=False)
    assert stats.max_active >= 2
    for r in reqs:
        assert not isinstance(mix[r.rid], Exception), mix[r.rid]
        assert np.all(np.isfinite(mix[r.rid]))
    for rid, tr in alone.items():
        np.testing.assert_allclose(mix[rid], tr, rtol=0, atol=MIX_TOL)
    s = stats.summary()
    assert s["requests"] == 5 and s["p99_ms"] >= s["p50_ms"] > 0 and s["state_steps_per_s"] > 0


def test_served_trace_matches_fp64():
    rng = np.random.default_rng(5)
    r = serve.draw_request(rng, 0, 0.0, jmax_range=(11, 11), t_end=0.2, max_vectors=24)
    job = serve.Job(r)
    trace = job.run()
    wl = job.wl
    td = TDSE(t_start=0.0, t_end=r.t_end, dt=r.dt)
    tc = td.time_grid()
    v = np.zeros((job.nvec, job.dim), np.complex128)
    v[np.arange(job.nvec), job.index] = 1.0
    ref = torch.from_numpy(v).cuda()
    plan = wl.cos2.device_operator()
    worst = 0.0
    for i, t in enumerate(tc):
        ref, _ = td.update(wl.hamiltonian(t), H0=wl.h0, vecs=ref, inplace=True, check=False)
        y = torch.empty_like(ref)
        plan.matvec(ref, y)
        e = torch.sum(torch.conj(ref) * y, dim=1).real.cpu().numpy()
        worst = max(worst, abs(float(job.weights @ e) + 1.0 / 3.0 - trace[i]))
    assert worst < FP64_TOL, worst


def test_realtime_stream_reports_latency():
    rs = serve.poisson_requests(3, rate=40.0, duration=0.2, jmax_range=(10, 12), t_end=0.05, max_vectors=64)
    assert len(rs) >= 2
    results, stats = serve.Server(budget_bytes=40e9, max_active=8).serve(rs, realtime=True)
    assert all(not isinstance(v, Exception) for v in results.values())
    s = stats.summary()
    assert s["requests"] == len(rs) and s["p50_ms"] > 0


def test_many_jobs_created_and_stepped_at_once():
    """Twelve jobs on twelve host threads at once, every one building its
    operators, recording its step graph and stepping while the others do the
    same (the library serialises its recordings and allocations): every trace
    equals the same request run alone."""
    reqs = small_requests(12, seed=23)
    alone = {}
    for r in reqs[:3]:
        res, _ = serve.Server(budget_bytes=40e9, max_active=1).serve([r], realtime=False)
        alone[r.rid] = res[r.rid]
    # without prebuild every job thread builds its own factors and operators
    # while the others record and step; with it, one builder thread feeds them
    for prebuild in (False, True):
        mix, stats = serve.Server(budget_bytes=80e9, max_active=12, prebuild=prebuild).serve(reqs, realtime=False)
        assert stats.max_active >= (4 if not prebuild else 2)
        for r in reqs:
            assert not isinstance(mix[r.rid], Exception), mix[r.rid]
        for rid, tr in alone.items():
            np.testing.assert_allclose(mix[rid], tr, rtol=0, atol=MIX_TOL)
