"""A time-step loop recorded as a CUDA graph (richmol_gb300.graph.StepGraph)
against the same steps run one call at a time: the same kernels on the same
inputs, so the states agree to the last bit; and the autotuned choice of the
batched mat-vec kernel."""
import numpy as np
import pytest
import torch

from richmol_gb300 import TDSE, workloads
from richmol_gb300.graph import StepGraph

pytestmark = pytest.mark.gpu


def test_recorded_steps_equal_eager_steps():
    wl = workloads.asym_top(Jmax=12, dt=0.005, nsteps=400)
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    v0 = td.init_state(wl.h0, temp=5, thresh=1e-3)[:3]
    times = tc[150:170]  # through the rising pulse
    eager = torch.from_numpy(np.ascontiguousarray(v0)).cuda()
    td_e = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    td_e.time_grid()
    for t in times:
        eager, _ = td_e.update(wl.hamiltonian(t), H0=wl.h0, vecs=eager, inplace=True, check=False)
    rec = torch.from_numpy(np.ascontiguousarray(v0)).cuda()
    g = StepGraph(td, wl.h0, rec, wl.hamiltonian, times)
    assert float((rec - torch.from_numpy(v0).cuda()).abs().max()) == 0.0  # recording ran nothing
    g.replay()
    torch.cuda.synchronize()
    assert float((rec - eager).abs().max()) == 0.0
    # a second replay continues from the new state: the same as 20 more eager steps
    # with the recorded fields
    g.replay()
    for t in times:
        eager, _ = td_e.update(wl.hamiltonian(t), H0=wl.h0, vecs=eager, inplace=True, check=False)
    assert float((rec - eager).abs().max()) == 0.0


def test_autotuned_matvec_kind(tmp_path, monkeypatch):
    """matvec="auto": every kind timed on the operator, the fastest kept and
    cached in the tuning file; a second ensemble of the same shape reads the
    choice from the file."""
    from richmol_gb300 import tune
    from richmol_gb300.batch import Ensemble
    monkeypatch.setenv(tune.CACHE_ENV, str(tmp_path / "tune.json"))
    wl, ensd = workloads.thermal_asym_top(Jmax=12, nvec=256)
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    ens = Ensemble(td, wl.h0, 256, tol=1e-8, matvec="auto")
    ens.load(ensd.vectors(wl.dim))
    ens.step(wl.hamiltonian(tc[100]))
    from richmol_gb300.batch import _KINDS
    assert set(ens.tuned) == set(_KINDS) and all(t > 0 for t in ens.tuned.values())
    assert ens.matvec == min(ens.tuned, key=ens.tuned.get) and not ens.tuned_from_cache
    again = Ensemble(td, wl.h0, 256, tol=1e-8, matvec="auto")
    again.load(ensd.vectors(wl.dim))
    again.step(wl.hamiltonian(tc[100]))
    assert again.tuned_from_cache and again.matvec == ens.matvec
    ref = Ensemble(td, wl.h0, 256, tol=1e-8, matvec="fp32")
    ref.load(ensd.vectors(wl.dim))
    ref.step(wl.hamiltonian(tc[100]))
    assert float((ens.store() - ref.store()).abs().max()) < 1e-5


def _ensemble_setup(nvec=256):
    from richmol_gb300.batch import Ensemble
    wl, ensd = workloads.thermal_asym_top(Jmax=12, nvec=nvec)
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    ens = Ensemble(td, wl.h0, nvec, tol=1e-8)
    ens.load(ensd.vectors(wl.dim))
    return wl, ensd, td, tc, ens


def test_recorded_ensemble_steps_equal_eager_steps():
    """Batched steps recorded into one CUDA graph (field launches and the
    steps' device-side Krylov loops) replay to the same bits as the same steps
    called one at a time."""
    from richmol_gb300.graph import EnsembleGraph
    wl, ensd, td, tc, eager = _ensemble_setup()
    _, _, _, _, rec = _ensemble_setup()
    times = tc[90:102]  # through the pulse maximum (Krylov orders rise)
    for t in times:
        eager.step(wl.hamiltonian(t))
    g = EnsembleGraph(rec, wl.hamiltonian, times)
    assert torch.equal(rec.store(), torch.from_numpy(ensd.vectors(wl.dim)).cuda())  # recording ran nothing
    g.replay()
    assert torch.equal(rec.store(), eager.store())
    for t in times:
        eager.step(wl.hamiltonian(t))
    g.replay()
    assert torch.equal(rec.store(), eager.store())


def test_unsynchronised_steps_equal_synchronised_steps():
    """Ensemble.step(sync=False) queues the whole step (no host read-back
    between Krylov iterations); the results equal the synchronised calls and
    Ensemble.sync() reports the last step's largest Krylov order."""
    wl, ensd, td, tc, a = _ensemble_setup()
    _, _, _, _, b = _ensemble_setup()
    for t in tc[95:101]:
        a.step(wl.hamiltonian(t))
        b.step(wl.hamiltonian(t), sync=False)
    b.sync()
    assert b.last_kmax == a.last_kmax > 0
    assert torch.equal(a.store(), b.store())


def test_unsynchronised_step_error_reported_by_sync():
    """A step that needs more Krylov vectors than the batch holds: with
    sync=False the error waits in the batch until sync() raises it; the steps
    queued behind it leave the states as they are; after the report the batch
    steps again."""
    from richmol_gb300 import _native
    from richmol_gb300.batch import Ensemble
    wl, ensd = workloads.thermal_asym_top(Jmax=12, nvec=128)
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    ens = Ensemble(td, wl.h0, 128, tol=1e-14, mmax=2)
    ens.load(ensd.vectors(wl.dim))
    ens.step(wl.hamiltonian(tc[100]), sync=False)
    torch.cuda.synchronize()
    after_error = ens.store()
    ens.step(wl.hamiltonian(tc[101]), sync=False)  # skipped: an error is pending
    assert torch.equal(ens.store(), after_error)
    with pytest.raises(_native.KrylovError) as e:
        ens.sync()
    assert e.value.code == _native.KR_ERR_MAXORDER
    ens.sync()  # reported once
    ok = Ensemble(td, wl.h0, 128, tol=1e-8, mmax=20)
    ok.load(ensd.vectors(wl.dim))
    ok.step(wl.hamiltonian(tc[100]))
    assert ok.last_kmax > 2
