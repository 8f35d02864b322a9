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


def test_autotuned_matvec_kind():
    from richmol_gb300.batch import Ensemble
    wl, ensd = workloads.thermal_asym_top(Jmax=12, nvec=256)
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    ens = Ensemble(td, wl.h0, 256, tol=1e-8, matvec="auto")
    ens.load(ensd.vectors(wl.dim))
    ens.step(wl.hamiltonian(tc[100]))
    assert set(ens.tuned) == {"tensor", "fp32"} and all(t > 0 for t in ens.tuned.values())
    assert ens.matvec == min(ens.tuned, key=ens.tuned.get)
    ref = Ensemble(td, wl.h0, 256, tol=1e-8, matvec="fp32")
    ref.load(ensd.vectors(wl.dim))
    ref.step(wl.hamiltonian(tc[100]))
    assert float((ens.store() - ref.store()).abs().max()) < 1e-5
