"""Field schedule (kr_set_field_schedule / kr_set_field_step): the fields of
many steps uploaded once, each step's field then set from device memory. The
field products are the same arithmetic on the same coefficients as a per-step
kr_set_field, so the steps agree with the call-by-call ones; a CUDA graph of
steps over an operator of more than 16 parts records them from the schedule."""
import operator
from functools import reduce

import numpy as np
import pytest
import torch

from richmol_gb300 import TDSE, _native, workloads
from richmol_gb300.graph import StepGraph
from richmol_gb300.molecules import MoleculeSet

pytestmark = pytest.mark.gpu

# the same field products either way; 1e-13 leaves room for a different
# instruction order of the two coefficient loads (kernel parameter / memory)
STATE_TOL = 1e-13


def _setup(Jmax=10):
    wl = workloads.asym_top(Jmax=Jmax, dt=0.005, nsteps=400)
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    v0 = td.init_state(wl.h0, temp=5, thresh=1e-3)[:3]
    return wl, td, tc, np.ascontiguousarray(v0)


def test_schedule_steps_equal_per_step_fields():
    wl, td, tc, v0 = _setup()
    times = tc[150:162]
    plan = wl.hamiltonian(times[0]).device_operator()
    plan.set_field_schedule([wl.hamiltonian(t)._part_states() for t in times])
    phase = td._h0_phase(wl.h0, td.exp_fac, torch.device("cuda"))
    a = torch.from_numpy(v0).cuda()
    b = a.clone()
    ka, kb = np.zeros(3, np.int32), np.zeros(3, np.int32)
    for i, t in enumerate(times):
        assert wl.hamiltonian(t).device_operator() is plan  # per-step kr_set_field
        plan.step(a, phase, td.exp_fac, 1e-15, korder=ka)
        plan.set_field_step(i)
        plan.step(b, phase, td.exp_fac, 1e-15, korder=kb)
        assert np.array_equal(ka, kb), (i, ka, kb)
    assert float((a - b).abs().max()) <= STATE_TOL
    assert float((a - torch.from_numpy(v0).cuda()).abs().max()) > 1e-3  # the field acted


def test_schedule_step_out_of_range_is_an_argument_error():
    wl, td, tc, _ = _setup(Jmax=4)
    plan = wl.hamiltonian(tc[0]).device_operator()
    plan.set_field_schedule([wl.hamiltonian(t)._part_states() for t in tc[:5]])
    for bad in (-1, 5):
        with pytest.raises(_native.KrylovError) as e:
            plan.set_field_step(bad)
        assert e.value.code == _native.KR_ERR_ARG
    plan.set_field_step(4)
    plan.sync_status()


def test_recorded_steps_beyond_16_parts():
    """H(t) as a sum of 18 parts (nine copies of the two-part H(t), each
    scaled by 1/9): the recording sets each step's field from the schedule;
    the call-by-call steps stage the coefficients through host memory; both
    read them from device memory, so they agree to the last bit, and both
    agree with the two-part operator to rounding."""
    wl, td, tc, v0 = _setup()
    times = tc[150:162]

    def h18(t):
        return reduce(operator.add, [wl.hamiltonian(t) * (1.0 / 9.0) for _ in range(9)])

    assert len(h18(times[0])._parts) == 18
    rec = torch.from_numpy(v0).cuda()
    g = StepGraph(td, wl.h0, rec, h18, times)
    assert g.schedule
    g.replay()
    torch.cuda.synchronize()
    eager = torch.from_numpy(v0).cuda()
    two = eager.clone()
    td_e = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    td_e.time_grid()
    td_2 = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    td_2.time_grid()
    for t in times:
        eager, _ = td_e.update(h18(t), H0=wl.h0, vecs=eager, inplace=True, check=False)
        two, _ = td_2.update(wl.hamiltonian(t), H0=wl.h0, vecs=two, inplace=True, check=False)
    assert float((rec - eager).abs().max()) == 0.0
    assert float((rec - two).abs().max()) < 1e-12


def test_recorded_steps_from_schedule_below_16_parts():
    wl, td, tc, v0 = _setup()
    times = tc[150:162]
    rec = torch.from_numpy(v0).cuda()
    g = StepGraph(td, wl.h0, rec, wl.hamiltonian, times, schedule=True)
    g.replay()
    eager = torch.from_numpy(v0).cuda()
    td_e = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    td_e.time_grid()
    for t in times:
        eager, _ = td_e.update(wl.hamiltonian(t), H0=wl.h0, vecs=eager, inplace=True, check=False)
    torch.cuda.synchronize()
    assert float((rec - eager).abs().max()) <= STATE_TOL
    # a new schedule frees the one the recording reads: its replay is refused
    g.plan.set_field_schedule([wl.hamiltonian(t)._part_states() for t in times])
    with pytest.raises(RuntimeError, match="replaced"):
        g.replay()


def test_molecule_set_with_field_schedule():
    wls = workloads.uneven_molecules(20, seed=8, jmax_range=(3, 7), t_end=1.0)
    td = TDSE(t_start=0.0, t_end=wls[0].t_end, dt=wls[0].dt)
    tc = td.time_grid()
    i0 = len(tc) // 2 - 3
    v0 = [workloads.ground_state(w) for w in wls]
    ms_a = MoleculeSet(td, [w.h0 for w in wls], [w.Hac for w in wls])
    ms_b = MoleculeSet(td, [w.h0 for w in wls], [w.Hac for w in wls])

    def set_fields(i):
        for w in wls:
            w.hamiltonian(tc[i0 + i])

    ms_b.set_field_schedule(set_fields, 6)
    a, b = ms_a.join(v0), ms_b.join(v0)
    for i in range(6):
        set_fields(i)
        ms_a.step(a)
        ms_b.step(b, field_step=i)
        assert np.array_equal(ms_a.last_korder, ms_b.last_korder)
    assert float((a - b).abs().max()) == 0.0  # both read the coefficients from device memory
