"""kr_observables: <v|O|v> of FP64 states on the device (OperatorPlan.observables)
against the host product with the assembled matrix (CarTens.tomat, the route of
examples/ocs_alignment.py:70,99-100), the Boltzmann-weighted sum, and the
vectors taken in chunks (products of more than 256 MiB) against one at a time."""
import numpy as np
import pytest
import torch

from richmol_gb300 import TDSE, workloads

pytestmark = pytest.mark.gpu


def _cos2(wl):
    O = wl.cos2
    if O._parts[0].prods is None:
        O.field([0, 0, 1])
    return O


def test_observables_match_host_matrix():
    wl = workloads.asym_top(Jmax=10, dt=0.005, nsteps=400)
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    v = torch.from_numpy(np.ascontiguousarray(td.init_state(wl.h0, temp=5, thresh=1e-3)[:6])).cuda()
    for t in tc[140:150]:  # mixes the eigenstates
        v, _ = td.update(wl.hamiltonian(t), H0=wl.h0, vecs=v, inplace=True, check=False)
    O = _cos2(wl)
    plan = O.device_operator()
    w = np.linspace(0.4, 0.05, 6)
    vals, wsum = plan.observables(v, weights=w)
    vh = v.cpu().numpy()
    M = O.tomat(form="full")
    ref = np.array([np.vdot(x, M @ x) for x in vh])
    assert np.abs(vals - ref).max() < 1e-13
    assert np.abs(vals.imag).max() < 1e-13  # Hermitian observable
    assert abs(wsum - float(w @ ref.real)) < 1e-13
    vals2, wsum2 = plan.observables(v, weights=w)
    assert np.array_equal(vals, vals2) and wsum == wsum2  # fixed summation order
    _, plain = plan.observables(v)
    assert abs(plain - float(ref.real.sum())) < 1e-13


def test_observables_in_chunks():
    """430 vectors at J <= 30 (dim 39,711): the products of 422 vectors fill
    256 MiB, so the call runs two chunks."""
    wl, _ = workloads.thermal_asym_top(Jmax=30, nvec=128)
    O = _cos2(wl)
    plan = O.device_operator()
    g = torch.Generator(device="cuda").manual_seed(5)
    v = torch.randn((430, wl.dim), dtype=torch.complex128, device="cuda", generator=g)
    v /= torch.linalg.vector_norm(v, dim=1, keepdim=True)
    vals, _ = plan.observables(v)
    one = np.array([plan.observables(v[i:i + 1])[0][0] for i in (0, 1, 421, 422, 429)])
    assert np.abs(vals[[0, 1, 421, 422, 429]] - one).max() < 1e-14
    y = torch.empty_like(v[:8])
    plan.matvec(v[:8].contiguous(), y)
    ref = torch.sum(torch.conj(v[:8]) * y, dim=1).cpu().numpy()
    assert np.abs(vals[:8] - ref).max() < 1e-13
