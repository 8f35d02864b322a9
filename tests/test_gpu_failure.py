"""Failure detection on the GPU without a fault: the bounded grid-barrier wait
of the step kernels, in a launch where one CTA never arrives (a rank that never
joins), gives up after its limit and reports KR_ERR_TIMEOUT to the host instead
of hanging; the context stays usable, so the next step runs and is right."""
import ctypes

import numpy as np
import pytest
import torch

from richmol_gb300 import TDSE, _native, workloads
from richmol_gb300.device import context

pytestmark = pytest.mark.gpu


def test_wait_nothing_ends_gives_up_with_timeout_status():
    ctx = context(0)
    st, waited = ctypes.c_int32(-1), ctypes.c_double(0.0)
    _native.check(_native.lib().kr_probe_wait(ctx, ctypes.byref(st), ctypes.byref(waited)), ctx)
    assert st.value == _native.KR_ERR_TIMEOUT
    assert 1.0 <= waited.value < 10.0  # the 2 s limit (or the spin cap) of a grid-barrier wait, then return

    # the context is still usable: steps run and keep the norms (the rows of a
    # thermal init_state carry sqrt of their Boltzmann weights, tdse.py:239-258)
    wl = workloads.asym_top(Jmax=6, dt=0.005, nsteps=400)
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    v0 = np.ascontiguousarray(td.init_state(wl.h0, temp=5, thresh=1e-3)[:3])
    v = torch.from_numpy(v0).cuda()
    for t in tc[150:155]:
        v, _ = td.update(wl.hamiltonian(t), H0=wl.h0, vecs=v, inplace=True, check=False)
    torch.cuda.synchronize()
    nrm = torch.linalg.vector_norm(v, dim=1).cpu().numpy()
    # the Lanczos stopping test (squared distance of successive solutions below
    # tol = 1e-15, tdse.py:476) leaves each step's last correction up to
    # sqrt(1e-15) ~ 3.2e-8, so five steps keep the norms to about 1.6e-7
    assert np.allclose(nrm, np.linalg.norm(v0, axis=1), rtol=0, atol=1e-7)
    assert float((v - torch.from_numpy(v0).cuda()).abs().max()) > 1e-6  # the steps moved the states
