"""Uneven-size batch on the GPU: a MoleculeSet (all molecules in one
block-diagonal operator, one persistent step launch per time step) against
each molecule propagated alone through TDSE.update (plain FP64 path, itself
parity-tested against the CPU oracle)."""
import numpy as np
import pytest
import torch

from richmol_gb300 import TDSE, workloads
from richmol_gb300.molecules import MoleculeSet

pytestmark = pytest.mark.gpu

# The same FP64 Lanczos per molecule on both sides (the segmented step keeps
# each molecule's scalars, stopping test and Krylov order); only the order of
# the floating-point sums differs. Bound of the plain path's parity tests.
STATE_TOL = 1e-10


# The mixed form (FP32 mat-vec products, FP64 everything else) against the
# same FP64 propagation: the bound of the mixed-precision forms (1e-6).
MIXED_TOL = 1e-6


def _run(wls, nsteps, precision="f64", check_orders=True):
    td = TDSE(t_start=0.0, t_end=wls[0].t_end, dt=wls[0].dt)
    tc = td.time_grid()
    ms = MoleculeSet(td, [w.h0 for w in wls], [w.Hac for w in wls], precision=precision)
    v0 = [workloads.ground_state(w) for w in wls]
    state = ms.join(v0)
    alone = [torch.from_numpy(v).cuda().reshape(1, -1) for v in v0]
    tds = [TDSE(t_start=0.0, t_end=w.t_end, dt=w.dt) for w in wls]
    for td_ in tds:
        td_.time_grid()
    i0 = len(tc) // 2 - nsteps // 2  # through the pulse maximum
    for i in range(i0, i0 + nsteps):
        for w in wls:
            w.hamiltonian(tc[i])
        ms.step(state)
        for m, w in enumerate(wls):
            alone[m], _ = tds[m].update(w.hamiltonian(tc[i]), H0=w.h0, vecs=alone[m], inplace=True)
            if check_orders:
                assert int(tds[m].last_korder[0]) == int(ms.last_korder[m]), (i, m)
    worst = 0.0
    for m, v in enumerate(ms.split(state)):
        worst = max(worst, float((v - alone[m].reshape(-1)).abs().max()))
    return ms, state, worst


def test_molecule_set_matches_each_molecule_alone():
    wls = workloads.uneven_molecules(5, seed=3, jmax_range=(10, 14), t_end=1.0)
    ms, state, worst = _run(wls, 6)
    assert worst < STATE_TOL, worst
    assert ms.last_korder.min() >= 2
    nrm = [float(torch.linalg.vector_norm(v)) for v in ms.split(state)]
    assert np.allclose(nrm, 1.0, atol=1e-12)


def test_molecule_set_beyond_16_parts():
    """20 molecules: the field coefficients go to the device as a buffer."""
    wls = workloads.uneven_molecules(20, seed=8, jmax_range=(3, 7), t_end=1.0)
    ms, state, worst = _run(wls, 4)
    assert ms.plan.nblock == 20 and len(ms.plan.sources) == 20
    assert worst < STATE_TOL, worst
    c2 = ms.expect([w.cos2 for w in wls], state) + 1.0 / 3.0  # the tensor is cos^2 theta - 1/3
    assert np.all((c2 > 0.0) & (c2 < 1.0))


def test_mixed_precision_molecule_set_within_bound():
    """precision="mixed": the mat-vec products in FP32, states, Krylov vectors
    and Lanczos scalars in FP64; states and <cos^2> within 1e-6 of each
    molecule's FP64 TDSE.update, norms kept to the Lanczos tolerance."""
    wls = workloads.uneven_molecules(6, seed=3, jmax_range=(10, 16), t_end=1.0)
    ms, state, worst = _run(wls, 8, precision="mixed", check_orders=False)
    assert worst < MIXED_TOL, worst
    nrm = [float(torch.linalg.vector_norm(v)) for v in ms.split(state)]
    assert np.allclose(nrm, 1.0, atol=1e-6)
