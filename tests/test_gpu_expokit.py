"""GPU: the expokit-scheme propagator (richmol's propag='external',
tdse.py:383-392) through the C ABI (kr_expv, kr_op_norm1) against the oracle
restatement (oracle/expokit.py, itself pinned to the exact exponential), and
TDSE.update(propag='external') against the reference's golden trajectories,
which the internal scheme produced: both schemes approximate the same
exponential to about 1e-14, so the states agree to the parity tolerance."""
import os

import numpy as np
import pytest
import scipy.linalg

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

STATE_RTOL = 1e-10


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _load(name):
    from oracle import fixtures
    return fixtures.load(os.path.join(GOLDEN, name))


def _ct(case, name):
    from richmol_gb300 import CarTens
    return CarTens(os.path.join(GOLDEN, case), name=name)


def _dressed_pol(case):
    from oracle import fixtures
    d, meta = _load(case)
    o = fixtures.tensor(d, meta, "pol")
    o.field(meta["field_vec"])
    T = _ct(case, "pol")
    T.field(meta["field_vec"])
    return d, meta, o, T


@pytest.mark.parametrize("case", ["ocs_j6.npz", "asym_j4.npz"])
def test_norm1_estimate_bounds_exact_norm(case):
    _, _, o, T = _dressed_pol(case)
    exact = np.abs(o.tomat(form="full").toarray()).sum(axis=0).max()
    est = T.device_operator().norm1()
    assert est <= exact * (1 + 1e-12)
    assert est >= 0.5 * exact


@pytest.mark.parametrize("case", ["ocs_j6.npz", "asym_j4.npz"])
def test_expv_matches_oracle_and_exact_exponential(case):
    from oracle.cartens import flat, split
    from oracle.expokit import zhexpv
    _, _, o, T = _dressed_pol(case)
    plan = T.device_operator()
    anorm = plan.norm1()
    Hd = o.tomat(form="full").toarray()
    rng = np.random.default_rng(4)
    v = rng.standard_normal(Hd.shape[0]) + 1j * rng.standard_normal(Hd.shape[0])
    t = -8.0 / anorm
    st = {}
    ref = zhexpv(v, anorm, 12, t, lambda x: flat(o, o.vec(split(o, x)), "1"), tol=1e-15, stats=st, c=1j)
    x = torch.from_numpy(v.copy()).cuda()
    nstep, _, _ = plan.expv(x, t, 12, 1e-15, anorm)
    # step-size decisions at the acceptance boundary may differ by rounding
    assert abs(nstep - st["nstep"]) <= 1
    got = x.cpu().numpy()
    assert _rel(got, ref) < 1e-12
    assert _rel(got, scipy.linalg.expm(t * 1j * Hd) @ v) < 1e-11


def test_update_external_split_operator_matches_reference():
    from richmol_gb300 import TDSE
    d, meta = _load("ocs_j6.npz")
    h0 = _ct("ocs_j6.npz", "h0")
    sp = meta["split"]
    Hac = _ct("ocs_j6.npz", "pol") * sp["scale"]
    td = TDSE(t_start=sp["t_start"], t_end=sp["t_end"], dt=sp["dt"])
    tc = td.time_grid()
    vecs = td.init_state(h0, temp=0)
    for i in range(len(tc)):
        Hac.field(d["split/fields"][i])
        vecs, _ = td.update(Hac, H0=h0, vecs=vecs, propag="external")
        assert _rel(vecs, d["split/states"][i]) < STATE_RTOL


def test_update_external_multivector_matches_reference():
    from richmol_gb300 import TDSE
    d, meta = _load("asym_j4.npz")
    sc = meta["scales"]
    h0 = _ct("asym_j4.npz", "h0")
    Hdc = (_ct("asym_j4.npz", "dip") * meta["dc"]) * sc["dc"]
    Hac = _ct("asym_j4.npz", "pol") * sc["ac"]
    sp = meta["split"]
    td = TDSE(t_start=sp["t_start"], t_end=sp["t_end"], dt=sp["dt"])
    tc = td.time_grid()
    vecs = td.init_state(h0, temp=5, thresh=1e-3)
    for i in range(len(tc)):
        Hac.field(d["split/fields"][i])
        vecs, _ = td.update(Hdc + Hac, H0=h0, vecs=vecs, propag="external")
    assert _rel(vecs, d["split/final"]) < STATE_RTOL


def test_expv_small_invariant_subspace_breaks_down():
    """The OCS ground state under a z field spans J = 0, 2, 4, 6 (m = 0): the
    Lanczos breaks down after 4 mat-vecs and one step covers the interval."""
    d, meta = _load("ocs_j6.npz")
    sp = meta["split"]
    T = _ct("ocs_j6.npz", "pol") * sp["scale"]
    T.field(d["split/fields"][0])
    plan = T.device_operator()
    x = torch.from_numpy(d["split/vec0"][0].copy()).cuda()
    assert plan.expv(x, -0.0018836515673088528, 12, 1e-15, plan.norm1()) == (1, 4, 0)


def test_expv_rejects_bad_sizes():
    """m >= dim is the reference's "bad input arguments" (pyexpokit.py:9-11)."""
    from richmol_gb300 import _native
    _, _, o, T = _dressed_pol("ocs_j6.npz")
    plan = T.device_operator()
    n = o.tomat(form="full").shape[0]
    x = torch.ones(n, dtype=torch.complex128, device="cuda")
    with pytest.raises(_native.KrylovError) as e:
        plan.expv(x, -0.1, n, 1e-15, 1.0)
    assert e.value.code == _native.KR_ERR_ARG


def test_expv_zero_vector_stays_zero():
    _, _, o, T = _dressed_pol("asym_j4.npz")
    plan = T.device_operator()
    n = o.tomat(form="full").shape[0]
    x = torch.zeros(n, dtype=torch.complex128, device="cuda")
    assert plan.expv(x, -0.1, 12, 1e-15, plan.norm1()) == (0, 0, 0)
    assert torch.count_nonzero(x).item() == 0
