"""GPU parity at the benchmark configurations, through the C ABI.

Against the reference's own propagation (fixtures of tests/golden/make_golden.py):
* ocs_c1_j20: the CPU-runnable configuration exactly as configured (linear OCS
  J <= 20 all M, dim 441, 300 steps of 10 fs through the 5e11 W/cm^2 pulse);
* asym_j10: the D2 asymmetric top at J <= 10 (dim 1,771) with DC field and
  the 35-degree pulse, 50 steps through the pulse maximum, 22-vector T = 5 K
  ensemble, <cos^2>, <cos> and J-populations of every vector at every step;
* c1_j10: a C1 molecule (complex K factors) at J <= 10.
Against the CPU oracle on the same factors (the in-house builder's, at sizes
the reference cannot build here):
* J <= 40 (dim 91,881, the plain FP64 drop-in configuration): 10 steps of 5 fs
  through the pulse maximum;
* J <= 30 (dim 39,711, the batched ensemble configuration): 10 steps of 10 fs
  through the pulse maximum for 256 vectors of the thermal ensemble on the
  batched mixed-precision path, four of them checked against the oracle.

Tolerances: plain path, states 1e-10 relative per step and observables 1e-9
absolute, with FP64 products and with double-float ones (products="df");
batched mixed-precision path, observables 1e-6 absolute (the stated bound of
that form) and states 1e-6 relative.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

STATE_RTOL = 1e-10
OBS_ATOL = 1e-9
MIXED_OBS_ATOL = 1e-6
MIXED_STATE_RTOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _built():
    from richmol_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        _native.build_library()
    assert torch.cuda.is_available()


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _load(name):
    from oracle import fixtures
    return fixtures.load(os.path.join(GOLDEN, name))


def _ct(case, name):
    from richmol_gb300 import CarTens
    return CarTens(os.path.join(GOLDEN, case), name=name)


def _dev_expect(O, states):
    """<v|O|v> of every row of a CUDA tensor, on the device (kr_observables)."""
    if O._parts[0].prods is None:
        O.field([0, 0, 1])
    vals, _ = O.device_operator().observables(states)
    return vals.real


def _pops(T, v):
    """J-populations of the rows of v (numpy) from the tensor's slab table."""
    basis = T._parts[0].src.basis("1")
    Js = sorted({b[0] for b in basis})
    out = np.zeros((v.shape[0], len(Js)))
    off = 0
    for J, _, dm, dk in basis:
        n = dm * dk
        out[:, Js.index(J)] += np.sum(np.abs(v[:, off: off + n]) ** 2, axis=1)
        off += n
    return out


PRODUCTS = ["f64", "df"]


@pytest.mark.parametrize("products", PRODUCTS)
def test_ocs_c1_configuration_matches_reference(products):
    from richmol_gb300 import TDSE
    case = "ocs_c1_j20.npz"
    d, meta = _load(case)
    h0 = _ct(case, "h0")
    Hac = _ct(case, "pol") * meta["scale"]
    cos2, cos = _ct(case, "cos2"), _ct(case, "cos")
    p = meta["tdse"]
    td = TDSE(t_start=p["t_start"], t_end=p["t_end"], dt=p["dt"])
    tc = td.time_grid()
    v0 = td.init_state(h0, temp=0)
    assert np.array_equal(v0, d["vec0"])
    v = torch.from_numpy(v0).cuda()
    saved = {int(s): k for k, s in enumerate(d["state_steps"])}
    worst = dict(state=0.0, cos2=0.0, cos=0.0, pops=0.0)
    for i in range(len(tc)):
        Hac.field(d["fields"][i])
        v, t2 = td.update(Hac, v, H0=h0, products=products)
        assert abs(t2 - d["times"][i]) < 1e-12
        vh = v.cpu().numpy()
        worst["cos2"] = max(worst["cos2"], abs(_dev_expect(cos2, v)[0] + 1 / 3 - d["cos2"][i]))
        worst["cos"] = max(worst["cos"], abs(_dev_expect(cos, v)[0] - d["cos"][i]))
        worst["pops"] = max(worst["pops"], np.abs(_pops(h0, vh)[0] - d["pops"][i]).max())
        if i in saved:
            worst["state"] = max(worst["state"], _rel(vh[0], d["states"][saved[i]]))
    print("ocs c1 (300 steps, %s products):" % products, worst)
    assert worst["state"] < STATE_RTOL
    assert worst["cos2"] < OBS_ATOL and worst["cos"] < OBS_ATOL and worst["pops"] < OBS_ATOL


def _asym_j10():
    from richmol_gb300 import TDSE
    case = "asym_j10.npz"
    d, meta = _load(case)
    sc = meta["scales"]
    h0 = _ct(case, "h0")
    Hdc = (_ct(case, "dip") * meta["dc"]) * sc["dc"]
    Hac = _ct(case, "pol") * sc["ac"]
    p = meta["tdse"]
    td = TDSE(t_start=p["t_start"], t_end=p["t_end"], dt=p["dt"])
    tc = td.time_grid()
    return case, d, h0, Hdc, Hac, td, tc


@pytest.mark.parametrize("products", PRODUCTS)
def test_asym_j10_ensemble_matches_reference(products):
    case, d, h0, Hdc, Hac, td, tc = _asym_j10()
    cos2, cos = _ct(case, "cos2"), _ct(case, "cos")
    v0 = td.init_state(h0, temp=5, thresh=1e-3)
    assert v0.shape == d["vec0"].shape and np.abs(v0 - d["vec0"]).max() < 1e-14
    v = torch.from_numpy(v0).cuda()
    saved = {int(s): k for k, s in enumerate(d["state_steps"])}
    worst = dict(state=0.0, cos2=0.0, cos=0.0, pops=0.0)
    for i in range(len(tc)):
        Hac.field(d["fields"][i])
        v, _ = td.update(Hdc + Hac, v, H0=h0, products=products)
        vh = v.cpu().numpy()
        worst["cos2"] = max(worst["cos2"], np.abs(_dev_expect(cos2, v) - d["cos2"][i]).max())
        worst["cos"] = max(worst["cos"], np.abs(_dev_expect(cos, v) - d["cos"][i]).max())
        worst["pops"] = max(worst["pops"], np.abs(_pops(h0, vh) - d["pops"][i]).max())
        if i in saved:
            worst["state"] = max(worst["state"], _rel(vh[:2], d["states"][saved[i]]))
    worst["state"] = max(worst["state"], _rel(v.cpu().numpy(), d["final"]))
    print("asym j10 (50 steps, 22 vectors, %s products):" % products, worst)
    assert worst["state"] < STATE_RTOL
    assert worst["cos2"] < OBS_ATOL and worst["cos"] < OBS_ATOL and worst["pops"] < OBS_ATOL


def test_asym_j10_batched_ensemble_within_mixed_precision_bound():
    """The same 50 steps on the batched mixed-precision path (complex64
    mat-vec and Krylov basis, FP64 Lanczos scalars, double-float state)."""
    from richmol_gb300.batch import Ensemble
    case, d, h0, Hdc, Hac, td, tc = _asym_j10()
    cos2, cos = _ct(case, "cos2"), _ct(case, "cos")
    v0 = td.init_state(h0, temp=5, thresh=1e-3)
    ens = Ensemble(td, h0, v0.shape[0], tol=1e-8)
    ens.load(v0)
    worst = dict(cos2=0.0, cos=0.0, pops=0.0)
    for i in range(len(tc)):
        Hac.field(d["fields"][i])
        ens.step(Hdc + Hac)
        worst["cos2"] = max(worst["cos2"], np.abs(ens.expect(cos2).real - d["cos2"][i]).max())
        worst["cos"] = max(worst["cos"], np.abs(ens.expect(cos).real - d["cos"][i]).max())
        pj = ens.populations()
        pops = np.stack([pj[J] for J in sorted(pj)], axis=1)
        worst["pops"] = max(worst["pops"], np.abs(pops - d["pops"][i]).max())
    state = _rel(ens.store().cpu().numpy(), d["final"])
    print("asym j10 batched (50 steps, 22 vectors):", worst, "state", state)
    assert worst["cos2"] < MIXED_OBS_ATOL and worst["cos"] < MIXED_OBS_ATOL and worst["pops"] < MIXED_OBS_ATOL
    assert state < MIXED_STATE_RTOL


@pytest.mark.parametrize("products", PRODUCTS)
def test_c1_molecule_matches_reference(products):
    from richmol_gb300 import TDSE
    case = "c1_j10.npz"
    d, meta = _load(case)
    h0 = _ct(case, "h0")
    Hac = _ct(case, "pol") * meta["scale"]
    cos2 = _ct(case, "cos2")
    p = meta["tdse"]
    td = TDSE(t_start=p["t_start"], t_end=p["t_end"], dt=p["dt"])
    tc = td.time_grid()
    v0 = td.init_state(h0, temp=2, thresh=1e-2)
    v = torch.from_numpy(v0).cuda()
    worst = 0.0
    for i in range(len(tc)):
        Hac.field(d["fields"][i])
        v, _ = td.update(Hac, v, H0=h0, products=products)
        worst = max(worst, np.abs(_dev_expect(cos2, v) - d["cos2"][i]).max())
    state = _rel(v.cpu().numpy()[:4], d["final"])
    print("c1 j10 (10 steps, %s products):" % products, worst, state)
    assert worst < OBS_ATOL and state < STATE_RTOL


def _oracle_ops(wl):
    from oracle.fixtures import from_cartens
    from richmol_gb300.convert_units import AUdip_x_Vm_to_invcm
    oh0 = from_cartens(wl.h0)
    oHac = from_cartens(wl.Hac)
    oHdc = (from_cartens(wl.dip) * list(wl.dc)) * (-1 * AUdip_x_Vm_to_invcm())
    return oh0, oHdc, oHac


def test_plain_j40_steps_through_pulse_match_oracle():
    """The plain FP64 drop-in configuration's operator (J <= 40, dim 91,881,
    builder factors), 10 steps of 5 fs through the pulse maximum from the
    ground state, against the oracle on the same factors."""
    from oracle.cartens import add_cartens
    from oracle.tdse import OTDSE
    from richmol_gb300 import TDSE, workloads
    wl = workloads.asym_top(Jmax=40)
    oh0, oHdc, oHac = _oracle_ops(wl)
    i0 = 195  # t = 0.975 ps: the pulse maximum at 1 ps lies inside the 10 steps
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    ot = OTDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    ot.time_grid()
    v0 = td.init_state(wl.h0, temp=0)
    vs = {p: torch.from_numpy(v0).cuda() for p in PRODUCTS}  # FP64 and double-float products
    r = v0.copy()
    c2 = from_oracle_mat(wl.cos2)
    c1 = from_oracle_mat(wl.cos)
    worst = {p: dict(state=0.0, cos2=0.0, cos=0.0) for p in PRODUCTS}
    for i in range(i0, i0 + 10):
        H = wl.hamiltonian(tc[i])
        oHac.field(wl.field(tc[i]))
        r, _ = ot.update(add_cartens(oHdc, oHac), r, H0=oh0)
        for p in PRODUCTS:
            v, _ = td.update(H, vs[p], H0=wl.h0, products=p)
            vs[p] = v
            vh = v.cpu().numpy()
            w = worst[p]
            w["state"] = max(w["state"], _rel(vh, r))
            w["cos2"] = max(w["cos2"], abs(_dev_expect(wl.cos2, v)[0] - np.vdot(r[0], c2.dot(r[0])).real))
            w["cos"] = max(w["cos"], abs(_dev_expect(wl.cos, v)[0] - np.vdot(r[0], c1.dot(r[0])).real))
    print("J<=40 plain (10 steps through the pulse):", worst, "Krylov orders", td.last_korder.tolist())
    for p in PRODUCTS:
        w = worst[p]
        assert w["state"] < STATE_RTOL and w["cos2"] < OBS_ATOL and w["cos"] < OBS_ATOL, p


def from_oracle_mat(T):
    from oracle.fixtures import from_cartens
    return from_cartens(T).tomat(form="full", cart="0")


def test_batched_j30_ensemble_through_pulse_matches_oracle():
    """The batched ensemble configuration's operator (J <= 30, dim 39,711):
    256 vectors of its thermal ensemble (the 25 with Boltzmann weight >= 1e-5
    and the next padding states) on the batched mixed-precision path, 10 steps
    of 10 fs through the pulse maximum; vectors 0, 1, 24 and 200 against the
    oracle (FP64) on the same factors."""
    from oracle.cartens import add_cartens
    from oracle.tdse import OTDSE
    from richmol_gb300 import TDSE, workloads
    from richmol_gb300.batch import Ensemble
    wl, ensd = workloads.thermal_asym_top(Jmax=30, nvec=256)
    oh0, oHdc, oHac = _oracle_ops(wl)
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    ot = OTDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    ot.time_grid()
    V0 = ensd.vectors(wl.dim)
    ens = Ensemble(td, wl.h0, 256, tol=1e-8)
    ens.load(V0)
    pick = [0, 1, 24, 200]
    r = V0[pick].copy()
    c2, c1 = from_oracle_mat(wl.cos2), from_oracle_mat(wl.cos)
    i0 = 95  # t = 0.95 - 1.05 ps
    worst = dict(state=0.0, cos2=0.0, cos=0.0, pops=0.0)
    for i in range(i0, i0 + 10):
        ens.step(wl.hamiltonian(tc[i]))
        oHac.field(wl.field(tc[i]))
        r, _ = ot.update(add_cartens(oHdc, oHac), r, H0=oh0)
        e2 = ens.expect(wl.cos2).real[pick]
        e1 = ens.expect(wl.cos).real[pick]
        worst["cos2"] = max(worst["cos2"], np.abs(e2 - [np.vdot(x, c2.dot(x)).real for x in r]).max())
        worst["cos"] = max(worst["cos"], np.abs(e1 - [np.vdot(x, c1.dot(x)).real for x in r]).max())
        pj = ens.populations()
        pops = np.stack([pj[J][pick] for J in sorted(pj)], axis=1)
        worst["pops"] = max(worst["pops"], np.abs(pops - _pops(wl.h0, r)).max())
    vs = ens.store().cpu().numpy()[pick]
    worst["state"] = max(_rel(vs[k], r[k]) for k in range(len(pick)))
    print("J<=30 batched (10 steps through the pulse):", worst, "Krylov orders", np.bincount(ens.korder()))
    assert worst["cos2"] < MIXED_OBS_ATOL and worst["cos"] < MIXED_OBS_ATOL and worst["pops"] < MIXED_OBS_ATOL
    assert worst["state"] < MIXED_STATE_RTOL
