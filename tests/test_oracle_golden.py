"""Pins the CPU oracle against outputs of the reference itself.

The fixtures in tests/golden were produced by running the reference
(CFEL-CMI/richmol) in the development container, see tests/golden/make_golden.py.
These tests run on CPU only.
"""
import os

import numpy as np
import pytest

from oracle import fixtures
from oracle.cartens import add_cartens, flat, split
from oracle.tdse import MaxOrderError, OTDSE, expmv_lanczos

from conftest import GOLDEN


def _load(name):
    return fixtures.load(os.path.join(GOLDEN, name))


def _close(a, b, rel=1e-12):
    a, b = np.asarray(a), np.asarray(b)
    scale = max(np.abs(b).max(), 1e-300)
    assert np.abs(a - b).max() <= rel * scale, (np.abs(a - b).max(), scale)


@pytest.mark.parametrize("case", ["ocs_j6.npz", "asym_j4.npz"])
@pytest.mark.parametrize("tens", ["pol", "dip"])
def test_field_matches_reference_mfmat(case, tens):
    d, meta = _load(case)
    T = fixtures.tensor(d, meta, tens)
    ref_mf = T.mfmat
    T.field(meta["field_vec"])
    assert set(T.mfmat.keys()) == set(ref_mf.keys())
    for Jp, mJ in ref_mf.items():
        assert set(T.mfmat[Jp].keys()) == set(mJ.keys())
        for sp, mS in mJ.items():
            assert set(T.mfmat[Jp][sp].keys()) == set(mS.keys())
            for irrep, m in mS.items():
                _close(T.mfmat[Jp][sp][irrep].toarray(), m.toarray(), 1e-14)


def test_field_threshold_matches_reference():
    d, meta = _load("ocs_j6.npz")
    pol = fixtures.tensor(d, meta, "pol")
    ref = fixtures.tensor(d, meta, "pol_thresh").mfmat
    f, thr = meta["thresh_field"]
    pol.field(f, thresh=thr)
    assert set(pol.mfmat.keys()) == set(ref.keys())
    for Jp in ref:
        for sp in ref[Jp]:
            for irrep in ref[Jp][sp]:
                # pol_thresh was scaled by -0.5*AUpol; compare the sparsity pattern
                a = pol.mfmat[Jp][sp][irrep]
                b = ref[Jp][sp][irrep]
                assert a.nnz == b.nnz
                assert (a.indices == b.indices).all()


@pytest.mark.parametrize("case", ["ocs_j6.npz", "asym_j4.npz"])
@pytest.mark.parametrize("tens", ["pol", "dip"])
def test_vec_matches_reference(case, tens):
    d, meta = _load(case)
    T = fixtures.tensor(d, meta, tens)
    T.field(meta["field_vec"])
    for x, y in zip(d[tens + "/vec_x"], d[tens + "/vec_y"]):
        _close(flat(T, T.vec(split(T, x)), "1"), y, 1e-13)


def test_sum_vec_matches_reference():
    d, meta = _load("asym_j4.npz")
    dip = fixtures.tensor(d, meta, "dip")
    pol = fixtures.tensor(d, meta, "pol")
    sc = meta["scales"]
    Hdc = (dip * meta["dc"]) * sc["dc"]
    Hac = (pol * sc["ac"]) * meta["field_vec"]
    H = add_cartens(Hdc, Hac)
    x, y = d["sum/vec_x"][0], d["sum/vec_y"][0]
    _close(flat(H, H.vec(split(H, x)), "1"), y, 1e-13)


def test_lanczos_matches_reference():
    d, meta = _load("lanczos.npz")
    H = d["H"]
    for ic, c in enumerate(meta["cases"][:3]):
        fac = complex(*c["fac"])
        st = {}
        u = expmv_lanczos(d["v%d" % ic], fac, lambda x: H.dot(x), stats=st)
        assert st["nmatvec"] == c["nmatvec"]
        _close(u, d["u%d" % ic], 1e-12)
        # and it is the exact exponential to the convergence tolerance
        w, Q = np.linalg.eigh(H)
        exact = Q @ (np.exp(fac * w) * (Q.conj().T @ d["v%d" % ic]))
        assert np.abs(u - exact).max() < 1e-7
    assert meta["cases"][3]["maxorder_error"]
    with pytest.raises(MaxOrderError):
        expmv_lanczos(d["v1"], -20j, lambda x: H.dot(x), maxorder=6)
    u0 = expmv_lanczos(d["v0"], -0.1j, lambda x: np.zeros_like(x))
    assert np.array_equal(u0, d["u_zero"])


def test_split_operator_ocs_matches_reference():
    d, meta = _load("ocs_j6.npz")
    h0 = fixtures.tensor(d, meta, "h0")
    pol = fixtures.tensor(d, meta, "pol")
    sp = meta["split"]
    Hac = pol * sp["scale"]
    td = OTDSE(t_start=sp["t_start"], t_end=sp["t_end"], dt=sp["dt"])
    tc = td.time_grid()
    np.testing.assert_allclose(tc, d["split/tc"], rtol=0, atol=1e-15)
    vecs = td.init_state(h0, temp=0)
    _close(vecs, d["split/vec0"], 0)
    for i in range(len(tc)):
        Hac.field(d["split/fields"][i])
        vecs, t2 = td.update(Hac, vecs, H0=h0)
        assert abs(t2 - d["split/times"][i]) < 1e-15
        _close(vecs, d["split/states"][i], 1e-10)


def test_full_h_ocs_matches_reference():
    d, meta = _load("ocs_j6.npz")
    h0 = fixtures.tensor(d, meta, "h0")
    pol = fixtures.tensor(d, meta, "pol")
    f = meta["full"]
    Hac = pol * meta["split"]["scale"]
    td = OTDSE(t_start=f["t_start"], t_end=f["t_end"], dt=f["dt"])
    td.time_grid()
    vecs = d["full/vec0"]
    for i in range(5):
        Hac.field(f["field"])
        H = add_cartens(Hac, h0)
        vecs, _ = td.update(H, vecs)
        _close(vecs, d["full/states"][i], 1e-10)


def test_split_operator_asym_multivector_matches_reference():
    d, meta = _load("asym_j4.npz")
    h0 = fixtures.tensor(d, meta, "h0")
    dip = fixtures.tensor(d, meta, "dip")
    pol = fixtures.tensor(d, meta, "pol")
    sc = meta["scales"]
    Hdc = (dip * meta["dc"]) * sc["dc"]
    Hac = pol * sc["ac"]
    sp = meta["split"]
    td = OTDSE(t_start=sp["t_start"], t_end=sp["t_end"], dt=sp["dt"])
    tc = td.time_grid()
    assert len(tc) == len(d["split/tc"]) == 19  # int((1.0-0.9)/0.005) truncates
    vecs = td.init_state(h0, temp=5, thresh=1e-3)
    _close(vecs, d["split/vec0"], 1e-15)
    for i in range(len(tc)):
        Hac.field(d["split/fields"][i])
        vecs, _ = td.update(add_cartens(Hdc, Hac), vecs, H0=h0)
        _close(vecs[:2], d["split/states_first2"][i], 1e-10)
    _close(vecs, d["split/final"], 1e-10)


@pytest.mark.parametrize("lab,kw", [("t0", dict(temp=0)), ("t5", dict(temp=5, thresh=1e-3)),
                                    ("t50", dict(temp=50, thresh=1e-6)), ("tnone", dict(temp=None))])
def test_init_state_matches_reference(lab, kw):
    d, meta = _load("asym_j4.npz")
    h0 = fixtures.tensor(d, meta, "h0")
    td = OTDSE(t_end=1.0, dt=0.01)
    v = td.init_state(h0, **kw)
    _close(v, fixtures.init_rows(d, "init/" + lab), 1e-14)


def test_init_state_dense_eigh_matches_reference_up_to_phase():
    d, meta = _load("asym_j4.npz")
    h0 = fixtures.tensor(d, meta, "h0")
    dip = fixtures.tensor(d, meta, "dip")
    Hdc = (dip * meta["dc"]) * meta["scales"]["dc"]
    td = OTDSE(t_end=1.0, dt=0.01)
    v = td.init_state(add_cartens(h0, Hdc), temp=0)[0]
    r = d["init/dressed_t0"][0]
    assert abs(abs(np.vdot(v, r)) - 1) < 1e-12


def test_legacy_ocs_alignment_populations():
    """tests/benchmarks/data/alignment_ocs: J-populations of the reference's own
    known answer (pop_reference.txt) to 1e-3 (tests/test_tdse.py:107-110), and
    the reference's own replay to 1e-10."""
    d, meta = _load("ocs_trove.npz")
    h0 = fixtures.tensor(d, meta, "h0")
    alpha = fixtures.tensor(d, meta, "alpha")
    Hbar = alpha * meta["scale"]
    n = meta["nsteps"]
    td = OTDSE(t_end=n * 0.01, dt=0.01)
    td.time_grid()
    vecs = td.init_state(h0, temp=0)
    pops, states = [], []
    for i in range(n):
        Hbar.field(d["fields"][i])
        vecs, _ = td.update(Hbar, vecs, H0=h0)
        if i % 10 == 0:
            pops.append(np.abs(vecs[0][:7]) ** 2)
        if i % 50 == 49:
            states.append(vecs.copy())
    pops = np.array(pops)
    assert np.abs(pops - d["pop_reference"][: len(pops)]).max() < 1e-3
    _close(pops, d["pops"], 1e-9)
    _close(np.array(states), d["states"], 1e-9)


@pytest.mark.slow
def test_readme_truncated_pulse_trace():
    """README.md:246-330 known answer, OCS J<=10: the reference's own replay to
    1e-9 and the published <cos^2 theta> trace (0.1 ps samples) to 5e-3."""
    path = os.path.join(GOLDEN, "trunc_pulse_j10.npz")
    if not os.path.exists(path):
        pytest.skip("trunc_pulse fixture not generated")
    d, meta = fixtures.load(path)
    h0 = fixtures.tensor(d, meta, "h0")
    pol = fixtures.tensor(d, meta, "pol")
    cos2 = fixtures.tensor(d, meta, "cos2")
    c2 = cos2.tomat(form="full", cart="0")
    n = 600  # 6 ps keeps the CPU suite short; the fixture holds the full replay
    td = OTDSE(t_start=0, t_end=meta["nsteps"] * 0.01, dt=0.01)
    td.time_grid()
    vecs = td.init_state(h0, temp=0)
    H = pol * meta["scale"]
    out = []
    for i in range(n):
        H.field([0, 0, d["fields"][i, 2]])
        vecs, t2 = td.update(H, vecs, H0=h0)
        out.append(np.vdot(vecs[0], c2.dot(vecs[0])).real + 1 / 3)
    out = np.array(out)
    assert np.abs(out - d["cos2"][:n]).max() < 1e-9
    ref = d["cos2_reference"]
    times = d["times"][:n]
    sel = ref[:, 0] <= times[-1]
    dev = np.abs(np.interp(ref[sel, 0], times, out) - ref[sel, 1])
    assert dev.max() < 5e-3
