"""State filters of CarTens (richmol/field.py:187-447, filter at 1859-1882)
against the reference's own filtered tensors (tests/golden/filter_j4.npz,
make_golden.py case_filter: its D2 asymmetric top at J <= 4, h0 and pol, with
their state quanta). The filters (restated from make_golden.filter_predicates):
m = 0 on both sides; bra states below 60 cm^-1 and ket states with J <= 3 and
not B3; m = 0 with elements below 1e-3 dropped. The cut blocks are slices of
the same matrices, so they must agree exactly. CPU only."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASE = os.path.join(GOLDEN, "filter_j4.npz")


def _predicates():
    m0 = lambda **kw: kw["m"] == 0 if "m" in kw else True
    low = lambda **kw: kw["enr"] < 60.0 if "enr" in kw else True
    j3 = lambda **kw: kw["J"] <= 3 and kw["sym"] != "B3"
    return {"m0": (m0, m0, None), "enr_j": (low, j3, None), "m0_thresh": (m0, m0, 1e-3)}


def _blocks(src):
    out = {}
    for Jp, kJ in src.kmat.items():
        for sp, kS in kJ.items():
            for irrep, m in kS.items():
                out[("k", Jp, sp, irrep, None)] = m.toarray()
    for Jp, mJ in src.mmat.items():
        for sp, mS in mJ.items():
            for irrep, mI in mS.items():
                for c, m in mI.items():
                    out[("m", Jp, sp, irrep, c)] = m.toarray()
    return out


@pytest.mark.parametrize("fname", ["m0", "enr_j", "m0_thresh"])
@pytest.mark.parametrize("name", ["h0", "pol"])
def test_filter_matches_reference(name, fname):
    from richmol_gb300.field import CarTens, filter
    bra, ket, thresh = _predicates()[fname]
    T = CarTens(CASE, name=name)
    ours = filter(T, bra, ket, thresh=thresh)._first()
    ref = CarTens(CASE, name=f"{name}_{fname}")._first()
    for side in ("1", "2"):
        for attr in ("Jlist", "symlist", "dim_m", "dim_k", "quanta_m"):
            assert getattr(ours, attr + side) == getattr(ref, attr + side), (attr, side)
        qa, qb = getattr(ours, "quanta_k" + side), getattr(ref, "quanta_k" + side)
        assert {J: {s: [q for q, _ in v] for s, v in d.items()} for J, d in qa.items()} == \
               {J: {s: [q for q, _ in v] for s, v in d.items()} for J, d in qb.items()}
        assert all(abs(a[1] - b[1]) < 1e-12 for J in qa for s in qa[J] for a, b in zip(qa[J][s], qb[J][s]))
    a, b = _blocks(ours), _blocks(ref)
    assert set(a) == set(b)
    for k in b:
        assert a[k].shape == b[k].shape and np.array_equal(a[k], b[k]), k
    # the original is left as it was
    assert CarTens(CASE, name=name)._first().dim_m1 == T._first().dim_m1


def test_filter_in_place_keeps_fields_and_sums():
    """CarTens.filter cuts every part of a sum alike and keeps the field
    products; reading with bra/ket filters (CarTens(filename, name, bra=, ket=),
    field.py:172) gives the same tensor as filtering after reading."""
    from richmol_gb300.field import CarTens, filter
    bra, ket, _ = _predicates()["enr_j"]
    h0 = CarTens(CASE, name="h0")
    pol = CarTens(CASE, name="pol")
    pol.field([1e3, -2e3, 5e3])
    H = h0 + pol
    Hf = filter(H, bra, ket)
    assert Hf._is_sum and len(Hf._parts) == 2
    assert Hf._parts[1].prods == H._parts[1].prods
    assert Hf.Jlist2 == [0.0, 1.0, 2.0, 3.0] and all("B3" not in Hf.symlist2[J] for J in Hf.Jlist2)
    read = CarTens(CASE, name="pol", bra=bra, ket=ket)
    cut = filter(CarTens(CASE, name="pol"), bra, ket)
    assert _blocks(read._first()).keys() == _blocks(cut._first()).keys()
    # the full matrix of the cut tensor is the matching sub-matrix of the full one
    fm = pol.tomat(form="full", cart="zz").toarray()
    pf = filter(pol, bra, ket)
    cm = pf.tomat(form="full", cart="zz").toarray()

    def keep(T, Tf, side):
        idx, off = [], 0
        qk, qm = getattr(T._first(), "quanta_k" + side), getattr(T._first(), "quanta_m" + side)
        qkf, qmf = getattr(Tf._first(), "quanta_k" + side), getattr(Tf._first(), "quanta_m" + side)
        for J in getattr(T, "Jlist" + side):
            for s in getattr(T, "symlist" + side)[J]:
                nm, nk = len(qm[J][s]), len(qk[J][s])
                if J in qkf and s in qkf[J]:
                    km = [i for i, q in enumerate(qk[J][s]) if q in qkf[J][s]]
                    mm = [i for i, q in enumerate(qm[J][s]) if q in qmf[J][s]]
                    idx += [off + a * nk + b for a in mm for b in km]
                off += nm * nk
        return idx

    r, c = keep(pol, pf, "1"), keep(pol, pf, "2")
    assert cm.shape == (len(r), len(c))
    assert np.array_equal(cm, fm[np.ix_(r, c)])


def test_filter_m_subset_dimensions_match_notebook():
    """rotations_quickstart.ipynb printed the dimensions of water's dipole
    (water.h5, J <= 5) filtered to one m at a time: 11, 20, 27, 32, 35, 36,
    35, 32, 27, 20, 11 for m = -5..5."""
    import tempfile
    from richmol_gb300.field import CarTens, filter
    d = np.load(os.path.join(GOLDEN, "h5_files.npz"))
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "water.h5")
        with open(path, "wb") as f:
            f.write(d["water_h5"].tobytes())
        dip = CarTens(path, name="dip")
        dims = []
        for m_ in range(-5, 6):
            flt = lambda **kw: kw["m"] == m_ if "m" in kw else True
            dims.append(filter(dip, flt, flt).tomat(form="full", cart="z").shape[0])
    assert dims == [11, 20, 27, 32, 35, 36, 35, 32, 27, 20, 11]


def test_assign_full_and_block_forms_follow_the_reference_order():
    """assign (field.py:572-657) lists the states in the row/column order of
    tomat; full_form and block_form (field.py:660-737) convert between the
    block dictionary and that matrix. For the reference's own D2 J<=4 h0 the
    diagonal of tomat carries each state's energy (its K label's energy)."""
    from richmol_gb300.field import CarTens, filter
    h0 = CarTens(CASE, name="h0")
    a1, a2 = h0.assign(form="full")
    H = h0.tomat(form="full", cart="0")
    assert len(a1["m"]) == H.shape[0] == sum(sum(v.values()) for v in h0.dim1.values())
    assert np.allclose(H.diagonal().real, [e for _, e in a1["k"]], atol=1e-9)
    blk = h0.assign(form="block")[0]
    J, s = 2.0, "A"
    assert blk[J][s]["m"][: h0.dim_k1[J][s]] == [-2] * h0.dim_k1[J][s]  # m outer, k inner
    pol = CarTens(CASE, name="pol")
    pol.field([0.2, -0.4, 1.0])
    full = pol.tomat(form="full", repres="csr_matrix")
    b = pol.block_form(full)
    back = pol.full_form(b)
    assert abs(back - full).max() == 0
    dense = pol.block_form(full.toarray())
    assert set(dense) == set(b)
    # after a filter the assignment lists only the kept states
    m0 = lambda **kw: kw["m"] == 0 if "m" in kw else True
    f1, _ = filter(h0, m0, m0).assign(form="full")
    assert set(f1["m"]) == {0} and len(f1["m"]) == sum(sum(v.values()) for v in filter(h0, m0, m0).dim1.values())
