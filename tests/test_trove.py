"""CarTensTrove (richmol/trove.py:9-672) reading the legacy OCS TROVE files
(their bytes in tests/golden/trove_files.npz) against the reference's own
CarTensTrove objects of the same files with the same state filter (even J <= 30,
m = 0; tests/golden/ocs_trove.npz, make_golden.py case_ocs_trove): the
field-free Hamiltonian and the polarizability, every block equal. CPU only."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _filt(**kw):
    ok = True
    if "J" in kw:
        ok = ok and kw["J"] <= 30 and kw["J"] % 2 == 0
    if "m" in kw:
        ok = ok and float(kw["m"]) == 0.0
    return ok


@pytest.fixture(scope="module")
def files(tmp_path_factory):
    from oracle import fixtures
    d, meta = fixtures.load(os.path.join(GOLDEN, "trove_files.npz"))
    root = tmp_path_factory.mktemp("trove")
    for i, fn in enumerate(meta["files"]):
        (root / fn).write_bytes(d[f"file{i}"].tobytes())
    return str(root)


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


@pytest.mark.parametrize("name", ["h0", "alpha"])
def test_trove_reader_matches_reference(files, name):
    from richmol_gb300 import CarTens
    from richmol_gb300.trove import CarTensTrove
    states = os.path.join(files, "ocs_energies_j0_j30.rchm")
    if name == "h0":
        T = CarTensTrove(states, bra=_filt, ket=_filt)
    else:
        T = CarTensTrove(states, os.path.join(files, "ocs_matelem_alpha_j<j1>_j<j2>.rchm"), bra=_filt, ket=_filt)
    ours, ref = T._first(), CarTens(os.path.join(GOLDEN, "ocs_trove.npz"), name=name)._first()
    for attr in ("Jlist1", "Jlist2", "symlist1", "symlist2", "dim_m1", "dim_k1", "dim_m2", "dim_k2"):
        assert getattr(ours, attr) == getattr(ref, attr), attr
    assert sorted(ours.carts) == sorted(ref.carts) and ours.rank == ref.rank
    a, b = _blocks(ours), _blocks(ref)
    assert set(a) == set(b)
    for k in b:
        assert np.array_equal(a[k], b[k]), k


def test_trove_states_and_errors(files, tmp_path):
    from richmol_gb300.trove import CarTensTrove
    states = os.path.join(files, "ocs_energies_j0_j30.rchm")
    H0 = CarTensTrove(states)  # no filter: J = 0..30, all m
    assert H0.Jlist1 == [float(J) for J in range(31)] and H0.dim_m1[30.0]["A"] == 61
    assert H0.quanta_k1[2.0]["A"][0][1] == pytest.approx(1.22063626)
    assert H0.quanta_m1[1.0]["A"] == [-1.0, 0.0, 1.0]
    bad = tmp_path / "bad_j0_j0.rchm"
    bad.write_text("Not richmol\n")
    with pytest.raises(ValueError):
        CarTensTrove(states, str(tmp_path / "bad_j<j1>_j<j2>.rchm"))
    with pytest.raises(ValueError):
        CarTensTrove(states, str(tmp_path / "none_j<j1>_j<j2>.rchm"))
