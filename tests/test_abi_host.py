"""CPU checks of the boundary: the C-ABI library loads and exports every entry
point declared in include/*.h, and the host-side plan compilation (ELL
conversion, K classification, factor files) is correct. No compute call runs."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest
from scipy.sparse import random as sprandom

from conftest import GOLDEN, ROOT


def _declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(kr_\w+)\s*\(", txt))
    return names


@pytest.fixture(scope="module")
def libpath():
    from richmol_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        _native.build_library()
    return _native.LIB_PATH


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    declared = _declared_symbols()
    assert len(declared) >= 11
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, missing
    from richmol_gb300 import _native
    assert set(_native.EXPORTED) <= declared


def test_header_cites_reference():
    txt = open(os.path.join(ROOT, "include", "richmol_gb300.h")).read()
    for cite in ("tdse.py:265-414", "tdse.py:417-486", "field.py:1073-1142", "field.py:1145-1245"):
        assert cite in txt


def test_ell_matches_dense():
    from richmol_gb300.plan import _ell
    rng = np.random.default_rng(0)
    mats = [sprandom(7, 9, density=0.3, random_state=s, format="csr") * (1 + 1j) for s in range(3)]
    width, col, val = _ell(mats, 7, 9)
    for ci, m in enumerate(mats):
        dense = np.zeros((7, 9), complex)
        for i in range(7):
            for w in range(width):
                dense[i, col[i * width + w]] += val[ci, i * width + w]
        assert np.allclose(dense, m.toarray())


def test_k_classification():
    from richmol_gb300 import _native
    from richmol_gb300.plan import _ktype
    assert _ktype(np.array([[1.0, 2.0]], complex))[0] == _native.KR_K_REAL
    assert _ktype(np.array([[1j, 0]], complex))[0] == _native.KR_K_IMAG
    assert _ktype(np.array([[1 + 1j, 0]], complex))[0] == _native.KR_K_COMPLEX


def test_compiled_source_terms_cover_reference_blocks():
    """Every (J1,J2,s1,s2,irrep) present in both kmat and mmat becomes one term,
    and D2 symmetry pairs share M groups."""
    from richmol_gb300 import CarTens
    from richmol_gb300.plan import compiled
    T = CarTens(os.path.join(GOLDEN, "asym_j4.npz"), name="pol")
    src = T._parts[0].src
    cs = compiled(src)
    nblocks = sum(1 for Jp in src.kmat for sp in src.kmat[Jp] for i in src.kmat[Jp][sp]
                  if Jp in src.mmat and sp in src.mmat[Jp] and i in src.mmat[Jp][sp])
    assert len(cs.terms) == nblocks
    assert len(cs.groups) < nblocks


def test_factor_file_roundtrip(tmp_path):
    from richmol_gb300 import CarTens
    T = CarTens(os.path.join(GOLDEN, "ocs_j6.npz"), name="dip") * 2.5
    f = str(tmp_path / "dip.npz")
    T.store(f, "dip")
    U = CarTens(f, name="dip")
    for Jp in T.kmat:
        for sp in T.kmat[Jp]:
            for i in T.kmat[Jp][sp]:
                assert np.allclose(T.kmat[Jp][sp][i].toarray(), U.kmat[Jp][sp][i].toarray())


def test_host_algebra_matches_oracle():
    """Sum/scale/field bookkeeping of the facade gives the same assembled
    matrix as the oracle restatement of field.py (host tomat path)."""
    from oracle import fixtures
    from oracle.cartens import add_cartens
    from richmol_gb300 import CarTens
    d, meta = fixtures.load(os.path.join(GOLDEN, "asym_j4.npz"))
    sc = meta["scales"]
    o_dip, o_pol = fixtures.tensor(d, meta, "dip"), fixtures.tensor(d, meta, "pol")
    o_H = add_cartens((o_dip * meta["dc"]) * sc["dc"], (o_pol * sc["ac"]) * meta["field_vec"])
    p = os.path.join(GOLDEN, "asym_j4.npz")
    H = (CarTens(p, name="dip") * meta["dc"]) * sc["dc"] + (CarTens(p, name="pol") * sc["ac"]) * meta["field_vec"]
    a = H.tomat(form="full").toarray()
    b = o_H.tomat(form="full").toarray()
    assert np.abs(a - b).max() <= 1e-14 * np.abs(b).max()
