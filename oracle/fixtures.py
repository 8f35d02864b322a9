"""Reader of the golden fixtures (tests/golden/*.npz) into oracle CarTens objects.

The fixture layout is written by tests/golden/make_golden.py: all CSR blocks of
one tensor are concatenated into ``<name>/csr_data|csr_indices|csr_indptr`` with
a ``<name>/csr_table`` of (data_off, nnz, indptr_off, nrows, ncols) rows, and the
JSON ``meta`` entry lists the blocks as (kind, J1, J2, sym1, sym2, irrep, cart,
matrix_index) with kind in {"k", "m", "mf"}.
"""
import json
from collections import defaultdict

import numpy as np
from scipy.sparse import csr_matrix

from .cartens import OCarTens


def _nested():
    return defaultdict(_nested)


def _jkey(J):
    return round(float(J), 1)


def load(path):
    d = np.load(path, allow_pickle=False)
    meta = json.loads(str(d["meta"]))
    return d, meta


def tensor(d, meta, name):
    """Builds an OCarTens holding the kmat/mmat/mfmat blocks of tensor ``name``."""
    info = meta[name]
    data = d[name + "/csr_data"]
    indices = d[name + "/csr_indices"]
    indptr = d[name + "/csr_indptr"]
    table = d[name + "/csr_table"]

    def mat(i):
        doff, nnz, poff, nr, nc = (int(x) for x in table[i])
        ip = indptr[poff: poff + nr + 1] - indptr[poff]
        return csr_matrix((data[doff: doff + nnz], indices[doff: doff + nnz], ip), shape=(nr, nc))

    T = OCarTens()
    for side in ("1", "2"):
        Jlist = [_jkey(J) for J in info["Jlist" + side]]
        syml = info["symlist" + side]
        setattr(T, "Jlist" + side, Jlist)
        setattr(T, "symlist" + side, {J: list(s) for J, s in zip(Jlist, syml)})
        dm = {J: dict(zip(syml[i], info["dim_m" + side][i])) for i, J in enumerate(Jlist)}
        dk = {J: dict(zip(syml[i], info["dim_k" + side][i])) for i, J in enumerate(Jlist)}
        setattr(T, "dim_m" + side, dm)
        setattr(T, "dim_k" + side, dk)
        setattr(T, "dim" + side, {J: {s: dm[J][s] * dk[J][s] for s in dm[J]} for J in Jlist})
    if "rank" in info:
        T.rank = info["rank"]
    if "cart" in info:
        T.cart = list(info["cart"])
    T.kmat = _nested()
    has_m = any(b[0] == "m" for b in info["blocks"])
    has_mf = any(b[0] == "mf" for b in info["blocks"])
    if has_m:
        T.mmat = _nested()
    if has_mf:
        T.mfmat = _nested()
    for kind, J1, J2, s1, s2, irrep, cart, idx in info["blocks"]:
        key = (_jkey(J1), _jkey(J2))
        if kind == "k":
            T.kmat[key][(s1, s2)][irrep] = mat(idx)
        elif kind == "m":
            T.mmat[key][(s1, s2)][irrep][cart] = mat(idx)
        else:
            T.mfmat[key][(s1, s2)][irrep] = mat(idx)
    return T


def init_rows(d, lab):
    """Dense initial-state array of a sparse-stored init_state fixture."""
    shape = tuple(int(x) for x in d[lab + "/shape"])
    v = np.zeros(shape, dtype=np.complex128)
    v[d[lab + "/rows"], d[lab + "/cols"]] = d[lab + "/vals"]
    return v


def from_cartens(T):
    """Oracle copy of a tensor made by the in-house factor builder
    (richmol_gb300.CarTens with one factor source): the same K and M blocks in
    an OCarTens, the part's scale applied as the reference's mul() would
    (field.py:932-1070). Test infrastructure: lets the oracle propagate the
    builder's operators at sizes the reference cannot build here."""
    src = T._parts[0].src
    o = OCarTens()
    for k in ("Jlist1", "Jlist2", "symlist1", "symlist2", "dim_m1", "dim_m2", "dim_k1", "dim_k2", "dim1", "dim2",
              "mmat", "rank"):
        setattr(o, k, getattr(src, k))
    # own copy of the K dictionaries: mul() replaces their entries
    o.kmat = {Jp: {sp: dict(kS) for sp, kS in kJ.items()} for Jp, kJ in src.kmat.items()}
    o.cart = src.carts
    if T._parts[0].kscale != 1:
        o.mul(T._parts[0].kscale)
    return o
