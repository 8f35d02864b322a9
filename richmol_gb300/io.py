"""Factor files: the blocks of Cartesian tensor operators in one ``.npz``.

Layout (one archive may hold several tensors, each under its own name):

* ``<name>/csr_data``    complex128, all CSR blocks' values, concatenated;
* ``<name>/csr_indices`` int64, their column indices;
* ``<name>/csr_indptr``  int64, their row pointers;
* ``<name>/csr_table``   int64 (nmat, 5): data offset, nnz, indptr offset, rows, cols;
* ``meta``               JSON: per tensor the bra/ket bases (Jlist, symlist,
  dim_m, dim_k), ``rank``, ``cart`` and the block list
  (kind, J1, J2, sym1, sym2, irrep, cart, matrix index), kind "k", "m" or "mf".

``read_tensor`` also reads the reference's own HDF5 files (richmol/field.py:
1304-1848: a group per tensor holding ``J:<J1>,<J2>/sym:<s1>,<s2>`` groups with
kmat_* / mmat_* datasets and their split attributes), through the numpy
HDF5 reader in richmol_gb300.hdf5, so factor files from richmol's database
load directly. Writing stays in the ``.npz`` layout above; the block keys and
the CSR content are the same in both.
"""
import json
import re
from collections import defaultdict

import numpy as np
from scipy.sparse import csr_matrix

from . import hdf5


def _nested():
    return defaultdict(_nested)


def jkey(J):
    return round(float(J), 1)


# group names of field.py:1885-1898 (J_group_key, sym_group_key)
_J_GROUP = re.compile(r"^J:(\d+\.\d+),(\d+\.\d+)$")
_SYM_GROUP = re.compile(r"^sym:(\w+),(\w+)$")


def _h5_attrs(group):
    """Attributes with the ``__json`` ones decoded (field.py:1647-1655)."""
    out = {}
    for key, val in group.attrs.items():
        if key.endswith("__json"):
            out[key[: -len("__json")]] = json.loads(val)
        else:
            out[key] = val
    return out


def _str(x):
    return x.decode("utf-8") if isinstance(x, (bytes, np.bytes_)) else str(x)


def _irrep(x):
    s = _str(x)
    try:
        return int(s)
    except ValueError:
        return s


def _h5_split(group, prefix, n):
    """The n CSR matrices of kmat_* or mmat_* (field.py:1755-1830): the
    concatenated datasets split by the per-matrix counts in the attributes."""
    a = group.attrs
    data = group[prefix + "_data"][()]
    ind = group[prefix + "_indices"][()]
    ptr = group[prefix + "_indptr"][()]
    cd, ci, cp = (np.concatenate([[0], np.cumsum(a[prefix + k])]) for k in ("_nnz", "_nind", "_nptr"))
    shape = np.asarray(a[prefix + "_shape"]).reshape(n, 2)
    out = []
    for i in range(n):
        out.append(csr_matrix((data[cd[i]: cd[i + 1]].astype(np.complex128),
                               ind[ci[i]: ci[i + 1]], ptr[cp[i]: cp[i + 1]]),
                              shape=(int(shape[i, 0]), int(shape[i, 1]))))
    return out


def read_tensor_h5(filename, name):
    """Reads a tensor stored by the reference's CarTens.store (field.py:
    1600-1848, without state filters or threshold). Returns the same tuple as
    read_tensor; mfmat is None (the reference stores kmat and mmat only)."""
    with hdf5.File(filename) as fl:
        if name not in fl:
            raise KeyError(f"file '{filename}' has no dataset with the name '{name}'")
        group = fl[name]
        attrs = _h5_attrs(group)
        cls = _str(attrs.get("__class_name__", ""))
        if not cls.endswith("CarTens") and not cls.endswith("LabTensor"):
            raise TypeError(f"dataset with the name '{name}' in file '{filename}' has different type: '{cls}'")
        basis = {}
        for side in ("1", "2"):
            Jlist = [jkey(J) for J in np.atleast_1d(attrs["Jlist" + side])]
            syml = {jkey(J): list(v) for J, v in attrs["symlist" + side].items()}
            basis["Jlist" + side] = Jlist
            basis["symlist" + side] = {J: syml[J] for J in Jlist}
            for kind in ("dim_m", "dim_k"):
                d = {jkey(J): {s: int(n) for s, n in v.items()} for J, v in attrs[kind + side].items()}
                basis[kind + side] = {J: d[J] for J in Jlist}
            # state quanta (field.py:58-170): m of each M row, (label, energy) of each K state
            if "quanta_m" + side in attrs:
                q = {jkey(J): {s: [int(m) for m in ms] for s, ms in v.items()}
                     for J, v in attrs["quanta_m" + side].items()}
                basis["quanta_m" + side] = {J: q[J] for J in Jlist}
            if "quanta_k" + side in attrs:
                q = {jkey(J): {s: [(str(a), None if e is None else float(e)) for a, e in ks] for s, ks in v.items()}
                     for J, v in attrs["quanta_k" + side].items()}
                basis["quanta_k" + side] = {J: q[J] for J in Jlist}
        rank = int(attrs["rank"])
        cart = [_str(c) for c in np.atleast_1d(attrs["cart"])]
        kmat, mmat = _nested(), _nested()
        for jname in group.keys():
            mj = _J_GROUP.match(jname)
            if mj is None:
                continue
            Jp = (jkey(mj.group(1)), jkey(mj.group(2)))
            gj = group[jname]
            for sname in gj.keys():
                ms = _SYM_GROUP.match(sname)
                if ms is None:
                    continue
                sp = (ms.group(1), ms.group(2))
                gs = gj[sname]
                if "kmat_irreps" in gs.attrs:
                    irreps = [_irrep(x) for x in np.atleast_1d(gs.attrs["kmat_irreps"])]
                    for irrep, m in zip(irreps, _h5_split(gs, "kmat", len(irreps))):
                        kmat[Jp][sp][irrep] = m
                if "mmat_irrep_cart" in gs.attrs:
                    ic = np.asarray(gs.attrs["mmat_irrep_cart"]).reshape(-1, 2)
                    for (irrep, c), m in zip(ic, _h5_split(gs, "mmat", len(ic))):
                        mmat[Jp][sp][_irrep(irrep)][_str(c)] = m
    return basis, kmat, mmat, None, rank, cart


def _drop_small(blocks, depth, thresh):
    """Zeroes elements below thresh in nested dicts of CSR matrices (depth =
    the number of dict levels above a matrix) and removes matrices, then
    dicts, left empty (field.py:1780-1840)."""
    for key in list(blocks.keys()):
        val = blocks[key]
        if depth == 1:
            m = val.copy()
            m.data[np.abs(m.data) < thresh] = 0
            m.eliminate_zeros()
            if m.nnz > 0:
                blocks[key] = m
            else:
                del blocks[key]
        else:
            _drop_small(val, depth - 1, thresh)
            if len(val) == 0:
                del blocks[key]


def read_tensor(filename, name, thresh=None):
    """Returns (basis dict, kmat, mmat, mfmat or None, rank, cart); with
    thresh, matrix elements below it are dropped (field.py:1600-1848)."""
    if hdf5.is_hdf5(filename):
        out = read_tensor_h5(filename, name)
    else:
        out = _read_tensor_npz(filename, name)
    if thresh is not None:
        basis, kmat, mmat, mfmat, rank, cart = out
        _drop_small(kmat, 3, thresh)   # [J pair][sym pair][irrep]
        _drop_small(mmat, 4, thresh)   # [J pair][sym pair][irrep][cart]
        if mfmat is not None:
            _drop_small(mfmat, 3, thresh)
    return out


def _read_tensor_npz(filename, name):
    d = np.load(filename, allow_pickle=False)
    meta = json.loads(str(d["meta"]))
    if name not in meta:
        raise KeyError(f"tensor '{name}' not found in '{filename}'")
    info = meta[name]
    data = d[name + "/csr_data"]
    indices = d[name + "/csr_indices"]
    indptr = d[name + "/csr_indptr"]
    table = d[name + "/csr_table"]

    def mat(i):
        doff, nnz, poff, nr, nc = (int(x) for x in table[i])
        ip = indptr[poff: poff + nr + 1] - indptr[poff]
        return csr_matrix((data[doff: doff + nnz], indices[doff: doff + nnz], ip), shape=(nr, nc))

    basis = {}
    for side in ("1", "2"):
        Jlist = [jkey(J) for J in info["Jlist" + side]]
        syml = info["symlist" + side]
        basis["Jlist" + side] = Jlist
        basis["symlist" + side] = {J: list(s) for J, s in zip(Jlist, syml)}
        basis["dim_m" + side] = {J: dict(zip(syml[i], info["dim_m" + side][i])) for i, J in enumerate(Jlist)}
        basis["dim_k" + side] = {J: dict(zip(syml[i], info["dim_k" + side][i])) for i, J in enumerate(Jlist)}
        if "quanta_m" + side in info:
            basis["quanta_m" + side] = {J: dict(zip(syml[i], info["quanta_m" + side][i])) for i, J in enumerate(Jlist)}
        if "quanta_k" + side in info:
            basis["quanta_k" + side] = {J: {s: [(str(a), e) for a, e in ks] for s, ks in zip(syml[i], info["quanta_k" + side][i])}
                                        for i, J in enumerate(Jlist)}
    kmat, mmat, mfmat = _nested(), _nested(), None
    for kind, J1, J2, s1, s2, irrep, cart, idx in info["blocks"]:
        key = (jkey(J1), jkey(J2))
        if kind == "k":
            kmat[key][(s1, s2)][irrep] = mat(idx)
        elif kind == "m":
            mmat[key][(s1, s2)][irrep][cart] = mat(idx)
        elif kind == "mf":
            if mfmat is None:
                mfmat = _nested()
            mfmat[key][(s1, s2)][irrep] = mat(idx)
    return basis, kmat, mmat, mfmat, info.get("rank"), info.get("cart")


def write_tensors(filename, tensors):
    """tensors: {name: CarTens}. Writes kmat (with the K scale applied) and mmat."""
    out, meta = {}, {}
    for name, T in tensors.items():
        src = T._single_source()
        scale = T._parts[0].kscale
        blocks, data, indices, indptr, table = [], [], [], [], []
        nd = ni = 0

        def add(m):
            nonlocal nd, ni
            m = csr_matrix(m)
            m.sort_indices()
            table.append((nd, m.nnz, ni, m.shape[0], m.shape[1]))
            data.append(m.data.astype(np.complex128))
            indices.append(m.indices.astype(np.int64))
            indptr.append(m.indptr.astype(np.int64))
            nd += m.nnz
            ni += m.shape[0] + 1
            return len(table) - 1

        for (J1, J2), kJ in src.kmat.items():
            for (s1, s2), kS in kJ.items():
                for irrep, km in kS.items():
                    blocks.append(("k", J1, J2, s1, s2, irrep, None, add(km * scale)))
        for (J1, J2), mJ in src.mmat.items():
            for (s1, s2), mS in mJ.items():
                for irrep, mI in mS.items():
                    for cart, mm in mI.items():
                        blocks.append(("m", J1, J2, s1, s2, irrep, cart, add(mm)))
        info = {"blocks": [list(b) for b in blocks], "rank": src.rank, "cart": list(src.carts)}
        for side in ("1", "2"):
            Jl = getattr(src, "Jlist" + side)
            sl = getattr(src, "symlist" + side)
            info["Jlist" + side] = list(Jl)
            info["symlist" + side] = [list(sl[J]) for J in Jl]
            info["dim_m" + side] = [[int(getattr(src, "dim_m" + side)[J][s]) for s in sl[J]] for J in Jl]
            info["dim_k" + side] = [[int(getattr(src, "dim_k" + side)[J][s]) for s in sl[J]] for J in Jl]
            qm = getattr(src, "quanta_m" + side)
            qk = getattr(src, "quanta_k" + side)
            info["quanta_m" + side] = [[[int(m) for m in qm[J][s]] for s in sl[J]] for J in Jl]
            info["quanta_k" + side] = [[[[str(a), None if e is None else float(e)] for a, e in qk[J][s]] for s in sl[J]]
                                       for J in Jl]
        meta[name] = info
        cat = lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)
        out[name + "/csr_data"] = cat(data, np.complex128)
        out[name + "/csr_indices"] = cat(indices, np.int64)
        out[name + "/csr_indptr"] = cat(indptr, np.int64)
        out[name + "/csr_table"] = np.array(table, np.int64).reshape(-1, 5)
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(filename, **out)
