"""Factor files: the blocks of Cartesian tensor operators in one ``.npz``.

Layout (one archive may hold several tensors, each under its own name):

* ``<name>/csr_data``    complex128, all CSR blocks' values, concatenated;
* ``<name>/csr_indices`` int64, their column indices;
* ``<name>/csr_indptr``  int64, their row pointers;
* ``<name>/csr_table``   int64 (nmat, 5): data offset, nnz, indptr offset, rows, cols;
* ``meta``               JSON: per tensor the bra/ket bases (Jlist, symlist,
  dim_m, dim_k), ``rank``, ``cart`` and the block list
  (kind, J1, J2, sym1, sym2, irrep, cart, matrix index), kind "k", "m" or "mf".

This stands in for the reference's HDF5 layout (richmol/field.py:1304-1848,
groups ``J:<J1>,<J2>/sym:<s1>,<s2>`` with kmat_* / mmat_* datasets), which
needs h5py; the block keys and the CSR content are the same.
"""
import json
from collections import defaultdict

import numpy as np
from scipy.sparse import csr_matrix


def _nested():
    return defaultdict(_nested)


def jkey(J):
    return round(float(J), 1)


def read_tensor(filename, name):
    """Returns (basis dict, kmat, mmat, mfmat or None, rank, cart)."""
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
        meta[name] = info
        cat = lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)
        out[name + "/csr_data"] = cat(data, np.complex128)
        out[name + "/csr_indices"] = cat(indices, np.int64)
        out[name + "/csr_indptr"] = cat(indptr, np.int64)
        out[name + "/csr_table"] = np.array(table, np.int64).reshape(-1, 5)
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(filename, **out)
