"""Oracle restatement of the reference CarTens operations on the hot path.

Reference: richmol/field.py (CFEL-CMI/richmol). The container mirrors the
reference's attributes (Jlist1/2, symlist1/2, dim_m1/2, dim_k1/2, dim1/2, kmat,
mmat, mfmat) so that tests read like the reference's own usage.
"""
import copy
import itertools
from collections import defaultdict

import numpy as np
import scipy.sparse
from scipy.sparse import csr_matrix, kron


def _nested():
    return defaultdict(_nested)


class OCarTens:
    """Block-sparse Kronecker operator sum_{J1,J2,s1,s2,w} MF_w (x) K_w."""

    # ------------------------------------------------------------------
    # field.py:1073-1142  CarTens.field
    # ------------------------------------------------------------------
    def field(self, field, thresh=None):
        fx, fy, fz = field[:3]
        fxyz = np.array([fx, fy, fz])
        # field.py:1094-1097: all products of `rank` field components
        field_prod = {
            "".join("xyz"[c] for c in comb): np.prod(fxyz[list(comb)])
            for comb in itertools.product((0, 1, 2), repeat=self.rank)
        }
        field_prod["0"] = 1  # field.py:1099
        if thresh is not None:  # field.py:1101-1105
            field_prod = {k: v for k, v in field_prod.items() if abs(v) >= thresh}
        self.mfmat = _nested()
        if len(field_prod) == 0:
            return
        # field.py:1112-1142: MF_w = sum_cart prod_cart * M_{w,cart}
        for (J1, J2), mJ in self.mmat.items():
            for (s1, s2), mS in mJ.items():
                res = {}
                for irrep, mI in mS.items():
                    mats = [field_prod[c] * mI[c].toarray()
                            for c in list(set(mI.keys()) & set(field_prod.keys()))]
                    mat = csr_matrix(mats[0]) if len(mats) == 1 else csr_matrix(sum(mats))
                    if thresh is not None and thresh > 0:
                        mask = abs(mat.data) < thresh
                        mat.data[mask] = 0
                        mat.eliminate_zeros()
                    if mat.nnz > 0:
                        res[irrep] = mat
                if len(res) > 0:
                    self.mfmat[(J1, J2)][(s1, s2)] = res

    # ------------------------------------------------------------------
    # field.py:1145-1245  CarTens.vec (scipy branch, field.py:1185-1186)
    # ------------------------------------------------------------------
    def vec(self, vec):
        vec2 = {}
        for (J1, J2) in list(set(self.mfmat.keys()) & set(self.kmat.keys())):
            mfJ = self.mfmat[(J1, J2)]
            kJ = self.kmat[(J1, J2)]
            if J1 not in vec2:
                vec2[J1] = {}
            for (s1, s2) in list(set(mfJ.keys()) & set(kJ.keys())):
                mf = mfJ[(s1, s2)]
                km = kJ[(s1, s2)]
                dim1 = self.dim_m2[J2][s2]
                dim2 = self.dim_k2[J2][s2]
                dim = self.dim1[J1][s1]
                try:
                    # field.py:1229: X = vec[J2][sym2] as (dim_m2, dim_k2) row-major
                    vecT = np.transpose(vec[J2][s2].reshape(dim1, dim2))
                except KeyError:
                    continue
                res = []
                for irrep in list(set(mf.keys()) & set(km.keys())):
                    tmat = km[irrep].dot(vecT)  # field.py:1235  T = K X^T
                    res.append(mf[irrep].dot(np.transpose(tmat)).reshape(dim))  # MF T^T
                try:
                    vec2[J1][s1] += sum(res)
                except KeyError:
                    vec2[J1][s1] = sum(res)
        return vec2

    # ------------------------------------------------------------------
    # field.py:449-569 tomat(form='full') and field.py:659-695 full_form
    # ------------------------------------------------------------------
    def tomat(self, form="full", repres="csr_matrix", cart=None):
        blocks = {}
        if cart is None:
            for Jp in list(set(self.mfmat.keys()) & set(self.kmat.keys())):
                for sp in list(set(self.mfmat[Jp].keys()) & set(self.kmat[Jp].keys())):
                    mm, km = self.mfmat[Jp][sp], self.kmat[Jp][sp]
                    me = sum(kron(mm[i], km[i]) for i in list(set(mm.keys()) & set(km.keys())))
                    if not np.isscalar(me):
                        blocks[(Jp, sp)] = me
        else:
            for Jp in list(set(self.mmat.keys()) & set(self.kmat.keys())):
                for sp in list(set(self.mmat[Jp].keys()) & set(self.kmat[Jp].keys())):
                    mm = {i: v[cart] for i, v in self.mmat[Jp][sp].items() if cart in v}
                    km = self.kmat[Jp][sp]
                    me = sum(kron(mm[i], km[i]) for i in list(set(mm.keys()) & set(km.keys())))
                    if not np.isscalar(me):
                        blocks[(Jp, sp)] = me
        rows = [(J, s) for J in self.Jlist1 for s in self.symlist1[J]]
        cols = [(J, s) for J in self.Jlist2 for s in self.symlist2[J]]
        res = scipy.sparse.bmat([
            [blocks[((J1, J2), (s1, s2))] if ((J1, J2), (s1, s2)) in blocks
             else csr_matrix(np.zeros((self.dim1[J1][s1], self.dim2[J2][s2])))
             for (J2, s2) in cols] for (J1, s1) in rows])
        if repres == "dense":
            return res.toarray()
        return getattr(scipy.sparse, repres)(res)

    # ------------------------------------------------------------------
    # field.py:932-948 mul, field.py:1248-1301 __mul__/__add__/__sub__
    # ------------------------------------------------------------------
    def mul(self, arg):
        for Jp in self.kmat.keys():
            for sp in self.kmat[Jp].keys():
                self.kmat[Jp][sp] = {k: v * arg for k, v in self.kmat[Jp][sp].items()}

    def __mul__(self, arg):
        res = copy.deepcopy(self)
        if isinstance(arg, (list, tuple, np.ndarray)):
            res.field(arg)
        else:
            res.mul(arg)
        return res

    __rmul__ = __mul__

    def __add__(self, arg):
        return add_cartens(self, arg)

    def __sub__(self, arg):
        return add_cartens(self, arg * (-1))


def add_cartens(a, b):
    """field.py:951-1070: union of both term lists, irreps renamed '<w>_1' and
    '<w>_2'; H0-type tensors (cart == ['0']) are first given field([0,0,1])."""
    for T in (a, b):
        if getattr(T, "cart", [None])[0] == "0":
            T.field([0, 0, 1])
    res = OCarTens()
    res.__dict__.update(a.__dict__)
    for attr in ("os", "rank", "cart", "mmat"):
        if hasattr(res, attr):
            delattr(res, attr)
    res.kmat = _nested()
    res.mfmat = _nested()
    for T, tag in ((a, "_1"), (b, "_2")):
        for src, dst in ((T.kmat, res.kmat), (T.mfmat, res.mfmat)):
            for Jp in src.keys():
                for sp in src[Jp].keys():
                    dst[Jp][sp].update({str(i) + tag: v for i, v in src[Jp][sp].items()})
    return res


def flat(T, vec_dict, side="1"):
    """Concatenation of a {J: {sym: array}} vector in Jlist x symlist order
    (tdse.py:353-360)."""
    Jlist = getattr(T, "Jlist" + side)
    symlist = getattr(T, "symlist" + side)
    dim = getattr(T, "dim" + side)
    return np.concatenate([
        vec_dict[J][s] if (J in vec_dict and s in vec_dict[J]) else np.zeros(dim[J][s], np.complex128)
        for J in Jlist for s in symlist[J]])


def split(T, v, side="2"):
    """Views of a flat vector as {J: {sym: slab}} (tdse.py:343-348)."""
    out, ind = {}, 0
    for J in getattr(T, "Jlist" + side):
        out[J] = {}
        for s in getattr(T, "symlist" + side)[J]:
            n = getattr(T, "dim" + side)[J][s]
            out[J][s] = v[ind: ind + n]
            ind += n
    return out
