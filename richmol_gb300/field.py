"""CarTens: laboratory-frame Cartesian tensor operator, GPU drop-in for
richmol.field.CarTens (CFEL-CMI/richmol, richmol/field.py:25-1301).

The attribute surface follows the reference (Jlist1/2, symlist1/2, dim_m1/2,
dim_k1/2, dim1/2, kmat, mmat, mfmat, rank, cart) and so do the operations on
the propagation path:

* ``field(E, thresh)``  records the field products (field.py:1094-1105); the
  contraction MF = sum_c E_c M_c happens on the GPU at the next product;
* ``vec(vec)``          the Kronecker mat-vec on the GPU (field.py:1145-1245);
* ``tomat``             host (scipy) assembly for set-up and observables
                        (field.py:449-569);
* ``*``, ``+``, ``-``   scalar and field multiplication and sums
                        (field.py:932-1070, 1248-1301).

Internally a tensor is a list of parts, one per factor source, each with its
K scale and field state; a sum concatenates the parts (the reference renames
irreps '<w>_1', '<w>_2' and snapshots mfmat, field.py:1012-1068). Factor
sources are immutable and their device copies are shared by every operator
built from them.
"""
import copy
import itertools
from collections import defaultdict
from collections.abc import Mapping

import numpy as np
import scipy.sparse
from scipy.sparse import csr_matrix, kron

from . import io as _io

_SCALAR = (int, float, complex, np.integer, np.floating, np.complexfloating)

CART_INDEX = {
    1: ["x", "y", "z"],
    2: ["xx", "xy", "xz", "yx", "yy", "yz", "zx", "zy", "zz"],
}


def _nested():
    return defaultdict(_nested)


class FactorSource:
    """Immutable factor blocks of one tensor: bases, kmat, mmat, rank, cart.

    The bases carry the reference's state quanta (field.py:58-170): per J and
    symmetry ``quanta_m`` (the m of each M row) and ``quanta_k`` ((label,
    energy) of each K state). Sources without them get m = -J..J for full M
    sets and labels "J sym i" with no energy."""

    def __init__(self, basis, kmat, mmat, rank, carts):
        for k, v in basis.items():
            setattr(self, k, v)
        for side in ("1", "2"):
            dm = getattr(self, "dim_m" + side)
            dk = getattr(self, "dim_k" + side)
            setattr(self, "dim" + side, {J: {s: dm[J][s] * dk[J][s] for s in dm[J]} for J in dm})
            sl = getattr(self, "symlist" + side)
            if not hasattr(self, "quanta_m" + side):
                setattr(self, "quanta_m" + side, {
                    J: {s: (list(range(-int(J), int(J) + 1)) if dm[J][s] == 2 * int(J) + 1 else list(range(dm[J][s])))
                        for s in sl[J]} for J in getattr(self, "Jlist" + side)})
            if not hasattr(self, "quanta_k" + side):
                setattr(self, "quanta_k" + side, {
                    J: {s: [(f"{int(J)} {s} {i}", None) for i in range(dk[J][s])] for s in sl[J]}
                    for J in getattr(self, "Jlist" + side)})
        self.kmat = kmat
        self.mmat = mmat
        self.rank = rank
        self.carts = list(carts)

    def filtered(self, bra, ket, thresh=None):
        """A new source with the states for which bra (rows) and ket (columns)
        hold (field.py:187-447): K states are tested with (J, sym, k=label,
        enr=energy), M rows with (J, sym, m); J values and symmetries left
        without states are dropped (symmetries sorted, as the reference), the
        blocks are cut to the kept rows and columns, elements below thresh
        dropped, and irreps whose K or M blocks end up empty removed."""
        basis, ind = {}, {}
        for side, f in (("1", bra), ("2", ket)):
            Jl = getattr(self, "Jlist" + side)
            sl = getattr(self, "symlist" + side)
            qk = getattr(self, "quanta_k" + side)
            qm = getattr(self, "quanta_m" + side)
            ik = {J: {s: [i for i, (q, e) in enumerate(qk[J][s]) if f(J=J, sym=s, k=q, enr=e)] for s in sl[J]}
                  for J in Jl}
            im = {J: {s: [i for i, q in enumerate(qm[J][s]) if f(J=J, sym=s, m=q)] for s in sl[J]} for J in Jl}
            ik = {J: {s: v for s, v in d.items() if v} for J, d in ik.items()}
            im = {J: {s: v for s, v in d.items() if v} for J, d in im.items()}
            Jnew = sorted(J for J in Jl if ik[J] and im[J])
            snew = {J: sorted(set(ik[J]) & set(im[J])) for J in Jnew}
            Jnew = [J for J in Jnew if snew[J]]
            basis["Jlist" + side] = Jnew
            basis["symlist" + side] = {J: snew[J] for J in Jnew}
            basis["dim_m" + side] = {J: {s: len(im[J][s]) for s in snew[J]} for J in Jnew}
            basis["dim_k" + side] = {J: {s: len(ik[J][s]) for s in snew[J]} for J in Jnew}
            basis["quanta_m" + side] = {J: {s: [qm[J][s][i] for i in im[J][s]] for s in snew[J]} for J in Jnew}
            basis["quanta_k" + side] = {J: {s: [qk[J][s][i] for i in ik[J][s]] for s in snew[J]} for J in Jnew}
            ind[side] = (ik, im, basis["symlist" + side])

        def cut(mat, rows, cols):
            return csr_matrix(mat)[rows, :].tocsc()[:, cols].tocsr()

        def drop(m):
            m.data[np.abs(m.data) < thresh] = 0
            m.eliminate_zeros()
            return m

        kmat, mmat = _nested(), _nested()
        (ik1, im1, s1l), (ik2, im2, s2l) = ind["1"], ind["2"]
        for Jp in set(self.kmat.keys()) & set(self.mmat.keys()):
            J1, J2 = Jp
            if J1 not in s1l or J2 not in s2l:
                continue
            for sp in set(self.kmat[Jp].keys()) & set(self.mmat[Jp].keys()):
                a, b = sp
                if a not in s1l[J1] or b not in s2l[J2]:
                    continue
                kS = {irrep: cut(m, ik1[J1][a], ik2[J2][b]) for irrep, m in self.kmat[Jp][sp].items()}
                mS = {irrep: {c: cut(m, im1[J1][a], im2[J2][b]) for c, m in mI.items()}
                      for irrep, mI in self.mmat[Jp][sp].items()}
                # irreps in both: thresh, then dropped if K or every M is empty
                # (irreps in one of them only stay as cut, field.py:417-443)
                for irrep in set(kS) & set(mS):
                    if thresh is not None:
                        kS[irrep] = drop(kS[irrep])
                        mS[irrep] = {c: m for c, m in ((c, drop(m)) for c, m in mS[irrep].items()) if m.nnz > 0}
                    if kS[irrep].nnz == 0 or len(mS[irrep]) == 0:
                        del kS[irrep], mS[irrep]
                if kS and mS:
                    for irrep, m in kS.items():
                        kmat[Jp][sp][irrep] = m
                    for irrep, mI in mS.items():
                        for c, m in mI.items():
                            mmat[Jp][sp][irrep][c] = m
        return FactorSource(basis, kmat, mmat, self.rank, self.carts)

    def basis(self, side):
        Jl = getattr(self, "Jlist" + side)
        sl = getattr(self, "symlist" + side)
        dm = getattr(self, "dim_m" + side)
        dk = getattr(self, "dim_k" + side)
        return [(J, s, int(dm[J][s]), int(dk[J][s])) for J in Jl for s in sl[J]]


class _Part:
    __slots__ = ("src", "kscale", "prods", "thresh")

    def __init__(self, src, kscale=1.0, prods=None, thresh=None):
        self.src = src
        self.kscale = kscale
        self.prods = prods      # field products {cart: value} after field(); None before
        self.thresh = thresh


# plan cache: tuple of factor sources -> OperatorPlan (strong references keep
# the sources alive while their plan exists)
_PLANS = {}


def clear_plan_cache():
    _PLANS.clear()


class CarTens:
    """GPU drop-in for richmol.field.CarTens on the propagation path.

    Args:
        filename : str   factor file: ``.npz`` (richmol_gb300.io) or the
                         reference's HDF5 layout (field.py:1304-1848)
        name : str       tensor name inside the file
        thresh : float   matrix elements below it are dropped on reading, and
                         blocks left empty with them (field.py:1600-1848 read)
    """

    def __init__(self, filename=None, name=None, **kwargs):
        self._parts = []
        self._is_sum = False
        if filename is not None:
            if name is None:
                raise ValueError(f"please specify the name of the data group in file '{filename}'")
            basis, kmat, mmat, mfmat, rank, cart = _io.read_tensor(filename, name, thresh=kwargs.get("thresh"))
            if not mmat and mfmat is not None:
                # stored field-contracted operator: a frozen single-component source
                mmat = _nested()
                for Jp, mJ in mfmat.items():
                    for sp, mS in mJ.items():
                        for irrep, m in mS.items():
                            mmat[Jp][sp][irrep]["0"] = m
                rank, cart = 0, ["0"]
            self._init_source(FactorSource(basis, kmat, mmat, rank, cart))
            if "bra" in kwargs or "ket" in kwargs:  # field.py:172, read with state filters
                self.filter(bra=kwargs.get("bra", lambda **kw: True), ket=kwargs.get("ket", lambda **kw: True))

    @classmethod
    def from_factors(cls, basis, kmat, mmat, rank, cart):
        T = cls()
        T._init_source(FactorSource(basis, kmat, mmat, rank, cart))
        return T

    def _init_source(self, src):
        self._parts = [_Part(src)]
        self._is_sum = False

    # ------------------------------------------------------------------
    # reference attributes
    # ------------------------------------------------------------------
    def _first(self):
        if not self._parts:
            raise AttributeError("empty CarTens")
        return self._parts[0].src

    def __getattr__(self, name):
        if name in ("Jlist1", "Jlist2", "symlist1", "symlist2", "dim_m1", "dim_m2", "dim_k1", "dim_k2",
                    "dim1", "dim2", "quanta_m1", "quanta_m2", "quanta_k1", "quanta_k2"):
            return getattr(self._first(), name)
        if name in ("rank", "cart", "mmat") and not self.__dict__.get("_is_sum", False):
            src = self._first()
            return {"rank": src.rank, "cart": src.carts, "mmat": src.mmat}[name]
        if name == "kmat":
            return self._kmat()
        if name == "mfmat":
            return self._mfmat()
        raise AttributeError(f"'{type(self).__name__}' object has no attribute '{name}'")

    def _single_source(self):
        if self._is_sum or len(self._parts) != 1:
            raise AttributeError("operation needs a single (non-sum) tensor")
        return self._parts[0].src

    def _irrep_name(self, irrep, p):
        return f"{irrep}_{p + 1}" if self._is_sum else irrep

    def _kmat(self):
        res = _nested()
        for p, part in enumerate(self._parts):
            for Jp, kJ in part.src.kmat.items():
                for sp, kS in kJ.items():
                    for irrep, km in kS.items():
                        res[Jp][sp][self._irrep_name(irrep, p)] = km * part.kscale
        return res

    def _mfmat(self):
        if not self._is_sum and self._parts[0].prods is None:
            raise AttributeError("'CarTens' object has no attribute 'mfmat' (call field() first)")
        res = _nested()
        for p, part in enumerate(self._parts):
            if part.prods is None:
                continue
            for Jp, mJ in part.src.mmat.items():
                for sp, mS in mJ.items():
                    blk = {}
                    for irrep, mI in mS.items():
                        mats = [part.prods[c] * mI[c].toarray() for c in set(mI.keys()) & set(part.prods.keys())]
                        if not mats:
                            continue
                        mat = csr_matrix(sum(mats)) if len(mats) > 1 else csr_matrix(mats[0])
                        if part.thresh is not None and part.thresh > 0:
                            mat.data[np.abs(mat.data) < part.thresh] = 0
                            mat.eliminate_zeros()
                        if mat.nnz > 0:
                            blk[self._irrep_name(irrep, p)] = mat
                    if blk:
                        res[Jp][sp].update(blk)
        return res

    # ------------------------------------------------------------------
    # field.py:1073-1142
    # ------------------------------------------------------------------
    def field(self, field, thresh=None):
        """In-place multiplication with the field (E_x, E_y, E_z)."""
        if self._is_sum:
            raise AttributeError("'CarTens' sum has no attribute 'rank' (field() needs a single tensor)")
        try:
            fx, fy, fz = field[:3]
            fxyz = np.array([fx, fy, fz])
        except (TypeError, IndexError):
            raise IndexError("field variable must be an iterable with three items which represent "
                             "field's X, Y, and Z components") from None
        src = self._parts[0].src
        prods = {"".join("xyz"[c] for c in comb): np.prod(fxyz[list(comb)])
                 for comb in itertools.product((0, 1, 2), repeat=src.rank)}
        prods["0"] = 1
        if thresh is not None:
            prods = {k: v for k, v in prods.items() if abs(v) >= thresh}
        self._parts[0].prods = prods
        self._parts[0].thresh = thresh

    def _has_field_terms(self):
        """True when the operator carries a non-zero field product for a
        Cartesian component present in its M factors (len(mfmat) > 0 of
        tdse.py:377, up to blocks whose elements all fall below thresh, which
        contribute an exact zero)."""
        for part in self._parts:
            if part.prods is None:
                continue
            if any(v != 0 and c in part.src.carts for c, v in part.prods.items()):
                return True
        return False

    # ------------------------------------------------------------------
    # algebra: field.py:932-1070, 1248-1301
    # ------------------------------------------------------------------
    def mul(self, arg):
        if not isinstance(arg, _SCALAR):
            raise TypeError(f"bad argument type for `arg` : '{type(arg)}'")
        for part in self._parts:
            part.kscale = part.kscale * arg

    def filter(self, thresh=None, bra=lambda **kw: True, ket=lambda **kw: True):
        """Keeps the states for which ``bra`` (bra states) and ``ket`` (ket
        states) return True (field.py:187-447): each is called with J, sym and
        k (the state's label), enr (its energy) for K states, and with J, sym
        and m for M states. Every part of a sum is cut alike; the field
        products are kept. Matrix elements below ``thresh`` are dropped."""
        done = {}
        for p in self._parts:
            if id(p.src) not in done:
                done[id(p.src)] = p.src.filtered(bra, ket, thresh)
            p.src = done[id(p.src)]

    def assign(self, form="block"):
        """Quantum numbers of the bra and ket states (field.py:572-657), in the
        order of the rows and columns of ``tomat``: per J and symmetry the
        product of the M states (outer) and K states (inner). form 'block':
        assign[J][sym]['m'] and ['k']; form 'full': lists 'm', 'k', 'sym', 'J'
        over the whole basis. A K entry is the state's (label, energy)."""
        assert form in ("block", "full"), f"bad value of argument 'form' = '{form}' (use 'block' or 'full')"
        out = []
        for side in ("1", "2"):
            Jl, sl = getattr(self, "Jlist" + side), getattr(self, "symlist" + side)
            qm, qk = getattr(self, "quanta_m" + side), getattr(self, "quanta_k" + side)
            if form == "block":
                a = _nested()
                for J in Jl:
                    for sym in sl[J]:
                        mk = list(itertools.product(qm[J][sym], qk[J][sym]))
                        a[J][sym]["m"] = [e[0] for e in mk]
                        a[J][sym]["k"] = [e[1] for e in mk]
            else:
                a = {"m": [], "k": [], "sym": [], "J": []}
                for J in Jl:
                    for sym in sl[J]:
                        mk = list(itertools.product(qm[J][sym], qk[J][sym]))
                        a["m"] += [e[0] for e in mk]
                        a["k"] += [e[1] for e in mk]
                        a["sym"] += [sym] * len(mk)
                        a["J"] += [J] * len(mk)
            out.append(a)
        return tuple(out)

    def full_form(self, mat, repres="csr_matrix", thresh=None):
        """Block matrix {(J1, J2): {(sym1, sym2): block}} -> one 2D matrix in the
        basis order of ``tomat`` (field.py:660-693); missing blocks are zero."""
        rows = [(J, s) for J in self.Jlist1 for s in self.symlist1[J]]
        cols = [(J, s) for J in self.Jlist2 for s in self.symlist2[J]]
        res = scipy.sparse.bmat([[mat[(J1, J2)][(s1, s2)]
                                  if (J1, J2) in mat and (s1, s2) in mat[(J1, J2)]
                                  else csr_matrix((self.dim1[J1][s1], self.dim2[J2][s2]))
                                  for J2, s2 in cols] for J1, s1 in rows])
        if thresh is not None:
            res = csr_matrix(res)
            res.data[np.abs(res.data) < thresh] = 0
            res.eliminate_zeros()
        return res.toarray() if repres == "dense" else getattr(scipy.sparse, repres)(res)

    def block_form(self, mat):
        """2D matrix -> {(J1, J2): {(sym1, sym2): block}} for the bra and ket
        J/symmetry slabs (field.py:696-737); all-zero blocks are left out, sparse
        input gives blocks of its own format."""
        rows = [(J, s) for J in self.Jlist1 for s in self.symlist1[J]]
        cols = [(J, s) for J in self.Jlist2 for s in self.symlist2[J]]
        r0 = np.cumsum([0] + [self.dim1[J][s] for J, s in rows])
        c0 = np.cumsum([0] + [self.dim2[J][s] for J, s in cols])
        sparse = scipy.sparse.issparse(mat)
        m = csr_matrix(mat) if sparse else np.asarray(mat)
        res = {}
        for i, (J1, s1) in enumerate(rows):
            for j, (J2, s2) in enumerate(cols):
                blk = m[r0[i]:r0[i + 1], c0[j]:c0[j + 1]]
                if sparse:
                    blk = getattr(scipy.sparse, mat.getformat() + "_matrix")(blk)
                    blk.eliminate_zeros()
                    if blk.nnz == 0:
                        continue
                elif not np.any(blk):
                    continue
                res.setdefault((J1, J2), {})[(s1, s2)] = blk
        return res

    def _copy(self):
        res = CarTens()
        res._parts = [_Part(p.src, p.kscale, None if p.prods is None else dict(p.prods), p.thresh)
                      for p in self._parts]
        res._is_sum = self._is_sum
        return res

    def __mul__(self, arg):
        if isinstance(arg, _SCALAR):
            res = self._copy()
            res.mul(arg)
        elif isinstance(arg, (np.ndarray, list, tuple)):
            res = self._copy()
            res.field(arg)
        elif isinstance(arg, dict):
            return self.vec(arg)
        else:
            raise TypeError(f"unsupported operand type(s) for '*': 'CarTens' and '{type(arg)}'")
        return res

    __rmul__ = __mul__

    def __add__(self, arg):
        if not isinstance(arg, CarTens):
            raise TypeError(f"unsupported operand type(s) for '+': 'CarTens' and '{type(arg)}'")
        for attr in ("Jlist1", "Jlist2", "symlist1", "symlist2", "dim1", "dim2", "dim_k1", "dim_k2",
                     "dim_m1", "dim_m2"):
            if getattr(self, attr) != getattr(arg, attr):
                raise ValueError("tensors defined with respect to different basis sets")
        for T in (self, arg):  # field.py:995-1004: H0-type tensors get field([0,0,1])
            if not T._is_sum and T._parts[0].src.carts[0] == "0":
                T.field([0, 0, 1])
        res = CarTens()
        res._parts = self._copy()._parts + arg._copy()._parts
        res._is_sum = True
        return res

    __radd__ = __add__

    def __sub__(self, arg):
        if not isinstance(arg, CarTens):
            raise TypeError(f"unsupported operand type(s) for '-': 'CarTens' and '{type(arg)}'")
        return self.__add__(arg * (-1))

    # ------------------------------------------------------------------
    # GPU operator
    # ------------------------------------------------------------------
    def _plan(self, maxorder=100, split=None):
        from .plan import OperatorPlan
        key = (tuple(id(p.src) for p in self._parts), int(maxorder), split)
        plan = _PLANS.get(key)
        if plan is None:
            src0 = self._parts[0].src
            plan = OperatorPlan([p.src for p in self._parts], src0.basis("1"), src0.basis("2"), maxorder=maxorder,
                                split=split)
            _PLANS[key] = plan
        return plan

    def _part_states(self):
        return [((p.prods or {}), p.kscale, p.thresh) for p in self._parts]

    def device_operator(self, maxorder=100, stream=None, split=None):
        """The OperatorPlan of this tensor with the current field applied
        (split: column chunks of the batched path, see OperatorPlan)."""
        if not self._is_sum and self._parts[0].prods is None:
            raise AttributeError("you need to multiply tensor with field before applying it to a vector")
        plan = self._plan(maxorder, split)
        plan.set_field(self._part_states(), stream)
        return plan

    def vec_device(self, x, out=None, stream=None):
        """y = H x for complex128 CUDA tensors x (nvec, dim2) -> (nvec, dim1)."""
        import torch
        plan = self.device_operator(stream=stream)
        x2 = x if x.dim() == 2 else x.reshape(1, -1)
        if out is None:
            out = torch.empty((x2.shape[0], plan.dim_out), dtype=torch.complex128, device=x.device)
        plan.matvec(x2.contiguous(), out, stream)
        return out if x.dim() == 2 else out.reshape(-1)

    def vec(self, vec, matvec_lib="scipy"):
        """Product with a {J: {sym: array}} vector (field.py:1145-1245) on the GPU."""
        import torch
        if not isinstance(vec, Mapping):
            raise TypeError(f"bad argument type for `vec`: '{type(vec)}'")
        assert matvec_lib in ["scipy", "numba", "cupy"], \
            f"bad argument for `matvec_lib`: '{matvec_lib}' (must be 'scipy', 'numba', 'cupy')"
        src = self._parts[0].src
        x = np.concatenate([
            np.asarray(vec[J][s], dtype=np.complex128).reshape(-1) if (J in vec and s in vec[J])
            else np.zeros(src.dim2[J][s], np.complex128)
            for J in src.Jlist2 for s in src.symlist2[J]])
        from .device import require_cuda
        require_cuda()  # the product runs on the GPU only: no CPU fallback
        xd = torch.from_numpy(x).cuda()
        y = self.vec_device(xd).cpu().numpy()
        out, ind = {}, 0
        for J in src.Jlist1:
            for s in src.symlist1[J]:
                n = src.dim1[J][s]
                out.setdefault(J, {})[s] = y[ind: ind + n]
                ind += n
        return out

    # ------------------------------------------------------------------
    # field.py:449-569, 659-695 (host assembly)
    # ------------------------------------------------------------------
    def tomat(self, form="block", repres="csr_matrix", thresh=None, cart=None):
        assert form in ("block", "full"), f"`form` unknown: '{form}' (use 'block', 'full')"
        blocks = {}
        if cart is None:
            mf = self.mfmat
            km = self.kmat
            for Jp in set(mf.keys()) & set(km.keys()):
                for sp in set(mf[Jp].keys()) & set(km[Jp].keys()):
                    me = sum(kron(mf[Jp][sp][i], km[Jp][sp][i]) for i in set(mf[Jp][sp]) & set(km[Jp][sp]))
                    if not np.isscalar(me):
                        blocks[(Jp, sp)] = me
        else:
            src = self._single_source()
            if cart not in src.carts:
                raise ValueError(f"specified Cartesian component '{cart}' is not contained in tensor "
                                 f"components '{src.carts}'")
            km = self.kmat
            for Jp in set(src.mmat.keys()) & set(km.keys()):
                for sp in set(src.mmat[Jp].keys()) & set(km[Jp].keys()):
                    mm = {i: v[cart] for i, v in src.mmat[Jp][sp].items() if cart in v}
                    me = sum(kron(mm[i], km[Jp][sp][i]) for i in set(mm) & set(km[Jp][sp]))
                    if not np.isscalar(me):
                        blocks[(Jp, sp)] = me
        if thresh is not None and thresh > 0:
            for key, m in blocks.items():
                m = m.tocsr()
                m.data[np.abs(m.data) <= thresh] = 0
                m.eliminate_zeros()
                blocks[key] = m
        src = self._parts[0].src
        if form == "block":
            res = _nested()
            for ((J1, J2), (s1, s2)), m in blocks.items():
                res[(J1, J2)][(s1, s2)] = m.toarray() if repres == "dense" else getattr(scipy.sparse, repres)(m)
            return res
        rows = [(J, s) for J in src.Jlist1 for s in src.symlist1[J]]
        cols = [(J, s) for J in src.Jlist2 for s in src.symlist2[J]]
        full = scipy.sparse.bmat([
            [blocks[((J1, J2), (s1, s2))] if ((J1, J2), (s1, s2)) in blocks
             else csr_matrix((src.dim1[J1][s1], src.dim2[J2][s2]), dtype=np.complex128)
             for (J2, s2) in cols] for (J1, s1) in rows])
        if repres == "dense":
            return full.toarray()
        return getattr(scipy.sparse, repres)(full)

    def store(self, filename, name):
        """Writes the factors (K scale applied) to a factor file."""
        _io.write_tensors(filename, {name: self})


def filter(obj, bra, ket, thresh=None):
    """A copy of ``obj`` with the state filters applied (field.py:1859-1882)."""
    if not isinstance(obj, CarTens):
        raise TypeError(f"bad argument type for 'obj': '{type(obj)}'")
    res = obj._copy()
    res.filter(bra=bra, ket=ket, thresh=thresh)
    return res
