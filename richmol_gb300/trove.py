"""CarTensTrove: tensors from the TROVE text files richmol reads
(richmol/trove.py:9-672), on the GPU propagation path like CarTens.

* the states file: one line per state, ``J id sym ndeg energy assignment...``
  (each of the ndeg degenerate components is a state of its own); it alone
  gives the field-free Hamiltonian: K = diag(energies), M = identity per J
  and symmetry (rank 0, trove.py:52-322);
* the matrix-element files, one per (J1, J2) pair, named by a template with
  ``<j1>``/``<j2>`` (integer J) or ``<f1>``/``<f2>`` (one decimal): between
  ``Start richmol format`` and ``End richmol format`` a header ``name nirrep
  ncart``, an ``M-tensor`` section (per Cartesian component a line ``alpha i
  icmplx cart``, then rows ``m1 m2`` and one value per irrep) and a
  ``K-tensor icmplx`` section (rows ``id1 id2 ideg1 ideg2`` and one value per
  irrep); icmplx = -1 marks imaginary values. When only the file of (J2, J1)
  exists its transpose serves (J1, J2); a file read the right way round is
  conjugated, since the format stores ket-bra order (trove.py:325-665).

State filters (``bra``, ``ket``) and ``thresh`` act as in CarTens.filter.
"""
import os
import re
from collections import defaultdict

import numpy as np
from scipy.sparse import csr_matrix

from .field import CarTens, FactorSource

# irreps of a Cartesian tensor by (number of Cartesian components, number of
# irreps), and its rank by the number of components (trove.py:360-372)
_IRREPS = {
    (3, 1): [(1, -1), (1, 0), (1, 1)],
    (9, 1): [(2, -2), (2, -1), (2, 0), (2, 1), (2, 2)],
    (9, 2): [(0, 0), (2, -2), (2, -1), (2, 0), (2, 1), (2, 2)],
    (6, 2): [(0, 0), (2, -2), (2, -1), (2, 0), (2, 1), (2, 2)],
    (9, 3): [(0, 0), (1, -1), (1, 0), (1, 1), (2, -2), (2, -1), (2, 0), (2, 1), (2, 2)],
}
_RANKS = {3: 1, 9: 2, 6: 2}


def _nested():
    return defaultdict(_nested)


def read_states(filename):
    """(Jlist, symlist, energies, labels, index map (J, id, ideg) -> (i, sym))."""
    energy, label, kmap = {}, {}, {}
    with open(filename) as fl:
        for line in fl:
            w = line.split()
            if not w:
                continue
            try:
                J = round(float(w[0]), 1)
                sid, sym, ndeg, enr = int(w[1]), w[2], int(w[3]), float(w[4])
            except (IndexError, ValueError):
                raise ValueError(f"error while reading file '{filename}'") from None
            q = " ".join(w[5:])
            for ideg in range(ndeg):
                energy.setdefault(J, {}).setdefault(sym, []).append(enr)
                label.setdefault(J, {}).setdefault(sym, []).append(q)
                kmap[(J, sid, ideg + 1)] = (len(energy[J][sym]) - 1, sym)
    if not energy:
        raise ValueError(f"zero number of states in file '{filename}'")
    Jlist = list(energy.keys())
    symlist = {J: list(energy[J].keys()) for J in Jlist}
    return Jlist, symlist, energy, label, kmap


def _file_for(template, J1, J2):
    name = re.sub(r"<f1>", str(round(J1, 1)), template)
    name = re.sub(r"<f2>", str(round(J2, 1)), name)
    name = re.sub(r"<j1>", str(int(round(J1, 0))), name)
    return re.sub(r"<j2>", str(int(round(J2, 0))), name)


def read_trans(template, Jlist, symlist, dim_m, dim_k, kmap, mind, thresh=None):
    """(kmat, mmat, rank, carts) of the matrix-element files of template."""
    kmat, mmat = _nested(), _nested()
    carts, meta = set(), {}
    for J1_ in Jlist:
        for J2_ in Jlist:
            J1, J2, transp = J1_, J2_, False
            fname = _file_for(template, J1, J2)
            if not os.path.exists(fname):
                J1, J2, transp = J2_, J1_, True
                fname = _file_for(template, J1, J2)
                if not os.path.exists(fname):
                    continue
            mrow, mcol, mdat = _nested(), _nested(), _nested()
            krow, kcol, kdat = _nested(), _nested(), _nested()
            section, cart, fac_m, fac_k, eof = None, None, 1.0, 1.0, False
            with open(fname) as fl:
                lines = [ln.rstrip("\n") for ln in fl]
            if not lines or lines[0] != "Start richmol format":
                raise ValueError(f"file '{fname}' has bogus header '{lines[0] if lines else ''}'")
            for iline, line in enumerate(lines[1:], start=1):
                if line == "End richmol format":
                    eof = True
                    break
                w = line.split()
                if iline == 1:
                    try:
                        nirrep, ncart = int(w[1]), int(w[2])
                    except (IndexError, ValueError):
                        raise ValueError(f"error while reading file '{fname}', line = {iline}") from None
                    if meta and meta["key"] != (ncart, nirrep):
                        raise ValueError(f"file '{fname}': (ncart, nirrep) = {(ncart, nirrep)} differs from "
                                         f"{meta['key']} read from previous files")
                    if (ncart, nirrep) not in _IRREPS:
                        raise ValueError(f"can't infer Cartesian tensor irreps from the number of Cartesian "
                                         f"components '{ncart}' and number of irreps = '{nirrep}'")
                    meta = {"key": (ncart, nirrep), "rank": _RANKS[ncart],
                            "omegas": sorted(set(o for o, _ in _IRREPS[(ncart, nirrep)]))}
                    continue
                if line == "M-tensor":
                    section = "m"
                    continue
                if "K-tensor" in line:
                    section = "k"
                    fac_k = (1j, 1.0)[int(w[1]) + 1] if len(w) > 1 else 1.0
                    continue
                if section == "m" and w and w[0] == "alpha":
                    try:
                        fac_m = (1j, 1.0)[int(w[2]) + 1]
                        cart = w[3].lower()
                    except (IndexError, ValueError):
                        raise ValueError(f"error while reading file '{fname}', line = '{iline}'") from None
                    carts.add(cart)
                    continue
                try:
                    if section == "m":
                        m1, m2 = round(float(w[0]), 1), round(float(w[1]), 1)
                        vals = [float(v) * fac_m for v in w[2:]]
                        i1, i2 = mind[(J1, m1)], mind[(J2, m2)]
                        for o, val in zip(meta["omegas"], vals):
                            if thresh is not None and abs(val) < thresh:
                                continue
                            mrow[o].setdefault(cart, []).append(i1)
                            mcol[o].setdefault(cart, []).append(i2)
                            mdat[o].setdefault(cart, []).append(val)
                    elif section == "k":
                        id1, id2, g1, g2 = (int(x) for x in w[:4])
                        vals = [float(v) * fac_k for v in w[4:]]
                        (s1i, s1), (s2i, s2) = kmap[(J1, id1, g1)], kmap[(J2, id2, g2)]
                        for o, val in zip(meta["omegas"], vals):
                            if thresh is not None and abs(val) < thresh:
                                continue
                            krow[(s1, s2)].setdefault(o, []).append(s1i)
                            kcol[(s1, s2)].setdefault(o, []).append(s2i)
                            kdat[(s1, s2)].setdefault(o, []).append(val)
                except (IndexError, ValueError, KeyError):
                    raise ValueError(f"error while reading file '{fname}', line = '{iline}'") from None
            if not eof:
                raise ValueError(f"'{fname}' has bogus footer")
            for sp in kdat:
                a, b = (sp[1], sp[0]) if transp else sp
                if a not in symlist[J1_] or b not in symlist[J2_]:
                    continue
                mshape = (dim_m[J1_][a], dim_m[J2_][b])
                kshape = (dim_k[J1_][a], dim_k[J2_][b])
                if transp:  # the (J2, J1) file: its transpose
                    mm = {o: {c: csr_matrix((np.asarray(mdat[o][c], complex), (mcol[o][c], mrow[o][c])), shape=mshape)
                              for c in mdat[o]} for o in mdat}
                    km = {o: csr_matrix((np.asarray(kdat[sp][o], complex), (kcol[sp][o], krow[sp][o])), shape=kshape)
                          for o in kdat[sp]}
                else:  # ket-bra order in the file: conjugate
                    mm = {o: {c: csr_matrix((np.conj(mdat[o][c]), (mrow[o][c], mcol[o][c])), shape=mshape)
                              for c in mdat[o]} for o in mdat}
                    km = {o: csr_matrix((np.conj(kdat[sp][o]), (krow[sp][o], kcol[sp][o])), shape=kshape)
                          for o in kdat[sp]}
                for o, mI in mm.items():
                    for c, m in mI.items():
                        mmat[(J1_, J2_)][(a, b)][o][c] = m
                for o, m in km.items():
                    kmat[(J1_, J2_)][(a, b)][o] = m
    if not meta:
        raise ValueError(f"no matrix-element files found for the template '{template}'")
    return kmat, mmat, meta["rank"], sorted(carts)


class CarTensTrove(CarTens):
    """richmol.trove.CarTensTrove (trove.py:9-50): the states file alone gives
    the field-free Hamiltonian; with ``matelem`` (the file-name template of the
    matrix-element files) the tensor they hold. kwargs: ``bra``, ``ket`` (state
    filters) and ``thresh``. ``coefs`` (the rovibrational coefficients, used by
    the reference for densities only) is accepted and not read."""

    def __init__(self, filename=None, matelem=None, coefs=None, **kwargs):
        super().__init__()
        if filename is None:
            return
        Jlist, symlist, energy, label, kmap = read_states(filename)
        mq = {J: [round(float(m), 1) for m in np.linspace(-J, J, int(2 * J) + 1)] for J in Jlist}
        mind = {(J, m): i for J in Jlist for i, m in enumerate(mq[J])}
        dim_m = {J: {s: len(mq[J]) for s in symlist[J]} for J in Jlist}
        dim_k = {J: {s: len(energy[J][s]) for s in symlist[J]} for J in Jlist}
        basis = {}
        for side in ("1", "2"):
            basis["Jlist" + side] = list(Jlist)
            basis["symlist" + side] = {J: list(symlist[J]) for J in Jlist}
            basis["dim_m" + side] = dim_m
            basis["dim_k" + side] = dim_k
            basis["quanta_m" + side] = {J: {s: list(mq[J]) for s in symlist[J]} for J in Jlist}
            basis["quanta_k" + side] = {J: {s: list(zip(label[J][s], energy[J][s])) for s in symlist[J]}
                                        for J in Jlist}
        thresh = kwargs.get("thresh")
        if matelem is None:
            kmat, mmat = _nested(), _nested()
            for J in Jlist:
                for s in symlist[J]:
                    mmat[(J, J)][(s, s)][0]["0"] = csr_matrix(np.eye(len(mq[J]), dtype=np.complex128))
                    kmat[(J, J)][(s, s)][0] = csr_matrix(np.diag(np.asarray(energy[J][s], dtype=np.complex128)))
            rank, carts = 0, ["0"]
        else:
            kmat, mmat, rank, carts = read_trans(matelem, Jlist, symlist, dim_m, dim_k, kmap, mind, thresh)
        self._init_source(FactorSource(basis, kmat, mmat, rank, carts))
        self.filter(thresh=thresh, bra=kwargs.get("bra", lambda **kw: True), ket=kwargs.get("ket", lambda **kw: True))
