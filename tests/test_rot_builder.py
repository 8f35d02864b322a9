"""The in-house factor builder (richmol_gb300.rot) against the reference's own
factors (tests/golden, produced by rot.LabTensor / rot.solve of the reference).

M factors involve no eigenvectors and must agree element by element; K factors
agree up to the sign of each eigenvector, so their magnitudes are compared;
energies per (J, symmetry) agree to rounding. CPU only."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _mol_ocs():
    from richmol_gb300 import rot
    return rot.Molecule(xyz=[("C", 0, 0, 0), ("O", 0, 0, -1.16), ("S", 0, 0, 1.56)],
                        dip=[0, 0, 0.28], pol=np.diag([35.0, 35.0, 80.0]))


def _mol_asym():
    from richmol_gb300 import rot
    return rot.Molecule(B=(9.0, 5.0, 3.2), sym="D2", watson=dict(DeltaJ=1e-3, DeltaJK=1e-3, DeltaK=1e-3),
                        dip=[0, 0, -0.73], pol=np.diag([9.1, 9.9, 9.4]))


def _mol_c1():
    """The C1 molecule of tests/golden/c1_j10.npz (its parameters are in the
    fixture's meta, written by make_golden.py's c1_molecule)."""
    import json
    from richmol_gb300 import rot
    m = json.loads(str(np.load(os.path.join(GOLDEN, "c1_j10.npz"))["meta"]))["mol"]
    return rot.Molecule(B=tuple(m["B"]), sym="C1", dip=m["dip"], pol=np.array(m["pol"]))


CASES = [
    ("ocs_j6.npz", _mol_ocs, 6, ["dip", "pol", "cos2", "cos", "h0"]),
    ("asym_j4.npz", _mol_asym, 4, ["dip", "pol", "cos2", "h0"]),
    ("asym_j10.npz", _mol_asym, 10, ["dip", "pol", "cos2", "cos", "h0"]),
    ("c1_j10.npz", _mol_c1, 10, ["dip", "pol", "cos2", "h0"]),
]
ARGS = {"cos2": "cos2theta", "cos": "costheta", "h0": "h0"}


# Eigenvalues of one (J, sym) closer than this (cm^-1) form a cluster: inside
# it the eigenvectors are fixed only up to a unitary mixing whose size is the
# eigensolver's round-off over the gap (near-prolate C1 tops have K doublets
# split by 1e-10 cm^-1 at J = 10), so K factors are compared there through
# invariants of that mixing (singular values of each cluster-pair sub-block).
CLUSTER_GAP = 1e-2


def _clusters(e):
    order = np.argsort(e, kind="stable")
    out, cur = [], [int(order[0])]
    for a, b in zip(order[:-1], order[1:]):
        if e[b] - e[a] < CLUSTER_GAP:
            cur.append(int(b))
        else:
            out.append(cur)
            cur = [int(b)]
    out.append(cur)
    return out


def _k_equivalent(a, b, ca, cb, tol):
    """|a| == |b| element by element outside multi-state clusters (signs and
    phases of single eigenvectors are free); singular values of the
    sub-blocks of clusters with more than one state."""
    for ia in ca:
        for ib in cb:
            sa, sb = a[np.ix_(ia, ib)], b[np.ix_(ia, ib)]
            if len(ia) == 1 and len(ib) == 1:
                if abs(abs(sa[0, 0]) - abs(sb[0, 0])) > tol:
                    return False
            else:
                if np.abs(np.linalg.svd(sa, compute_uv=False) - np.linalg.svd(sb, compute_uv=False)).max() > tol:
                    return False
    return True


@pytest.mark.parametrize("case,mk,Jmax,names", CASES)
def test_factors_match_reference(case, mk, Jmax, names):
    from oracle import fixtures
    from richmol_gb300 import rot
    d, meta = fixtures.load(os.path.join(GOLDEN, case))
    mol = mk()
    sol = rot.Solution(mol, Jmax=Jmax)
    # reference energies per (J, sym), when the fixture holds them
    enr, clus = {}, {}
    if "enr_keys" in meta:
        i = 0
        for J, s, n in meta["enr_keys"]:
            enr[(float(J), s)] = d["enr"][i: i + n]
            i += n
        clus = {k: _clusters(e) for k, e in enr.items()}
    for nm in names:
        ref = fixtures.tensor(d, meta, nm)
        arg = ARGS.get(nm, mol.dip if nm == "dip" else mol.pol)
        src = rot.lab_tensor(arg, sol)._parts[0].src
        assert src.Jlist1 == ref.Jlist1
        assert src.symlist1 == ref.symlist1
        assert src.dim_k1 == ref.dim_k1 and src.dim_m1 == ref.dim_m1
        for Jp in ref.kmat:
            for sp in ref.kmat[Jp]:
                for i in ref.kmat[Jp][sp]:
                    a = ref.kmat[Jp][sp][i].toarray()
                    try:
                        b = src.kmat[Jp][sp][i].toarray()
                    except (KeyError, AttributeError):
                        # the reference keeps round-off blocks above machine epsilon
                        b = np.zeros_like(a)
                    tol = 1e-12 * max(1.0, np.abs(a).max())
                    k1, k2 = (float(Jp[0]), sp[0]), (float(Jp[1]), sp[1])
                    if k1 in clus and k2 in clus and a.shape == (len(enr[k1]), len(enr[k2])):
                        assert _k_equivalent(a, b, clus[k1], clus[k2], 1e-10 * max(1.0, np.abs(a).max())), \
                            (nm, Jp, sp, i)
                    else:
                        assert np.abs(np.abs(a) - np.abs(b)).max() < tol, (nm, Jp, sp, i)
        for Jp in ref.mmat:
            for sp in ref.mmat[Jp]:
                for i in ref.mmat[Jp][sp]:
                    for c in ref.mmat[Jp][sp][i]:
                        a = ref.mmat[Jp][sp][i][c].toarray()
                        b = src.mmat[Jp][sp][i][c].toarray()
                        assert np.abs(a - b).max() < 1e-14, (nm, Jp, sp, i, c)


@pytest.mark.parametrize("case,mk,Jmax", [("asym_j4.npz", _mol_asym, 4), ("asym_j10.npz", _mol_asym, 10),
                                          ("c1_j10.npz", _mol_c1, 10)])
def test_energies_match_reference(case, mk, Jmax):
    from oracle import fixtures
    from richmol_gb300 import rot
    d, meta = fixtures.load(os.path.join(GOLDEN, case))
    sol = rot.Solution(mk(), Jmax=Jmax)
    i = 0
    for J, s, n in meta["enr_keys"]:
        e = sol.states[J][s][0]
        assert len(e) == n
        assert np.abs(e - d["enr"][i: i + n]).max() < 1e-10
        i += n


def test_ocs_rotational_constant_from_geometry():
    import json
    meta = json.loads(str(np.load(os.path.join(GOLDEN, "ocs_j6.npz"))["meta"]))
    assert np.allclose(_mol_ocs().B, meta["B"], rtol=1e-14, atol=0)


def test_three_j_against_exact_reference_stub():
    import sys
    sys.path.insert(0, os.path.join(GOLDEN, "refshim"))
    try:
        import py3nj
    finally:
        sys.path.pop(0)
    from richmol_gb300 import rot
    rng = np.random.default_rng(0)
    for _ in range(200):
        j1 = int(rng.integers(0, 45))
        w = int(rng.integers(0, 3))
        j2 = int(rng.integers(max(0, j1 - w), j1 + w + 1))
        a = int(rng.integers(-j1, j1 + 1))
        s = int(rng.integers(-w, w + 1))
        if abs(a + s) > j2:
            continue
        ref = py3nj.wigner3j(2 * j1, 2 * w, 2 * j2, 2 * a, 2 * s, -2 * (a + s))[0]
        assert abs(rot.three_j(j1, w, j2, a, s, -(a + s)) - ref) < 1e-15


def test_propagation_observable_is_basis_invariant():
    """Propagating the reference fixture's initial state with the builder's
    factors gives the reference's <cos^2 theta> trace (the oracle runs both)."""
    from oracle import fixtures
    from oracle.cartens import OCarTens
    from oracle.tdse import OTDSE
    from richmol_gb300 import rot
    d, meta = fixtures.load(os.path.join(GOLDEN, "ocs_j6.npz"))
    sp = meta["split"]
    sol = rot.Solution(_mol_ocs(), Jmax=6)

    def to_oracle(T):
        src = T._parts[0].src
        o = OCarTens()
        for k in ("Jlist1", "Jlist2", "symlist1", "symlist2", "dim_m1", "dim_m2", "dim_k1", "dim_k2",
                  "dim1", "dim2", "kmat", "mmat", "rank"):
            setattr(o, k, getattr(src, k))
        o.cart = src.carts
        return o
    h0 = to_oracle(rot.lab_tensor("h0", sol))
    Hac = to_oracle(rot.lab_tensor(_mol_ocs().pol, sol)) * sp["scale"]
    c2 = to_oracle(rot.lab_tensor("cos2theta", sol)).tomat(form="full", cart="0")
    td = OTDSE(t_start=sp["t_start"], t_end=sp["t_end"], dt=sp["dt"])
    tc = td.time_grid()
    vecs = td.init_state(h0, temp=0)
    for i in range(len(tc)):
        Hac.field(d["split/fields"][i])
        vecs, _ = td.update(Hac, vecs, H0=h0)
        c = np.vdot(vecs[0], c2.dot(vecs[0])).real + 1 / 3
        assert abs(c - d["split/cos2"][i]) < 1e-9


def test_g_matrix_energies_do_not_depend_on_the_frame():
    """The rigid rotor 1/2 G_ab J_a J_b of one geometry in three frames
    (principal axes, a random rotation, the polarizability's axes): the
    rotational energies agree to rounding, and the symmetric-top basis
    solution (the real part of H in the Wang basis, as rot/solution.py:207
    diagonalises) equals the full Hermitian diagonalisation, so nothing is
    dropped with the imaginary part for a non-diagonal G."""
    from richmol_gb300 import rot
    rng = np.random.default_rng(17)
    atoms = [(a, *rng.uniform(-1.5, 1.5, 3)) for a in ("C", "O", "N", "H", "H")]
    p = rng.normal(size=(3, 3))
    pol = p @ p.T + 20 * np.eye(3)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    mols = [rot.Molecule.from_geometry(atoms, frame=f, pol=pol, center=True) for f in ("ipas", q, "diag(pol)")]
    assert np.abs(mols[0].G - np.diag(np.diag(mols[0].G))).max() < 1e-12
    assert min(np.abs(m.G - np.diag(np.diag(m.G))).max() for m in mols[1:]) > 1e-3
    # the reference's own form keeps the input origin: an off-centre geometry's
    # G carries the parallel-axis term, a centred one gives the same G
    off = rot.Molecule.from_geometry(atoms, frame="ipas", pol=pol)
    assert np.abs(off.G - mols[0].G).max() > 1e-3
    m = np.array([rot.MASSES[a[0]] for a in atoms])
    r = np.array([a[1:] for a in atoms])
    r0 = r - (m[:, None] * r).sum(0) / m.sum()
    cen = rot.Molecule.from_geometry([(a[0], *x) for a, x in zip(atoms, r0)], frame="ipas", pol=pol)
    assert np.abs(cen.G - mols[0].G).max() < 1e-12 * np.abs(cen.G).max()
    for J in (1, 4, 8):
        full = [np.linalg.eigvalsh(m.hamiltonian(J)) for m in mols]
        sol = [np.sort(rot.Solution(m, Jmin=J, Jmax=J).states[J]["A"][0]) for m in mols]
        scale = max(1.0, np.abs(full[0]).max())
        for f, s in zip(full, sol):
            assert np.abs(f - full[0]).max() < 1e-13 * scale, J
            assert np.abs(s - f).max() < 1e-13 * scale, J
