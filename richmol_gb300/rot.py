"""In-house rotational factor builder: field-free solutions and the M (x) K
factors of laboratory-frame tensors, vectorised with numpy.

Stands in for the reference's set-up chain (CFEL-CMI/richmol), which cannot
run on the GPU machine and takes hours at J >= 30:

* symmetric-top basis and Wang combinations   rot/basis.py:702-801
* D2 / C1 symmetrisation by projection        rot/symmetry.py:31-209
* rigid rotor + Watson-A diagonal terms       rot/solution.py:160-334, rot/J.py
* K and M factors from Wigner 3j symbols      rot/labtens.py:411-638
* named observables cos(theta), cos^2(theta)  rot/labtens.py:362-385
* field-free Hamiltonian as a tensor          rot/labtens.py:388-408

Conventions follow the reference so that symmetry labels, block shapes and
energies agree with it; eigenvector signs may differ (both use LAPACK eigh),
which changes no observable.
"""
import math
from collections import defaultdict
from fractions import Fraction
from functools import lru_cache

import numpy as np
import scipy.constants as const
from scipy.sparse import csr_matrix

from .field import CarTens

# Cartesian-to-spherical transformation of rank-1 and rank-2 tensors
# (rot/labtens.py:89-100); rows follow IRREP_IND, columns CART_IND.
_S2 = math.sqrt(2.0)
TMAT_S = {
    1: np.array([[_S2 / 2, -_S2 * 1j / 2, 0],
                 [0, 0, 1.0],
                 [-_S2 / 2, -_S2 * 1j / 2, 0]], dtype=np.complex128),
    2: np.array([[-1 / math.sqrt(3), 0, 0, 0, -1 / math.sqrt(3), 0, 0, 0, -1 / math.sqrt(3)],
                 [0, 0, -0.5, 0, 0, 0.5j, 0.5, -0.5j, 0],
                 [0, 1 / _S2 * 1j, 0, -1 / _S2 * 1j, 0, 0, 0, 0, 0],
                 [0, 0, -0.5, 0, 0, -0.5j, 0.5, 0.5j, 0],
                 [0.5, -0.5j, 0, -0.5j, -0.5, 0, 0, 0, 0],
                 [0, 0, 0.5, 0, 0, -0.5j, 0.5, -0.5j, 0],
                 [-1 / math.sqrt(6), 0, 0, 0, -1 / math.sqrt(6), 0, 0, 0, (1 / 3) * math.sqrt(6)],
                 [0, 0, -0.5, 0, 0, -0.5j, -0.5, -0.5j, 0],
                 [0.5, 0.5j, 0, 0.5j, -0.5, 0, 0, 0, 0]], dtype=np.complex128),
}
# The reference inverts with np.linalg.pinv (rot/labtens.py:104); the maps are
# unitary, so the exact inverse is the conjugate transpose. It agrees with pinv
# to 2.5e-16 and keeps purely real / imaginary entries free of round-off.
TMAT_X = {k: np.ascontiguousarray(v.conj().T) for k, v in TMAT_S.items()}
CART_IND = {1: ["x", "y", "z"], 2: ["xx", "xy", "xz", "yx", "yy", "yz", "zx", "zy", "zz"]}
IRREP_IND = {1: [(1, -1), (1, 0), (1, 1)], 2: [(o, s) for o in range(3) for s in range(-o, o + 1)]}

# isotope masses of the most abundant isotopes (u)
MASSES = {"H": 1.00782503223, "C": 12.0, "N": 14.00307400443, "O": 15.99491461957, "S": 31.9720711744}


# ---------------------------------------------------------------------------
# Wigner 3j symbols (Racah's formula, exact rational arithmetic)
# ---------------------------------------------------------------------------
@lru_cache(maxsize=None)
def _fact(n):
    return math.factorial(n)


def three_j(j1, j2, j3, m1, m2, m3):
    """(j1 j2 j3; m1 m2 m3) for integer arguments."""
    if m1 + m2 + m3 != 0 or abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.0
    if j3 > j1 + j2 or j3 < abs(j1 - j2):
        return 0.0
    f = _fact
    pre = Fraction(f(j1 + j2 - j3) * f(j1 - j2 + j3) * f(-j1 + j2 + j3) * f(j1 + m1) * f(j1 - m1)
                   * f(j2 + m2) * f(j2 - m2) * f(j3 + m3) * f(j3 - m3), f(j1 + j2 + j3 + 1))
    tmin = max(0, j2 - j3 - m1, j1 - j3 + m2)
    tmax = min(j1 + j2 - j3, j1 - m1, j2 + m2)
    s = Fraction(0)
    for t in range(tmin, tmax + 1):
        s += Fraction((-1) ** t, f(t) * f(j3 - j2 + t + m1) * f(j3 - j1 + t - m2) * f(j1 + j2 - j3 - t)
                      * f(j1 - t - m1) * f(j2 - t + m2))
    if s == 0:
        return 0.0
    sign = (-1 if (j1 - j2 - m3) % 2 else 1) * (1 if s > 0 else -1)
    return sign * math.sqrt(float(pre * s * s))


@lru_cache(maxsize=None)
def three_j_rows(j1, w, j2):
    """T[sigma + w, a + j1] = (j1 w j2; a sigma -(a+sigma)) for a = -j1..j1."""
    T = np.zeros((2 * w + 1, 2 * j1 + 1))
    for si, sigma in enumerate(range(-w, w + 1)):
        for ai, a in enumerate(range(-j1, j1 + 1)):
            if abs(a + sigma) <= j2:
                T[si, ai] = three_j(j1, w, j2, a, sigma, -(a + sigma))
    return T


# ---------------------------------------------------------------------------
# symmetric-top basis, Wang functions and symmetrisation
# ---------------------------------------------------------------------------
def wang_coefficients(J, linear):
    """Columns: Wang functions |J,k,tau> (k = 0..J, tau = 0, 1), rows k = -J..J
    (rot/basis.py:714-801); the linear case keeps k = 0 only."""
    if linear:
        return np.array([[1.0 if J % 2 == 0 else 1j]], dtype=np.complex128), [(0, J % 2)]
    bas = []
    for k in range(0, J + 1):
        for t in ([J % 2] if k == 0 else [0, 1]):
            bas.append((k, t))
    C = np.zeros((2 * J + 1, len(bas)), dtype=np.complex128)
    for ib, (k, tau) in enumerate(bas):
        sigma = (k % 3) * tau
        fac1 = (-1.0) ** sigma / math.sqrt(2.0)
        fac2 = fac1 * (-1.0) ** (J + k)
        if tau == 0:
            vals = [1.0] if k == 0 else [fac1, fac2]
        else:
            vals = [1j] if k == 0 else [1j * fac1, -1j * fac2]
        for kk, c in zip([k, -k], vals):
            C[kk + J, ib] = c
            if k == 0:
                break
    return C, bas


def _wigner_d(J, beta):
    """d^J(beta)[m, k] in the reference's convention (rot/wig.py:5-29)."""
    x = lambda m: math.sqrt((J + m) * (J - m + 1))
    n = 2 * J + 1
    A = np.zeros((n, n), dtype=np.complex128)
    ms = np.arange(-J, J + 1)
    for i in range(n - 1):
        A[i + 1, i] = 0.5j * x(ms[i + 1])
        A[i, i + 1] = np.conj(A[i + 1, i])
    _, V = np.linalg.eigh(A)
    e = np.exp(-1j * ms * beta)
    return np.einsum("i,mi,ki->mk", e, np.conj(V), V)


_D2 = dict(
    labels=["A", "B1", "B2", "B3"],
    # characters over E, C2(z), C2(y), C2(x) (rot/symmetry.py:180-209)
    chars=np.array([[1, 1, 1, 1], [1, 1, -1, -1], [1, -1, 1, -1], [1, -1, -1, 1]], dtype=float),
    euler=[(0, 0, 0), (np.pi, 0, 0), (0, np.pi, 0), (0.5 * np.pi, np.pi, 1.5 * np.pi)],
)


def symmetrize(J, C, sym, linear):
    """Splits Wang columns by irreducible representation: {label: column idx}."""
    if sym == "C1" or linear:
        return {"A": list(range(C.shape[1]))}
    if sym != "D2":
        raise NotImplementedError(f"symmetry '{sym}' is not implemented (use 'C1' or 'D2')")
    ks = np.arange(-J, J + 1)
    Ds = []
    for a, b, g in _D2["euler"]:
        d = _wigner_d(J, b)
        Ds.append(np.exp(1j * a * ks)[:, None] * np.exp(1j * g * ks)[None, :] * d)
    out = {}
    for ir, lab in enumerate(_D2["labels"]):
        P = sum(_D2["chars"][ir, g] / 4.0 * Ds[g] for g in range(4))
        pc = P @ C
        cols = [i for i in range(C.shape[1]) if np.abs(pc[:, i]).max() > 1e-12]
        if cols:
            out[lab] = cols
    assert sum(len(v) for v in out.values()) == C.shape[1]
    return out


def _j_matrices(J):
    """Molecular-frame Jx, Jy, Jz on |J,k>, k = -J..J (rot/J.py: J+ lowers k)."""
    n = 2 * J + 1
    ks = np.arange(-J, J + 1)
    Jp = np.zeros((n, n))
    Jm = np.zeros((n, n))
    for i, k in enumerate(ks):
        if abs(k - 1) <= J:
            Jp[i - 1, i] = math.sqrt(J * (J + 1) - k * (k - 1))
        if abs(k + 1) <= J:
            Jm[i + 1, i] = math.sqrt(J * (J + 1) - k * (k + 1))
    Jx = 0.5 * (Jp + Jm)
    Jy = (Jp - Jm) / 2j
    return Jx, Jy, np.diag(ks.astype(float))


def _inertia_origin(m, r):
    """Inertia tensor about the coordinate origin, sum_i m_i (|r_i|^2 - r_i r_i^T).
    The reference's G matrix (rot/molecule.py:189-260) is the inverse of this
    tensor of the frame-rotated coordinates, not shifted to the centre of mass."""
    return np.eye(3) * np.sum(m * np.sum(r * r, axis=1)) - (m[:, None] * r).T @ r


def _inertia_com(m, r):
    """Inertia tensor about the centre of mass (rot/molecule.py:169-186)."""
    r0 = r - (m[:, None] * r).sum(0) / m.sum()
    return _inertia_origin(m, r0)


# h N_A 1e16 / (4 pi^2 c) 1e5: amu*Angstrom^2 -> cm^-1 for G (rot/molecule.py:191-192)
_G_CONV = (const.value("Planck constant") * const.value("Avogadro constant") * 1e16
           / (4.0 * np.pi ** 2 * const.value("speed of light in vacuum")) * 1e5)


class Molecule:
    """Rotational constants (cm^-1), Watson-A centrifugal terms, symmetry and
    molecular-frame tensors (dipole, polarizability) of one molecule.

    The rigid-rotor part is either B = (Bx, By, Bz), H = sum_a B_a J_a^2
    (rot/solution.py:251-257), or a full rotational kinetic-energy matrix G
    (cm^-1), H = 1/2 sum_ab G_ab J_a J_b (rot/solution.py:259-272), as the
    reference builds for a geometry in a frame where the inertia tensor is not
    diagonal (``from_geometry``)."""

    def __init__(self, B=None, xyz=None, linear=None, sym="C1", watson=None, dip=None, pol=None, G=None):
        self.G = None if G is None else np.asarray(G, dtype=np.float64).reshape(3, 3)
        if B is None and xyz is not None:
            B = self.B_from_geometry(xyz)
        if B is None and self.G is not None:
            B = 0.5 * np.diag(self.G)
        self.B = tuple(float(b) for b in B)
        self.linear = linear if linear is not None else (sum(b == 0 for b in self.B) == 1)
        if self.G is not None and self.linear:
            raise ValueError("a G matrix describes a non-linear molecule; give B for a linear one")
        self.sym = sym
        self.watson = dict(watson or {})
        self.dip = None if dip is None else np.asarray(dip, dtype=np.float64)
        self.pol = None if pol is None else np.asarray(pol, dtype=np.float64)
        self.frame_rotation = np.eye(3)

    @staticmethod
    def frame_matrix(frame, masses, xyz, pol=None):
        """Rotation R to a molecular frame, r' = R r (rot/mol_frames.py:29-140):
        None or "eye" (identity), "ipas" / "diag(inertia)" (eigenvectors of the
        centre-of-mass inertia tensor, ascending), "diag(pol)" (of the
        polarizability), or an explicit 3x3 matrix."""
        if frame is None or (isinstance(frame, str) and frame.lower() in ("eye", "none", "null")):
            return np.eye(3)
        if not isinstance(frame, str):
            R = np.asarray(frame, dtype=np.float64).reshape(3, 3)
        else:
            f = frame.strip().lower()
            if f in ("ipas", "diag(inertia)"):
                mat = _inertia_com(masses, xyz)
            elif f == "diag(pol)":
                if pol is None:
                    raise TypeError("tensor 'pol' is not available")
                mat = np.asarray(pol, dtype=np.float64)
                if np.any(np.abs(mat - mat.T) > 1e-12):
                    raise ValueError("tensor is not symmetric")
            else:
                raise ValueError(f"frame '{frame}' is not available")
            _, vec = np.linalg.eigh(mat)
            R = vec.T
        if np.abs(R @ R.T - np.eye(3)).max() > 1e-12:
            raise ValueError("frame rotation matrix is not orthogonal")
        return R

    @classmethod
    def from_geometry(cls, atoms, frame=None, sym="C1", dip=None, pol=None, watson=None, units="angstrom",
                      center=False):
        """Molecule from atoms [(label, x, y, z)] or [(label, mass, x, y, z)].

        Coordinates, dipole and polarizability are rotated to ``frame``
        (r' = R r, mu' = R mu, alpha' = R alpha R^T, as the reference's tensors
        follow its frame, rot/molecule.py:45-165). The Hamiltonian takes the G
        matrix of the rotated coordinates (rot/molecule.py:189-260): the
        inverse of their inertia tensor about the origin times h N_A/(4 pi^2 c),
        through an SVD with singular values below 1e-12 rejected. ``units``:
        "angstrom" or "bohr" (Bohr radius from scipy.constants, as
        rot/atomdata.py:89-90). The reference keeps the input origin (its G of
        an off-centre geometry carries the parallel-axis term); ``center=True``
        moves the origin to the centre of mass first."""
        labels, masses, xyz = [], [], []
        for a in atoms:
            if len(a) == 5:
                lab, mass, x, y, z = a
            else:
                lab, x, y, z = a
                mass = MASSES[lab]
            labels.append(lab)
            masses.append(float(mass))
            xyz.append((float(x), float(y), float(z)))
        m = np.array(masses)
        r = np.array(xyz)
        if units.lower() == "bohr":
            r = r * const.value("Bohr radius") * 1e10
        elif units.lower() != "angstrom":
            raise ValueError(f"unknown units '{units}'")
        if center:
            r = r - (m[:, None] * r).sum(0) / m.sum()
        R = cls.frame_matrix(frame, m, r, pol)
        r = r @ R.T
        u, sv, vt = np.linalg.svd(_inertia_origin(m, r))
        if np.any(sv <= 1e-12):
            raise ValueError("rotational kinetic energy matrix is singular (linear molecule?): give B instead")
        G = (u @ np.diag(1.0 / sv) @ vt) * _G_CONV
        dip_r = None if dip is None else R @ np.asarray(dip, dtype=np.float64)
        pol_r = None if pol is None else R @ np.asarray(pol, dtype=np.float64) @ R.T
        mol = cls(G=G, sym=sym, dip=dip_r, pol=pol_r, watson=watson)
        mol.frame_rotation = R
        mol.atoms = list(zip(labels, masses, map(tuple, r)))
        return mol

    @classmethod
    def read(cls, filename, name, sym="C1", dip=None, pol=None, watson=None):
        """Molecule stored by the reference's Molecule.store (rot/molecule.py:
        390-470): atoms (label, mass, xyz in Angstrom) and frame_rotation; the
        G matrix follows from them as in ``from_geometry``. Tensors given here
        are in the input frame and are rotated with the stored frame."""
        import json
        from . import hdf5
        with hdf5.File(filename) as fl:
            if name not in fl:
                raise KeyError(f"file '{filename}' has no dataset with the name '{name}'")
            at = fl[name].attrs
            atoms = json.loads(at["atoms__json"])["val"]
            R = np.asarray(at.get("frame_rotation", np.eye(3)), dtype=np.float64)
        rows = [(a[0], a[1], *(a[2]["val"] if isinstance(a[2], dict) else a[2])) for a in atoms]
        return cls.from_geometry(rows, frame=R, sym=sym, dip=dip, pol=pol, watson=watson)

    @staticmethod
    def B_from_geometry(xyz):
        """xyz: [(atom, x, y, z)] in Angstrom; principal axes along x, y, z
        (rot/molecule.py:169-300)."""
        m = np.array([MASSES[a] for a, *_ in xyz])
        r = np.array([p for _, *p in xyz], dtype=np.float64)
        r = r - (m[:, None] * r).sum(0) / m.sum()
        I = np.diag([np.sum(m * (r[:, 1] ** 2 + r[:, 2] ** 2)), np.sum(m * (r[:, 0] ** 2 + r[:, 2] ** 2)),
                     np.sum(m * (r[:, 0] ** 2 + r[:, 1] ** 2))])
        conv = (const.value("Planck constant") * const.value("Avogadro constant") * 1e16
                / (8.0 * np.pi ** 2 * const.value("speed of light in vacuum")) * 1e5)
        return [conv / v if abs(v) > 1e-12 else 0.0 for v in np.diag(I)]

    def hamiltonian(self, J):
        """Rotational Hamiltonian on |J,k> (rot/solution.py:227-334)."""
        if self.linear:
            Bl = [b for b in self.B if b != 0][0]
            return np.array([[Bl * J * (J + 1)]], dtype=np.complex128)
        Jx, Jy, Jz = _j_matrices(J)
        if self.G is not None:
            Js = (Jx, Jy, Jz)
            H = 0.5 * sum(self.G[a, b] * (Js[a] @ Js[b]) for a in range(3) for b in range(3))
        else:
            H = self.B[0] * Jx @ Jx + self.B[1] * Jy @ Jy + self.B[2] * Jz @ Jz
        J2 = J * (J + 1)
        Jz2 = Jz @ Jz
        w = self.watson
        H = H - w.get("DeltaJ", 0.0) * J2 * J2 * np.eye(2 * J + 1) - w.get("DeltaJK", 0.0) * J2 * Jz2 \
            - w.get("DeltaK", 0.0) * Jz2 @ Jz2
        for key in ("deltaJ", "deltaK", "HJ", "HJK", "HKJ", "HK", "phiJ", "phiJK", "phiK"):
            if w.get(key, 0.0) != 0.0:
                raise NotImplementedError(f"Watson term '{key}' is not implemented")
        return H


class Solution:
    """Field-free eigenfunctions per (J, sym): coefficients on |J,k>, k=-J..J."""

    def __init__(self, mol, Jmin=0, Jmax=10):
        self.mol = mol
        self.Jlist = list(range(Jmin, Jmax + 1))
        self.states = {}   # J -> {sym: (energies, coefficients[k, state])}
        for J in self.Jlist:
            C, _ = wang_coefficients(J, mol.linear)
            H = mol.hamiltonian(J)
            self.states[J] = {}
            for lab, cols in symmetrize(J, C, mol.sym, mol.linear).items():
                Cs = C[:, cols]
                hmat = (np.conj(Cs.T) @ H @ Cs).real
                e, v = np.linalg.eigh(hmat)
                self.states[J][lab] = (e, Cs @ v)

    @classmethod
    def read(cls, filename, name, mol):
        """Solutions stored by the reference's Solution.store (rot/solution.py:
        60-130, the ``data__json`` attribute): per J and symmetry the energies
        and the states' coefficients on the symmetric-top functions |J,k> (each
        row of ``k.table`` a primitive (J, k) and its coefficient in every
        state). ``mol`` gives what the factors need besides (linear or not)."""
        import json
        from . import hdf5

        def cplx(x):
            return complex(x["real"], x["imag"]) if isinstance(x, dict) else complex(x)

        with hdf5.File(filename) as fl:
            if name not in fl:
                raise KeyError(f"file '{filename}' has no dataset with the name '{name}'")
            data = json.loads(fl[name].attrs["data__json"])
        sol = cls.__new__(cls)
        sol.mol = mol
        sol.Jlist = sorted(int(J) for J in data)
        sol.states = {}
        for J in sol.Jlist:
            sol.states[J] = {}
            for sym, tab in data[str(J)].items():
                enr = np.asarray(tab["enr"], dtype=np.float64)
                C = np.zeros((1 if mol.linear else 2 * J + 1, len(enr)), dtype=np.complex128)
                for prim, _, c in tab["k.table"]["val"]:
                    j, k = (int(x) for x in (prim["val"] if isinstance(prim, dict) else prim))
                    if j != J:
                        raise ValueError(f"primitive J = {j} in the table of J = {J}")
                    C[0 if mol.linear else k + J] = [cplx(x) for x in (c["val"] if isinstance(c, dict) else c)]
                sol.states[J][sym] = (enr, C)
        return sol

    def quanta(self):
        """{J: {sym: [(label, energy), ...]}} in the reference's form
        (quanta_k of field.py:58-170, labels of rot/solution.py): J, then k and
        tau of the state's largest Wang component and its weight |c|^2 as
        "%9.6f", joined by spaces."""
        out = {}
        for J in self.Jlist:
            Cw, bas = wang_coefficients(J, self.mol.linear)
            out[float(J)] = {}
            for sym, (e, C) in self.states[J].items():
                w = np.abs(np.conj(Cw.T) @ C) ** 2
                lead = np.argmax(w, axis=0)
                out[float(J)][sym] = [(" ".join([str(J), str(bas[i][0]), str(bas[i][1]), "%9.6f" % w[i, n]]),
                                       float(e[n])) for n, i in enumerate(lead)]
        return out

    def basis(self):
        Jl = [float(J) for J in self.Jlist]
        syml = {float(J): list(self.states[J].keys()) for J in self.Jlist}
        dm = {float(J): {s: 2 * J + 1 for s in self.states[J]} for J in self.Jlist}
        dk = {float(J): {s: self.states[J][s][1].shape[1] for s in self.states[J]} for J in self.Jlist}
        b = {}
        qk = self.quanta()
        qm = {float(J): {s: list(range(-J, J + 1)) for s in self.states[J]} for J in self.Jlist}
        for side in ("1", "2"):
            b["Jlist" + side] = Jl
            b["symlist" + side] = syml
            b["dim_m" + side] = dm
            b["dim_k" + side] = dk
            b["quanta_k" + side] = qk
            b["quanta_m" + side] = qm
        return b


def _nested():
    return defaultdict(_nested)


def _tensor_spherical(arg):
    """(rank, cart list, irrep list, Us, Ux, tens_flat) of a molecular tensor or
    a named observable (rot/labtens.py:234-385)."""
    if isinstance(arg, str):
        name = arg.lower()
        if name == "costheta":
            return 0, ["0"], [(1, 0)], np.ones((1, 1), complex), np.ones((1, 1), complex), np.ones(1)
        if name == "cos2theta":
            return 0, ["0"], [(2, 0)], np.ones((1, 1), complex), np.full((1, 1), 2.0 / 3.0, complex), np.ones(1)
        raise ValueError(f"unknown name for tensor operator: '{arg}'")
    tens = np.asarray(arg, dtype=np.float64)
    rank = tens.ndim
    carts = CART_IND[rank]
    flat = np.array([tens.item(tuple("xyz".index(c) for c in cart)) for cart in carts])
    Us, Ux = TMAT_S[rank].copy(), TMAT_X[rank].copy()
    irreps = list(IRREP_IND[rank])
    eps = np.finfo(np.complex128).eps
    Us[np.abs(Us) < eps] = 0
    Ux[np.abs(Ux) < eps] = 0
    return rank, carts, irreps, Us, Ux, flat


@lru_cache(maxsize=None)
def _m_factors(carts, uxo_bytes, sigmas, J1, J2, o, thr):
    """M factors of one (J1, J2, omega) block: sqrt((2J1+1)(2J2+1)) (-1)^|b|
    sum_sigma Ux[c, sigma] (J2 omega J1; a sigma -b) per Cartesian component c,
    as CSR matrices. They depend on the tensor's rank and lab-frame
    transformation only, not on the molecule, so every molecule with the same
    J pair shares them (a set of molecules builds each once)."""
    Uxo = np.frombuffer(uxo_bytes, dtype=np.complex128).reshape(len(carts), len(sigmas))
    T = three_j_rows(J2, o, J1)
    mfull = np.zeros((len(carts), 2 * J1 + 1, 2 * J2 + 1), dtype=np.complex128)
    fac_m = math.sqrt((2 * J1 + 1) * (2 * J2 + 1))
    a = np.arange(-J2, J2 + 1)
    for si, sg in enumerate(sigmas):
        b = a + sg
        ok = np.abs(b) <= J1
        aa, bb = a[ok], b[ok]
        v = T[sg + o, aa + J2] * np.where(bb % 2, -1.0, 1.0)
        mfull[:, bb + J1, aa + J2] += fac_m * v[None, :] * Uxo[:, si][:, None]
    mfull[np.abs(mfull) < thr] = 0
    return {cart: csr_matrix(mfull[ci]) for ci, cart in enumerate(carts) if np.any(mfull[ci])}


def lab_tensor(arg, sol, thresh=None):
    """LabTensor equivalent: the K and M factors of a lab-frame tensor, a named
    observable ('costheta', 'cos2theta'), or the field-free Hamiltonian
    (arg == 'h0'), as a CarTens."""
    thr = np.finfo(np.complex128).eps if thresh is None else thresh
    basis = sol.basis()
    kmat, mmat = _nested(), _nested()
    if isinstance(arg, str) and arg == "h0":
        for J in sol.Jlist:
            for s, (e, _) in sol.states[J].items():
                kmat[(float(J), float(J))][(s, s)][0] = csr_matrix(np.diag(e).astype(np.complex128))
                mmat[(float(J), float(J))][(s, s)][0]["0"] = csr_matrix(np.eye(2 * J + 1, dtype=np.complex128))
        return CarTens.from_factors(basis, kmat, mmat, 0, ["0"])

    rank, carts, irreps, Us, Ux, flat = _tensor_spherical(arg)
    omegas = sorted(set(o for o, _ in irreps))
    sig = {o: [i for i, (oo, s) in enumerate(irreps) if oo == o] for o in omegas}
    # K-side molecular-frame spherical components, M-side lab transformation
    UsT = {o: Us[sig[o], :] @ flat for o in omegas}
    Uxo = {o: Ux[:, sig[o]] for o in omegas}
    wmax = max(omegas)
    for J2 in sol.Jlist:          # ket
        for J1 in sol.Jlist:      # bra
            if abs(J1 - J2) > wmax:
                continue
            for o in omegas:
                if abs(J1 - J2) > o:
                    continue
                T = three_j_rows(J2, o, J1)  # (J2 o J1; a sigma -(a+sigma))
                sigmas = tuple(irreps[i][1] for i in sig[o])
                # primitive matrix elements <J1,b| . |J2,a>, b = a + sigma:
                # K: (-1)^|b| sum_s 3j * UsT[s]; M: sqrt((2J1+1)(2J2+1)) (-1)^|b| sum_s Ux[c,s] 3j
                lin = sol.mol.linear
                kfull = np.zeros((2 * J1 + 1, 2 * J2 + 1), dtype=np.complex128)
                a = np.arange(-J2, J2 + 1)
                for si, sg in enumerate(sigmas):
                    b = a + sg
                    ok = np.abs(b) <= J1
                    aa, bb = a[ok], b[ok]
                    v = T[sg + o, aa + J2] * np.where(bb % 2, -1.0, 1.0)
                    kfull[bb + J1, aa + J2] += v * UsT[o][si]
                kprim = kfull[J1:J1 + 1, J2:J2 + 1] if lin else kfull
                mcsr = _m_factors(tuple(carts), Uxo[o].tobytes(), sigmas, J1, J2, o, float(thr))
                for s2, (_, C2) in sol.states[J2].items():
                    for s1, (_, C1) in sol.states[J1].items():
                        K = np.conj(C1.T) @ kprim @ C2
                        K[np.abs(K) < thr] = 0
                        if np.any(K):
                            kmat[(float(J1), float(J2))][(s1, s2)][o] = csr_matrix(K)
                        for cart, M in mcsr.items():
                            mmat[(float(J1), float(J2))][(s1, s2)][o][cart] = M
    # keep only blocks present in both (rot/labtens.py:598-636 stores each
    # separately; CarTens products use the intersection)
    return CarTens.from_factors(basis, kmat, mmat, rank, carts)


def pulse_field(t, t0, fwhm, intensity_wcm2, direction):
    """Cycle-averaged Gaussian pulse (E_a, E_b products equal the cycle average
    E0^2/2 envelope^2), E0 = sqrt(2 I / (c eps0)); times in ps, I in W/cm^2."""
    e0 = np.sqrt(2 * intensity_wcm2 * 1e4 / (const.c * const.epsilon_0))
    env = np.exp(-2 * np.log(2) * (t - t0) ** 2 / fwhm ** 2)
    d = np.asarray(direction, dtype=np.float64)
    d = d / np.linalg.norm(d)
    return e0 * env / np.sqrt(2) * d
