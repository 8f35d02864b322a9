"""Generates the golden fixtures in this folder by running the reference
implementation (CFEL-CMI/richmol, Python) in this container.

The reference cannot travel to the GPU machine, so every quantity that the tests
compare against is written here into small ``.npz`` files:

* the tensor factors (``kmat`` / ``mmat`` CSR blocks) of every operator, exported
  with the exact (J, sym, irrep, cart) keys the reference uses;
* outputs of ``CarTens.field`` (``mfmat``) and ``CarTens.vec`` on seeded vectors;
* per-step state vectors from ``TDSE.update`` (split-operator and full-H forms);
* ``TDSE.init_state`` outputs;
* direct calls of ``tdse._expmv_lanczos``;
* the reference's own known answers for the path: the legacy OCS alignment
  J-populations (tests/benchmarks/data/alignment_ocs/pop_reference.txt) and the
  README truncated-pulse <cos^2 theta> trace (docs/source/notebooks/
  trunc_pulse_cos2theta.txt), together with the inputs that reproduce them.

Run from the repository root:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py [case ...]

The stand-in modules in ``refshim/`` are put ahead of the reference on sys.path
(see refshim/README.txt).
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = "/root/reference"
sys.path[:0] = [os.path.join(HERE, "refshim"), REF]
np.float_ = np.float64  # numpy-2 alias the reference still uses (field.py:935)

from richmol.field import CarTens  # noqa: E402
from richmol.rot import LabTensor, Molecule, solve  # noqa: E402
from richmol.tdse import TDSE, _expmv_lanczos  # noqa: E402
from richmol.trove import CarTensTrove  # noqa: E402
from richmol.convert_units import AUdip_x_Vm_to_invcm, AUpol_x_Vm_to_invcm  # noqa: E402
import scipy.constants as const  # noqa: E402


# ---------------------------------------------------------------------------
# export of CarTens objects into flat arrays
# ---------------------------------------------------------------------------

class Packer:
    """Collects CSR matrices into flat arrays and keeps a JSON index."""

    def __init__(self):
        self.data, self.indices, self.indptr = [], [], []
        self.nd = 0
        self.ni = 0
        self.mats = []  # (data_off, nnz, indptr_off, nrows, ncols)

    def add(self, mat):
        mat = mat.tocsr()
        mat.sort_indices()
        idx = len(self.mats)
        self.mats.append((self.nd, int(mat.nnz), self.ni, int(mat.shape[0]), int(mat.shape[1])))
        self.data.append(np.asarray(mat.data, dtype=np.complex128))
        self.indices.append(np.asarray(mat.indices, dtype=np.int64))
        self.indptr.append(np.asarray(mat.indptr, dtype=np.int64))
        self.nd += int(mat.nnz)
        self.ni += int(mat.shape[0]) + 1
        return idx

    def arrays(self, prefix):
        cat = lambda lst, dt: np.concatenate(lst).astype(dt) if lst else np.zeros(0, dt)
        return {
            prefix + "csr_data": cat(self.data, np.complex128),
            prefix + "csr_indices": cat(self.indices, np.int64),
            prefix + "csr_indptr": cat(self.indptr, np.int64),
            prefix + "csr_table": np.array(self.mats, dtype=np.int64).reshape(-1, 5),
        }


def _key(x):
    """JSON-safe key for J / irrep / cart values."""
    if isinstance(x, (np.integer, int)):
        return int(x)
    if isinstance(x, (np.floating, float)):
        return float(x)
    return str(x)


def export_cartens(T, prefix, out, meta, with_mmat=True, with_mfmat=True, with_quanta=False):
    pk = Packer()
    info = {}
    for side in ("1", "2"):
        Jlist = getattr(T, "Jlist" + side)
        symlist = getattr(T, "symlist" + side)
        info["Jlist" + side] = [_key(J) for J in Jlist]
        info["symlist" + side] = [[str(s) for s in symlist[J]] for J in Jlist]
        for attr in ("dim_m", "dim_k"):
            d = getattr(T, attr + side)
            info[attr + side] = [[int(d[J][s]) for s in symlist[J]] for J in Jlist]
        if with_quanta:  # state quanta: m of each M row, (label, energy) of each K state
            qm, qk = getattr(T, "quanta_m" + side), getattr(T, "quanta_k" + side)
            info["quanta_m" + side] = [[[int(m) for m in qm[J][s]] for s in symlist[J]] for J in Jlist]
            info["quanta_k" + side] = [[[[str(q), float(e)] for q, e in qk[J][s]] for s in symlist[J]]
                                       for J in Jlist]
    for attr in ("rank", "cart", "os"):
        if hasattr(T, attr):
            v = getattr(T, attr)
            info[attr] = [list(map(_key, e)) if isinstance(e, tuple) else _key(e) for e in v] \
                if isinstance(v, (list, tuple)) else _key(v)
    blocks = []
    for (J1, J2), kJ in T.kmat.items():
        for (s1, s2), kS in kJ.items():
            for irrep, km in kS.items():
                blocks.append(("k", _key(J1), _key(J2), str(s1), str(s2), _key(irrep), None, pk.add(km)))
    if with_mmat and hasattr(T, "mmat"):
        for (J1, J2), mJ in T.mmat.items():
            for (s1, s2), mS in mJ.items():
                for irrep, mI in mS.items():
                    for cart, mm in mI.items():
                        blocks.append(("m", _key(J1), _key(J2), str(s1), str(s2), _key(irrep), str(cart), pk.add(mm)))
    if with_mfmat and hasattr(T, "mfmat"):
        for (J1, J2), mJ in T.mfmat.items():
            for (s1, s2), mS in mJ.items():
                for irrep, mm in mS.items():
                    blocks.append(("mf", _key(J1), _key(J2), str(s1), str(s2), _key(irrep), None, pk.add(mm)))
    info["blocks"] = blocks
    meta[prefix] = info
    out.update(pk.arrays(prefix + "/"))


def flat(T, vec_dict, side="2"):
    """Concatenate a {J: {sym: array}} vector in Jlist x symlist order
    (the order of tdse.py:343-360)."""
    Jlist = getattr(T, "Jlist" + side)
    symlist = getattr(T, "symlist" + side)
    dim = getattr(T, "dim" + side)
    return np.concatenate([
        vec_dict[J][s] if (J in vec_dict and s in vec_dict[J]) else np.zeros(dim[J][s], np.complex128)
        for J in Jlist for s in symlist[J]])


def split(T, v, side="2"):
    Jlist = getattr(T, "Jlist" + side)
    symlist = getattr(T, "symlist" + side)
    dim = getattr(T, "dim" + side)
    out, ind = {}, 0
    for J in Jlist:
        out[J] = {}
        for s in symlist[J]:
            out[J][s] = v[ind: ind + dim[J][s]]
            ind += dim[J][s]
    return out


def total_dim(T, side="2"):
    dim = getattr(T, "dim" + side)
    return sum(dim[J][s] for J in getattr(T, "Jlist" + side) for s in getattr(T, "symlist" + side)[J])


def save(name, out, meta):
    out["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {os.path.getsize(path) / 1024:.1f} KiB")


def gaussian_field(t, t0, fwhm, intensity_wcm2, direction):
    """Cycle-averaged Gaussian pulse: E_a(t) with E_a E_b equal to the
    cycle average of the laser field product (E0^2/2 envelope^2)."""
    e0 = np.sqrt(2 * intensity_wcm2 * 1e4 / (const.c * const.epsilon_0))
    env = np.exp(-2 * np.log(2) * (t - t0) ** 2 / fwhm ** 2)
    d = np.asarray(direction, dtype=np.float64)
    d = d / np.linalg.norm(d)
    return list(e0 * env / np.sqrt(2) * d)


# ---------------------------------------------------------------------------
# cases
# ---------------------------------------------------------------------------

def ocs_molecule():
    """Linear OCS: C-O 1.16 A and C-S 1.56 A on z, mu_z = 0.28 au,
    alpha = diag(35, 35, 80) au."""
    ocs = Molecule()
    ocs.XYZ = ("angstrom", "C", 0.0, 0.0, 0.0, "O", 0.0, 0.0, -1.16, "S", 0.0, 0.0, 1.56)
    ocs.dip = [0, 0, 0.28]
    ocs.pol = [[35.0, 0, 0], [0, 35.0, 0], [0, 0, 80.0]]
    return ocs


def asym_molecule():
    """Asymmetric top, Watson A with diagonal quartic terms, D2."""
    m = Molecule()
    m.B = (9.0, 5.0, 3.2)  # (Bx, By, Bz) = (A, B, C)
    m.watson = "watson_a"
    m.DeltaJ = 1e-3
    m.DeltaJK = 1e-3
    m.DeltaK = 1e-3
    m.sym = "D2"
    m.dip = [0, 0, -0.73]
    m.pol = [[9.1, 0, 0], [0, 9.9, 0], [0, 0, 9.4]]
    return m


def vec_checks(name, T, out, rng, nvec=2):
    n2 = total_dim(T, "2")
    xs, ys = [], []
    for _ in range(nvec):
        x = rng.standard_normal(n2) + 1j * rng.standard_normal(n2)
        y = T.vec(split(T, x, "2"))
        xs.append(x)
        ys.append(flat(T, y, "1"))
    out[name + "/vec_x"] = np.array(xs)
    out[name + "/vec_y"] = np.array(ys)


def case_ocs_small(Jmax=6):
    out, meta = {}, {"Jmax": Jmax}
    rng = np.random.default_rng(1234)
    mol = ocs_molecule()
    sol = solve(mol, Jmax=Jmax)
    h0 = LabTensor(mol, sol)
    dip = LabTensor(mol.dip, sol)
    pol = LabTensor(mol.pol, sol)
    cos2 = LabTensor("cos2theta", sol)
    cos = LabTensor("costheta", sol)
    meta["B"] = [float(b) for b in mol.B]

    # generic (tilted) field: exercises x, y and z Cartesian components
    field_vec = [3.0e8, -1.5e8, 9.0e8]
    pol.field(field_vec)
    dip.field(field_vec)
    meta["field_vec"] = field_vec
    for nm, T in (("h0", h0), ("dip", dip), ("pol", pol), ("cos2", cos2), ("cos", cos)):
        export_cartens(T, nm, out, meta, with_mfmat=nm in ("dip", "pol"))
    vec_checks("pol", pol, out, rng)
    vec_checks("dip", dip, out, rng)

    # thresholded field: thresh drops small field products and MF elements
    pol_t = -0.5 * pol * AUpol_x_Vm_to_invcm()
    pol_t.field([2.0e6, 0.0, 9.0e8], thresh=1e13)
    export_cartens(pol_t, "pol_thresh", out, meta, with_mmat=False)
    meta["thresh_field"] = [[2.0e6, 0.0, 9.0e8], 1e13]

    # split-operator propagation through the pulse maximum (z-polarised,
    # 5e11 W/cm^2, FWHM 300 fs, centred at 1 ps)
    Hac = -0.5 * pol * AUpol_x_Vm_to_invcm()
    tdse = TDSE(t_start=0.85, t_end=1.15, dt=0.01, t_units="ps", enr_units="invcm")
    tgrid = tdse.time_grid()
    vecs = tdse.init_state(h0, temp=0)
    out["split/vec0"] = vecs.copy()
    fields, states, times = [], [], []
    for t in tgrid:
        f = gaussian_field(t, 1.0, 0.3, 5e11, [0, 0, 1])
        Hac.field(f)
        vecs, t2 = tdse.update(Hac, H0=h0, vecs=vecs)
        fields.append(f)
        states.append(vecs.copy())
        times.append(t2)
    out["split/fields"] = np.array(fields)
    out["split/states"] = np.array(states)
    out["split/times"] = np.array(times)
    out["split/tc"] = np.asarray(tgrid)
    meta["split"] = dict(t_start=0.85, t_end=1.15, dt=0.01, scale=-0.5 * AUpol_x_Vm_to_invcm())
    c2 = cos2.tomat(form="full", cart="0")
    out["split/cos2"] = np.array([np.vdot(s[0], c2.dot(s[0])).real + 1 / 3 for s in states])

    # full-H form (no H0 kwarg): H = Hac + h0 at a tilted field
    tdse2 = TDSE(t_start=0.0, t_end=0.05, dt=0.01, t_units="ps", enr_units="invcm")
    tdse2.time_grid()
    rng2 = np.random.default_rng(7)
    n = total_dim(h0)
    v0 = rng2.standard_normal((2, n)) + 1j * rng2.standard_normal((2, n))
    v0 /= np.linalg.norm(v0, axis=1)[:, None]
    out["full/vec0"] = v0.copy()
    vecs = v0
    states = []
    for i in range(5):
        Hac.field([1.0e9, 0.0, 2.0e9])
        H = Hac + h0
        vecs, _ = tdse2.update(H, vecs)
        states.append(vecs.copy())
    out["full/states"] = np.array(states)
    meta["full"] = dict(t_start=0.0, t_end=0.05, dt=0.01, field=[1.0e9, 0.0, 2.0e9])
    save("ocs_j%d" % Jmax, out, meta)


def case_asym_small(Jmax=4):
    out, meta = {}, {"Jmax": Jmax}
    rng = np.random.default_rng(4321)
    mol = asym_molecule()
    sol = solve(mol, Jmax=Jmax)
    h0 = LabTensor(mol, sol, thresh=1e-9)
    dip = LabTensor(mol.dip, sol)
    pol = LabTensor(mol.pol, sol)
    cos2 = LabTensor("cos2theta", sol)
    field_vec = [4.0e8, 2.5e8, -7.0e8]
    pol.field(field_vec)
    dip.field(field_vec)
    meta["field_vec"] = field_vec
    for nm, T in (("h0", h0), ("dip", dip), ("pol", pol), ("cos2", cos2)):
        export_cartens(T, nm, out, meta, with_mfmat=nm in ("dip", "pol"))
    vec_checks("pol", pol, out, rng)
    vec_checks("dip", dip, out, rng)

    # energies of the field-free solution, per (J, sym), for the factor builder
    out["enr"] = np.concatenate([np.asarray(sol[J][s].enr) for J in sol.keys() for s in sol[J].keys()])
    meta["enr_keys"] = [[int(J), str(s), len(sol[J][s].enr)] for J in sol.keys() for s in sol[J].keys()]

    # DC field 20 kV/cm along z plus a 1e12 W/cm^2 FWHM 500 fs pulse at 35 deg
    dc = [0.0, 0.0, 20e3 * 1e2]
    beta = np.deg2rad(35.0)
    Hdc = -1 * dip * dc * AUdip_x_Vm_to_invcm()
    Hac = -0.5 * pol * AUpol_x_Vm_to_invcm()
    meta["dc"] = dc
    meta["scales"] = dict(dc=-1 * AUdip_x_Vm_to_invcm(), ac=-0.5 * AUpol_x_Vm_to_invcm())
    sum_vec = Hdc + (Hac * field_vec)
    vec_checks("sum", sum_vec, out, rng, nvec=1)

    tdse = TDSE(t_start=0.9, t_end=1.0, dt=0.005, t_units="ps", enr_units="invcm")
    tgrid = tdse.time_grid()
    vecs = tdse.init_state(h0, temp=5, thresh=1e-3)
    out["split/vec0"] = vecs.copy()
    fields, states = [], []
    for t in tgrid:
        f = gaussian_field(t, 1.0, 0.5, 1e12, [np.sin(beta), 0, np.cos(beta)])
        Hac.field(f)
        vecs, _ = tdse.update(Hdc + Hac, H0=h0, vecs=vecs)
        fields.append(f)
        states.append(vecs.copy())
    out["split/fields"] = np.array(fields)
    out["split/states_first2"] = np.array(states)[:, :2]
    out["split/final"] = states[-1]
    out["split/tc"] = np.asarray(tgrid)
    meta["split"] = dict(t_start=0.9, t_end=1.0, dt=0.005)

    # initial states
    tdse_i = TDSE(t_end=1.0, dt=0.01)
    for lab, kw in (("t0", dict(temp=0)), ("t5", dict(temp=5, thresh=1e-3)),
                    ("t50", dict(temp=50, thresh=1e-6)), ("tnone", dict(temp=None))):
        v = tdse_i.init_state(h0, **kw)
        rows, cols = np.nonzero(v)
        out["init/" + lab + "/shape"] = np.array(v.shape)
        out["init/" + lab + "/rows"] = rows
        out["init/" + lab + "/cols"] = cols
        out["init/" + lab + "/vals"] = v[rows, cols]
    # field-dressed ground state through the dense eigh path (tdse.py:231-233)
    out["init/dressed_t0"] = tdse_i.init_state(h0 + Hdc, temp=0)
    save("asym_j%d" % Jmax, out, meta)


def case_lanczos():
    """Direct calls of _expmv_lanczos (tdse.py:417-486) on dense matrices."""
    out, meta = {}, {}
    rng = np.random.default_rng(99)
    n = 40
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    H = (A + A.conj().T) / 2
    out["H"] = H
    cases = []
    for ic, (fac, scale) in enumerate(((-0.05j, 1.0), (-0.3j, 1.0), (-0.05j, 0.2))):
        v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        v = v / np.linalg.norm(v) * scale  # scale != 1: unnormalised first vector
        calls = [0]

        def mv(x):
            calls[0] += 1
            return H.dot(x)
        u = _expmv_lanczos(v, fac, mv)
        out["v%d" % ic] = v
        out["u%d" % ic] = u
        cases.append(dict(fac=[fac.real, fac.imag], nmatvec=calls[0]))
    # maximum-order failure
    try:
        _expmv_lanczos(out["v1"], -20j, lambda x: H.dot(x), maxorder=6)
        cases.append(dict(maxorder_error=False))
    except ValueError:
        cases.append(dict(maxorder_error=True))
    # zero operator (breakdown branch, tdse.py:459-465)
    v = out["v0"]
    out["u_zero"] = _expmv_lanczos(v, -0.1j, lambda x: np.zeros_like(x))
    meta["cases"] = cases
    save("lanczos", out, meta)


def case_ocs_trove(nsteps=600):
    """Legacy OCS alignment: even J<=30, M=0 (tests/benchmarks/data/alignment_ocs)."""
    out, meta = {}, {}
    path = os.path.join(REF, "tests/benchmarks/data/alignment_ocs/")

    def filt(**kw):
        ok = True
        if "J" in kw:
            ok = ok and kw["J"] <= 30 and kw["J"] % 2 == 0
        if "m" in kw:
            ok = ok and float(kw["m"]) == 0.0
        return ok
    H0 = CarTensTrove(path + "matelem/ocs_energies_j0_j30.rchm", bra=filt, ket=filt)
    scale = -0.5 * AUpol_x_Vm_to_invcm()
    alpha = CarTensTrove(path + "matelem/ocs_energies_j0_j30.rchm",
                         path + "matelem/ocs_matelem_alpha_j<j1>_j<j2>.rchm", bra=filt, ket=filt)
    export_cartens(H0, "h0", out, meta)
    export_cartens(alpha, "alpha", out, meta, with_mfmat=False)
    Hbar = alpha * scale
    meta["scale"] = scale
    fields = np.array([[0.0, 0.0, 1e2 * float(l.split()[3])] for l in open(path + "field.txt")][:nsteps])
    out["fields"] = fields
    ref = []
    with open(path + "pop_reference.txt") as f:
        next(f)
        for line in f:
            s = line.split()
            ref.append([float(s[2 + 6 * j]) if 6 * (j + 1) < len(s) else 0.0 for j in range(7)])
    out["pop_reference"] = np.array(ref[: nsteps // 10 + 1])
    tdse = TDSE(t_end=nsteps * 0.01, dt=0.01)
    tgrid = tdse.time_grid()
    vecs = tdse.init_state(H0, temp=0)
    out["vec0"] = vecs.copy()
    pops, states = [], []
    t0 = time.time()
    for i, _ in enumerate(tgrid):
        Hbar.field(fields[i])
        vecs, _ = tdse.update(Hbar, vecs, H0=H0)
        if i % 10 == 0:
            pops.append(np.abs(vecs[0][:7]) ** 2)
        if i % 50 == 49:
            states.append(vecs.copy())
    print("trove replay", time.time() - t0, "s")
    out["pops"] = np.array(pops)
    out["states"] = np.array(states)
    meta["nsteps"] = nsteps
    meta["J_order"] = [int(J) for J in H0.Jlist1]
    save("ocs_trove", out, meta)


def case_trunc_pulse(nsteps=3000):
    """README known answer: OCS J<=10 truncated-pulse alignment (README.md:246-330)."""
    out, meta = {}, {}
    ocs = Molecule()
    ocs.XYZ = ("angstrom",
               "C", 0.0, 0.0, -0.522939783141,
               "O", 0.0, 0.0, -1.680839357,
               "S", 0.0, 0.0, 1.037160128)
    ocs.dip = [0, 0, -0.31093]
    ocs.pol = [[25.5778097, 0, 0], [0, 25.5778097, 0], [0, 0, 52.4651140]]
    sol = solve(ocs, Jmax=10)
    pol = LabTensor(ocs.pol, sol)
    h0 = LabTensor(ocs, sol)
    cos2 = LabTensor("cos2theta", sol)
    for nm, T in (("h0", h0), ("pol", pol), ("cos2", cos2)):
        export_cartens(T, nm, out, meta, with_mfmat=False)
    d = os.path.join(REF, "docs/source/notebooks/")
    field = np.array([[float(e) for e in l.split()[1:]] for l in open(d + "trunc_pulse.txt")])[:nsteps] * 1e2
    ref = np.array([[float(e) for e in l.split()[:2]] for l in open(d + "trunc_pulse_cos2theta.txt")])
    out["fields"] = field
    out["cos2_reference"] = ref[ref[:, 0] <= nsteps * 0.01 + 1e-9]
    tdse = TDSE(t_start=0, t_end=nsteps * 0.01, dt=0.01, t_units="ps", enr_units="invcm")
    vecs = tdse.init_state(h0, temp=0)
    H = -0.5 * pol * AUpol_x_Vm_to_invcm()
    meta["scale"] = -0.5 * AUpol_x_Vm_to_invcm()
    c2 = cos2.tomat(form="full", cart="0")
    cos2_t, times = [], []
    t0 = time.time()
    for i, t in enumerate(tdse.time_grid()):
        H.field([0, 0, field[i, 2]])
        vecs, t2 = tdse.update(H, H0=h0, vecs=vecs)
        cos2_t.append(np.vdot(vecs[0], c2.dot(vecs[0])).real + 1 / 3)
        times.append(t2)
    print("trunc pulse replay", time.time() - t0, "s")
    out["cos2"] = np.array(cos2_t)
    out["times"] = np.array(times)
    out["final"] = vecs.copy()
    meta["nsteps"] = nsteps
    save("trunc_pulse_j10", out, meta)


def slab_populations(T, vecs):
    """J-populations of each row of vecs: sum of |v|^2 over the slabs of each J
    (the observable of tests/test_tdse.py:63-67), as an (nvec, nJ) array."""
    out = np.zeros((vecs.shape[0], len(T.Jlist1)))
    for v in range(vecs.shape[0]):
        d = split(T, vecs[v], "1")
        for iJ, J in enumerate(T.Jlist1):
            out[v, iJ] = sum(float(np.sum(np.abs(d[J][s]) ** 2)) for s in T.symlist1[J])
    return out


def expect_rows(mat, vecs):
    """<v|O|v> of each row (complex)."""
    return np.array([np.vdot(v, mat.dot(v)) for v in vecs])


def case_ocs_c1(nsteps=300):
    """The CPU-runnable configuration as configured: linear OCS (C-O 1.16 A,
    C-S 1.56 A), mu_z 0.28 au, alpha diag(35, 35, 80) au, J = 0..20 with all M
    (dim 441), |J=0,M=0>, z-polarised cycle-averaged Gaussian pulse 5e11 W/cm^2,
    FWHM 300 fs at 1 ps, 0-3 ps at dt = 10 fs (300 steps), split operator with
    the reference's internal Lanczos (its expokit path, whose Krylov dimension
    is 12, needs the Fortran extension). Per step: <cos^2>, <cos> and the
    J-populations; states every 10 steps."""
    out, meta = {}, {"Jmax": 20}
    mol = ocs_molecule()
    sol = solve(mol, Jmax=20)
    h0 = LabTensor(mol, sol)
    pol = LabTensor(mol.pol, sol)
    cos2 = LabTensor("cos2theta", sol)
    cos = LabTensor("costheta", sol)
    for nm, T in (("h0", h0), ("pol", pol), ("cos2", cos2), ("cos", cos)):
        export_cartens(T, nm, out, meta, with_mfmat=False)
    scale = -0.5 * AUpol_x_Vm_to_invcm()
    meta["scale"] = scale
    Hac = pol * scale
    tdse = TDSE(t_start=0.0, t_end=nsteps * 0.01, dt=0.01, t_units="ps", enr_units="invcm")
    tgrid = tdse.time_grid()
    vecs = tdse.init_state(h0, temp=0)
    out["vec0"] = vecs.copy()
    c2 = cos2.tomat(form="full", cart="0")
    c1 = cos.tomat(form="full", cart="0")
    fields, saved, saved_steps, cos2_t, cos_t, pops, times = [], [], [], [], [], [], []
    t0 = time.time()
    for i, t in enumerate(tgrid):
        f = gaussian_field(t, 1.0, 0.3, 5e11, [0, 0, 1])
        Hac.field(f)
        vecs, t2 = tdse.update(Hac, H0=h0, vecs=vecs)
        fields.append(f)
        times.append(t2)
        cos2_t.append(expect_rows(c2, vecs).real.sum() + 1 / 3)
        cos_t.append(expect_rows(c1, vecs).real.sum())
        pops.append(slab_populations(h0, vecs).sum(axis=0))
        if i % 10 == 9 or i < 3:
            saved.append(vecs[0].copy())
            saved_steps.append(i)
    print("ocs c1 replay", time.time() - t0, "s")
    out["fields"] = np.array(fields)
    out["times"] = np.array(times)
    out["tc"] = np.asarray(tgrid)
    out["cos2"] = np.array(cos2_t)
    out["cos"] = np.array(cos_t)
    out["pops"] = np.array(pops)
    out["states"] = np.array(saved)
    out["state_steps"] = np.array(saved_steps)
    meta["tdse"] = dict(t_start=0.0, t_end=nsteps * 0.01, dt=0.01)
    meta["pulse"] = dict(t0=1.0, fwhm=0.3, intensity=5e11, direction=[0, 0, 1])
    save("ocs_c1_j20", out, meta)


def case_asym_j10(nsteps=50):
    """The asymmetric top of the larger configurations (A, B, C = 9.0, 5.0,
    3.2 cm^-1, Watson A, D2, mu (0, 0, -0.73) au, alpha diag(9.1, 9.9, 9.4) au) at
    J = 0..10 (dim 1,771): DC 20 kV/cm along z plus the 1e12 W/cm^2 FWHM 500 fs
    pulse at 35 deg, dt = 5 fs, 50 steps through the pulse maximum at 1 ps, from
    the T = 5 K ensemble (thresh 1e-3). Per step and vector: <cos^2>, <cos>,
    J-populations; states of two vectors every 10 steps, all vectors at the end."""
    out, meta = {}, {"Jmax": 10}
    mol = asym_molecule()
    sol = solve(mol, Jmax=10)
    t0 = time.time()
    h0 = LabTensor(mol, sol, thresh=1e-9)
    dip = LabTensor(mol.dip, sol)
    pol = LabTensor(mol.pol, sol)
    cos2 = LabTensor("cos2theta", sol)
    cos = LabTensor("costheta", sol)
    print("asym j10 factors", time.time() - t0, "s")
    for nm, T in (("h0", h0), ("dip", dip), ("pol", pol), ("cos2", cos2), ("cos", cos)):
        export_cartens(T, nm, out, meta, with_mfmat=False)
    out["enr"] = np.concatenate([np.asarray(sol[J][s].enr) for J in sol.keys() for s in sol[J].keys()])
    meta["enr_keys"] = [[int(J), str(s), len(sol[J][s].enr)] for J in sol.keys() for s in sol[J].keys()]
    dc = [0.0, 0.0, 20e3 * 1e2]
    beta = np.deg2rad(35.0)
    direction = [np.sin(beta), 0, np.cos(beta)]
    Hdc = -1 * dip * dc * AUdip_x_Vm_to_invcm()
    Hac = -0.5 * pol * AUpol_x_Vm_to_invcm()
    meta["dc"] = dc
    meta["scales"] = dict(dc=-1 * AUdip_x_Vm_to_invcm(), ac=-0.5 * AUpol_x_Vm_to_invcm())
    t_start = 1.0 - nsteps * 0.005 / 2
    tdse = TDSE(t_start=t_start, t_end=t_start + nsteps * 0.005, dt=0.005, t_units="ps", enr_units="invcm")
    tgrid = tdse.time_grid()
    vecs = tdse.init_state(h0, temp=5, thresh=1e-3)
    out["vec0"] = vecs.copy()
    c2 = cos2.tomat(form="full", cart="0")
    c1 = cos.tomat(form="full", cart="0")
    fields, saved, saved_steps, cos2_t, cos_t, pops = [], [], [], [], [], []
    t0 = time.time()
    for i, t in enumerate(tgrid):
        f = gaussian_field(t, 1.0, 0.5, 1e12, direction)
        Hac.field(f)
        vecs, _ = tdse.update(Hdc + Hac, H0=h0, vecs=vecs)
        fields.append(f)
        cos2_t.append(expect_rows(c2, vecs).real)
        cos_t.append(expect_rows(c1, vecs).real)
        pops.append(slab_populations(h0, vecs))
        if i % 10 == 9:
            saved.append(vecs[:2].copy())
            saved_steps.append(i)
    print("asym j10 replay", time.time() - t0, "s,", vecs.shape[0], "vectors")
    out["fields"] = np.array(fields)
    out["tc"] = np.asarray(tgrid)
    out["cos2"] = np.array(cos2_t)        # (nsteps, nvec), without the 1/3
    out["cos"] = np.array(cos_t)          # (nsteps, nvec)
    out["pops"] = np.array(pops)          # (nsteps, nvec, nJ)
    out["states"] = np.array(saved)       # (nsaved, 2, dim)
    out["state_steps"] = np.array(saved_steps)
    out["final"] = vecs.copy()
    meta["tdse"] = dict(t_start=t_start, t_end=t_start + nsteps * 0.005, dt=0.005)
    meta["pulse"] = dict(t0=1.0, fwhm=0.5, intensity=1e12, direction=direction)
    save("asym_j10", out, meta)


def c1_molecule():
    """An asymmetric top without symmetry (C1), drawn like the uneven-size
    batch's molecules: rotational constants (Bx, By, Bz) = (2.3, 0.71, 0.38)
    cm^-1, dipole (0.31, -0.52, 0.17) au, a non-diagonal symmetric positive
    definite polarizability (eigenvalues 12, 37, 81 au)."""
    m = Molecule()
    m.B = (2.3, 0.71, 0.38)
    m.sym = "C1"
    m.dip = [0.31, -0.52, 0.17]
    q, _ = np.linalg.qr(np.random.default_rng(11).standard_normal((3, 3)))
    p = q @ np.diag([12.0, 37.0, 81.0]) @ q.T
    m.pol = ((p + p.T) / 2).tolist()
    return m


def case_c1_j10(nsteps=10):
    """Factors of a C1 molecule at J = 0..10 (dim 1,771; n_k = 2J + 1) for the
    factor builder, and a short propagation from its T = 2 K ensemble under a
    tilted pulse (the C1 propagation of the uneven-size and serving workloads)."""
    out, meta = {}, {"Jmax": 10}
    mol = c1_molecule()
    sol = solve(mol, Jmax=10)
    t0 = time.time()
    h0 = LabTensor(mol, sol, thresh=1e-9)
    dip = LabTensor(mol.dip, sol)
    pol = LabTensor(mol.pol, sol)
    cos2 = LabTensor("cos2theta", sol)
    print("c1 j10 factors", time.time() - t0, "s")
    for nm, T in (("h0", h0), ("dip", dip), ("pol", pol), ("cos2", cos2)):
        export_cartens(T, nm, out, meta, with_mfmat=False)
    out["enr"] = np.concatenate([np.asarray(sol[J][s].enr) for J in sol.keys() for s in sol[J].keys()])
    meta["enr_keys"] = [[int(J), str(s), len(sol[J][s].enr)] for J in sol.keys() for s in sol[J].keys()]
    meta["mol"] = dict(B=list(mol.B), dip=list(map(float, mol.dip)), pol=np.asarray(mol.pol).tolist())
    direction = [0.48, -0.36, 0.8]
    Hac = -0.5 * pol * AUpol_x_Vm_to_invcm()
    meta["scale"] = -0.5 * AUpol_x_Vm_to_invcm()
    tdse = TDSE(t_start=0.45, t_end=0.45 + nsteps * 0.01, dt=0.01, t_units="ps", enr_units="invcm")
    tgrid = tdse.time_grid()
    vecs = tdse.init_state(h0, temp=2, thresh=1e-2)
    out["vec0"] = vecs.copy()
    c2 = cos2.tomat(form="full", cart="0")
    fields, cos2_t = [], []
    for t in tgrid:
        f = gaussian_field(t, 0.5, 0.2, 3e12, direction)
        Hac.field(f)
        vecs, _ = tdse.update(Hac, H0=h0, vecs=vecs)
        fields.append(f)
        cos2_t.append(expect_rows(c2, vecs).real)
    out["fields"] = np.array(fields)
    out["tc"] = np.asarray(tgrid)
    out["cos2"] = np.array(cos2_t)        # (nsteps, nvec), without the 1/3
    out["final"] = vecs[:4].copy()        # the first four vectors (the file stays small)
    meta["tdse"] = dict(t_start=0.45, t_end=0.45 + nsteps * 0.01, dt=0.01)
    meta["pulse"] = dict(t0=0.5, fwhm=0.2, intensity=3e12, direction=direction)
    save("c1_j10", out, meta)


def filter_predicates():
    """The state filters of case_filter, as (bra, ket, thresh) per name; the
    test restates them."""
    m0 = lambda **kw: kw["m"] == 0 if "m" in kw else True
    low = lambda **kw: kw["enr"] < 60.0 if "enr" in kw else True
    j3 = lambda **kw: kw["J"] <= 3 and kw["sym"] != "B3"
    return {"m0": (m0, m0, None), "enr_j": (low, j3, None), "m0_thresh": (m0, m0, 1e-3)}


def case_filter(Jmax=4):
    """The reference's state filters (field.py:187-447, 1859-1882) applied to
    its own D2 asymmetric-top tensors at J <= 4: the unfiltered h0 and pol with
    their state quanta, and for each filter of filter_predicates the filtered
    tensors (bases, quanta and blocks)."""
    import copy

    def ref_filter(T, bra, ket, thresh=None):
        # field.py:1859-1882 (deepcopy, then CarTens.filter). The reference's
        # filter raises RuntimeError when a filter removes a symmetry of a J it
        # keeps and the tensor holds symtop_basis (field.py:348-352 deletes
        # from the dict it iterates over); that loop only trims symtop_basis,
        # which the blocks do not depend on, so the copy drops it first.
        res = copy.deepcopy(T)
        if hasattr(res, "symtop_basis"):
            del res.symtop_basis
        res.filter(bra=bra, ket=ket, thresh=thresh)
        return res

    out, meta = {}, {"Jmax": Jmax}
    mol = asym_molecule()
    sol = solve(mol, Jmax=Jmax)
    h0 = LabTensor(mol, sol, thresh=1e-9)
    pol = LabTensor(mol.pol, sol)
    for nm, T in (("h0", h0), ("pol", pol)):
        export_cartens(T, nm, out, meta, with_mfmat=False, with_quanta=True)
        for fname, (bra, ket, thresh) in filter_predicates().items():
            export_cartens(ref_filter(T, bra, ket, thresh=thresh), f"{nm}_{fname}", out, meta, with_mfmat=False,
                           with_quanta=True)
    save("filter_j4", out, meta)


def case_trove_files():
    """The legacy OCS TROVE files (tests/benchmarks/data/alignment_ocs/matelem:
    the states file and the alpha matrix-element files) as bytes, so that
    richmol_gb300.trove is tested against ocs_trove.npz (the reference's own
    CarTensTrove objects of the same files) where the reference is absent."""
    out, meta = {}, {"files": []}
    mdir = os.path.join(REF, "tests/benchmarks/data/alignment_ocs/matelem")
    for i, fn in enumerate(sorted(f for f in os.listdir(mdir) if "energies" in f or "alpha" in f)):
        with open(os.path.join(mdir, fn), "rb") as f:
            out[f"file{i}"] = np.frombuffer(f.read(), dtype=np.uint8)
        meta["files"].append(fn)
    save("trove_files", out, meta)


def _notebook_outputs(nb, cell):
    """Text output of the cell-th code cell of a reference notebook."""
    with open(os.path.join(REF, "docs/source/notebooks", nb)) as f:
        cells = [c for c in json.load(f)["cells"] if c["cell_type"] == "code"]
    return "".join("".join(o.get("text", [])) for o in cells[cell].get("outputs", []))


def case_h5_files():
    """The reference's own HDF5 factor files (docs/source/notebooks/water.h5
    and camphor.h5, written by CarTens.store, Molecule.store and
    Solution.store of the reference) as compressed bytes, so that the reader
    of richmol_gb300.hdf5 is tested where the reference is absent, with what
    the reference's notebooks printed from the same files:

    * rotations_quickstart.ipynb, code cell 4: the entries scipy printed of
      the full-matrix dipole X, polarizability XZ and H0 of water.h5;
    * hdf5_files.ipynb, code cell 3: camphor's J = 0..10 energies (6 decimals);

    and the inputs those notebooks gave (water: geometry in bohr, frame ipas,
    D2, J <= 5, dipole and polarizability; camphor: dipole and polarizability
    in the input frame, frame diag(pol), C1, J <= 10)."""
    out, meta = {}, {}
    nbdir = os.path.join(REF, "docs/source/notebooks")
    for nm in ("water", "camphor"):
        with open(os.path.join(nbdir, nm + ".h5"), "rb") as f:
            out[nm + "_h5"] = np.frombuffer(f.read(), dtype=np.uint8)
    text = _notebook_outputs("rotations_quickstart.ipynb", 3)
    sections, cur = {}, None
    for line in text.splitlines():
        for key, tag in (("dipole X:", "dip_x"), ("polarizability XZ:", "pol_xz"), ("field-free Hamiltonian:", "h0")):
            if line.startswith(key):
                cur = tag
                line = line[len(key):]
        if cur is None:
            continue
        line = line.strip()
        if line.startswith("("):
            ij, val = line.split("\t")
            i, j = (int(x) for x in ij.strip("()").split(","))
            sections.setdefault(cur, []).append((i, j, complex(val.strip("()"))))
    for tag, rows in sections.items():
        out["water_" + tag + "_ij"] = np.array([[i, j] for i, j, _ in rows], np.int64)
        out["water_" + tag + "_val"] = np.array([v for _, _, v in rows], np.complex128)
    enr = []
    for line in _notebook_outputs("hdf5_files.ipynb", 2).splitlines():
        w = line.split()
        if len(w) == 6 and w[0].isdigit():
            enr.append((int(w[0]), w[1], int(w[2]), float(w[3])))
    out["camphor_enr_J"] = np.array([e[0] for e in enr], np.int64)
    out["camphor_enr_i"] = np.array([e[2] for e in enr], np.int64)
    out["camphor_enr"] = np.array([e[3] for e in enr])
    meta["water"] = dict(atoms=[["O", 0.0, 0.0, 0.12395915], ["H", 0.0, -1.43102686, -0.98366080],
                                ["H", 0.0, 1.43102686, -0.98366080]], units="bohr", frame="ipas",
                         sym="D2", Jmax=5, dip=[0, 0, -0.7288],
                         pol=[[9.1369, 0, 0], [0, 9.8701, 0], [0, 0, 9.4486]])
    meta["camphor"] = dict(frame="diag(pol)", sym="C1", Jmax=10, dip=[1.21615, -0.30746, 0.01140],
                           pol=[[115.80434, -0.58739, 0.03276], [-0.58739, 112.28245, 1.36146],
                                [0.03276, 1.36146, 108.47809]])
    save("h5_files", out, meta)


CASES = {
    "trove_files": case_trove_files,
    "filter": case_filter,
    "h5_files": case_h5_files,
    "ocs_c1": case_ocs_c1,
    "asym_j10": case_asym_j10,
    "c1_j10": case_c1_j10,
    "ocs_small": case_ocs_small,
    "asym_small": case_asym_small,
    "lanczos": case_lanczos,
    "ocs_trove": case_ocs_trove,
    "trunc_pulse": case_trunc_pulse,
}

if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    for nm in names:
        t0 = time.time()
        CASES[nm]()
        print(nm, "done in %.1f s" % (time.time() - t0))
