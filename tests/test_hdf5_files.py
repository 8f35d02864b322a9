"""The reference's own HDF5 factor files, read by richmol_gb300.hdf5 and
richmol_gb300.io (CarTens(filename=..., name=...)), and rebuilt by the factor
builder from the molecules they were computed for.

The files (tests/golden/h5_files.npz holds their bytes) were written by the
reference's CarTens.store / Molecule.store / Solution.store (richmol/field.py:
1304-1598, rot/molecule.py:390-470): water (D2, J <= 5, frame ipas) in
docs/source/notebooks/water.h5 and camphor (C1, J <= 10, frame diag(pol)) in
camphor.h5. The reader is pinned by what the reference's notebooks printed
from the same files; the builder by the files' factors (M element by element,
K up to eigenvector phases, energies to rounding). CPU only."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_rot_builder import _clusters, _k_equivalent


@pytest.fixture(scope="module")
def h5(tmp_path_factory):
    from oracle import fixtures
    d, meta = fixtures.load(os.path.join(GOLDEN, "h5_files.npz"))
    root = tmp_path_factory.mktemp("h5")
    paths = {}
    for nm in ("water", "camphor"):
        p = root / (nm + ".h5")
        p.write_bytes(d[nm + "_h5"].tobytes())
        paths[nm] = str(p)
    return d, meta, paths


def test_reader_reproduces_notebook_printout(h5):
    """rotations_quickstart.ipynb printed entries of dip.tomat(cart='x'),
    pol.tomat(cart='xz') and h0.tomat(cart='0') after reading water.h5 with the
    reference's CarTens (field.py:1600-1848); the same entries here."""
    from richmol_gb300.field import CarTens
    d, _, paths = h5
    for name, cart, tag in (("dip", "x", "dip_x"), ("pol", "xz", "pol_xz"), ("h0", "0", "h0")):
        T = CarTens(filename=paths["water"], name=name)
        mat = T.tomat(form="full", cart=cart).tocsr()
        assert mat.shape == (286, 286)
        ij, val = d["water_" + tag + "_ij"], d["water_" + tag + "_val"]
        assert len(ij) >= 6
        got = np.array([mat[i, j] for i, j in ij])
        assert np.abs(got - val).max() <= 1e-15 * np.abs(val).max(), tag


def test_reader_energies_match_camphor_notebook(h5):
    """hdf5_files.ipynb printed camphor's energies (6 decimals) for J <= 10;
    the diagonal of the stored field-free tensor 'h' gives them."""
    from richmol_gb300.field import CarTens
    d, _, paths = h5
    h = CarTens(filename=paths["camphor"], name="h")
    for J, i, e in zip(d["camphor_enr_J"], d["camphor_enr_i"], d["camphor_enr"]):
        blk = h.kmat[(float(J), float(J))][("A", "A")]
        k = np.sort(blk[0].toarray().diagonal().real) if 0 in blk else np.zeros(1)
        assert abs(k[i] - e) < 6e-7, (J, i)


def test_reader_structure_and_attributes(h5):
    from richmol_gb300 import hdf5
    _, _, paths = h5
    assert hdf5.is_hdf5(paths["water"]) and not hdf5.is_hdf5(os.path.join(GOLDEN, "c1_j10.npz"))
    with hdf5.File(paths["camphor"]) as f:
        assert sorted(f.keys()) == ["camphor", "dip", "h", "pol", "sol"]
        assert f["dip"].attrs["__class_name__"] == "richmol.field.CarTens"
        assert int(f["pol"].attrs["rank"]) == 2
        assert list(f["pol"].attrs["cart"]) == ["xx", "xy", "xz", "yx", "yy", "yz", "zx", "zy", "zz"]
        g = f["dip/J:0.0,1.0/sym:A,A"]
        ds = g["kmat_data"]
        assert ds.dtype == np.complex128 and ds.shape == (int(np.sum(g.attrs["kmat_nnz"])),)
        assert "J:0.0,1.0/sym:A,A/mmat_indptr" in f["dip"]
        assert "J:0.0,9.0" not in f["dip"]
        with pytest.raises(KeyError):
            f["nothing"]


def test_reader_errors(h5, tmp_path):
    from richmol_gb300 import hdf5, io
    from richmol_gb300.field import CarTens
    _, _, paths = h5
    with pytest.raises(KeyError):
        CarTens(filename=paths["water"], name="alpha")
    with pytest.raises(TypeError):
        io.read_tensor_h5(paths["camphor"], "camphor")  # a Molecule, not a tensor
    bad = tmp_path / "bad.h5"
    bad.write_bytes(hdf5.SIGNATURE + bytes([9]) + bytes(100))
    with pytest.raises(hdf5.HDF5Error):
        hdf5.File(str(bad))
    empty = tmp_path / "empty.h5"
    empty.write_bytes(b"")
    with pytest.raises(hdf5.HDF5Error):
        hdf5.File(str(empty))


def _energies(T):
    out = {}
    for J in T.Jlist1:
        for s in T.symlist1[J]:
            n = T.dim_k1[J][s]
            blk = T.kmat.get((J, J), {}).get((s, s), {})
            out[(J, s)] = blk[0].toarray().diagonal().real if 0 in blk else np.zeros(n)
    return out


def _compare_factors(ref, ours, enr, tol_m=1e-14):
    """ref, ours: CarTens. M element by element; K through the cluster-aware
    comparison of the builder tests (signs and phases of eigenvectors free)."""
    clus = {k: _clusters(e) for k, e in enr.items()}
    assert ours.Jlist1 == ref.Jlist1 and ours.symlist1 == ref.symlist1
    assert ours.dim_k1 == ref.dim_k1 and ours.dim_m1 == ref.dim_m1
    nk = nm = 0
    for Jp in ref.kmat:
        for sp in ref.kmat[Jp]:
            for i in ref.kmat[Jp][sp]:
                a = ref.kmat[Jp][sp][i].toarray()
                try:
                    b = ours.kmat[Jp][sp][i].toarray()
                except (KeyError, AttributeError):
                    b = np.zeros_like(a)
                k1, k2 = (Jp[0], sp[0]), (Jp[1], sp[1])
                assert _k_equivalent(a, b, clus[k1], clus[k2], 1e-10 * max(1.0, np.abs(a).max())), (Jp, sp, i)
                nk += 1
    for Jp in ref.mmat:
        for sp in ref.mmat[Jp]:
            for i in ref.mmat[Jp][sp]:
                for c in ref.mmat[Jp][sp][i]:
                    a = ref.mmat[Jp][sp][i][c].toarray()
                    b = ours.mmat[Jp][sp][i][c].toarray()
                    assert np.abs(a - b).max() < tol_m, (Jp, sp, i, c)
                    nm += 1
    return nk, nm


def _check_file(path, mol, Jmax, names, e_tol):
    from richmol_gb300 import hdf5, rot
    from richmol_gb300.field import CarTens
    sol = rot.Solution(mol, Jmax=Jmax)
    h_name = names[0]
    href = CarTens(filename=path, name=h_name)
    enr = _energies(href)
    for J in sol.Jlist:
        for s, (e, _) in sol.states[J].items():
            assert np.abs(np.sort(e) - np.sort(enr[(float(J), s)])).max() < e_tol * max(1.0, np.abs(e).max()), (J, s)
    with hdf5.File(path) as f:
        flat = {nm: np.asarray(f[nm].attrs["tens_flat"]) for nm in names[1:]}
    counts = {}
    for nm in names[1:]:
        tens = mol.dip if flat[nm].size == 3 else mol.pol
        # the tensor the reference built from, in its molecular frame
        assert np.abs(np.asarray(tens).reshape(-1) - flat[nm]).max() < 1e-12, nm
        ref = CarTens(filename=path, name=nm)
        ours = rot.lab_tensor(tens, sol)._parts[0].src
        counts[nm] = _compare_factors(ref, ours, enr)
    return counts


def test_builder_reproduces_water_file(h5):
    """water.h5: geometry in bohr, frame = principal axes of inertia, D2,
    J <= 5 (rotations_quickstart.ipynb). Energies to 2e-9 relative: the file
    was written with the CODATA 2018 Bohr radius (5.29177210903e-11 m), this
    scipy holds CODATA 2022 (5.29177210544e-11 m), and energies scale with
    1/r^2, a relative shift of 1.36e-9."""
    from richmol_gb300 import rot
    _, meta, paths = h5
    w = meta["water"]
    mol = rot.Molecule.from_geometry([tuple(a) for a in w["atoms"]], frame=w["frame"], sym=w["sym"],
                                     dip=w["dip"], pol=np.array(w["pol"]), units=w["units"])
    counts = _check_file(paths["water"], mol, w["Jmax"], ["h0", "dip", "pol"], 2e-9)
    assert all(nk > 20 and nm > 20 for nk, nm in counts.values()), counts


def test_builder_reproduces_camphor_file(h5):
    """camphor.h5: the stored molecule (atoms with masses, frame_rotation),
    C1, J <= 10 (dim 1,771). Its frame, diag(pol), leaves the inertia tensor
    non-diagonal, so the Hamiltonian is the full 1/2 G_ab J_a J_b form."""
    from richmol_gb300 import rot
    _, meta, paths = h5
    c = meta["camphor"]
    mol = rot.Molecule.read(paths["camphor"], "camphor", sym=c["sym"], dip=c["dip"], pol=np.array(c["pol"]))
    # the stored rotation is the reference's diag(pol) frame of the input tensors
    R = rot.Molecule.frame_matrix(c["frame"], None, None, np.array(c["pol"]))
    assert np.abs(R - mol.frame_rotation).max() < 1e-12
    assert np.abs(mol.G - np.diag(np.diag(mol.G))).max() > 1e-4  # a genuinely non-diagonal G
    counts = _check_file(paths["camphor"], mol, c["Jmax"], ["h", "dip", "pol"], 1e-12)
    # every J pair with |J1 - J2| <= rank: dip 30 K blocks (J = 0 with itself vanishes), pol 57
    assert counts["dip"][0] == 30 and counts["pol"][0] == 57 and min(c[1] for c in counts.values()) >= 90, counts


def test_molecule_frame_rules():
    from richmol_gb300 import rot
    m = np.array([16.0, 1.0, 1.0])
    r = np.array([[0, 0, 0.12], [0, -0.76, -0.47], [0, 0.76, -0.47]])
    assert np.array_equal(rot.Molecule.frame_matrix(None, m, r), np.eye(3))
    R = rot.Molecule.frame_matrix("ipas", m, r)
    I = rot._inertia_com(m, r @ R.T)
    assert np.abs(I - np.diag(np.diag(I))).max() < 1e-12 and np.all(np.diff(np.diag(I)) >= 0)
    with pytest.raises(ValueError):
        rot.Molecule.frame_matrix("diag(pol)", m, r, np.array([[1, 2, 0], [0, 1, 0], [0, 0, 1.0]]))
    with pytest.raises(ValueError):
        rot.Molecule.frame_matrix(np.ones((3, 3)), m, r)
    with pytest.raises(ValueError):
        rot.Molecule.frame_matrix("zxy", m, r)
    with pytest.raises(ValueError):
        rot.Molecule.from_geometry([("C", 0, 0, 0), ("O", 0, 0, -1.16), ("S", 0, 0, 1.56)])  # linear: B only


def test_reader_matlab_user_block_file():
    """A file written by another HDF5 library (MATLAB 7.3 format, in scipy's
    test data): the superblock sits behind a 512-byte user block and its
    addresses are relative to that base; one contiguous float64 dataset
    (linspace(0, 2 pi, 9) as a 9 x 1 column) with a fixed-length string
    attribute."""
    scipy_io = pytest.importorskip("scipy.io.matlab")
    from richmol_gb300 import hdf5
    path = os.path.join(os.path.dirname(scipy_io.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
    if not os.path.exists(path):
        pytest.skip("scipy's MATLAB test data is not installed")
    assert not hdf5.is_hdf5(path)  # the signature is not at offset 0
    with hdf5.File(path) as f:
        assert f.keys() == ["testdouble"]
        ds = f["testdouble"]
        assert ds.shape == (9, 1) and ds.dtype == np.float64
        assert np.array_equal(ds[()][:, 0], np.linspace(0, 2 * np.pi, 9))
        assert ds.attrs["MATLAB_class"] == b"double"


def test_stored_solution_gives_the_files_k_factors_element_by_element(h5):
    """camphor.h5 also holds the reference's rotational solutions (sol, the
    eigenvectors the stored dip and pol were built from). With those
    eigenvectors there is no phase freedom left: the builder's K factors equal
    the file's element by element, and the stored energies the builder's."""
    from richmol_gb300 import rot
    from richmol_gb300.field import CarTens
    from richmol_gb300 import hdf5
    _, meta, paths = h5
    c = meta["camphor"]
    mol = rot.Molecule.read(paths["camphor"], "camphor", sym=c["sym"], dip=c["dip"], pol=np.array(c["pol"]))
    stored = rot.Solution.read(paths["camphor"], "sol", mol)
    ours = rot.Solution(mol, Jmax=c["Jmax"])
    assert stored.Jlist == ours.Jlist
    for J in ours.Jlist:
        e, C = stored.states[J]["A"]
        assert np.abs(e - ours.states[J]["A"][0]).max() < 1e-12 * max(1.0, np.abs(e).max())
        assert np.abs(C.conj().T @ C - np.eye(C.shape[1])).max() < 1e-12  # orthonormal states
    with hdf5.File(paths["camphor"]) as f:
        flat = {nm: np.asarray(f[nm].attrs["tens_flat"]) for nm in ("dip", "pol")}
    for nm, tens in (("dip", mol.dip), ("pol", mol.pol)):
        assert np.abs(np.asarray(tens).reshape(-1) - flat[nm]).max() < 1e-12
        ref = CarTens(filename=paths["camphor"], name=nm)
        got = rot.lab_tensor(tens, stored)._parts[0].src
        n = 0
        for Jp in ref.kmat:
            for sp in ref.kmat[Jp]:
                for i in ref.kmat[Jp][sp]:
                    a = ref.kmat[Jp][sp][i].toarray()
                    b = got.kmat[Jp][sp][i].toarray()
                    assert np.abs(a - b).max() < 1e-12 * max(1.0, np.abs(a).max()), (nm, Jp, i)
                    n += 1
        assert n == (30 if nm == "dip" else 57)


def test_builder_state_labels_match_the_files(h5):
    """The builder's state quanta (label: J, k and tau of the largest Wang
    component and its weight; energy) against the quanta_k the reference
    stored with water's and camphor's tensors. Inside K doublets closer than
    1e-2 cm^-1 (camphor at J >= 8: 6e-10 apart) the eigenvectors mix by the
    eigensolver's round-off, so there the weight is compared to 1e-4."""
    import json
    from richmol_gb300 import hdf5, rot
    from test_rot_builder import CLUSTER_GAP
    _, meta, paths = h5
    w, c = meta["water"], meta["camphor"]
    cases = [
        (paths["water"], "dip", rot.Molecule.from_geometry([tuple(a) for a in w["atoms"]], frame=w["frame"],
                                                            sym=w["sym"], dip=w["dip"], pol=np.array(w["pol"]),
                                                            units=w["units"]), w["Jmax"], 2e-9),
        (paths["camphor"], "dip", rot.Molecule.read(paths["camphor"], "camphor", sym=c["sym"], dip=c["dip"],
                                                    pol=np.array(c["pol"])), c["Jmax"], 1e-12),
    ]
    for path, name, mol, Jmax, etol in cases:
        q = rot.Solution(mol, Jmax=Jmax).quanta()
        with hdf5.File(path) as f:
            ref = json.loads(f[name].attrs["quanta_k1__json"])
        n = 0
        for J in range(Jmax + 1):
            for s, states in ref[f"{J}.0"].items():
                e = np.array([x[1] for x in states])
                for i, ((a, ea), (b, eb)) in enumerate(zip(q[float(J)][s], states)):
                    assert abs(ea - eb) < etol * max(1.0, abs(eb)), (J, s, i)
                    near = np.sort(np.abs(e - e[i]))[1:2] if len(e) > 1 else np.array([np.inf])
                    if near.size and near[0] < CLUSTER_GAP:
                        assert a.split()[:3] == b.split()[:3] and abs(float(a.split()[3]) - float(b.split()[3])) < 1e-4
                    else:
                        assert a == b, (J, s, i, a, b)
                    n += 1
        assert n == sum(len(v) for d in ref.values() for v in d.values())
