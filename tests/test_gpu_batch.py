"""GPU: the batched mixed-precision ensemble against the plain FP64 path.

Tolerance of the batched form (stated by the propagation contract): every
observable within 1e-6 of the FP64 propagation; the states themselves agree to
the single-precision mat-vec (about 1e-6 relative over these runs)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

OBS_ATOL = 1e-6
# relative max-norm error of one batched mat-vec against the FP64 mat-vec, per
# kind: FP32 products (2^-24 rounding) and split-TF32 tensor-core products
# (about 2^-21 per product)
MV_RTOL = {"fp32": 2e-6, "fp32_reg": 2e-6, "tensor": 1e-5, "tensor_tmem": 1e-5}
MATVECS = ["tensor", "tensor_tmem", "fp32", "fp32_reg"]


def _ct(case, name):
    from richmol_gb300 import CarTens
    return CarTens(os.path.join(GOLDEN, case), name=name)


@pytest.mark.parametrize("matvec", MATVECS)
def test_batch_matches_plain_fp64_fixture_ensemble(matvec):
    """22-vector Boltzmann ensemble of the asymmetric-top fixture (J<=4), DC +
    pulse, 19 split-operator steps: batched vs plain FP64."""
    from oracle import fixtures
    from richmol_gb300 import TDSE
    from richmol_gb300.batch import Ensemble
    d, meta = fixtures.load(os.path.join(GOLDEN, "asym_j4.npz"))
    sc = meta["scales"]
    h0 = _ct("asym_j4.npz", "h0")
    cos2 = _ct("asym_j4.npz", "cos2")
    Hdc = (_ct("asym_j4.npz", "dip") * meta["dc"]) * sc["dc"]
    Hac = _ct("asym_j4.npz", "pol") * sc["ac"]
    sp = meta["split"]
    td = TDSE(t_start=sp["t_start"], t_end=sp["t_end"], dt=sp["dt"])
    tc = td.time_grid()
    v0 = td.init_state(h0, temp=5, thresh=1e-3)
    ens = Ensemble(td, h0, v0.shape[0], tol=1e-10, matvec=matvec)
    ens.load(v0)
    vecs = v0
    c2 = cos2.tomat(form="full", cart="0")
    for i in range(len(tc)):
        Hac.field(d["split/fields"][i])
        H = Hdc + Hac
        ens.step(H)
        vecs, _ = td.update(H, H0=h0, vecs=vecs)
        e = ens.expect(cos2)
        ref = np.array([np.vdot(v, c2.dot(v)) for v in vecs])
        assert np.abs(e - ref).max() < OBS_ATOL
    got = ens.store().cpu().numpy()
    assert np.abs(got - vecs).max() / np.abs(vecs).max() < 1e-5
    assert np.abs(got - d["split/final"]).max() / np.abs(d["split/final"]).max() < 1e-5


@pytest.mark.parametrize("matvec", MATVECS)
def test_batch_thermal_ensemble_observable_within_1e6(matvec):
    """Asymmetric top J<=8 (D2), 64 lowest eigenstates as unit vectors, 300
    steps of 5 fs through the pulse: the Boltzmann-weighted <cos^2 theta> of the
    batch stays within 1e-6 of the plain FP64 propagation at every step."""
    import scipy.constants as const
    from richmol_gb300 import TDSE, workloads
    from richmol_gb300.batch import Ensemble
    wl = workloads.asym_top(Jmax=8)
    td = TDSE(t_start=0.3, t_end=1.8, dt=0.005)
    tc = td.time_grid()
    wl.h0.field([0, 0, 1])
    enr = wl.h0.tomat(form="full").diagonal().real
    order = np.argsort(enr, kind="stable")[:64]
    v0 = np.zeros((64, wl.dim), np.complex128)
    v0[np.arange(64), order] = 1.0
    w = np.exp(-(enr[order] - enr[order[0]]) * (const.h * const.c * 100) / (const.k * 5.0))
    w /= w.sum()
    ens = Ensemble(td, wl.h0, 64, tol=1e-8, matvec=matvec)
    ens.load(v0)
    ref = torch.from_numpy(v0).cuda()
    c2 = wl.cos2.tomat(form="full", cart="0")
    worst = 0.0
    for i in range(len(tc)):
        H = wl.hamiltonian(tc[i])
        ens.step(H)
        ref, _ = td.update(H, H0=wl.h0, vecs=ref, inplace=True)
        if i % 10 == 9 or i == len(tc) - 1:
            e = ens.expect(wl.cos2).real
            r = ref.cpu().numpy()
            er = np.array([np.vdot(x, c2.dot(x)).real for x in r])
            worst = max(worst, abs(np.dot(w, e) - np.dot(w, er)))
            assert np.abs(e - er).max() < 1e-5
    assert worst < OBS_ATOL, worst


@pytest.mark.parametrize("matvec", MATVECS)
@pytest.mark.parametrize("jmax,nvec", [(12, 40), (30, 96), (30, 384), (34, 128)])
def test_batched_matvec_matches_fp64(jmax, nvec, matvec):
    """The complex64 batched mat-vec against the FP64 mat-vec of the same
    operator (DC + tilted pulse, all Delta J couplings) on random vectors; J<=12
    crosses the tile shapes, J<=30 is the ensemble workload's basis, J<=34 has
    slabs with n_k = 17, 18 (the K extent 32 tiles)."""
    from richmol_gb300 import TDSE, workloads
    from richmol_gb300.batch import Ensemble
    wl = workloads.asym_top(Jmax=jmax)
    td = TDSE(t_end=1.0, dt=0.01)
    td.time_grid()
    H = wl.hamiltonian(1.0)
    ens = Ensemble(td, wl.h0, nvec, matvec=matvec)
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn((nvec, wl.dim), dtype=torch.complex128, device="cuda", generator=g)
    y32 = ens.apply(H, x)
    plan = H.device_operator()
    y64 = torch.empty_like(x)
    plan.matvec(x, y64)
    err = (y32 - y64).abs().max().item() / y64.abs().max().item()
    assert err < MV_RTOL[matvec], err


def _scrambled(T, seed):
    """The tensor T with the columns of every M block permuted: the same
    numbers of entries per row on a scattered (non-banded) pattern, which the
    batched mat-vec takes through stored columns instead of diagonal offsets."""
    from scipy.sparse import csr_matrix
    from richmol_gb300 import CarTens
    src = T._parts[0].src
    rng = np.random.default_rng(seed)
    perms, mmat = {}, {}
    for JJ, mJ in src.mmat.items():
        for ss, mS in mJ.items():
            for irrep, mI in mS.items():
                for cart, m in mI.items():
                    n = m.shape[1]
                    p = perms.setdefault(n, rng.permutation(n))
                    d = m.toarray() if hasattr(m, "toarray") else np.asarray(m)
                    mmat.setdefault(JJ, {}).setdefault(ss, {}).setdefault(irrep, {})[cart] = csr_matrix(d[:, p])
    basis = {k: getattr(src, k) for k in ("Jlist1", "Jlist2", "symlist1", "symlist2",
                                          "dim_m1", "dim_m2", "dim_k1", "dim_k2")}
    return CarTens.from_factors(basis, src.kmat, mmat, src.rank, src.carts)


@pytest.mark.parametrize("matvec", MATVECS)
def test_batched_matvec_scattered_m_matches_fp64(matvec):
    from richmol_gb300 import TDSE, workloads
    from richmol_gb300.batch import Ensemble
    from richmol_gb300.convert_units import AUpol_x_Vm_to_invcm
    wl = workloads.asym_top(Jmax=12)
    H = _scrambled(wl.pol, 5) * (-0.5 * AUpol_x_Vm_to_invcm())
    H.field(wl.field(1.0))
    td = TDSE(t_end=1.0, dt=0.01)
    td.time_grid()
    nvec = 64
    ens = Ensemble(td, wl.h0, nvec, matvec=matvec)
    g = torch.Generator(device="cuda").manual_seed(11)
    x = torch.randn((nvec, wl.dim), dtype=torch.complex128, device="cuda", generator=g)
    y32 = ens.apply(H, x)
    y64 = torch.empty_like(x)
    H.device_operator().matvec(x, y64)
    err = (y32 - y64).abs().max().item() / y64.abs().max().item()
    assert err < MV_RTOL[matvec], err


@pytest.mark.parametrize("matvec", MATVECS)
def test_batched_matvec_complex_k_c1_molecule(matvec):
    """A C1 molecule (no symmetry) with a general dipole and polarisability in a
    tilted DC + AC field: complex K blocks (both products of the complex
    contraction) and n_k up to 17 (both tile K extents)."""
    from richmol_gb300 import TDSE, rot
    from richmol_gb300.batch import Ensemble
    from richmol_gb300.convert_units import AUdip_x_Vm_to_invcm, AUpol_x_Vm_to_invcm
    pol_m = np.array([[9.0, 0.5, 0.2], [0.5, 8.0, 0.1], [0.2, 0.1, 7.0]])
    mol = rot.Molecule(B=(2.0, 1.2, 0.8), sym="C1", dip=[0.3, -0.4, 0.5], pol=pol_m)
    sol = rot.Solution(mol, Jmax=8)
    h0 = rot.lab_tensor("h0", sol)
    Hdc = (rot.lab_tensor(mol.dip, sol) * [1e6, 2e6, 3e6]) * (-AUdip_x_Vm_to_invcm())
    Hac = rot.lab_tensor(mol.pol, sol) * (-0.5 * AUpol_x_Vm_to_invcm())
    Hac.field([4e8, -2e8, 6e8])
    H = Hdc + Hac
    td = TDSE(t_end=1.0, dt=0.01)
    td.time_grid()
    nvec = 128
    ens = Ensemble(td, h0, nvec, matvec=matvec)
    g = torch.Generator(device="cuda").manual_seed(17)
    x = torch.randn((nvec, ens.dim), dtype=torch.complex128, device="cuda", generator=g)
    y32 = ens.apply(H, x)
    y64 = torch.empty_like(x)
    H.device_operator().matvec(x, y64)
    err = (y32 - y64).abs().max().item() / y64.abs().max().item()
    assert err < MV_RTOL[matvec], err


def _asym_fixture_setup():
    from oracle import fixtures
    from richmol_gb300 import TDSE
    d, meta = fixtures.load(os.path.join(GOLDEN, "asym_j4.npz"))
    sc = meta["scales"]
    h0 = _ct("asym_j4.npz", "h0")
    Hdc = (_ct("asym_j4.npz", "dip") * meta["dc"]) * sc["dc"]
    Hac = _ct("asym_j4.npz", "pol") * sc["ac"]
    sp = meta["split"]
    td = TDSE(t_start=sp["t_start"], t_end=sp["t_end"], dt=sp["dt"])
    tc = td.time_grid()
    return d, h0, Hdc, Hac, td, tc


@pytest.mark.parametrize("nvec", [1, 129])
def test_batch_ragged_ensemble_sizes_and_zero_vector(nvec):
    """One vector (127 padding lanes) and 129 vectors (two 128-vector groups,
    the second almost all padding), one of them zero: every vector follows the
    plain FP64 path over 5 steps, the zero vector stays zero."""
    from richmol_gb300.batch import Ensemble
    d, h0, Hdc, Hac, td, tc = _asym_fixture_setup()
    dim = sum(b[2] * b[3] for b in h0._parts[0].src.basis("1"))
    rng = np.random.default_rng(nvec)
    v0 = rng.standard_normal((nvec, dim)) + 1j * rng.standard_normal((nvec, dim))
    v0 /= np.linalg.norm(v0, axis=1, keepdims=True)
    if nvec > 1:
        v0[nvec // 2] = 0.0
    ens = Ensemble(td, h0, nvec, tol=1e-10)
    ens.load(v0)
    live = np.linalg.norm(v0, axis=1) > 0
    vecs = v0[live].copy()  # the plain path follows the reference's Lanczos, not meant for zero vectors
    for i in range(5):
        Hac.field(d["split/fields"][i])
        H = Hdc + Hac
        ens.step(H)
        vecs, _ = td.update(H, H0=h0, vecs=vecs, check=False)
    got = ens.store().cpu().numpy()
    assert np.abs(got[live] - vecs).max() < 1e-5
    if nvec > 1:
        assert np.count_nonzero(got[nvec // 2]) == 0
        assert (ens.korder()[nvec // 2]) == 0


def test_batch_zero_field_matvec_is_exactly_zero():
    """A field that makes every MF zero leaves every term empty: the mat-vec
    writes exact zeros (both kinds)."""
    from richmol_gb300.batch import Ensemble
    _, h0, _, Hac, td, _ = _asym_fixture_setup()
    Hac.field([0.0, 0.0, 0.0])
    nvec = 8
    ens = Ensemble(td, h0, nvec)
    x = torch.randn((nvec, ens.dim), dtype=torch.complex128, device="cuda")
    from richmol_gb300.batch import _KINDS
    for kind in _KINDS:
        from richmol_gb300 import _native
        _native.check(_native.lib().kr_batch_set_matvec(
            ens.handle, _KINDS[kind]), ens.ctx)
        y = ens.apply(Hac, x)
        assert torch.count_nonzero(y).item() == 0, kind


def test_batch_maxorder_raises():
    """A step that needs more Krylov vectors than the batch holds is an error
    (the reference's ValueError at maxorder, tdse.py:480-484)."""
    from richmol_gb300 import _native
    from richmol_gb300.batch import Ensemble
    d, h0, Hdc, Hac, td, tc = _asym_fixture_setup()
    Hac.field(np.asarray(d["split/fields"][0]) * 30.0)
    v0 = td.init_state(h0, temp=5, thresh=1e-3)
    ens = Ensemble(td, h0, v0.shape[0], tol=1e-12, mmax=2)
    ens.load(v0)
    with pytest.raises(_native.KrylovError) as e:
        ens.step(Hdc + Hac)
    assert e.value.code == _native.KR_ERR_MAXORDER


def test_batch_populations_match_plain_fp64():
    """J-populations of the 22-vector fixture ensemble after 5 steps against the
    same sums over the plain FP64 vectors."""
    from richmol_gb300.batch import Ensemble
    d, h0, Hdc, Hac, td, tc = _asym_fixture_setup()
    v0 = td.init_state(h0, temp=5, thresh=1e-3)
    ens = Ensemble(td, h0, v0.shape[0], tol=1e-10)
    ens.load(v0)
    vecs = v0
    for i in range(5):
        Hac.field(d["split/fields"][i])
        H = Hdc + Hac
        ens.step(H)
        vecs, _ = td.update(H, H0=h0, vecs=vecs)
    pops = ens.populations()
    off = 0
    ref = {}
    for J, _s, dm, dk in h0._parts[0].src.basis("1"):
        ref[J] = ref.get(J, 0.0) + (np.abs(vecs[:, off:off + dm * dk]) ** 2).sum(axis=1)
        off += dm * dk
    assert sorted(pops) == sorted(ref)
    for J in ref:
        assert np.abs(pops[J] - ref[J]).max() < 1e-6, J
    total = sum(pops.values())
    assert np.abs(total - (np.abs(vecs) ** 2).sum(axis=1)).max() < 1e-6


def _c1_workload(jmax, seed=4):
    """An asymmetric top without symmetry (n_k = 2J + 1, up to 2 jmax + 1),
    random polarizability, pulse polarised off the axes."""
    from richmol_gb300 import rot, workloads
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    pol = (q * np.sign(np.diag(r))) @ np.diag([12.0, 40.0, 75.0]) @ (q * np.sign(np.diag(r))).T
    mol = rot.Molecule(B=(0.9, 0.5, 0.31), sym="C1", pol=0.5 * (pol + pol.T))
    d = np.array([0.3, -0.5, 0.81])
    return workloads.Workload("c1_j%d" % jmax, mol, jmax, 0.0, 0.2, 0.01, None,
                              (0.1, 0.08, 5e12, d / np.linalg.norm(d)))


@pytest.mark.parametrize("matvec", MATVECS)
def test_batch_wide_k_column_chunks_match_fp64(matvec):
    """n_k up to 37 (J <= 18, C1): the batched path splits every slab wider
    than 32 into column chunks with K sub-blocks (row stride = n_k); single
    mat-vecs, states, <cos^2> and J-populations against the plain FP64 path,
    which takes the slabs whole."""
    from richmol_gb300 import TDSE
    from richmol_gb300.batch import Ensemble
    wl = _c1_workload(18)
    basis = wl.h0._parts[0].src.basis("1")
    assert max(b[3] for b in basis) == 37
    td = TDSE(t_start=0.0, t_end=0.12, dt=0.01)
    tc = td.time_grid()
    nvec = 40
    wl.h0.field([0, 0, 1])
    order = np.argsort(wl.h0.tomat(form="full").diagonal().real, kind="stable")
    v0 = np.zeros((nvec, wl.dim), np.complex128)
    v0[np.arange(nvec), order[:nvec]] = 1.0
    ens = Ensemble(td, wl.h0, nvec, tol=1e-10, matvec=matvec)
    assert ens.split == 32 and ens._plan0.split == 32
    ens.load(v0)
    # one mat-vec with the pulse on: chunked complex64 against whole-slab FP64
    H = wl.hamiltonian(0.1)
    x = torch.randn(nvec, wl.dim, dtype=torch.complex128, device="cuda")
    y = ens.apply(H, x)
    y64 = torch.empty_like(x)
    H.device_operator().matvec(x, y64)
    assert float((y - y64).abs().max() / y64.abs().max()) < MV_RTOL[matvec]
    # the plain FP64 path refuses the chunked operator
    from richmol_gb300 import _native
    with pytest.raises(_native.KrylovError) as ei:
        H.device_operator(split=32).matvec(x, torch.empty_like(x))
    assert ei.value.code == _native.KR_ERR_UNSUPPORTED
    c2 = wl.cos2
    ref = torch.from_numpy(v0).cuda()
    for i in range(len(tc)):
        H = wl.hamiltonian(tc[i])
        ens.step(H)
        ref, _ = td.update(H, H0=wl.h0, vecs=ref, inplace=True, check=False)
    e = ens.expect(c2).real
    plan = c2.device_operator()
    yy = torch.empty_like(ref)
    plan.matvec(ref, yy)
    r = torch.sum(torch.conj(ref) * yy, dim=1).real.cpu().numpy()
    assert np.abs(e - r).max() < OBS_ATOL
    got = ens.store()
    assert float((got - ref).abs().max() / ref.abs().max()) < 1e-5
    pops = ens.populations()
    tot = sum(pops.values())
    assert np.allclose(tot, 1.0, atol=1e-9)
    refn = ref.cpu().numpy()
    off = 0
    for J, s, dm, dk in basis:
        blk = refn[:, off:off + dm * dk]
        off += dm * dk
        pops_ref = np.sum(np.abs(blk) ** 2, axis=1)
        pops[J] = pops[J] - pops_ref
    assert max(np.abs(p).max() for p in pops.values()) < 1e-6


def test_batch_expect_on_device_matches_host_expect():
    """Ensemble.expect_into (the weighted observable written to device memory,
    no synchronisation) against the weighted sum of Ensemble.expect, over a trace
    of unsynchronised steps read once at the end."""
    from oracle import fixtures
    from richmol_gb300 import TDSE
    from richmol_gb300.batch import Ensemble
    d, meta = fixtures.load(os.path.join(GOLDEN, "asym_j4.npz"))
    sc = meta["scales"]
    h0 = _ct("asym_j4.npz", "h0")
    cos2 = _ct("asym_j4.npz", "cos2")
    Hdc = (_ct("asym_j4.npz", "dip") * meta["dc"]) * sc["dc"]
    Hac = _ct("asym_j4.npz", "pol") * sc["ac"]
    sp = meta["split"]
    td = TDSE(t_start=sp["t_start"], t_end=sp["t_end"], dt=sp["dt"])
    tc = td.time_grid()
    v0 = td.init_state(h0, temp=5, thresh=1e-3)
    w = np.random.default_rng(3).uniform(0.1, 1.0, v0.shape[0])
    wd = torch.from_numpy(w).cuda()
    a = Ensemble(td, h0, v0.shape[0], tol=1e-10, matvec="tensor_tmem")
    b = Ensemble(td, h0, v0.shape[0], tol=1e-10, matvec="tensor_tmem")
    a.load(v0)
    b.load(v0)
    n = len(tc)
    trace = torch.zeros(n, dtype=torch.float64, device="cuda")
    ones = torch.zeros(n, dtype=torch.float64, device="cuda")
    ref, ref1 = np.zeros(n), np.zeros(n)
    for i in range(n):
        Hac.field(d["split/fields"][i])
        a.step(Hdc + Hac, sync=False)
        a.expect_into(cos2, trace[i:i + 1], wd)
        a.expect_into(cos2, ones[i:i + 1])
        b.step(Hdc + Hac)
        e = b.expect(cos2).real
        ref[i] = float(w @ e)
        ref1[i] = float(e.sum())
    a.sync()
    assert np.abs(trace.cpu().numpy() - ref).max() < 1e-13
    assert np.abs(ones.cpu().numpy() - ref1).max() < 1e-13


def test_batch_expect_on_device_skips_zero_weight_groups():
    """Vector groups of zero weight are left out of the device observable's
    mat-vec; the weighted sum equals the host one over the weighted vectors."""
    from oracle import fixtures
    from richmol_gb300 import TDSE
    from richmol_gb300.batch import Ensemble
    d, meta = fixtures.load(os.path.join(GOLDEN, "asym_j4.npz"))
    sc = meta["scales"]
    h0 = _ct("asym_j4.npz", "h0")
    cos2 = _ct("asym_j4.npz", "cos2")
    Hac = _ct("asym_j4.npz", "pol") * sc["ac"]
    sp = meta["split"]
    td = TDSE(t_start=sp["t_start"], t_end=sp["t_end"], dt=sp["dt"])
    tc = td.time_grid()
    v0 = td.init_state(h0, temp=5, thresh=1e-3)
    nvec = 96
    rng = np.random.default_rng(5)
    v = np.zeros((nvec, v0.shape[1]), np.complex128)
    v[: v0.shape[0]] = v0
    v[v0.shape[0]:] = rng.normal(size=(nvec - v0.shape[0], v0.shape[1]))
    v[v0.shape[0]:] /= np.linalg.norm(v[v0.shape[0]:], axis=1)[:, None]
    w = np.zeros(nvec)
    w[: v0.shape[0]] = rng.uniform(0.1, 1.0, v0.shape[0])
    w[70] = 0.5  # one weighted vector in the third group
    ens = Ensemble(td, h0, nvec, tol=1e-10, matvec="tensor_tmem")
    ens.load(v)
    Hac.field(d["split/fields"][0])
    ens.step(Hac)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    ens.expect_into(cos2, out, torch.from_numpy(w).cuda())
    e = ens.expect(cos2).real
    assert abs(float(out.cpu()[0]) - float(w @ e)) < 1e-13


@pytest.mark.parametrize("matvec", ["tensor_tmem", "fp32"])
def test_batch_next_prologue_kept_through_calls_between_steps(matvec):
    """The state combination of a step also writes the next step's first
    Krylov vector (H0 half-phase times the state) and its norm partials, so the
    next prologue skips its pass over the state. Observables, device
    observables, populations and a standalone product between the steps use
    other buffers: the states come out bit for bit as without them. A reload
    after every step (the prologue then recomputes the vector from the state)
    agrees to the rounding of the store/load round trip."""
    from oracle import fixtures
    from richmol_gb300 import TDSE
    from richmol_gb300.batch import Ensemble
    d, meta = fixtures.load(os.path.join(GOLDEN, "asym_j4.npz"))
    sc = meta["scales"]
    h0 = _ct("asym_j4.npz", "h0")
    cos2 = _ct("asym_j4.npz", "cos2")
    Hdc = (_ct("asym_j4.npz", "dip") * meta["dc"]) * sc["dc"]
    Hac = _ct("asym_j4.npz", "pol") * sc["ac"]
    sp = meta["split"]
    td = TDSE(t_start=sp["t_start"], t_end=sp["t_end"], dt=sp["dt"])
    tc = td.time_grid()
    v0 = td.init_state(h0, temp=5, thresh=1e-3)
    n = v0.shape[0]
    ens = {k: Ensemble(td, h0, n, tol=1e-10, matvec=matvec) for k in ("plain", "calls", "reload")}
    for e in ens.values():
        e.load(v0)
    w = torch.full((n,), 1.0 / n, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    x = torch.from_numpy(np.ascontiguousarray(v0)).cuda()
    for i in range(len(tc)):
        Hac.field(d["split/fields"][i])
        H = Hdc + Hac
        for k, e in ens.items():
            e.step(H)
            if k == "calls":
                e.expect(cos2)
                e.expect_into(cos2, out, w)
                e.populations()
                e.apply(H, x)
            elif k == "reload":
                e.load(e.store())
    a = ens["plain"].store()
    assert torch.equal(a, ens["calls"].store())
    r = ens["reload"].store()
    assert (r - a).abs().max().item() <= 1e-13 * a.abs().max().item()


def test_batch_full_h_without_phase_matches_reference():
    """Full-H steps (no H0 split, so no phase array: the first Krylov vector the
    state combination keeps for the next step is the state itself) on the
    batched path against the reference's own full-H states (linear OCS J<=6,
    five steps), with observables and populations read between the steps."""
    from oracle import fixtures
    from richmol_gb300 import TDSE
    from richmol_gb300.batch import Ensemble
    d, meta = fixtures.load(os.path.join(GOLDEN, "ocs_j6.npz"))
    h0 = _ct("ocs_j6.npz", "h0")
    cos2 = _ct("ocs_j6.npz", "cos2")
    f = meta["full"]
    Hac = _ct("ocs_j6.npz", "pol") * meta["split"]["scale"]
    td = TDSE(t_start=f["t_start"], t_end=f["t_end"], dt=f["dt"])
    td.time_grid()
    v0 = np.atleast_2d(d["full/vec0"])
    ens = Ensemble(td, None, v0.shape[0], tol=1e-8, template=h0, matvec="fp32")
    ens.load(v0)
    for i in range(5):
        Hac.field(f["field"])
        ens.step(Hac + h0)
        ens.expect(cos2)
        ens.populations()
        got = ens.store().cpu().numpy()
        ref = np.atleast_2d(d["full/states"][i])
        assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-5, i
