"""Field-dressed initial states (tdse.py:177-262 with a non-diagonal H) through
the block eigensolver of richmol_gb300.tdse: against the reference's golden
dressed ground state (dense eigh in the reference, equal up to phase) and
against dense eigh on scrambled block matrices. Runs on the host here; the
GPU variant (cuSOLVER per block) is in the -m gpu set."""
import os

import numpy as np
import pytest
from scipy.sparse import csr_matrix

from conftest import GOLDEN


def _ct(case, name):
    from richmol_gb300 import CarTens
    return CarTens(os.path.join(GOLDEN, case), name=name)


def _dressed_ground_state():
    from oracle import fixtures
    from richmol_gb300 import TDSE
    d, meta = fixtures.load(os.path.join(GOLDEN, "asym_j4.npz"))
    h0 = _ct("asym_j4.npz", "h0")
    Hdc = (_ct("asym_j4.npz", "dip") * meta["dc"]) * meta["scales"]["dc"]
    td = TDSE(t_end=1.0, dt=0.01)
    return td.init_state(h0 + Hdc, temp=0)[0], d["init/dressed_t0"][0]


def test_dressed_ground_state_matches_reference_up_to_phase():
    v, r = _dressed_ground_state()
    assert abs(abs(np.vdot(v, r)) - 1) < 1e-12


@pytest.mark.gpu
def test_dressed_ground_state_on_gpu_matches_reference_up_to_phase():
    import torch
    assert torch.cuda.is_available()
    v, r = _dressed_ground_state()
    assert abs(abs(np.vdot(v, r)) - 1) < 1e-12


def _scrambled_blocks(sizes, seed):
    rng = np.random.default_rng(seed)
    n = sum(sizes)
    H = np.zeros((n, n), np.complex128)
    o = 0
    for s in sizes:
        a = rng.standard_normal((s, s)) + 1j * rng.standard_normal((s, s))
        H[o:o + s, o:o + s] = (a + a.conj().T) / 2
        o += s
    p = rng.permutation(n)
    return H[np.ix_(p, p)]


def test_block_eigh_matches_dense_eigh():
    from richmol_gb300.tdse import BlockEigh
    H = _scrambled_blocks([7, 1, 12, 7, 30, 3], 4)
    eig = BlockEigh(csr_matrix(H))
    assert len(eig.blocks) == 6
    w = np.linalg.eigvalsh(H)
    assert np.abs(eig.values - w).max() < 1e-12 * np.abs(w).max()
    V = eig.vectors(np.arange(H.shape[0])).toarray()  # rows
    assert np.abs(V @ H.T - eig.values[:, None] * V).max() < 1e-12 * np.abs(w).max()  # rows: v^T H^T = w v^T
    assert np.abs(V.conj() @ V.T - np.eye(H.shape[0])).max() < 1e-12


def test_all_states_reconstruct_the_matrix():
    from richmol_gb300.tdse import BlockEigh
    H = _scrambled_blocks([5, 5, 9], 5)
    vals, vecs = BlockEigh(csr_matrix(H)).all()  # eigenvectors as columns
    V = vecs.toarray()
    assert np.abs(V @ np.diag(vals) @ V.conj().T - H).max() < 1e-12 * np.abs(H).max()
