"""CPU: the oracle's restatement of the expokit propagator (ZHEXPV scheme,
richmol propag='external') against the exact exponential. The reference's own
Fortran does not build here (no gfortran), so this variant is pinned to
exp(tA)v itself, in the form richmol drives it (A = i H, t = Im(exp_fac),
tdse.py:383-392) and in the Hermitian form the scheme was written for."""
import numpy as np
import pytest
import scipy.linalg

from oracle.expokit import ExpokitError, zhexpv


def _herm(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return (a + a.conj().T) / 2, v


@pytest.mark.parametrize("t", [-0.05, -0.5, 0.2])
def test_richmol_form_matches_expm(t):
    H, v = _herm(60, 0)
    anorm = np.abs(H).sum(axis=0).max()
    st = {}
    w = zhexpv(v, anorm, 12, t, lambda x: H @ x, tol=1e-15, stats=st, c=1j)
    ref = scipy.linalg.expm(t * 1j * H) @ v
    assert np.abs(w - ref).max() / np.abs(ref).max() < 1e-12
    assert st["nstep"] >= 1 and st["nmult"] == 13 * st["nstep"]


def test_hermitian_form_matches_expm():
    H, v = _herm(50, 1)
    anorm = np.abs(H).sum(axis=0).max()
    w = zhexpv(v, anorm, 12, 0.05, lambda x: H @ x, tol=1e-14)
    ref = scipy.linalg.expm(0.05 * H) @ v
    assert np.abs(w - ref).max() / np.abs(ref).max() < 1e-12


@pytest.mark.parametrize("c", [1.0, 1j])
def test_happy_breakdown_is_exact(c):
    """A Krylov space of dimension 3 (three distinct eigenvalues): breakdown at
    j = 3 and one step over the whole interval, in both forms."""
    n = 30
    d = np.repeat([1.0, 2.5, -4.0], 10)
    rng = np.random.default_rng(2)
    q, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    H = q @ np.diag(d) @ q.conj().T
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    st = {}
    w = zhexpv(v, np.abs(H).sum(axis=0).max(), 12, -0.7, lambda x: H @ x, tol=1e-15, stats=st, c=c)
    ref = scipy.linalg.expm(-0.7 * c * H) @ v
    assert np.abs(w - ref).max() / np.abs(ref).max() < 1e-12
    assert st["nstep"] == 1


def test_bad_sizes_raise():
    H, v = _herm(10, 3)
    with pytest.raises(ExpokitError):
        zhexpv(v, 1.0, 12, 0.1, lambda x: H @ x)
