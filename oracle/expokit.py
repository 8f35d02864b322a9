"""TEST INFRASTRUCTURE ONLY - numpy restatement of the expokit Krylov
propagator that richmol's ``propag='external'`` calls (richmol/tdse.py:383-392,
richmol/pyexpokit.py:55-89): EXPOKIT's ZHEXPV (R. B. Sidje, ACM Trans. Math.
Softw. 24 (1998) 130-156), vendored by the reference as expokit/expokit.f:2783-3113.

The published algorithm, with the constants of that routine:
  * fixed Krylov dimension m (richmol passes 12), Hermitian three-term
    recurrence (Lanczos) on the Hermitian operator M, happy breakdown at
    ||p_j|| <= 1e-7; the exponent is exp(t c M) with c = 1 (ZHEXPV's own use)
    or c = i (richmol: it passes A = i H as the operator, tdse.py:389; the
    recurrence, written for Hermitian A, then loses orthogonality and misses
    the breakdown of vectors with a small invariant subspace, e.g. the OCS
    ground state under a z field; here the Lanczos runs on H and the projected
    matrix is c T, the same exponential);
  * time stepping over [0, |t|]: first step from the a-priori bound
    (expokit.f:2946-2949), each step accepted when the local error estimate
    (two extra terms of the augmented (m+2) x (m+2) exponential,
    expokit.f:3042-3055) is <= delta * t_step * tol, else the step shrinks
    by gamma * (t_step * tol / err)^(1/m) and is retried (no limit on
    rejections); next step from the same formula; step sizes rounded to 2
    significant digits (expokit.f:2948-2949);
  * delta = 1.2, gamma = 0.9, at most 500 steps (then "maximum number of
    steps reached"), tol raised to sqrt(eps) when <= eps;
  * the small exponential by Pade (6, 6) with scaling and squaring (ZGPADM);
    scipy's expm (Pade 13) is used here - both exact to rounding.
"""
import math

import numpy as np
import scipy.linalg


class ExpokitError(Exception):
    pass


MXSTEP = 500
DELTA = 1.2
GAMMA = 0.9
BREAK_TOL = 1e-7


def _nint(x):
    return math.copysign(math.floor(abs(x) + 0.5), x)


def _round2(x):
    """Step-size rounding of expokit.f:2948-2949: two significant digits."""
    p1 = 10.0 ** (_nint(math.log10(x) - math.sqrt(0.1)) - 1)
    return math.trunc(x / p1 + 0.55) * p1


MXREJECT = 500  # rejections per step (the routine allows any number)


def zhexpv(v, anorm, m, t, matvec, tol=0.0, stats=None, c=1.0):
    """w = exp(t c M) v with the ZHEXPV scheme; ``matvec(x)`` returns M x for a
    Hermitian M, c = 1 or 1j. Raises ExpokitError like richmol/pyexpokit.py:9-18."""
    v = np.asarray(v, dtype=np.complex128).ravel()
    n = v.size
    if m >= n or m <= 0:
        raise ExpokitError("bad input arguments")
    eps = np.finfo(np.float64).eps
    if tol <= eps:
        tol = math.sqrt(eps)
    rndoff = eps * anorm
    t_out = abs(t)
    sgn = 1.0 if t >= 0 else -1.0
    w = v.copy()
    beta = np.linalg.norm(w)
    xm = 1.0 / m
    p2 = tol * ((m + 1) / 2.72) ** (m + 1) * math.sqrt(2.0 * 3.14 * (m + 1))
    t_new = _round2((1.0 / anorm) * (p2 / (4.0 * beta * anorm)) ** xm)
    t_now = 0.0
    nstep = 0
    nmult = 0
    nreject = 0
    mh = m + 2
    while t_now < t_out:
        nstep += 1
        t_step = min(t_out - t_now, t_new)
        beta = np.linalg.norm(w)
        V = np.zeros((m + 1, n), np.complex128)
        Hm = np.zeros((mh, mh), np.complex128)
        V[0] = w / beta
        k1 = 2
        mbrkdwn = m
        avnorm = 0.0
        for j in range(m):
            p = matvec(V[j])
            nmult += 1
            if j > 0:
                p = p - (Hm[j - 1, j] / c) * V[j - 1]
            hjj = np.vdot(V[j], p)
            p = p - hjj * V[j]
            hj1j = np.linalg.norm(p)
            Hm[j, j] = c * hjj
            if hj1j <= BREAK_TOL:
                k1 = 0
                mbrkdwn = j + 1
                t_step = t_out - t_now
                break
            Hm[j, j + 1] = c * hj1j
            Hm[j + 1, j] = c * hj1j
            V[j + 1] = p / hj1j
        if k1 != 0:
            avnorm = np.linalg.norm(matvec(V[m]))
            nmult += 1
        # augmented matrix: h_{m+1,m} = beta_m stays below the diagonal, the
        # entry above it is cleared, and a 1 at (m+2, m+1) (expokit.f:3021-3022)
        Hm[m - 1, m] = 0.0
        Hm[m + 1, m] = 1.0
        nreject_step = 0
        while True:
            if nreject_step > MXREJECT:
                raise ExpokitError("requested tolerance was too high")
            mx = mbrkdwn + k1
            F = scipy.linalg.expm(sgn * t_step * Hm[:mx, :mx])
            if k1 == 0:
                err_loc = tol
                break
            p1 = abs(F[m, 0]) * beta
            p2 = abs(F[m + 1, 0]) * beta * avnorm
            if p1 > 10.0 * p2:
                err_loc, xm = p2, 1.0 / m
            elif p1 > p2:
                err_loc, xm = (p1 * p2) / (p1 - p2), 1.0 / m
            else:
                err_loc, xm = p1, 1.0 / (m - 1)
            if not math.isfinite(err_loc):
                raise ExpokitError("requested tolerance was too high")
            if err_loc <= DELTA * t_step * tol:
                break
            t_step = _round2(GAMMA * t_step * (t_step * tol / err_loc) ** xm)
            nreject += 1
            nreject_step += 1
        mx = mbrkdwn + max(0, k1 - 1)
        w = beta * (F[:mx, 0] @ V[:mx])
        t_new = _round2(GAMMA * t_step * (t_step * tol / err_loc) ** xm)
        t_now += t_step
        if nstep >= MXSTEP:
            raise ExpokitError("maximum number of steps reached without convergence")
    if stats is not None:
        stats.update(nstep=nstep, nmult=nmult, nreject=nreject)
    return w
