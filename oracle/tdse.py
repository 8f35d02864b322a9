"""Oracle restatement of the reference time propagator.

Reference: richmol/tdse.py (CFEL-CMI/richmol). Same units, time convention,
split-operator order and Lanczos recurrence, including its quirks:

* the first Krylov vector is the input vector itself, not normalised
  (tdse.py:443-446);
* re-orthogonalisation happens only on exact breakdown, starting from a
  vector of ones (tdse.py:455-465);
* the stopping test is on the *squared* distance of successive solutions
  against ``tol`` (default 1e-15, tdse.py:333 and 476);
* expm of the leading (k+1)x(k+1) block of T and the full rebuild of the
  solution on every iteration (tdse.py:474-475).
"""
import numpy as np
import scipy.constants as const
from scipy.sparse import csr_matrix, diags
from scipy.sparse.linalg import expm

from .cartens import flat, split

# convert_units.py:14-19 and tdse.py:129-143
_J_TO_INVCM = 1.0 / (const.value("Planck constant") * 1e2 * const.value("speed of light in vacuum"))
_MHZ_TO_INVCM = 1.0 / const.value("speed of light in vacuum") * 1e4
T_UNITS = {"fs": 1e-15, "ps": 1e-12, "ns": 1e-9, "au": const.value("atomic unit of time")}
ENR_UNITS = {"invcm": 1.0 / _J_TO_INVCM, "mhz": _MHZ_TO_INVCM / _J_TO_INVCM}


class OTDSE:
    """tdse.py:27-414."""

    def __init__(self, t_start=0.0, t_end=None, dt=None, t_units="ps", enr_units="invcm"):
        self._ncalls = {}
        self._t_start = t_start
        self._t_end = t_end
        self._dt = dt
        self._t_to_s = T_UNITS[t_units]
        self._enr_to_J = ENR_UNITS[enr_units.lower()]

    def time_grid(self):
        """tdse.py:146-174: interval starts t1, ends t2 and centres tc."""
        n = int((self._t_end - self._t_start) / self._dt)
        t1 = np.linspace(self._t_start, self._t_end, num=n, endpoint=False)
        self._time_grid = (t1, t1 + self._dt, t1 + self._dt / 2)
        return self._time_grid[2]

    @property
    def exp_fac(self):
        """tdse.py:336-337."""
        return -1j * self._dt * self._t_to_s * self._enr_to_J / const.value("reduced Planck constant")

    def init_state(self, H, temp=None, thresh=1e-3, zpe=None):
        """tdse.py:177-262 (dense output)."""
        H_is_diag = False
        if getattr(H, "cart", [None])[0] == "0":
            H.field([0, 0, 1])
            H_is_diag = True
        if H_is_diag:
            enrs = H.tomat(form="full", repres="csr_matrix").diagonal()
            vecs = diags(np.ones(len(enrs)), format="csr")
        else:
            hmat = H.tomat(form="full", repres="dense")
            enrs, vecs = np.linalg.eigh(hmat)
            vecs = csr_matrix(vecs)
        if zpe is None:
            zpe = enrs[0]
        enrs = enrs - zpe
        vecs = vecs.transpose()
        if temp is None:
            pass
        elif temp == 0:
            vecs = vecs.getrow(0)
        else:
            enrs = enrs * self._enr_to_J
            beta = 1.0 / (const.value("Boltzmann constant") * temp)
            w = np.exp(-beta * enrs)
            w /= np.sum(w)
            # tdse.py:254-255: cumulative sum in basis order
            inds = [i for i in range(len(w)) if (1 - np.sum(w[: i + 1])) > thresh]
            vecs = csr_matrix(vecs)[inds].multiply(np.sqrt(w[inds])[:, None])
        return csr_matrix(vecs).toarray().astype(np.complex128)

    def update(self, H, vecs, H0=None, tol=1e-15):
        """tdse.py:265-414 with propag='internal'. Returns (vecs2, t2)."""
        exp_fac = self.exp_fac

        def cartensvec(v):
            return flat(H, H.vec(split(H, v, "2")), "1")

        if H0 is not None:
            if not hasattr(self, "_exp_fac_H0"):
                h0 = H0.tomat(form="full", cart="0")
                assert (h0 - diags(h0.diagonal())).nnz == 0, "H0 is not diagonal"
                self._exp_fac_H0 = np.exp(exp_fac / 2 * h0.diagonal())
            vecs2 = vecs * self._exp_fac_H0
            if hasattr(H, "mfmat") and len(H.mfmat) > 0:
                for i, v in enumerate(vecs2):
                    vecs2[i] = expmv_lanczos(v, exp_fac, cartensvec, tol=tol)
            vecs2 *= self._exp_fac_H0
        else:
            vecs2 = np.empty(vecs.shape, dtype=vecs.dtype)
            for i, v in enumerate(vecs):
                vecs2[i] = expmv_lanczos(v, exp_fac, cartensvec, tol=tol)
        icall = self._ncalls.get("update", 0)
        self._ncalls["update"] = icall + 1
        return vecs2, self._time_grid[1][icall]


class MaxOrderError(ValueError):
    pass


def expmv_lanczos(vec, fac, matvec, maxorder=100, tol=1e-15, stats=None):
    """tdse.py:417-486: exp(fac*H) vec by the in-house Lanczos recurrence."""
    V, W = [], []
    T = np.zeros((maxorder, maxorder), dtype=vec.dtype)
    V.append(vec)
    w = matvec(V[0])
    T[0, 0] = np.vdot(w, V[0])
    W.append(w - T[0, 0] * V[0])
    u_k, conv_k, k = V[0], 1, 1
    while k < maxorder and conv_k > tol:
        T[k - 1, k] = np.sqrt(sum(np.abs(W[k - 1]) ** 2))
        T[k, k - 1] = T[k - 1, k]
        if not T[k - 1, k] == 0:
            V.append(W[k - 1] / T[k - 1, k])
        else:
            v = np.ones(V[k - 1].shape, dtype=np.complex128)
            for j in range(k):
                v = v - np.vdot(V[j], v) * V[j]
            V.append(v / np.sqrt(sum(np.abs(v) ** 2)))
        w = matvec(V[k])
        T[k, k] = np.vdot(w, V[k])
        w = w - T[k, k] * V[k] - T[k - 1, k] * V[k - 1]
        W.append(w)
        u_km1 = u_k
        expT = expm(fac * T[: k + 1, : k + 1])
        u_k = sum([expT[i, 0] * v_i for i, v_i in enumerate(V)])
        conv_k = sum(np.abs(u_k - u_km1) ** 2)
        k += 1
    if stats is not None:
        stats["k"] = k
        stats["nmatvec"] = k
    if k == maxorder:
        raise MaxOrderError(f"Lanczos reached maximum order of '{maxorder}' without convergence")
    return u_k
