"""TDSE: time propagator, GPU drop-in for richmol.tdse.TDSE
(CFEL-CMI/richmol, richmol/tdse.py:27-414).

Same constructor keywords, time grid, units, initial states and update
signature; ``update`` runs the Krylov step on the GPU through the C ABI
(kr_step): the reference's in-house Lanczos recurrence (tdse.py:417-486) in
FP64, with the H0 half-phases of the split-operator form (tdse.py:365-394)
fused into the same persistent kernel. ``matvec_lib`` is accepted for
compatibility and ignored: every product runs on the GPU.
"""
import functools

import numpy as np
import scipy.constants as const
import torch
from scipy.sparse import csr_matrix, diags

from . import _native
from .convert_units import J_to_invcm, MHz_to_invcm
from .device import require_cuda
from .field import CarTens


class ExpokitError(Exception):
    """Error of the external (expokit-scheme) propagator, as richmol.pyexpokit.ExpokitError."""


class BlockEigh:
    """Eigen-decomposition of a sparse Hermitian matrix through its independent
    blocks (connected components of the non-zero pattern): each block is
    diagonalised densely, on the GPU (batched over blocks of equal size) when
    one is present. Eigenvalues come sorted ascending (ties keep block order);
    eigenvectors are formed only for the states asked for."""

    def __init__(self, h):
        from scipy.sparse.csgraph import connected_components
        h = csr_matrix(h)
        self.n = h.shape[0]
        ncomp, labels = connected_components(h != 0, directed=False)
        order = np.argsort(labels, kind="stable")
        self.blocks = np.split(order, np.cumsum(np.bincount(labels, minlength=ncomp))[:-1])
        self._vals, self._vecs = [None] * ncomp, [None] * ncomp
        by_size = {}
        for b, idx in enumerate(self.blocks):
            by_size.setdefault(len(idx), []).append(b)
        use_gpu = torch.cuda.is_available()
        for size, bl in by_size.items():
            mats = np.stack([h[self.blocks[b]][:, self.blocks[b]].toarray() for b in bl]).astype(np.complex128)
            if use_gpu and size > 1:
                w, v = torch.linalg.eigh(torch.from_numpy(mats).cuda())
                w, v = w.cpu().numpy(), v.cpu().numpy()
            else:
                w, v = np.linalg.eigh(mats)
            for i, b in enumerate(bl):
                self._vals[b], self._vecs[b] = w[i], v[i]
        vals = np.concatenate(self._vals) if ncomp else np.zeros(0)
        owner = np.concatenate([np.full(len(self.blocks[b]), b) for b in range(ncomp)]) if ncomp else np.zeros(0, int)
        local = np.concatenate([np.arange(len(self.blocks[b])) for b in range(ncomp)]) if ncomp else np.zeros(0, int)
        srt = np.argsort(vals, kind="stable")
        self.values = vals[srt]
        self._owner, self._local = owner[srt], local[srt]

    def vectors(self, states):
        """Eigenvectors of the given sorted-state indices as rows of a CSR matrix."""
        rows, cols, data = [], [], []
        for r, st in enumerate(np.asarray(states, dtype=np.int64)):
            b, j = self._owner[st], self._local[st]
            idx = self.blocks[b]
            rows.append(np.full(len(idx), r))
            cols.append(idx)
            data.append(self._vecs[b][:, j])
        if not rows:
            return csr_matrix((0, self.n), dtype=np.complex128)
        return csr_matrix((np.concatenate(data), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(len(rows), self.n))

    def all(self):
        """(eigenvalues, eigenvectors as columns of a CSR matrix), like numpy's eigh."""
        return self.values, self.vectors(np.arange(self.n)).transpose().tocsr()


def update_counter(func):
    """tdse.py:11-24: returns (vecs, t2[icall]), the end of the interval."""
    @functools.wraps(func)
    def wrapper(self, *args, **kwargs):
        vecs = func(self, *args, **kwargs)
        name = func.__name__
        icall = self._ncalls.get(name, 0)
        self._ncalls[name] = icall + 1
        return vecs, self._time_grid[1][icall]
    return wrapper


class TDSE:
    """Time propagator (tdse.py:27-144)."""

    def __init__(self, **kwargs):
        self._ncalls = dict()
        if "t_start" in kwargs:
            assert type(kwargs["t_start"]) in [int, float], \
                f"`initial time `t_start` has bad type: '{type(kwargs['t_start'])}', (use 'int', 'float')"
            self._t_start = kwargs["t_start"]
        else:
            self._t_start = 0.0
        assert "t_end" in kwargs, "terminal time 't_end' not found in kwargs"
        assert type(kwargs["t_end"]) in [int, float], \
            f"terminal time `t_end` has bad type: '{type(kwargs['t_end'])}', (use 'int', 'float')"
        assert kwargs["t_end"] > self._t_start, \
            f"terminal time `t_end` has bad value: '{kwargs['t_end']}', (must be > '{self._t_start}')"
        self._t_end = kwargs["t_end"]
        assert "dt" in kwargs, "time step `dt` not found in kwargs"
        assert type(kwargs["dt"]) in [int, float], \
            f"time step `dt` has bad type: '{type(kwargs['dt'])}', (use 'int', 'float')"
        assert kwargs["dt"] <= (self._t_end - self._t_start), \
            f"time step `dt` has bad value : '{kwargs['dt']}', (must be <= '{self._t_end - self._t_start}')"
        self._dt = kwargs["dt"]
        t_units = {"fs": 1e-15, "ps": 1e-12, "ns": 1e-9, "au": const.value("atomic unit of time")}
        if "t_units" in kwargs:
            assert type(kwargs["t_units"]) == str, \
                f"time units `t_units` has bad type: '{type(kwargs['t_units'])}', (use 'str')"
            assert kwargs["t_units"] in list(t_units.keys()), \
                f"time units `t_units` has bad value: '{kwargs['t_units']}', (use 'fs', 'ps', 'ns', 'au')"
            self._t_to_s = t_units[kwargs["t_units"]]
        else:
            self._t_to_s = t_units["ps"]
        enr_units = {"invcm": 1 / J_to_invcm(), "mhz": MHz_to_invcm() / J_to_invcm()}
        if "enr_units" in kwargs:
            assert type(kwargs["enr_units"]) == str, \
                f"energy units `enr_units` has bad type: '{type(kwargs['enr_units'])}', (use 'str')"
            assert kwargs["enr_units"].lower() in list(enr_units.keys()), \
                f"energy units `enr_units` has bad value: '{kwargs['enr_units']}', (use 'invcm', 'MHz')"
            self._enr_to_J = enr_units[kwargs["enr_units"].lower()]
        else:
            self._enr_to_J = enr_units["invcm"]
        self.last_korder = None

    def time_grid(self, grid_type="equidistant"):
        """tdse.py:146-174."""
        assert grid_type.lower() in ["equidistant"], \
            f"time grid type `grid_type` has bad value: '{grid_type}', (use 'equidistant')"
        grid_size = int((self._t_end - self._t_start) / self._dt)
        t_1 = np.linspace(self._t_start, self._t_end, num=grid_size, endpoint=False)
        t_2 = t_1 + self._dt
        t_c = t_1 + self._dt / 2
        self._time_grid = (t_1, t_2, t_c)
        return t_c

    @property
    def exp_fac(self):
        """Factor in the exponent, tdse.py:336-337."""
        return -1j * self._dt * self._t_to_s * self._enr_to_J / const.value("reduced Planck constant")

    def init_state(self, H, temp=None, thresh=1e-3, zpe=None, sparse=False):
        """Initial state vectors, eigenfunctions of H (tdse.py:177-262), on the host."""
        if temp is not None:
            assert temp >= 0, f"temperature `temp` has negative value: '{temp}'"
        assert thresh >= 0, f"partition function threshold `thresh` has negative or zero value: '{thresh}'"
        H_is_diag = False
        try:
            if H.cart[0] == "0":
                H.field([0, 0, 1])
                H_is_diag = True
        except AttributeError:
            pass
        if not hasattr(H, "mfmat"):
            raise AttributeError("hamiltonian `H` has inappropriate type (must be Hamiltonian)") from None
        if H_is_diag:
            enrs = H.tomat(form="full", repres="csr_matrix").diagonal()
            eig = None
        else:
            # tdse.py:231-233 diagonalises the dense matrix; here the
            # independent blocks of H (with a field along z the dressed H
            # conserves m) are diagonalised one by one, and only the
            # eigenvectors of the states kept below are formed
            eig = BlockEigh(H.tomat(form="full", repres="csr_matrix"))
            enrs = eig.values

        def rows(states):  # eigenvectors of the given states, as CSR rows
            if eig is None:  # H diagonal: the basis functions, in basis order
                return diags(np.ones(len(enrs)), format="csr")[np.asarray(states, dtype=np.int64)]
            return eig.vectors(states)

        if zpe is not None:
            assert zpe <= abs(enrs[0]), \
                f"zero-point energy `zpe` has a value that is larger than the lowest energy: " \
                f"zpe = '{zpe}' > emin = '{enrs[0]}'"
        else:
            zpe = enrs[0]
        enrs = enrs - zpe
        if temp is None:
            vecs = rows(np.arange(len(enrs)))
        elif temp == 0:
            vecs = rows([0])
        else:
            enrs = enrs * self._enr_to_J
            beta = 1.0 / (const.value("Boltzmann constant") * temp)
            weights = np.exp(-beta * enrs)
            weights /= np.sum(weights)
            # cumulative sum in state order, as tdse.py:254-255
            cum = np.cumsum(weights)
            inds = [i for i in range(len(weights)) if (1 - np.sum(weights[: i + 1])) > thresh] \
                if len(weights) < 4096 else list(np.nonzero((1 - cum) > thresh)[0])
            sqrt_weights = np.sqrt(weights[inds])
            vecs = rows(inds).multiply(sqrt_weights[:, None])
        if not sparse:
            vecs = csr_matrix(vecs).toarray()
        return vecs.astype(np.complex128)

    def _h0_phase(self, H0, exp_fac, device):
        if "_exp_fac_H0" not in self.__dict__:
            H0_mat = H0.tomat(form="full", cart="0")
            assert (H0_mat - diags(H0_mat.diagonal())).nnz == 0, \
                "field-free Hamiltonian `H0` is not diagonal -> split-operator approach not implemented"
            self._exp_fac_H0 = np.exp(exp_fac / 2 * H0_mat.diagonal())
        dev = self.__dict__.get("_exp_fac_H0_dev")
        if dev is None or dev.device != device:
            dev = torch.from_numpy(np.ascontiguousarray(self._exp_fac_H0)).to(device)
            self._exp_fac_H0_dev = dev
        return dev

    @update_counter
    def update(self, H, vecs, **kwargs):
        """Propagates vectors by one time step (tdse.py:265-414).

        ``vecs`` is a numpy array (returned as a new numpy array) or a complex128
        CUDA tensor (returned as a new CUDA tensor; pass ``inplace=True`` to
        propagate it in place). ``products="df"`` computes the mat-vec products
        in double-float arithmetic on the FP32 pipes (about 1e-14 relative per
        product) instead of FP64; everything else stays FP64."""
        if "H0" in kwargs:
            assert isinstance(kwargs["H0"], CarTens), \
                f"field-free Hamiltonian `H0` is of bad (sub-)class: '{type(kwargs['H0'])}', " \
                f"(must be (sub-class of) '{CarTens}')"
            H0 = kwargs["H0"]
        else:
            H0 = None
        matvec_lib = kwargs.get("matvec_lib", "scipy")
        assert matvec_lib in ["scipy", "numba", "cupy"], \
            f"bad argument for `matvec_lib`: '{matvec_lib}' (must be 'scipy', 'numba', 'cupy')"
        if "propag" in kwargs:
            assert type(kwargs["propag"]) is str, \
                f"propagator 'propag' has bad type: '{type(kwargs['propag'])}', (must be 'str')"
            assert kwargs["propag"] in ["external", "internal"], \
                f"propagator 'propag' has bad value: '{kwargs['propag']}', (use 'external', 'internal')"
            propag = kwargs["propag"]
        else:
            propag = "internal"
        if "tol" in kwargs:
            assert type(kwargs["tol"]) in [int, float], \
                f"tolerance `tol` has bad type: '{type(kwargs['tol'])}', (must be 'int', 'float')"
            assert 0 < kwargs["tol"] <= 1, f"tolerance `tol` has bad value: '{kwargs['tol']}', (must be > 0 and <= 1)"
            tol = kwargs["tol"]
        else:
            tol = 1e-15
        maxorder = int(kwargs.get("maxorder", 100))
        check = bool(kwargs.get("check", True))
        # arithmetic of the mat-vec products (an extension): "f64" as the
        # reference, or "df", double-float products on the FP32 pipes
        products = kwargs.get("products", "f64")
        exp_fac = self.exp_fac

        require_cuda()  # the step runs on the GPU only: no CPU fallback
        as_numpy = isinstance(vecs, np.ndarray)
        if as_numpy:
            v = torch.from_numpy(np.ascontiguousarray(vecs, dtype=np.complex128)).cuda()
        else:
            if not (torch.is_tensor(vecs) and vecs.is_cuda and vecs.dtype == torch.complex128):
                raise TypeError("vecs must be a numpy array or a complex128 CUDA tensor")
            v = vecs if kwargs.get("inplace", False) else vecs.clone()
        v2 = v if v.dim() == 2 else v.reshape(1, -1)

        phase = None
        if H0 is not None:
            phase = self._h0_phase(H0, exp_fac, v.device)
        if not isinstance(H, CarTens):
            raise TypeError(f"hamiltonian `H` has inappropriate type: '{type(H)}'")
        has_field = H._has_field_terms()
        if H0 is not None and not has_field:
            # tdse.py:377: no field term, only the two half-phases
            plan = H0._plan(maxorder)
            plan.step(v2, phase, exp_fac, tol, flags=_native.KR_STEP_SKIP_KRYLOV)
        elif propag == "external":
            # tdse.py:383-392 / 400-411: expokit ZHEXPV per vector, m = 12,
            # A = i H, t = Im(exp_fac), 1-norm estimate of H
            plan = H.device_operator(maxorder=maxorder)
            anorm = plan.norm1()
            for ind in range(v2.shape[0]):
                try:
                    self.last_expv_stats = plan.expv(v2[ind], exp_fac.imag, 12, tol, anorm, phase=phase)
                except _native.KrylovError as e:
                    if e.code == _native.KR_ERR_MAXORDER:  # pyexpokit.py:9-18
                        raise ExpokitError("maximum number of steps reached without convergence") from None
                    if e.code == _native.KR_ERR_ARG:
                        raise ExpokitError("bad input arguments") from None
                    raise
        else:
            plan = H.device_operator(maxorder=maxorder)
            plan.set_precision(products)
            korder = np.zeros(v2.shape[0], np.int32) if check else None
            try:
                plan.step(v2, phase, exp_fac, tol, flags=0, korder=korder)
            except _native.KrylovError as e:
                if e.code == _native.KR_ERR_MAXORDER:  # tdse.py:480-484
                    raise ValueError(f"Lanczos reached maximum order of '{maxorder}' without convergence") from None
                raise
            self.last_korder = korder
        if as_numpy:
            return v.cpu().numpy()
        return v
