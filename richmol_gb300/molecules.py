"""Many molecules of uneven basis size propagated together, each with its own field.

The reference propagates one molecule per ``TDSE.update`` call
(richmol/tdse.py:265-414), each with its own H0 and field-dressed tensors. A
``MoleculeSet`` joins the molecules' vectors one after the other (molecule m
at ``offsets[m]``) and their field-coupled tensors into one block-diagonal
operator: the slab table of every molecule in one ragged block table, one
operator part per tensor of each molecule, carrying that molecule's field.
A time step is one field launch (kr_set_field: every molecule's M (x) field
products) and one persistent launch of the segmented FP64 step (kr_seg_step):
the mat-vec tasks of all molecules share the grid, while the Lanczos
recurrence of tdse.py:417-486 runs per molecule, with each molecule's own
coefficients, stopping test (squared distance of successive solutions below
``tol``, tdse.py:476) and Krylov order, and the H0 half-phases around it.
"""
import ctypes

import numpy as np
import torch
from scipy.sparse import diags

from . import _native
from .device import stream_ptr
from .plan import OperatorPlan


class MoleculeSet:
    """Args:
        tdse : richmol_gb300.TDSE     the shared time grid (dt, units)
        h0s : list of CarTens         field-free Hamiltonians, diagonal (split operator)
        tensors : list of CarTens     per molecule the field-coupled tensor or sum of
                                      tensors; its field is set by the caller
                                      (``tensors[m].field(E_m(t))``) before each step
        maxorder : int                Lanczos basis capacity (tdse.py default 100)
        tol : float                   stopping tolerance (tdse.py default 1e-15)
        precision : str               "f64" (default): every product in FP64, as the
                                      reference; "mixed": the mat-vec products in FP32
                                      on the FP32 pipes (complex64 accuracy, about 1e-7
                                      relative per mat-vec) with states, Krylov vectors,
                                      Lanczos scalars and the stopping test in FP64
    """

    def __init__(self, tdse, h0s, tensors, maxorder=100, tol=1e-15, precision="f64"):
        assert len(h0s) == len(tensors) and len(h0s) > 0
        self.tdse = tdse
        self.h0s, self.tensors = list(h0s), list(tensors)
        self.tol = float(tol)
        blocks, sources, sblock = [], [], []
        for m, (h0, T) in enumerate(zip(self.h0s, self.tensors)):
            src0 = h0._parts[0].src
            blocks.append((src0.basis("1"), src0.basis("2")))
            for part in T._parts:
                sources.append(part.src)
                sblock.append(m)
        self.nparts = [len(T._parts) for T in self.tensors]
        self.plan = OperatorPlan(sources, None, None, maxorder=maxorder, blocks=blocks, source_block=sblock)
        slab_seg = np.concatenate([np.full(len(b[0]), m, np.int32) for m, b in enumerate(blocks)])
        self._slab_seg = np.ascontiguousarray(slab_seg)
        h = ctypes.c_void_p()
        _native.check(_native.lib().kr_seg_create(self.plan.op, len(blocks), self._slab_seg.ctypes.data,
                                                  ctypes.byref(h)), self.plan.ctx)
        self.handle = h
        if precision not in ("f64", "mixed"):
            raise ValueError("precision must be 'f64' or 'mixed'")
        self.precision = precision
        _native.check(_native.lib().kr_seg_set_precision(
            h, _native.KR_SEG_F32_MATVEC if precision == "mixed" else _native.KR_SEG_F64), self.plan.ctx)
        self.dims = [sum(dm * dk for _, _, dm, dk in b[0]) for b in blocks]
        self.offsets = np.concatenate([[0], np.cumsum(self.dims)[:-1]]).astype(np.int64)
        self.dim = int(sum(self.dims))
        assert self.dim == self.plan.dim_out
        self._phase = None
        self.last_korder = None

    def _phase_dev(self):
        """exp(exp_fac / 2 * diag H0) of every molecule, one after the other
        (tdse.py:368-375, split operator)."""
        if self._phase is None:
            fac = self.tdse.exp_fac
            ph = []
            for h0 in self.h0s:
                if h0._parts[0].prods is None:
                    h0.field([0, 0, 1])
                H0 = h0.tomat(form="full", cart="0")
                assert (H0 - diags(H0.diagonal())).nnz == 0, "field-free Hamiltonian is not diagonal"
                ph.append(np.exp(fac / 2 * H0.diagonal()))
            self._phase = torch.from_numpy(np.ascontiguousarray(np.concatenate(ph))).cuda()
        return self._phase

    def join(self, vecs):
        """One complex128 CUDA vector from the molecules' vectors (numpy or torch)."""
        out = torch.empty(self.dim, dtype=torch.complex128, device="cuda")
        for m, v in enumerate(vecs):
            t = v if torch.is_tensor(v) else torch.from_numpy(np.ascontiguousarray(v, np.complex128))
            out[self.offsets[m]:self.offsets[m] + self.dims[m]] = t.reshape(-1).to(out.device)
        return out

    def split(self, state):
        """The molecules' vectors (views) of a joint vector."""
        return [state[self.offsets[m]:self.offsets[m] + self.dims[m]] for m in range(len(self.dims))]

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            try:
                _native.lib().kr_seg_destroy(h)
            except Exception:
                pass
            self.handle = None

    def set_field_schedule(self, set_fields, nsteps):
        """Uploads the fields of ``nsteps`` steps at once (kr_set_field_schedule):
        ``set_fields(i)`` sets step i's field on the tensors, as a caller does
        before ``step``. ``step(state, field_step=i)`` then takes step i's field
        from device memory: no host copy and no stream synchronisation per step
        (a set of more than 16 parts otherwise stages its coefficients through
        host memory every step)."""
        steps = []
        for i in range(nsteps):
            set_fields(i)
            steps.append([ps for T in self.tensors for ps in T._part_states()])
        self.plan.set_field_schedule(steps)

    def step(self, state, field_step=None):
        """One TDSE.update of every molecule, in place on the joint vector
        ``state`` ((dim,) complex128 CUDA tensor), each molecule with the field
        its tensor carries (or with step ``field_step`` of the uploaded field
        schedule). ``last_korder``: the Krylov order of each molecule."""
        if field_step is None:
            self.plan.set_field([ps for T in self.tensors for ps in T._part_states()])
        else:
            self.plan.set_field_step(field_step)
        korder = np.zeros(len(self.dims), np.int32)
        fac = self.tdse.exp_fac
        rc = _native.lib().kr_seg_step(self.handle, _native.ptr(state), _native.ptr(self._phase_dev()),
                                       float(fac.real), float(fac.imag), self.tol, korder.ctypes.data, stream_ptr())
        if rc == _native.KR_ERR_MAXORDER:  # tdse.py:480-484
            raise ValueError(f"Lanczos reached maximum order of '{self.plan.maxorder}' without convergence")
        _native.check(rc, self.plan.ctx)
        self.last_korder = korder
        return state

    def expect(self, ops, state):
        """<v_m|O_m|v_m> per molecule (numpy array) for per-molecule H0-type
        tensors ``ops`` (e.g. cos^2 theta), through kr_observables (the FP64
        mat-vec of each and a fixed-order FP64 dot product)."""
        out = np.zeros(len(ops))
        for m, (O, v) in enumerate(zip(ops, self.split(state))):
            if not O._is_sum and O._parts[0].prods is None:
                O.field([0, 0, 1])
            vals, _ = O.device_operator().observables(v.reshape(1, -1))
            out[m] = vals[0].real
        return out

    def launches(self):
        return self.plan.launches() + int(_native.lib().kr_seg_launch_count(self.handle))
