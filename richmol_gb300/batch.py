"""Batched mixed-precision propagation of ensembles (thermal ensembles, many
initial states) on the GPU.

The reference propagates the vectors of an ensemble one after another
(richmol/tdse.py:379-382) with the FP64 Lanczos of tdse.py:417-486. An
``Ensemble`` moves all vectors at once through the C ABI (kr_batch_*): complex64
mat-vec with FP32 accumulation, complex64 Krylov basis with full
orthogonalisation, FP64 Lanczos scalars, tridiagonal exponential and
a-posteriori error estimate (each vector stops at its own Krylov order), FP64
state and H0 half-phases. Observables are weighted sums of per-vector
expectation values, so Boltzmann weights can be applied at the end
(equivalent, by linearity, to the sqrt(w)-weighted vectors of tdse.py:256-257).
"""
import ctypes

import numpy as np
import torch

from . import _native
from .device import stream_ptr


_KINDS = {"tensor": _native.KR_MATVEC_TENSOR, "fp32": _native.KR_MATVEC_FP32,
          "tensor_tmem": _native.KR_MATVEC_TENSOR_TMEM, "fp32_reg": _native.KR_MATVEC_FP32_REG}


class Ensemble:
    """nvec state vectors of one basis, propagated together.

    Args:
        tdse : richmol_gb300.TDSE   time grid, units (exp factor)
        H0 : CarTens or None        field-free Hamiltonian for the split operator
        nvec : int
        tol : float                 per-vector error tolerance of the Krylov step
        mmax : int                  maximum Krylov order (<= 31)
        matvec : str                "tensor" (default): K contractions on the tensor cores
                                    as split-TF32 MMAs (about 2^-21 relative per product);
                                    "tensor_tmem": the same with the A operands in tensor
                                    memory; "fp32": every product an FP32 FMA; "fp32_reg":
                                    the same register-tiled (all terms of a tile
                                    summed in registers); "auto": at
                                    the first step the kind is picked by richmol_gb300.tune
                                    (the cached choice for this operator shape and vector
                                    count, else every kind timed on that step's operator and
                                    the fastest kept and cached; ``self.tuned``: ms per
                                    mat-vec of each)
        tune_cache : bool           "auto" reads and writes the tuning cache file
    """

    def __init__(self, tdse, H0, nvec, tol=1e-8, mmax=20, template=None, matvec="tensor", tune_cache=True):
        self.tdse = tdse
        self.H0 = H0
        self.nvec = int(nvec)
        self.tol = float(tol)
        self.mmax = int(mmax)
        self.template = template if template is not None else H0
        # n_k above 32: slabs go to the batched mat-vec as column chunks of 32
        basis = self.template._parts[0].src.basis("1")
        self.split = 32 if max(b[3] for b in basis) > 32 else None
        self._plan0 = self.template._plan(split=self.split)
        self.dim = self._plan0.dim_out
        self.ctx = self._plan0.ctx
        h = ctypes.c_void_p()
        _native.check(_native.lib().kr_batch_create(self._plan0.op, self.nvec, self.mmax, ctypes.byref(h)), self.ctx)
        self.handle = h
        if matvec not in tuple(_KINDS) + ("auto",):
            raise ValueError(f"matvec must be one of {sorted(_KINDS) + ['auto']}")
        self.matvec = matvec
        self.tuned = None
        self.tuned_from_cache = False
        self.tune_cache = bool(tune_cache)
        _native.check(_native.lib().kr_batch_set_matvec(h, _KINDS["tensor" if matvec == "auto" else matvec]),
                      self.ctx)
        self.phase = None
        self.last_kmax = 0

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            try:
                _native.lib().kr_batch_destroy(h)
            except Exception:
                pass
            self.handle = None

    def load(self, vecs):
        """vecs: (nvec, dim) complex128, numpy or CUDA tensor."""
        v = vecs if torch.is_tensor(vecs) else torch.from_numpy(np.ascontiguousarray(vecs, np.complex128))
        v = v.to("cuda", torch.complex128).contiguous()
        assert v.shape == (self.nvec, self.dim)
        self._keep = v
        _native.check(_native.lib().kr_batch_load(self.handle, v.data_ptr(), stream_ptr()), self.ctx)

    def store(self, out=None):
        if out is None:
            out = torch.empty((self.nvec, self.dim), dtype=torch.complex128, device="cuda")
        _native.check(_native.lib().kr_batch_store(self.handle, out.data_ptr(), stream_ptr()), self.ctx)
        return out

    def step(self, H, sync=True):
        """One TDSE.update of every vector with the field-dressed H.

        The Krylov loop runs on the device (the step is one CUDA graph). With
        ``sync=True`` the call waits for the step, sets ``last_kmax`` and raises
        on a step error (KrylovError with code KR_ERR_MAXORDER when a vector
        needs more than mmax Krylov vectors, the reference's maxorder error of
        tdse.py:480-484); with ``sync=False`` it returns at once and
        ``sync()`` reports errors later. Inside a CUDA-graph recording (a
        capturing stream) the step's nodes join the recording; use sync=False."""
        exp_fac = self.tdse.exp_fac
        phase = None
        if self.H0 is not None:
            phase = self.tdse._h0_phase(self.H0, exp_fac, torch.device("cuda", torch.cuda.current_device()))
        plan = H.device_operator(split=self.split)
        if self.matvec == "auto":
            self._tune(plan)
        self._step_plan(plan, phase, sync)

    def _step_plan(self, plan, phase, sync):
        """kr_batch_step on an operator plan whose field is set."""
        exp_fac = self.tdse.exp_fac
        kmax = ctypes.c_int32()
        rc = _native.lib().kr_batch_step(self.handle, plan.op, None if phase is None else phase.data_ptr(),
                                         float(exp_fac.real), float(exp_fac.imag), self.tol,
                                         ctypes.byref(kmax) if sync else None, stream_ptr())
        self._raise(rc)
        if sync:
            self.last_kmax = kmax.value

    def _raise(self, rc):
        _native.check(rc, self.ctx)  # KrylovError; code KR_ERR_MAXORDER when mmax was not enough

    def sync(self):
        """Waits for the steps launched so far and raises a pending step error;
        sets ``last_kmax`` (largest Krylov order of the last step)."""
        kmax = ctypes.c_int32()
        self._raise(_native.lib().kr_batch_sync(self.handle, ctypes.byref(kmax), stream_ptr()))
        self.last_kmax = kmax.value

    def _tune(self, plan, reps=3):
        """Picks the mat-vec kind for this operator shape and vector count
        (richmol_gb300.tune: from the cache file when the shape was tuned
        before, else every kind timed with CUDA events and the fastest kept
        and stored) and keeps it."""
        from . import tune
        L = _native.lib()

        def run(kind):
            _native.check(L.kr_batch_set_matvec(self.handle, _KINDS[kind]), self.ctx)
            _native.check(L.kr_batch_matvec(self.handle, plan.op, stream_ptr()), self.ctx)

        name = torch.cuda.get_device_name(torch.cuda.current_device())
        best, times, cached = tune.choose(plan, self.nvec, list(_KINDS), run, name, use_cache=self.tune_cache,
                                          reps=reps)
        _native.check(L.kr_batch_set_matvec(self.handle, _KINDS[best]), self.ctx)
        self.tuned = times
        self.tuned_from_cache = cached
        self.matvec = best

    def korder(self):
        out = np.zeros(self.nvec, np.int32)
        _native.check(_native.lib().kr_batch_korder(self.handle, out.ctypes.data, stream_ptr()), self.ctx)
        return out

    def expect(self, O):
        """<v|O|v> for every vector (complex128 numpy array). O is an H0-type
        tensor such as cos^2(theta); its field [0, 0, 1] is set here."""
        if not O._is_sum and O._parts[0].prods is None:
            O.field([0, 0, 1])
        plan = O.device_operator(split=self.split)
        out = np.zeros(2 * self.nvec, np.float64)
        _native.check(_native.lib().kr_batch_expect(self.handle, plan.op, out.ctypes.data, stream_ptr()), self.ctx)
        return out.view(np.complex128)

    def expect_into(self, O, out, weights=None):
        """sum_v w_v Re <v|O|v> into ``out`` (a float64 CUDA tensor of one element,
        e.g. one entry of a trace), ordered on the current stream without a host
        synchronisation (kr_batch_expect_dev); ``weights`` a float64 CUDA tensor of
        nvec weights, or None for all 1. O as in ``expect``."""
        if not O._is_sum and O._parts[0].prods is None:
            O.field([0, 0, 1])
        plan = O.device_operator(split=self.split)
        assert out.is_cuda and out.dtype == torch.float64 and out.numel() >= 1
        wp = None
        if weights is not None:
            assert weights.is_cuda and weights.dtype == torch.float64 and weights.numel() >= self.nvec
            wp = weights.data_ptr()
        _native.check(_native.lib().kr_batch_expect_dev(self.handle, plan.op, wp, out.data_ptr(), stream_ptr()),
                      self.ctx)

    def populations(self):
        """{J: (nvec,) array} J-populations of every vector (sum of |v|^2 over the
        slabs of each J), as the reference's observables (tests/test_tdse.py:63-67)."""
        basis = self.template._parts[0].src.basis("1")
        parent = self._plan0.slab_parent  # slab (or column chunk) -> basis slab
        out = np.zeros(len(parent) * self.nvec, np.float64)
        _native.check(_native.lib().kr_batch_populations(self.handle, out.ctypes.data, stream_ptr()), self.ctx)
        out = out.reshape(len(parent), self.nvec)
        pops = {}
        for p, row in zip(parent, out):
            J = basis[p][0]
            pops[J] = pops.get(J, 0.0) + row
        return pops

    def apply(self, H, x):
        """y = H x for (nvec, dim) complex128 CUDA tensors with the batched
        complex64 mat-vec (the single-precision CarTens.vec)."""
        plan = H.device_operator(split=self.split)
        x = x.contiguous()
        y = torch.empty_like(x)
        _native.check(_native.lib().kr_batch_apply(self.handle, plan.op, x.data_ptr(), y.data_ptr(), stream_ptr()),
                      self.ctx)
        return y

    def launches(self):
        return int(_native.lib().kr_batch_launch_count(self.handle))
