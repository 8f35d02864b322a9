"""Time-step loops recorded once as a CUDA graph and replayed with one launch.

A user loop over the reference's ``TDSE.update`` (richmol/tdse.py:265-414,
examples/ocs_alignment.py:70-100) sets the field, then steps, every time step.
``StepGraph`` records a run of such steps for the plain FP64 path: per step the
field launch (kr_set_field, the step's coefficients as kernel parameters, so
each recorded step carries its own field) and the persistent step launch
(kr_step, one per vector) on one stream; ``replay()`` then runs all of them with
no host work in between. The library allocates nothing while stepping, so the
recording holds only these launches and two small memsets per step.

``EnsembleGraph`` does the same for the batched ensemble path: per step the
field launch and the batched step's own nodes (its Krylov loop is a
conditional WHILE node on the device, so a recorded step needs no host
decision between iterations).

Operators of up to 16 parts record their field coefficients as kernel
parameters. Above that (or with ``schedule=True``) the fields of all recorded
steps are uploaded once before recording (kr_set_field_schedule) and each
recorded step sets its own from device memory (kr_set_field_step), since a
per-call copy from host memory cannot be repeated by a replay. No Krylov
orders are read back per step (a Lanczos error is sticky on the device and
raised by ``replay`` through kr_sync_status).
"""
import torch

from . import _native


class StepGraph:
    """Args:
        tdse : richmol_gb300.TDSE      time grid and units
        H0 : CarTens or None           field-free Hamiltonian (split operator)
        vecs : (nvec, dim) complex128 CUDA tensor, propagated in place by replay()
        hamiltonian : callable t -> CarTens with the field of time t set
        times : the times of the recorded steps (e.g. a slice of time_grid())
        tol, maxorder : as TDSE.update
        before_step : optional callable recorded ahead of every step (e.g. an
                      L2 flush for timing)
        schedule : None (fields from device memory above 16 parts), or True /
                   False to force either form
        products : "f64" or "df", the arithmetic of the mat-vec products (as
                   TDSE.update's products), fixed when the steps are recorded
    """

    def __init__(self, tdse, H0, vecs, hamiltonian, times, tol=1e-15, maxorder=100, before_step=None,
                 schedule=None, products="f64"):
        assert torch.is_tensor(vecs) and vecs.is_cuda and vecs.dtype == torch.complex128
        self.vecs = vecs if vecs.dim() == 2 else vecs.reshape(1, -1)
        self.times = list(times)
        fac = tdse.exp_fac
        phase = tdse._h0_phase(H0, fac, vecs.device) if H0 is not None else None
        # operators are created (and uploaded) outside the recording
        self.plan = hamiltonian(self.times[0]).device_operator(maxorder=maxorder)
        self.plan.set_precision(products)
        if schedule is None:
            schedule = len(self.plan.sources) > _native.KR_PART_INLINE
        elif not schedule and len(self.plan.sources) > _native.KR_PART_INLINE:
            raise ValueError(f"above {_native.KR_PART_INLINE} operator parts a recorded step needs the field schedule")
        self.schedule = bool(schedule)
        if self.schedule:
            steps = []
            for t in self.times:
                H = hamiltonian(t)
                if H._plan(maxorder) is not self.plan:
                    raise ValueError("the recorded steps must share one operator (the same factor sources)")
                steps.append(H._part_states())
            self.plan.set_field_schedule(steps)
            self._schedule_gen = self.plan.schedule_gen
        self.graph = torch.cuda.CUDAGraph()
        stream = torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.graph(self.graph, stream=stream):
            for i, t in enumerate(self.times):
                if before_step is not None:
                    before_step()
                if self.schedule:
                    plan = self.plan
                    plan.set_field_step(i)  # field launch of this step, from the schedule
                else:
                    plan = hamiltonian(t).device_operator(maxorder=maxorder)  # field launch of this step
                    plan.set_precision(products)
                plan.step(self.vecs, phase, fac, tol, flags=0, korder=None)
        torch.cuda.current_stream().wait_stream(stream)

    def replay(self):
        """Runs the recorded steps on the current stream's device and checks
        the Lanczos status afterwards (ValueError at maxorder, as tdse.py:480-484)."""
        if self.schedule and self.plan.schedule_gen != self._schedule_gen:
            raise RuntimeError("the operator's field schedule was replaced after this recording")
        self.graph.replay()
        try:
            self.plan.sync_status()
        except _native.KrylovError as e:
            if e.code == _native.KR_ERR_MAXORDER:
                raise ValueError("Lanczos reached maximum order without convergence") from None
            raise
        return self.vecs


class EnsembleGraph:
    """A run of batched ensemble steps (batch.Ensemble.step) recorded once as
    a CUDA graph and replayed with one launch.

    Args:
        ens : batch.Ensemble         the ensemble (its states are propagated in place)
        hamiltonian : callable t -> CarTens with the field of time t set
        times : the times of the recorded steps
        schedule : None (fields from device memory above 16 parts), or True /
                   False to force either form
    """

    def __init__(self, ens, hamiltonian, times, schedule=None):
        if ens.matvec == "auto":
            raise ValueError("tune the ensemble's mat-vec kind (one step) before recording")
        self.ens = ens
        self.times = list(times)
        dev = torch.device("cuda", torch.cuda.current_device())
        phase = ens.tdse._h0_phase(ens.H0, ens.tdse.exp_fac, dev) if ens.H0 is not None else None
        self.plan = hamiltonian(self.times[0]).device_operator(split=ens.split)
        if schedule is None:
            schedule = len(self.plan.sources) > _native.KR_PART_INLINE
        elif not schedule and len(self.plan.sources) > _native.KR_PART_INLINE:
            raise ValueError(f"above {_native.KR_PART_INLINE} operator parts a recorded step needs the field schedule")
        self.schedule = bool(schedule)
        if self.schedule:
            steps = []
            for t in self.times:
                H = hamiltonian(t)
                if H._plan(split=ens.split) is not self.plan:
                    raise ValueError("the recorded steps must share one operator (the same factor sources)")
                steps.append(H._part_states())
            self.plan.set_field_schedule(steps)
            self._schedule_gen = self.plan.schedule_gen
        self.graph = torch.cuda.CUDAGraph()
        stream = torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.graph(self.graph, stream=stream):
            for i, t in enumerate(self.times):
                if self.schedule:
                    self.plan.set_field_step(i)
                    ens._step_plan(self.plan, phase, sync=False)
                else:
                    ens.step(hamiltonian(t), sync=False)
        torch.cuda.current_stream().wait_stream(stream)

    def replay(self):
        """Runs the recorded steps and reports a step error afterwards
        (KrylovError, code KR_ERR_MAXORDER when mmax was not enough)."""
        if self.schedule and self.plan.schedule_gen != self._schedule_gen:
            raise RuntimeError("the operator's field schedule was replaced after this recording")
        self.graph.replay()
        self.ens.sync()
