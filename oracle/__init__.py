"""CPU oracle for the TDSE Krylov hot path — TEST INFRASTRUCTURE ONLY.

This package restates, in plain numpy/scipy, the reference algorithm of
CFEL-CMI/richmol for the time-propagation step:

* ``oracle.cartens``  — CarTens.field / CarTens.vec / tomat / scalar and sum
  algebra (reference richmol/field.py).
* ``oracle.tdse``     — TDSE.time_grid / init_state / update and the in-house
  Lanczos exponential _expmv_lanczos (reference richmol/tdse.py).
* ``oracle.fixtures`` — reader of the golden ``.npz`` fixtures written by
  tests/golden/make_golden.py from the reference itself.

Every function cites the reference file:line it follows. The oracle is pinned
against the reference's own outputs (tests/golden/*.npz, generated by running
the reference) and against the reference's known answers for this path
(legacy OCS alignment populations and the README truncated-pulse trace), see
tests/test_oracle_golden.py.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg /
``--impl reference`` arm of ``bench.py`` may import this package, and only as
the checker or the timed CPU baseline. The product package ``richmol_gb300``
never imports it and has no CPU fallback.
"""
