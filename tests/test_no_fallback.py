"""Without a GPU the product path fails loudly: there is no CPU fallback. The C
ABI reports KR_ERR_CUDA from kr_ctx_create, and every device entry point of the
Python facade (TDSE.update, CarTens.vec, Ensemble, MoleculeSet) raises before
computing anything. Runs only on machines without a CUDA device."""
import ctypes
import os

import numpy as np
import pytest
import torch

from richmol_gb300 import TDSE, _native, workloads

pytestmark = pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a GPU")

NO_GPU = "no CPU fallback"


@pytest.fixture(scope="module")
def wl():
    return workloads.asym_top(Jmax=3, dt=0.005, nsteps=400)


def test_c_abi_reports_no_device():
    if not os.path.exists(_native.LIB_PATH):
        _native.build_library()
    h = ctypes.c_void_p()
    rc = _native.lib().kr_ctx_create(0, ctypes.byref(h))
    assert rc == _native.KR_ERR_CUDA and not h.value
    assert "no CUDA device" in _native.last_error()


def test_update_raises(wl):
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    v = np.zeros((1, wl.dim), np.complex128)
    v[0, 0] = 1.0
    with pytest.raises(RuntimeError, match=NO_GPU):
        td.update(wl.hamiltonian(tc[10]), H0=wl.h0, vecs=v)


def test_vec_raises(wl):
    H = wl.hamiltonian(0.5)
    x = {J: {s: np.ones(dm * dk, np.complex128) for s, (dm, dk) in syms.items()}
         for J, syms in _slab_shapes(H).items()}
    with pytest.raises(RuntimeError, match=NO_GPU):
        H.vec(x)


def test_batched_and_molecule_paths_raise(wl):
    from richmol_gb300.batch import Ensemble
    from richmol_gb300.molecules import MoleculeSet
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    td.time_grid()
    with pytest.raises(RuntimeError, match=NO_GPU):
        Ensemble(td, wl.h0, 128)
    with pytest.raises(RuntimeError, match=NO_GPU):
        MoleculeSet(td, [wl.h0], [wl.Hac])


def _slab_shapes(H):
    """{J: {sym: (dim_m, dim_k)}} of the tensor's input basis."""
    out = {}
    for J in H.Jlist2:
        out[J] = {s: (H.dim_m2[J][s], H.dim_k2[J][s]) for s in H.symlist2[J]}
    return out
