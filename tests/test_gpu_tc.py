"""GPU: the tensor-core building block of the batched mat-vec - one
tcgen05.mma kind::tf32 tile (128 x 16 x 16) through kr_probe_mma: K-major
operand staging, shared-memory and instruction descriptors, TMEM allocation,
commit to an mbarrier, TMEM load."""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _probe(a, b, entry="kr_probe_mma"):
    from richmol_gb300 import _native
    from richmol_gb300.device import context
    if not os.path.exists(_native.LIB_PATH):
        _native.build_library()
    ctx = context(0)
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    d = np.zeros((128, 16), np.float32)
    _native.check(getattr(_native.lib(), entry)(ctx, a.ctypes.data, b.ctypes.data, d.ctypes.data), ctx)
    return d


def test_mma_small_integers_exact():
    rng = np.random.default_rng(1)
    a = rng.integers(-4, 5, (128, 16)).astype(np.float32)
    b = rng.integers(-4, 5, (16, 16)).astype(np.float32)
    d = _probe(a, b)
    assert np.array_equal(d, a @ b.T)


def test_mma_tf32_precision():
    """Random operands: TF32 keeps 10 explicit mantissa bits of each input."""
    rng = np.random.default_rng(2)
    a = rng.standard_normal((128, 16)).astype(np.float32)
    b = rng.standard_normal((16, 16)).astype(np.float32)
    d = _probe(a, b).astype(np.float64)
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    scale = np.abs(a).astype(np.float64) @ np.abs(b).astype(np.float64).T
    assert np.all(np.abs(d - ref) <= 2.0 ** -9 * scale + 1e-6)


def test_mma_with_a_in_tensor_memory():
    """A in TMEM (lane m = row m, K along the columns), B in shared memory: the
    same products as the shared-memory form, bit for bit."""
    rng = np.random.default_rng(3)
    a = rng.integers(-4, 5, (128, 16)).astype(np.float32)
    b = rng.integers(-4, 5, (16, 16)).astype(np.float32)
    assert np.array_equal(_probe(a, b, "kr_probe_mma_ta"), a @ b.T)
    a = rng.standard_normal((128, 16)).astype(np.float32)
    b = rng.standard_normal((16, 16)).astype(np.float32)
    assert np.array_equal(_probe(a, b, "kr_probe_mma_ta"), _probe(a, b))
