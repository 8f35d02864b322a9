"""Property tests of the host layout of an operator (hypothesis, CPU only):
the ELL form of M factors (plan._ell) rebuilds every matrix exactly with every
stored column inside the matrix, and column chunks (plan._chunks) cover every
element of the row-major slabs exactly once."""
import numpy as np
import pytest
from scipy.sparse import csr_matrix

from richmol_gb300 import plan

hyp = pytest.importorskip("hypothesis")
st = pytest.importorskip("hypothesis.strategies")
given, settings = hyp.given, hyp.settings


@st.composite
def sparse_sets(draw):
    """1-3 matrices of one shape with a shared random pattern (banded or not)."""
    nrows = draw(st.integers(1, 24))
    ncols = draw(st.integers(1, 24))
    ncart = draw(st.integers(1, 3))
    seed = draw(st.integers(0, 2 ** 31 - 1))
    rng = np.random.default_rng(seed)
    if draw(st.booleans()):  # a band of diagonals
        lo = draw(st.integers(-4, 4))
        offs = range(lo, lo + draw(st.integers(1, 5)))
        mask = np.zeros((nrows, ncols), bool)
        for i in range(nrows):
            for o in offs:
                if 0 <= i + o < ncols:
                    mask[i, i + o] = rng.random() < 0.9
    else:
        mask = rng.random((nrows, ncols)) < draw(st.floats(0.0, 0.6))
    mats = []
    for _ in range(ncart):
        m = np.zeros((nrows, ncols), np.complex128)
        m[mask] = rng.normal(size=mask.sum()) + 1j * rng.normal(size=mask.sum())
        mats.append(m)
    return nrows, ncols, mats


@settings(max_examples=150, deadline=None)
@given(sparse_sets())
def test_ell_rebuilds_every_matrix(case):
    nrows, ncols, mats = case
    width, col, val = plan._ell([csr_matrix(m) for m in mats], nrows, ncols)
    assert val.shape == (len(mats), nrows * width) and col.shape == (nrows * width,)
    if width == 0:
        assert all(not np.any(m) for m in mats)
        return
    assert col.min() >= 0 and col.max() < ncols  # padding columns stay inside the matrix
    rebuilt = np.zeros((len(mats), nrows, ncols), np.complex128)
    rows = np.repeat(np.arange(nrows), width)
    for c in range(len(mats)):
        np.add.at(rebuilt[c], (rows, col), val[c])
    assert np.array_equal(rebuilt, np.array(mats))
    # no two stored values of one row share a column (each entry is stored once)
    for i in range(nrows):
        cols = col[i * width:(i + 1) * width]
        live = np.any(val[:, i * width:(i + 1) * width] != 0, axis=0)
        assert len(set(cols[live])) == int(live.sum())


@settings(max_examples=150, deadline=None)
@given(st.lists(st.tuples(st.integers(1, 9), st.integers(1, 80)), min_size=1, max_size=8),
       st.sampled_from([8, 16, 32]))
def test_chunks_cover_each_element_once(slabs, width):
    dm = np.array([s[0] for s in slabs])
    dk = np.array([s[1] for s in slabs])
    off = np.concatenate([[0], np.cumsum(dm * dk)[:-1]])
    dim = int((dm * dk).sum())
    seen = np.zeros(dim, np.int32)
    for parent, c0, w, rows, o, stride in plan._chunks(dm, dk, off, width):
        assert 1 <= w <= width and rows == dm[parent] and stride == dk[parent]
        assert o == off[parent] + c0 and c0 + w <= dk[parent]
        idx = o + np.arange(rows)[:, None] * stride + np.arange(w)[None, :]
        seen[idx.reshape(-1)] += 1
    assert np.all(seen == 1)
