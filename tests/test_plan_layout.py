"""Host-side M-factor layout (richmol_gb300.plan._ell): the ELL tables must
reproduce every M matrix exactly, banded groups must come in diagonal slot
order (what kr_op_create detects for the batched mat-vec), and padding slots
of packed rows must stay inside the row's own band."""
import numpy as np
import pytest
from scipy.sparse import csr_matrix

from richmol_gb300 import plan


def dense_from_ell(width, col, val, nrows, ncols):
    out = np.zeros((val.shape[0], nrows, ncols), np.complex128)
    for c in range(val.shape[0]):
        for i in range(nrows):
            for w in range(width):
                out[c, i, col[i * width + w]] += val[c, i * width + w]
    return out


def banded(nrows, ncols, offsets, rng):
    m = np.zeros((nrows, ncols), np.complex128)
    for i in range(nrows):
        for o in offsets:
            j = i + o
            if 0 <= j < ncols:
                m[i, j] = rng.normal() + 1j * rng.normal()
    return m


@pytest.mark.parametrize("nrows,ncols,offsets", [(61, 61, range(-2, 3)), (61, 65, range(0, 5)),
                                                  (65, 61, range(-4, 1)), (1, 5, range(-2, 3)),
                                                  (5, 1, range(-2, 3)), (9, 9, [0]), (13, 11, [-3, -1, 1])])
def test_banded_groups_use_diagonal_slots(nrows, ncols, offsets):
    rng = np.random.default_rng(7)
    mats = [banded(nrows, ncols, offsets, rng) for _ in range(3)]
    width, col, val = plan._ell([csr_matrix(m) for m in mats], nrows, ncols)
    assert np.array_equal(dense_from_ell(width, col, val, nrows, ncols), np.array(mats))
    # diagonal slot order: slot w of row i is column i + d0 + w where that lies in the matrix
    nz = [(i, j) for m in mats for i, j in zip(*np.nonzero(m))]
    d0 = min(j - i for i, j in nz)
    wd = max(j - i for i, j in nz) - d0 + 1
    rowmax = max(np.bincount([i for i, _ in set(nz)]))
    if not (wd <= plan.DIAG_MAX and wd <= 2 * rowmax):
        assert width == rowmax  # too sparse for diagonal order: packed rows
        return
    assert width == wd
    c = col.reshape(nrows, width)
    v = np.abs(val).sum(0).reshape(nrows, width)
    for i in range(nrows):
        for w in range(width):
            j = i + d0 + w
            if 0 <= j < ncols:
                assert c[i, w] == j
            else:
                assert v[i, w] == 0 and 0 <= c[i, w] < ncols


def test_scattered_groups_pack_rows_with_in_band_padding():
    rng = np.random.default_rng(3)
    nrows, ncols = 40, 50
    m = np.zeros((nrows, ncols), np.complex128)
    for i in range(nrows):
        if i % 7 == 3:
            continue  # empty rows
        for j in rng.choice(ncols, size=rng.integers(1, 4), replace=False):
            m[i, j] = rng.normal() + 1j * rng.normal()
    width, col, val = plan._ell([csr_matrix(m)], nrows, ncols)
    assert np.array_equal(dense_from_ell(width, col, val, nrows, ncols)[0], m)
    c = col.reshape(nrows, width)
    for i in range(nrows):
        nzc = np.nonzero(m[i])[0]
        if len(nzc):
            assert c[i].min() >= nzc.min() and c[i].max() <= nzc.max()


def test_empty_group():
    width, col, val = plan._ell([csr_matrix((4, 6), dtype=np.complex128)], 4, 6)
    assert width == 0 and col.size == 0 and val.shape == (1, 0)
