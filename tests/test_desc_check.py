"""The descriptor checks of kr_op_create, run on the host with kr_op_check (no
device): the tables plan.build_tables makes pass (whole slabs, column chunks,
molecule blocks), and single planted faults are refused with the status and
message kr_op_create would give."""
import os
from types import SimpleNamespace

import numpy as np
import pytest

from richmol_gb300 import _native, workloads
from richmol_gb300.plan import build_tables, check_desc


@pytest.fixture(scope="module", autouse=True)
def library():
    if not os.path.exists(_native.LIB_PATH):
        _native.build_library()


@pytest.fixture(scope="module")
def mol():
    wl = workloads.uneven_molecules(1, seed=4, jmax_range=(18, 18), t_end=0.2)[0]
    srcs = [p.src for p in wl.pol._parts]
    return srcs, srcs[0].basis("1"), srcs[0].basis("2")


def _copy(T):
    return SimpleNamespace(**{**vars(T), "arrays": {k: v.copy() for k, v in T.arrays.items()}})


def _refused(T, npart, match, code=_native.KR_ERR_ARG, maxorder=100):
    with pytest.raises(_native.KrylovError, match=match) as e:
        check_desc(T, npart, maxorder)
    assert e.value.code == code


def test_built_tables_pass(mol):
    srcs, b1, b2 = mol
    check_desc(build_tables(srcs, b1, b2), len(srcs))
    check_desc(build_tables(srcs, b1, b2, split=32), len(srcs))
    wls = workloads.uneven_molecules(3, seed=9, jmax_range=(4, 8), t_end=0.2)
    blocks = [(w.h0._parts[0].src.basis("1"), w.h0._parts[0].src.basis("2")) for w in wls]
    sources = [w.pol._parts[0].src for w in wls]
    for split in (None, 32):
        T = build_tables(sources, None, None, split=split, blocks=blocks, source_block=[0, 1, 2])
        check_desc(T, 3)


def test_slab_tables(mol):
    srcs, b1, b2 = mol
    T = _copy(build_tables(srcs, b1, b2))
    T.dim_out += 1
    _refused(T, len(srcs), "dim_out does not match")
    T = _copy(build_tables(srcs, b1, b2))
    T.arrays["in_off"][1] += 1
    _refused(T, len(srcs), "malformed input slab table")
    _refused(build_tables(srcs, b1, b2), len(srcs), "maxorder out of range", maxorder=1)
    _refused(build_tables(srcs, b1, b2), _native.KR_MAXPART + 1, "npart out of range")


def test_column_chunk_coverage(mol):
    srcs, b1, b2 = mol
    base = build_tables(srcs, b1, b2, split=32)
    wide = int(np.flatnonzero(base.arrays["out_stride"] > base.arrays["out_dk"])[0])
    T = _copy(base)
    T.arrays["out_off"][wide] += 1  # shifted by one column: overlaps its neighbour
    _refused(T, len(srcs), "overlap|malformed slab chunk table")
    T = _copy(base)
    T.arrays["out_dk"][wide] -= 1  # one column of every row left out
    _refused(T, len(srcs), "do not cover|K block shape")
    T = _copy(base)
    T.arrays["out_stride"][wide] = T.arrays["out_dk"][wide] - 1  # stride below the width
    _refused(T, len(srcs), "malformed slab chunk table")


def test_terms_and_factors(mol):
    srcs, b1, b2 = mol
    base = build_tables(srcs, b1, b2)
    A = base.arrays
    # a term whose K block has another shape
    t = int(np.flatnonzero(A["k_rows"][A["t_k"]] != A["k_rows"][A["t_k"][0]])[0])
    T = _copy(base)
    T.arrays["t_k"][0] = T.arrays["t_k"][t]
    _refused(T, len(srcs), "K block shape does not match")
    # an M column outside the input slab
    T = _copy(base)
    T.arrays["m_col"][0] = 10 ** 6
    _refused(T, len(srcs), "M column outside the input slab")
    # an MF instance of a part the operator does not have
    T = _copy(base)
    T.arrays["mf_part"][0] = len(srcs)
    _refused(T, len(srcs), "malformed MF instance")
    # a term index past the tables
    T = _copy(base)
    T.arrays["t_out"][0] = len(A["out_dm"])
    _refused(T, len(srcs), "term index out of range")
    # a K block reaching past its data
    T = _copy(base)
    T.arrays["k_off"][-1] = T.arrays["k_data"].size
    _refused(T, len(srcs), "K block out of range")
    # more Cartesian components than a rank-2 tensor has
    T = _copy(base)
    T.arrays["m_ncart"][0] = _native.KR_MAXCART + 1
    _refused(T, len(srcs), "malformed M group")


def test_unsupported_width_is_not_an_argument_error(mol):
    """n_k above 128 without column chunks is a limit of the kernels, reported
    as KR_ERR_UNSUPPORTED (the batched path cuts such slabs into chunks)."""
    srcs, b1, b2 = mol
    T = _copy(build_tables(srcs, b1, b2))
    A = T.arrays
    A["out_dk"][0], A["out_dm"][0] = 129, 1  # same element count is not needed: width is checked first
    _refused(T, len(srcs), "n_k above 128", code=_native.KR_ERR_UNSUPPORTED)
