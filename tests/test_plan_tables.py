"""Host tables of an operator (richmol_gb300.plan.build_tables, the kr_op_desc
arrays) checked on the CPU: a numpy reading of the descriptor (the same
contraction the kernels perform, field.py:1212-1243: Y_s1 += MF X_s2 K^T over
strided slabs) applied to random vectors.

* column chunks (split=32, the batched form for n_k above 32) give the same
  operator as whole slabs;
* a block-diagonal operator over several molecules (blocks=..., the
  uneven-size batch) is the molecules' operators side by side, each part
  with its own field coefficients;
* the reading itself agrees with the host assembly CarTens.tomat, fed with
  the field input as kr_set_field receives it (plan.field_arrays)."""
import numpy as np
import pytest

from richmol_gb300 import _native, workloads
from richmol_gb300.plan import build_tables, field_arrays

RTOL = 1e-12


def emulate(T, coef, scale, x):
    """y = H x from the tables: MF = scale_p sum_c coef_{p,c} M_c per instance,
    then per term Y[i, a] += sum_b K[a, b] sum_w MF[i, w] X[col(i, w), b]."""
    A = T.arrays
    out_st = A.get("out_stride", A["out_dk"])
    in_st = A.get("in_stride", A["in_dk"])
    m_val = A["m_val"].view(np.complex128)
    mf = []
    for i in range(T.nmf):
        g, p = A["mf_group"][i], A["mf_part"][i]
        rows, W, nc = int(A["m_rows"][g]), int(A["m_width"][g]), int(A["m_ncart"][g])
        ne = rows * W
        vals = m_val[A["m_val_off"][g]:A["m_val_off"][g] + nc * ne].reshape(nc, ne)
        mfv = scale[p] * (coef[p][:nc, None] * vals).sum(0)
        cols = A["m_col"][A["m_col_off"][g]:A["m_col_off"][g] + ne]
        mf.append((mfv.reshape(rows, W), cols.reshape(rows, W)))
    y = np.zeros(T.dim_out, np.complex128)
    for t in range(T.nterm):
        s1, s2, kb, mi = A["t_out"][t], A["t_in"][t], A["t_k"][t], A["t_mf"][t]
        nk1, nk2, kt, ko = int(A["k_rows"][kb]), int(A["k_cols"][kb]), A["k_type"][kb], A["k_off"][kb]
        if kt == _native.KR_K_REAL:
            K = A["k_data"][ko:ko + nk1 * nk2].reshape(nk1, nk2).astype(np.complex128)
        elif kt == _native.KR_K_IMAG:
            K = 1j * A["k_data"][ko:ko + nk1 * nk2].reshape(nk1, nk2)
        else:
            K = A["k_data"][ko:ko + 2 * nk1 * nk2].view(np.complex128).reshape(nk1, nk2)
        assert nk1 == A["out_dk"][s1] and nk2 == A["in_dk"][s2]
        M, C = mf[mi]
        dm2 = int(A["in_dm"][s2])
        xi = A["in_off"][s2] + np.arange(dm2)[:, None] * in_st[s2] + np.arange(nk2)[None, :]
        X2 = x[xi]
        Z = np.einsum("iw,iwb->ib", M, X2[C])
        dm1 = int(A["out_dm"][s1])
        assert M.shape[0] == dm1
        yi = A["out_off"][s1] + np.arange(dm1)[:, None] * out_st[s1] + np.arange(nk1)[None, :]
        y[yi] += Z @ K.T
    return y


def _field(rng, T):
    coef = [rng.normal(size=len(c)) + 1j * rng.normal(size=len(c)) for c in T.part_carts]
    return coef, np.ones(len(coef), np.complex128)


@pytest.fixture(scope="module")
def c1_molecule():
    return workloads.uneven_molecules(1, seed=4, jmax_range=(18, 18), t_end=0.2)[0]


def test_column_chunks_reproduce_whole_slabs(c1_molecule):
    wl = c1_molecule
    srcs = [p.src for p in wl.pol._parts]
    b1, b2 = srcs[0].basis("1"), srcs[0].basis("2")
    assert max(b[3] for b in b1) == 37
    T0 = build_tables(srcs, b1, b2)
    T1 = build_tables(srcs, b1, b2, split=32)
    A1 = T1.arrays
    # chunks: at most 32 columns, row stride = the parent slab's n_k, every element once
    assert A1["out_dk"].max() <= 32 and A1["in_dk"].max() <= 32
    seen = np.zeros(T1.dim_out, np.int32)
    for s in range(len(A1["out_dm"])):
        par = b1[T1.slab_parent[s]]
        assert A1["out_stride"][s] == par[3] and A1["out_dm"][s] == par[2]
        idx = A1["out_off"][s] + np.arange(A1["out_dm"][s])[:, None] * A1["out_stride"][s] + \
            np.arange(A1["out_dk"][s])[None, :]
        seen[idx.reshape(-1)] += 1
    assert np.all(seen == 1)
    assert T1.nterm > T0.nterm
    rng = np.random.default_rng(0)
    coef, scale = _field(rng, T0)
    for _ in range(2):
        x = rng.normal(size=T0.dim_in) + 1j * rng.normal(size=T0.dim_in)
        y0 = emulate(T0, coef, scale, x)
        y1 = emulate(T1, coef, scale, x)
        assert np.abs(y1 - y0).max() <= RTOL * np.abs(y0).max()


def test_blocks_are_the_molecules_side_by_side():
    wls = workloads.uneven_molecules(3, seed=9, jmax_range=(4, 8), t_end=0.2)
    sources, sblock, blocks = [], [], []
    for m, wl in enumerate(wls):
        b = wl.h0._parts[0].src
        blocks.append((b.basis("1"), b.basis("2")))
        for part in wl.pol._parts:
            sources.append(part.src)
            sblock.append(m)
    T = build_tables(sources, None, None, blocks=blocks, source_block=sblock)
    assert T.nblock == 3 and len(T.part_carts) == 3
    rng = np.random.default_rng(1)
    coef, scale = _field(rng, T)
    x = rng.normal(size=T.dim_in) + 1j * rng.normal(size=T.dim_in)
    y = emulate(T, coef, scale, x)
    off = 0
    for m, wl in enumerate(wls):
        src = wl.pol._parts[0].src
        Tm = build_tables([src], src.basis("1"), src.basis("2"))
        n = Tm.dim_in
        ym = emulate(Tm, [coef[m]], scale[m:m + 1], x[off:off + n])
        assert np.abs(y[off:off + n] - ym).max() <= RTOL * np.abs(ym).max()
        off += n
    assert off == T.dim_out


def test_blocks_with_column_chunks():
    """Both at once: molecules side by side, slabs wider than 32 cut."""
    wls = workloads.uneven_molecules(2, seed=5, jmax_range=(16, 17), t_end=0.2)
    sources, sblock, blocks = [], [], []
    for m, wl in enumerate(wls):
        b = wl.h0._parts[0].src
        blocks.append((b.basis("1"), b.basis("2")))
        sources.append(wl.pol._parts[0].src)
        sblock.append(m)
    T0 = build_tables(sources, None, None, blocks=blocks, source_block=sblock)
    T1 = build_tables(sources, None, None, split=32, blocks=blocks, source_block=sblock)
    rng = np.random.default_rng(2)
    coef, scale = _field(rng, T0)
    x = rng.normal(size=T0.dim_in) + 1j * rng.normal(size=T0.dim_in)
    y0, y1 = emulate(T0, coef, scale, x), emulate(T1, coef, scale, x)
    assert np.abs(y1 - y0).max() <= RTOL * np.abs(y0).max()


def test_emulation_matches_the_host_matrix(c1_molecule):
    """The reading of the tables above against CarTens.tomat (the host scipy
    assembly of kron(MF, K), field.py:449-569) of the same field-dressed tensor,
    so the checks above compare operators that are right, not only alike."""
    wl = c1_molecule
    H = wl.Hac
    H.field(np.array([0.3, -0.7, 0.55]) * 1e7)
    srcs = [p.src for p in H._parts]
    T = build_tables(srcs, srcs[0].basis("1"), srcs[0].basis("2"))
    # the field input exactly as kr_set_field and the field schedule receive it
    coef, scale, thresh = field_arrays(T.part_carts, H._part_states())
    assert np.all(thresh == 0.0)
    rng = np.random.default_rng(3)
    x = rng.normal(size=T.dim_in) + 1j * rng.normal(size=T.dim_in)
    y = emulate(T, coef, scale, x)
    ref = H.tomat(form="full") @ x
    assert np.abs(y - ref).max() <= 1e-10 * np.abs(ref).max()


def test_field_arrays_layout():
    """Per part: coefficients in the part's own Cartesian order (zero where the
    field has no product), K scale, threshold (None: 0); the part count must
    match the operator's."""
    carts = [["x", "y", "z"], ["xx", "xy", "xz", "yy", "yz", "zz"]]
    states = [({"z": 2.0, "x": 1j}, 0.5, None), ({"zz": -3.0, "xy": 0.25}, 1 + 1j, 1e-12)]
    coef, scale, thresh = field_arrays(carts, states)
    assert coef.shape == (2, 9)
    assert coef[0].tolist() == [1j, 0, 2.0] + [0] * 6
    assert coef[1].tolist() == [0, 0.25, 0, 0, 0, -3.0] + [0] * 3
    assert scale.tolist() == [0.5, 1 + 1j] and thresh.tolist() == [0.0, 1e-12]
    with pytest.raises(ValueError):
        field_arrays(carts, states[:1])
