"""Compilation of CarTens factors into the device tables of one kr_op.

A CarTens operator is a sum of parts; each part is one factor source (the
kmat/mmat blocks of a tensor, field.py:58-170) with a K scale and a field
state. The device operator holds, per source,

* every K block  K[(J1,J2)][(s1,s2)][irrep]  as a dense n_k1 x n_k2 matrix,
  stored real, imaginary or complex (D2 blocks are purely one or the other);
* every M block set {cart: M[(J1,J2)][(s1,s2)][irrep][cart]} as one "group"
  in ELL form over the union sparsity pattern of its Cartesian components,
  de-duplicated by content (symmetry pairs share identical M blocks);

and, per part, one MF instance for each group it uses. Terms are the
(J1,s1) <- (J2,s2) products of field.py:1212-1243 present in both kmat and mmat.
"""
import ctypes
import hashlib

from types import SimpleNamespace

import numpy as np
import torch
from scipy.sparse import csr_matrix

from . import _native
from .device import context, stream_ptr


def _dense(m):
    return np.asarray(m.toarray() if hasattr(m, "toarray") else m, dtype=np.complex128)


def _kdense(kt, kd, shape):
    """The complex dense K block back from its stored kind and data."""
    if kt == _native.KR_K_REAL:
        return np.asarray(kd, np.float64).reshape(shape).astype(np.complex128)
    if kt == _native.KR_K_IMAG:
        return 1j * np.asarray(kd, np.float64).reshape(shape)
    return np.ascontiguousarray(kd).view(np.complex128).reshape(shape)


def _chunks(dm, dk, off, width):
    """Column chunks of at most ``width`` of row-major (dm, dk) slabs at ``off``:
    per chunk (parent slab, first column, columns, rows, offset, row stride)."""
    out = []
    for i in range(len(dm)):
        for c0 in range(0, int(dk[i]), width):
            out.append((i, c0, min(width, int(dk[i]) - c0), int(dm[i]), int(off[i]) + c0, int(dk[i])))
    return out


def _ktype(K):
    if not np.any(K.imag):
        return _native.KR_K_REAL, np.ascontiguousarray(K.real)
    if not np.any(K.real):
        return _native.KR_K_IMAG, np.ascontiguousarray(K.imag)
    return _native.KR_K_COMPLEX, np.ascontiguousarray(K).view(np.float64)


DIAG_MAX = 8  # widest band stored in diagonal slot order (the batched mat-vec's limit)


def _ell(mats, nrows, ncols):
    """Union-pattern ELL of a list of sparse matrices with equal shapes.
    Returns (width, col[nrows*width] int32, val[ncart, nrows*width] complex).

    A band of at most DIAG_MAX diagonals (d0 .. d0 + width - 1) is stored in
    diagonal slot order: slot w of row i holds column i + d0 + w, and where
    that column falls outside the matrix, the nearest column with value 0.
    Otherwise the entries of a row are packed by column, the padding slots
    repeating the last column of the row (or of the nearest non-empty row),
    so that a row's columns span only its own band."""
    coos = [m.tocoo() for m in mats]
    rows = np.concatenate([c.row for c in coos]).astype(np.int64) if coos else np.zeros(0, np.int64)
    cols = np.concatenate([c.col for c in coos]).astype(np.int64) if coos else np.zeros(0, np.int64)
    keys = np.unique(rows * ncols + cols)
    urow, ucol = keys // ncols, keys % ncols
    counts = np.bincount(urow, minlength=nrows)
    width = int(counts.max()) if len(keys) else 0
    if width == 0:
        return 0, np.zeros(0, np.int32), np.zeros((len(mats), 0), np.complex128)
    off = ucol - urow
    d0 = int(off.min())
    wd = int(off.max()) - d0 + 1
    if wd <= DIAG_MAX and wd <= 2 * width:
        width = wd
        slot = urow * width + (off - d0)
        col = np.clip(np.arange(nrows)[:, None] + d0 + np.arange(width)[None, :], 0, ncols - 1)
        col = np.ascontiguousarray(col.reshape(-1), dtype=np.int32)
    else:
        start = np.concatenate([[0], np.cumsum(counts)[:-1]])
        pos = np.arange(len(keys)) - start[urow]
        slot = urow * width + pos
        last = np.full(nrows, -1, np.int64)
        last[urow] = ucol  # keys are sorted: the last write per row is its largest column
        src = np.where(last >= 0, np.arange(nrows), -1)
        src = np.maximum.accumulate(src)
        src[src < 0] = int(np.flatnonzero(last >= 0)[0])
        col = np.repeat(last[src], width).astype(np.int32)
        col[slot] = ucol
    val = np.zeros((len(mats), nrows * width), dtype=np.complex128)
    for ci, c in enumerate(coos):
        idx = np.searchsorted(keys, c.row.astype(np.int64) * ncols + c.col)
        np.add.at(val[ci], slot[idx], c.data)
    return width, col, val


class CompiledSource:
    """Device-ready blocks of one factor source (cached on the source)."""

    def __init__(self, src):
        self.carts = list(src.carts)
        cidx = {c: i for i, c in enumerate(self.carts)}
        self.kblocks = []   # (ktype, data)
        self.kshape = []
        self.groups = []    # (rows, width, ncart, col, val)
        self.terms = []     # (J1, s1, J2, s2, kidx, gidx)
        self._keep = []
        gkey = {}
        gid = {}
        for (J1, J2), kJ in src.kmat.items():
            mJ = src.mmat.get((J1, J2)) if hasattr(src.mmat, "get") else src.mmat[(J1, J2)]
            if not mJ:
                continue
            for (s1, s2), kS in kJ.items():
                mS = mJ.get((s1, s2))
                if not mS:
                    continue
                for irrep, km in kS.items():
                    mI = mS.get(irrep)
                    if not mI:
                        continue
                    K = _dense(km)
                    kt, kd = _ktype(K)
                    kidx = len(self.kblocks)
                    self.kblocks.append((kt, kd))
                    self.kshape.append(K.shape)
                    mats = [None] * len(self.carts)
                    shape = None
                    for cart, mm in mI.items():
                        mats[cidx[cart]] = mm
                        shape = mm.shape
                    ikey = tuple(id(m) for m in mats)
                    g = gid.get(ikey)
                    if g is None:
                        full = [m if m is not None else csr_matrix(shape, dtype=np.complex128) for m in mats]
                        width, col, val = _ell(full, shape[0], shape[1])
                        h = hashlib.sha1()
                        h.update(np.array([shape[0], shape[1], width], np.int64).tobytes())
                        h.update(col.tobytes())
                        h.update(val.tobytes())
                        key = h.digest()
                        if key not in gkey:
                            gkey[key] = len(self.groups)
                            self.groups.append((shape[0], width, len(self.carts), col, val))
                        g = gkey[key]
                        gid[ikey] = g
                        self._keep.append(mats)  # ids stay valid while compiled
                    self.terms.append((J1, s1, J2, s2, kidx, g))


def compiled(src):
    c = getattr(src, "_compiled", None)
    if c is None:
        c = CompiledSource(src)
        src._compiled = c
    return c


def build_tables(sources, basis_out, basis_in, split=None, blocks=None, source_block=None):
    """Host tables of one operator (the kr_op_desc arrays) from its factor
    sources; no device work. Returns a SimpleNamespace: ``arrays`` (name -> numpy
    array, the descriptor fields), ``dim_out``, ``dim_in``, ``slab_parent``,
    ``part_carts``, ``nblock``, ``split``, ``nterm`` and the counts ``nk``,
    ``nm``, ``nmf``. Arguments as OperatorPlan."""
    sources = list(sources)
    split = int(split) if split else None
    if blocks is None:
        blocks = [(basis_out, basis_in)]
        source_block = [0] * len(sources)
    assert len(source_block) == len(sources)
    nblock = len(blocks)
    basis_out = [b for bo, _ in blocks for b in bo]
    basis_in = [b for _, bi in blocks for b in bi]
    slabs_out = [(k, J, s) for k, (bo, _) in enumerate(blocks) for J, s, _, _ in bo]
    slabs_in = [(k, J, s) for k, (_, bi) in enumerate(blocks) for J, s, _, _ in bi]
    sidx_out = {k: i for i, k in enumerate(slabs_out)}
    sidx_in = {k: i for i, k in enumerate(slabs_in)}
    out_dm = np.array([b[2] for b in basis_out], np.int32)
    out_dk = np.array([b[3] for b in basis_out], np.int32)
    in_dm = np.array([b[2] for b in basis_in], np.int32)
    in_dk = np.array([b[3] for b in basis_in], np.int32)
    out_off = np.concatenate([[0], np.cumsum(out_dm.astype(np.int64) * out_dk)[:-1]]).astype(np.int64)
    in_off = np.concatenate([[0], np.cumsum(in_dm.astype(np.int64) * in_dk)[:-1]]).astype(np.int64)
    dim_out = int((out_dm.astype(np.int64) * out_dk).sum())
    dim_in = int((in_dm.astype(np.int64) * in_dk).sum())
    if split:
        ch_out = _chunks(out_dm, out_dk, out_off, split)
        ch_in = _chunks(in_dm, in_dk, in_off, split)
        vout = [[] for _ in range(len(out_dm))]
        vin = [[] for _ in range(len(in_dm))]
        for v, c in enumerate(ch_out):
            vout[c[0]].append(v)
        for v, c in enumerate(ch_in):
            vin[c[0]].append(v)
        slab_parent = [c[0] for c in ch_out]
    else:
        slab_parent = list(range(len(out_dm)))

    k_off, k_rows, k_cols, k_type, k_data = [], [], [], [], []
    m_rows, m_width, m_ncart, m_col_off, m_val_off, m_col, m_val = [], [], [], [], [], [], []
    mf_group, mf_part = [], []
    t_out, t_in, t_k, t_mf = [], [], [], []
    koff = 0
    coff = 0
    voff = 0
    src_base = {}
    full_k, sub_k = [], {}

    def add_k(kt, kd, r, c, koff):
        if kt == _native.KR_K_COMPLEX and koff % 2:
            k_data.append(np.zeros(1))
            koff += 1
        k_off.append(koff)
        k_rows.append(r)
        k_cols.append(c)
        k_type.append(kt)
        flat = np.ascontiguousarray(kd, dtype=np.float64).reshape(-1)
        k_data.append(flat)
        return koff + flat.size

    part_carts = []
    for p, src in enumerate(sources):
        cs = compiled(src)
        part_carts.append(cs.carts)
        if id(src) not in src_base:
            kb0, g0 = (len(full_k) if split else len(k_type)), len(m_rows)
            for (kt, kd), (r, c) in zip(cs.kblocks, cs.kshape):
                if split:
                    full_k.append((kt, kd, (r, c)))
                else:
                    koff = add_k(kt, kd, r, c, koff)
            for rows, width, ncart, col, val in cs.groups:
                m_rows.append(rows)
                m_width.append(width)
                m_ncart.append(ncart)
                m_col_off.append(coff)
                m_val_off.append(voff)
                m_col.append(col)
                m_val.append(val.reshape(-1))
                coff += col.size
                voff += val.size
            src_base[id(src)] = (kb0, g0)
        kb0, g0 = src_base[id(src)]
        inst = {}
        for J1, s1, J2, s2, kidx, gidx in cs.terms:
            blk = source_block[p]
            if (blk, J1, s1) not in sidx_out or (blk, J2, s2) not in sidx_in:
                continue
            g = g0 + gidx
            if g not in inst:
                inst[g] = len(mf_group)
                mf_group.append(g)
                mf_part.append(p)
            so, si = sidx_out[(blk, J1, s1)], sidx_in[(blk, J2, s2)]
            if not split:
                t_out.append(so)
                t_in.append(si)
                t_k.append(kb0 + kidx)
                t_mf.append(inst[g])
                continue
            for vo in vout[so]:
                for vi in vin[si]:
                    key = (kb0 + kidx, ch_out[vo][1], ch_in[vi][1])
                    kb = sub_k.get(key, -2)
                    if kb == -2:
                        kt, kd, shp = full_k[kb0 + kidx]
                        a0, w1, b0_, w2 = ch_out[vo][1], ch_out[vo][2], ch_in[vi][1], ch_in[vi][2]
                        sub = _kdense(kt, kd, shp)[a0:a0 + w1, b0_:b0_ + w2]
                        kb = -1
                        if np.any(sub):
                            skt, skd = _ktype(np.ascontiguousarray(sub))
                            kb = len(k_type)
                            koff = add_k(skt, skd, w1, w2, koff)
                        sub_k[key] = kb
                    if kb < 0:
                        continue  # a zero K sub-block: no term
                    t_out.append(vo)
                    t_in.append(vi)
                    t_k.append(kb)
                    t_mf.append(inst[g])

    A = lambda x, dt: np.ascontiguousarray(np.array(x, dtype=dt).reshape(-1))
    cat = lambda xs, dt: np.ascontiguousarray(np.concatenate(xs).astype(dt)) if xs else np.zeros(1, dt)
    if split:
        out_dm = np.array([c[3] for c in ch_out], np.int32)
        out_dk = np.array([c[2] for c in ch_out], np.int32)
        out_off = np.array([c[4] for c in ch_out], np.int64)
        out_st = np.array([c[5] for c in ch_out], np.int32)
        in_dm = np.array([c[3] for c in ch_in], np.int32)
        in_dk = np.array([c[2] for c in ch_in], np.int32)
        in_off = np.array([c[4] for c in ch_in], np.int64)
        in_st = np.array([c[5] for c in ch_in], np.int32)
    keep = dict(
        out_dm=out_dm, out_dk=out_dk, out_off=out_off, in_dm=in_dm, in_dk=in_dk, in_off=in_off,
        k_off=A(k_off, np.int64), k_rows=A(k_rows, np.int32), k_cols=A(k_cols, np.int32),
        k_type=A(k_type, np.int32), k_data=cat(k_data, np.float64),
        m_rows=A(m_rows, np.int32), m_width=A(m_width, np.int32), m_ncart=A(m_ncart, np.int32),
        m_col_off=A(m_col_off, np.int64), m_val_off=A(m_val_off, np.int64),
        m_col=cat(m_col, np.int32), m_val=cat(m_val, np.complex128).view(np.float64),
        mf_group=A(mf_group, np.int32), mf_part=A(mf_part, np.int32),
        t_out=A(t_out, np.int32), t_in=A(t_in, np.int32), t_k=A(t_k, np.int32), t_mf=A(t_mf, np.int32),
    )
    if split:
        keep["out_stride"], keep["in_stride"] = out_st, in_st
    return SimpleNamespace(arrays=keep, dim_out=dim_out, dim_in=dim_in, slab_parent=slab_parent,
                           part_carts=part_carts, nblock=nblock, split=split, nterm=len(t_out),
                           nk=len(k_type), nm=len(m_rows), nmf=len(mf_group))


def make_desc(T, npart, maxorder=100):
    """The kr_op_desc of host tables T (build_tables): pointers into T.arrays,
    which must stay alive while the descriptor is used."""
    keep = T.arrays
    d = _native.kr_op_desc()
    d.nslab_out, d.nslab_in = len(keep["out_dm"]), len(keep["in_dm"])
    if T.split:
        d.out_stride, d.in_stride = keep["out_stride"].ctypes.data, keep["in_stride"].ctypes.data
    for f in ("out_dm", "out_dk", "out_off", "in_dm", "in_dk", "in_off", "k_off", "k_rows", "k_cols",
              "k_type", "k_data", "m_rows", "m_width", "m_ncart", "m_col_off", "m_val_off", "m_col",
              "m_val", "mf_group", "mf_part", "t_out", "t_in", "t_k", "t_mf"):
        setattr(d, f, keep[f].ctypes.data)
    d.dim_out, d.dim_in = T.dim_out, T.dim_in
    d.nk = T.nk
    d.k_data_len = keep["k_data"].size if T.nk else 0
    d.nm = T.nm
    d.m_col_len = keep["m_col"].size if T.nm else 0
    d.m_val_len = keep["m_val"].size if T.nm else 0
    d.npart = int(npart)
    d.nmf = T.nmf
    d.nterm = T.nterm
    d.maxorder = int(maxorder)
    return d


def check_desc(T, npart, maxorder=100):
    """kr_op_check of the descriptor of T on the host (no device): raises
    KrylovError with the library's message if kr_op_create would refuse it."""
    d = make_desc(T, npart, maxorder)
    buf = ctypes.create_string_buffer(256)
    rc = _native.lib().kr_op_check(ctypes.byref(d), buf, len(buf))
    if rc != _native.KR_OK:
        raise _native.KrylovError(rc, buf.value.decode(errors="replace"))


def field_arrays(part_carts, part_states, coef=None, scale=None, thresh=None):
    """The field input of kr_set_field (and of one step of a field schedule):
    coef[p, c] = the field product of part p's Cartesian component c (in the
    part's component order, part_carts[p]; zero where the field has none),
    scale[p] = the part's K scale, thresh[p] = its element threshold (None: 0,
    no threshold). part_states: per part (field_prod dict cart -> value, K
    scale, thresh), as CarTens._part_states() gives (field.py:1094-1139 forms
    the same products)."""
    n = max(1, len(part_carts))
    coef = np.zeros((n, _native.KR_MAXCART), np.complex128) if coef is None else coef
    scale = np.zeros(n, np.complex128) if scale is None else scale
    thresh = np.zeros(n, np.float64) if thresh is None else thresh
    if len(part_states) != len(part_carts):
        raise ValueError(f"{len(part_states)} part states for an operator of {len(part_carts)} parts")
    coef[:] = 0
    for p, (prods, sc, th) in enumerate(part_states):
        for ci, c in enumerate(part_carts[p]):
            v = prods.get(c)
            if v is not None:
                coef[p, ci] = v
        scale[p] = sc
        thresh[p] = 0.0 if th is None else float(th)
    return coef, scale, thresh


class OperatorPlan:
    """One kr_op: the device tables for a tuple of factor sources."""

    def __init__(self, sources, basis_out, basis_in, maxorder=100, device=None, split=None, blocks=None,
                 source_block=None):
        """split: None, or a width (32): slabs wider than it become column chunks
        of at most that many columns with the K blocks cut to match (the batched
        path's form for n_k above 32; the plain FP64 path refuses such operators).

        blocks: a block-diagonal operator over several bases (one molecule each),
        given as [(basis_out, basis_in), ...] in place of basis_out / basis_in;
        source_block[p] is the block of source p. The vector is the blocks'
        vectors one after the other, and every source is a part of its own
        (its own field coefficients in set_field)."""
        if len(sources) > _native.KR_MAXPART:
            raise ValueError(f"at most {_native.KR_MAXPART} operator parts are supported")
        self.ctx = context(device)
        self.sources = list(sources)
        L = _native.lib()
        T = build_tables(self.sources, basis_out, basis_in, split, blocks, source_block)
        self.tables = T
        self.nblock, self.dim_out, self.dim_in = T.nblock, T.dim_out, T.dim_in
        self.split, self.slab_parent, self.part_carts = T.split, T.slab_parent, T.part_carts
        d = make_desc(T, len(self.sources), maxorder)
        self.nterm = T.nterm
        self.maxorder = int(maxorder)
        h = ctypes.c_void_p()
        _native.check(L.kr_op_create(self.ctx, ctypes.byref(d), ctypes.byref(h)), self.ctx)
        self.op = h
        npart = max(1, len(self.sources))
        self._coef = np.zeros((npart, _native.KR_MAXCART), np.complex128)
        self._scale = np.zeros(npart, np.complex128)
        self._thresh = np.zeros(npart, np.float64)

    def __del__(self):
        op = getattr(self, "op", None)
        if op:
            try:
                _native.lib().kr_op_destroy(op)
            except Exception:
                pass
            self.op = None

    # ------------------------------------------------------------------
    def field_coefficients(self, part_states, coef=None, scale=None, thresh=None):
        """The kr_set_field arrays of one step (see field_arrays)."""
        if coef is None:
            coef, scale, thresh = np.zeros_like(self._coef), np.zeros_like(self._scale), np.zeros_like(self._thresh)
        return field_arrays(self.part_carts, part_states, coef, scale, thresh)

    def set_field(self, part_states, stream=None):
        """part_states: per part (field_prod dict cart -> value, K scale, thresh)."""
        self.field_coefficients(part_states, self._coef, self._scale, self._thresh)
        _native.check(_native.lib().kr_set_field(
            self.op, self._coef.ctypes.data, self._scale.ctypes.data, self._thresh.ctypes.data,
            stream_ptr(stream)), self.ctx)

    def set_field_schedule(self, steps, stream=None):
        """Uploads the field of many steps at once (kr_set_field_schedule);
        steps: per step the part_states of set_field. set_field_step(i) then
        sets step i's field with no host data (recordable at any part count)."""
        n = len(steps)
        if n == 0:
            raise ValueError("empty field schedule")
        coef = np.zeros((n,) + self._coef.shape, np.complex128)
        scale = np.zeros((n,) + self._scale.shape, np.complex128)
        thresh = np.zeros((n,) + self._thresh.shape, np.float64)
        for i, ps in enumerate(steps):
            self.field_coefficients(ps, coef[i], scale[i], thresh[i])
        _native.check(_native.lib().kr_set_field_schedule(
            self.op, n, coef.ctypes.data, scale.ctypes.data, thresh.ctypes.data, stream_ptr(stream)), self.ctx)
        self.schedule_steps = n
        # a replaced schedule's memory is freed: recordings of set_field_step
        # keep the generation they were made with and refuse another
        self.schedule_gen = getattr(self, "schedule_gen", 0) + 1

    def set_field_step(self, step, stream=None):
        """The field of step `step` of the uploaded schedule (kr_set_field_step)."""
        _native.check(_native.lib().kr_set_field_step(self.op, int(step), stream_ptr(stream)), self.ctx)

    def matvec(self, x, y, stream=None):
        assert x.dtype == torch.complex128 and y.dtype == torch.complex128 and x.is_cuda and y.is_cuda
        nvec = x.shape[0] if x.dim() == 2 else 1
        _native.check(_native.lib().kr_matvec(self.op, _native.ptr(x), _native.ptr(y), nvec,
                                              stream_ptr(stream)), self.ctx)

    def set_precision(self, products):
        """Arithmetic of the plain step's mat-vec products (kr_op_set_precision):
        "f64" (FP64, the default) or "df" (double-float on the FP32 pipes, about
        1e-14 relative per product; vectors, Lanczos scalars and exponential
        stay FP64)."""
        prec = {"f64": _native.KR_PREC_F64, "df": _native.KR_PREC_DF}.get(products)
        if prec is None:
            raise ValueError(f"products must be 'f64' or 'df', not {products!r}")
        _native.check(_native.lib().kr_op_set_precision(self.op, prec), self.ctx)
        self.products = products

    def step(self, states, phase, fac, tol, flags=0, korder=None, stream=None):
        nvec = states.shape[0] if states.dim() == 2 else 1
        kp = None
        if korder is not None:
            assert korder.dtype == np.int32 and korder.size >= nvec
            kp = korder.ctypes.data
        _native.check(_native.lib().kr_step(
            self.op, _native.ptr(states), nvec, _native.ptr(phase), float(fac.real), float(fac.imag),
            float(tol), int(flags), kp, stream_ptr(stream)), self.ctx)

    def observables(self, states, weights=None, stream=None):
        """<v_i|O|v_i> of the rows of ``states`` ((nvec, dim) or (dim,) complex128
        CUDA tensor) with this operator as O (kr_observables): a complex numpy
        array, and sum_i w_i Re <v_i|O|v_i> (weights: None = all 1)."""
        nvec = states.shape[0] if states.dim() == 2 else 1
        out = np.zeros(nvec, np.complex128)
        w = None
        if weights is not None:
            w = np.ascontiguousarray(weights, np.float64)
            assert w.size == nvec
        ws = ctypes.c_double()
        _native.check(_native.lib().kr_observables(
            self.op, _native.ptr(states), nvec, None if w is None else w.ctypes.data, out.ctypes.data,
            ctypes.byref(ws), stream_ptr(stream)), self.ctx)
        return out, ws.value

    def norm1(self, stream=None):
        """1-norm estimate of the operator with its current field (kr_op_norm1)."""
        out = ctypes.c_double()
        _native.check(_native.lib().kr_op_norm1(self.op, ctypes.byref(out), stream_ptr(stream)), self.ctx)
        return out.value

    def expv(self, x, t, m, tol, anorm, phase=None, stream=None):
        """x <- exp(t i H) x for one vector (complex128 CUDA tensor of dim elements),
        expokit ZHEXPV scheme (kr_expv); returns (substeps, mat-vecs, rejected)."""
        stats = np.zeros(3, np.int32)
        _native.check(_native.lib().kr_expv(
            self.op, _native.ptr(x), _native.ptr(phase), float(t), int(m), float(tol), float(anorm),
            stats.ctypes.data, stream_ptr(stream)), self.ctx)
        return tuple(int(s) for s in stats)

    def sync_status(self, stream=None):
        _native.check(_native.lib().kr_sync_status(self.op, stream_ptr(stream)), self.ctx)

    def launches(self):
        return int(_native.lib().kr_op_launch_count(self.op))

    def work(self):
        f, b = ctypes.c_double(), ctypes.c_double()
        _native.lib().kr_op_work(self.op, ctypes.byref(f), ctypes.byref(b))
        return f.value, b.value
