"""Branches of the numpy HDF5 reader that the reference's files do not use,
on files laid out here byte by byte from the HDF5 File Format Specification
(version 3.0): a version-2 superblock, version-2 object headers ("OHDR") with
link messages, a chunked dataset (version-1 chunk B-tree, edge chunks, the
shuffle + deflate + Fletcher-32 pipeline, one chunk stored with deflate skipped
by its filter mask), version-3 attribute messages of enumeration (h5py's bool),
array, variable-length sequence (global heap) and fixed-string types, and a
contiguous dataset with an unallocated address (fill value zero). The layout
code below is test infrastructure: it writes what the specification describes,
so it checks the reader's arithmetic, not an independent writer. CPU only."""
import struct
import zlib

import numpy as np
import pytest

UNDEF = 0xFFFFFFFFFFFFFFFF


def _ohdr(messages):
    """Version-2 object header: (type, body) messages, 4-byte chunk size."""
    body = b"".join(struct.pack("<BHB", t, len(m), 0) + m for t, m in messages)
    return b"OHDR" + bytes([2, 0x02]) + struct.pack("<I", len(body)) + body + b"\0\0\0\0"


def _dspace(shape):
    if shape == ():
        return bytes([2, 0, 0, 0])  # version 2, scalar
    return bytes([2, len(shape), 0, 1]) + b"".join(struct.pack("<Q", d) for d in shape)


F64 = bytes([0x11, 0x20, 63, 0]) + struct.pack("<I", 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
I32 = bytes([0x10, 0x08, 0, 0]) + struct.pack("<I", 4) + struct.pack("<HH", 0, 32)
I8 = bytes([0x10, 0x08, 0, 0]) + struct.pack("<I", 1) + struct.pack("<HH", 0, 8)


def _enum_bool():  # class 8, version 3, 2 members over int8
    return bytes([0x38, 2, 0, 0]) + struct.pack("<I", 1) + I8 + b"FALSE\0TRUE\0" + bytes([0, 1])


def _array_i32(dims):  # class 10, version 3
    return bytes([0x3A, 0, 0, 0]) + struct.pack("<I", 4 * int(np.prod(dims))) + bytes([len(dims)]) + \
        b"".join(struct.pack("<I", d) for d in dims) + I32


def _vlen_seq_i32():  # class 9, version 1, sequence of int32
    return bytes([0x19, 0, 0, 0]) + struct.pack("<I", 16) + I32


def _fixed_string(n):
    return bytes([0x13, 0, 0, 0]) + struct.pack("<I", n)


def _attr(name, dtype, shape, data):  # attribute message, version 3
    nm = name.encode() + b"\0"
    ds = _dspace(shape)
    return struct.pack("<BBHHHB", 3, 0, len(nm), len(dtype), len(ds), 0) + nm + dtype + ds + data


def _link(name, addr):  # link message, version 1, hard link, 1-byte name length
    nm = name.encode()
    return bytes([1, 0, len(nm)]) + nm + struct.pack("<Q", addr)


class _File:
    def __init__(self):
        self.buf = bytearray(48)  # the superblock goes in at the end

    def put(self, data, align=8):
        while len(self.buf) % align:
            self.buf.append(0)
        addr = len(self.buf)
        self.buf += data
        return addr

    def finish(self, root):
        sb = b"\x89HDF\r\n\x1a\n" + bytes([2, 8, 8, 0]) + struct.pack("<QQQQ", 0, UNDEF, len(self.buf), root)
        self.buf[:48] = sb + b"\0\0\0\0"
        return bytes(self.buf)


def _shuffle(raw, es):
    a = np.frombuffer(raw, np.uint8)
    n = len(a) // es
    return a[: n * es].reshape(n, es).T.reshape(-1).tobytes() + a[n * es:].tobytes()


@pytest.fixture(scope="module")
def layout_file(tmp_path_factory):
    f = _File()
    data = np.arange(7 * 5, dtype=np.float64).reshape(7, 5) * 0.25 - 3.0
    cs = (4, 3)  # chunks of 4 x 3; the edge chunks run past the 7 x 5 data
    chunks = []
    for i0 in range(0, 7, cs[0]):
        for j0 in range(0, 5, cs[1]):
            c = np.zeros(cs)
            blk = data[i0:i0 + cs[0], j0:j0 + cs[1]]
            c[: blk.shape[0], : blk.shape[1]] = blk
            raw = c.tobytes()
            mask = 0
            if (i0, j0) == (4, 3):  # this chunk skips deflate (filter 1 of the pipeline)
                stored = _shuffle(raw, 8) + b"\0\0\0\0"
                mask = 0b010
            else:
                stored = zlib.compress(_shuffle(raw, 8)) + b"\0\0\0\0"
            chunks.append((i0, j0, mask, f.put(stored), len(stored)))
    # chunk B-tree node: key (size, filter mask, offsets) and address per chunk,
    # then the closing key
    node = b"TREE" + bytes([1, 0]) + struct.pack("<H", len(chunks)) + struct.pack("<QQ", UNDEF, UNDEF)
    keys = b""
    for i0, j0, mask, addr, nbytes in chunks:
        keys += struct.pack("<II", nbytes, mask) + struct.pack("<QQQ", i0, j0, 0) + struct.pack("<Q", addr)
    keys += struct.pack("<II", 0, 0) + struct.pack("<QQQ", 7, 5, 0)
    btree = f.put(node + keys)
    pipeline = bytes([2, 3]) + struct.pack("<HHH", 2, 0, 1) + struct.pack("<I", 8) + \
        struct.pack("<HHH", 1, 0, 1) + struct.pack("<I", 6) + struct.pack("<HHH", 3, 0, 0)
    layout = bytes([3, 2, 3]) + struct.pack("<Q", btree) + struct.pack("<III", *cs, 8)
    # global heap with two sequences for the vlen attribute
    seqs = [np.array([7, -1, 4], np.int32), np.array([11], np.int32)]
    objs = b""
    for i, sq in enumerate(seqs, start=1):
        b = sq.tobytes()
        objs += struct.pack("<HHIQ", i, 1, 0, len(b)) + b + bytes((-len(b)) % 8)
    coll_size = 16 + len(objs) + 16
    gcol = f.put(b"GCOL" + bytes([1, 0, 0, 0]) + struct.pack("<Q", coll_size) + objs + struct.pack("<HHIQ", 0, 0, 0, 0))
    vlen_data = b"".join(struct.pack("<IQI", len(sq), gcol, i) for i, sq in enumerate(seqs, start=1))
    attrs = [
        (0x0C, _attr("flag", _enum_bool(), (), bytes([1]))),
        (0x0C, _attr("grid", _array_i32((2, 3)), (), np.arange(6, dtype=np.int32).tobytes())),
        (0x0C, _attr("seqs", _vlen_seq_i32(), (2,), vlen_data)),
        (0x0C, _attr("unit", _fixed_string(4), (), b"au\0\0")),
    ]
    dset = f.put(_ohdr([(0x01, _dspace((7, 5))), (0x03, F64), (0x0B, pipeline), (0x08, layout)] + attrs))
    empty = f.put(_ohdr([(0x01, _dspace((3,))), (0x03, I32),
                         (0x08, bytes([3, 1]) + struct.pack("<QQ", UNDEF, 12))]))
    sub = f.put(_ohdr([(0x06, _link("empty", empty))]))
    root = f.put(_ohdr([(0x06, _link("data", dset)), (0x06, _link("sub", sub))]))
    p = tmp_path_factory.mktemp("h5") / "layouts.h5"
    p.write_bytes(f.finish(root))
    return str(p), data, seqs


def test_v2_headers_links_and_chunked_filtered_data(layout_file):
    from richmol_gb300 import hdf5
    path, data, _ = layout_file
    with hdf5.File(path) as f:
        assert sorted(f.keys()) == ["data", "sub"]
        ds = f["data"]
        assert ds.shape == (7, 5) and ds.dtype == np.float64
        assert np.array_equal(ds[()], data)
        assert np.array_equal(f["sub/empty"][()], np.zeros(3, np.int32))


def test_v3_attribute_types(layout_file):
    from richmol_gb300 import hdf5
    path, _, seqs = layout_file
    with hdf5.File(path) as f:
        at = f["data"].attrs
        assert at["flag"] is np.True_ or at["flag"] == True  # noqa: E712
        assert np.array_equal(at["grid"], np.arange(6).reshape(2, 3))
        assert [list(s) for s in at["seqs"]] == [list(s) for s in seqs]
        assert at["unit"] == b"au"  # null padding dropped, as numpy's fixed-width bytes (and h5py) give it
