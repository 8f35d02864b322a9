"""Read-only HDF5 reader in numpy, for the factor files richmol stores.

The reference writes its tensors with h5py (richmol/field.py:1304-1598,
CarTens.store; richmol/rot/solution.py:60-130, richmol/rot/molecule.py:
390-460) and reads them back the same way (field.py:1600-1848). h5py is not
part of this framework's dependencies, so this module decodes the subset of
the HDF5 file format (version 0-3 superblocks) that such files use:

* superblock version 0/1 (symbol-table root) and 2/3 (object-header root);
* object headers version 1 and 2 ("OHDR"), with continuation blocks;
* groups as symbol tables (version-1 B-tree of "SNOD" nodes plus a local heap)
  or as compact link messages; dense link storage (a fractal heap) is
  reported as unsupported;
* dataspaces (scalar, simple, null), datatypes of class fixed-point, float,
  fixed string, bitfield, opaque, compound (``r``/``i`` pairs become complex),
  enumeration (h5py's bool), variable-length (strings and sequences, through
  the global heap) and array;
* data layouts compact, contiguous and chunked (version-1 B-tree index), with
  the deflate, shuffle and Fletcher-32 filters;
* attribute messages version 1-3 stored in the object header.

Names follow h5py: ``File(path)`` is the root ``Group``; ``group[name]`` (a
``/``-separated path) gives a ``Group`` or ``Dataset``; ``obj.attrs`` is a
dict of decoded values (strings as ``str``, fixed strings as ``bytes``, arrays
as numpy arrays); ``dataset[()]`` (or ``np.asarray(dataset)``) reads the data.
The layout is the one published in the HDF5 File Format Specification
(version 3.0); the code here is a restatement of those tables.
"""
import mmap
import struct
import zlib

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"


class HDF5Error(ValueError):
    pass


def is_hdf5(path):
    try:
        with open(path, "rb") as f:
            head = f.read(8)
    except OSError:
        return False
    return head == SIGNATURE


class _Reader:
    """Byte access to the file plus the superblock's sizes."""

    def __init__(self, path):
        self._f = open(path, "rb")
        try:
            self.buf = mmap.mmap(self._f.fileno(), 0, access=mmap.ACCESS_READ)
        except ValueError:  # empty file
            self._f.close()
            raise HDF5Error(f"'{path}' is empty") from None
        self.path = path
        self._gheaps = {}
        sb = self._find_superblock()
        self._parse_superblock(sb)

    def close(self):
        self.buf.close()
        self._f.close()

    def _find_superblock(self):
        off = 0
        n = len(self.buf)
        while off + 8 <= n:
            if self.buf[off: off + 8] == SIGNATURE:
                return off
            off = 512 if off == 0 else off * 2
        raise HDF5Error(f"'{self.path}' is not an HDF5 file")

    def u(self, pos, size):
        return int.from_bytes(self.buf[pos: pos + size], "little")

    def addr(self, pos):
        return self.u(pos, self.so)

    def length(self, pos):
        return self.u(pos, self.sl)

    def undefined(self, a):
        return a == (1 << (8 * self.so)) - 1

    def _parse_superblock(self, sb):
        b = self.buf
        ver = b[sb + 8]
        self.sb_version = ver
        if ver in (0, 1):
            self.so, self.sl = b[sb + 13], b[sb + 14]
            pos = sb + 24 + (4 if ver == 1 else 0)
            self.base = self.addr(pos)
            pos += 4 * self.so  # base, free-space, end of file, driver info
            # root group symbol table entry: name offset, object header address, cache
            self.root_addr = self.addr(pos + self.so)
        elif ver in (2, 3):
            self.so, self.sl = b[sb + 9], b[sb + 10]
            pos = sb + 12
            self.base = self.addr(pos)
            self.root_addr = self.addr(pos + 3 * self.so)
        else:
            raise HDF5Error(f"superblock version {ver} is not supported")
        if self.so not in (2, 4, 8) or self.sl not in (2, 4, 8):
            raise HDF5Error(f"unsupported offset/length sizes {self.so}/{self.sl}")

    # ------------------------------------------------------------------
    # object headers
    # ------------------------------------------------------------------
    def messages(self, addr):
        """[(type, flags, start, size)] of the object header at addr."""
        a = self.base + addr
        b = self.buf
        out = []
        if b[a: a + 4] == b"OHDR":
            ver = b[a + 4]
            if ver != 2:
                raise HDF5Error(f"object header version {ver} is not supported")
            flags = b[a + 5]
            pos = a + 6
            if flags & 0x20:
                pos += 16
            if flags & 0x10:
                pos += 4
            wsz = 1 << (flags & 3)
            chunk = self.u(pos, wsz)
            pos += wsz
            blocks = [(pos, chunk)]
            crt = bool(flags & 0x04)
            while blocks:
                start, size = blocks.pop(0)
                p, end = start, start + size
                while p + 4 + (2 if crt else 0) <= end:
                    mtype, msize, mflags = b[p], self.u(p + 1, 2), b[p + 3]
                    p += 4 + (2 if crt else 0)
                    out.append((mtype, mflags, p, msize))
                    if mtype == 0x10:
                        caddr, clen = self.addr(p), self.length(p + self.so)
                        c = self.base + caddr
                        if b[c: c + 4] != b"OCHK":
                            raise HDF5Error("bad object header continuation block")
                        blocks.append((c + 4, clen - 8))
                    p += msize
        else:
            ver = b[a]
            if ver != 1:
                raise HDF5Error(f"object header version {ver} at {addr} is not supported")
            nmsg = self.u(a + 2, 2)
            hsize = self.u(a + 8, 4)
            blocks = [(a + 16, hsize)]
            while blocks and len(out) < nmsg:
                start, size = blocks.pop(0)
                p, end = start, start + size
                while p + 8 <= end and len(out) < nmsg:
                    mtype, msize, mflags = self.u(p, 2), self.u(p + 2, 2), b[p + 4]
                    p += 8
                    out.append((mtype, mflags, p, msize))
                    if mtype == 0x10:
                        blocks.append((self.base + self.addr(p), self.length(p + self.so)))
                    p += msize
        for mtype, mflags, _, _ in out:
            if mflags & 0x02 and mtype not in (0, 0x10):
                raise HDF5Error(f"shared header message (type {mtype}) is not supported")
        return out

    # ------------------------------------------------------------------
    # groups
    # ------------------------------------------------------------------
    def local_heap_data(self, addr):
        a = self.base + addr
        if self.buf[a: a + 4] != b"HEAP":
            raise HDF5Error("bad local heap signature")
        dsize = self.length(a + 8)
        daddr = self.addr(a + 8 + 2 * self.sl)
        return self.base + daddr, dsize

    def cstring(self, pos):
        end = self.buf.find(b"\0", pos)
        return bytes(self.buf[pos: end]).decode("utf-8")

    def symbol_table_links(self, btree, heap):
        heap_data, _ = self.local_heap_data(heap)
        links = {}
        entry = 2 * self.so + 24

        def node(addr):
            a = self.base + addr
            if self.buf[a: a + 4] != b"TREE":
                raise HDF5Error("bad group B-tree node")
            level, used = self.buf[a + 5], self.u(a + 6, 2)
            pos = a + 8 + 2 * self.so + self.sl  # siblings, then key 0
            for _ in range(used):
                child = self.addr(pos)
                pos += self.so + self.sl
                if level > 0:
                    node(child)
                else:
                    snod(child)

        def snod(addr):
            a = self.base + addr
            if self.buf[a: a + 4] != b"SNOD":
                raise HDF5Error("bad symbol table node")
            nsym = self.u(a + 6, 2)
            pos = a + 8
            for _ in range(nsym):
                name = self.cstring(heap_data + self.length(pos))
                links[name] = self.addr(pos + self.so)
                pos += entry

        node(btree)
        return links

    def link_message(self, p):
        b = self.buf
        flags = b[p + 1]
        pos = p + 2
        ltype = 0
        if flags & 0x08:
            ltype = b[pos]
            pos += 1
        if flags & 0x04:
            pos += 8
        if flags & 0x10:
            pos += 1
        nsz = 1 << (flags & 3)
        nlen = self.u(pos, nsz)
        pos += nsz
        name = bytes(b[pos: pos + nlen]).decode("utf-8")
        pos += nlen
        if ltype == 0:
            return name, self.addr(pos)
        return name, None  # soft or external link: not followed

    def group_links(self, addr):
        links = {}
        for mtype, _, p, _ in self.messages(addr):
            if mtype == 0x11:
                links.update(self.symbol_table_links(self.addr(p), self.addr(p + self.so)))
            elif mtype == 0x06:
                name, target = self.link_message(p)
                if target is not None:
                    links[name] = target
            elif mtype == 0x02:
                flags = self.buf[p + 1]
                pos = p + 2 + (8 if flags & 1 else 0)
                if not self.undefined(self.addr(pos)):
                    raise HDF5Error("dense link storage (fractal heap) is not supported")
        return links

    # ------------------------------------------------------------------
    # datatypes, dataspaces, data
    # ------------------------------------------------------------------
    def datatype(self, p):
        """Returns (descriptor, size of the datatype message). A descriptor is a
        numpy dtype, or ('vlen', is_string, base descriptor, element size)."""
        b = self.buf
        cls, ver = b[p] & 0x0F, b[p] >> 4
        bits = self.u(p + 1, 3)
        size = self.u(p + 4, 4)
        q = p + 8
        bo = ">" if bits & 1 else "<"
        if cls == 0:  # fixed point
            return np.dtype(f"{bo}{'i' if bits & 0x08 else 'u'}{size}"), 12
        if cls == 1:  # floating point
            if size not in (2, 4, 8):
                raise HDF5Error(f"float of {size} bytes is not supported")
            return np.dtype(f"{bo}f{size}"), 20
        if cls == 3:  # fixed-length string
            return np.dtype(f"S{size}"), 8
        if cls == 4:  # bitfield
            return np.dtype(f"{bo}u{size}"), 12
        if cls == 5:  # opaque: ASCII tag padded to 8
            tag = self.buf.find(b"\0", q) - q + 1
            return np.dtype(f"V{size}"), 8 + ((tag + 7) // 8) * 8
        if cls == 6:  # compound
            nmem = bits & 0xFFFF
            names, formats, offsets = [], [], []
            for _ in range(nmem):
                end = b.find(b"\0", q)
                names.append(bytes(b[q: end]).decode("utf-8"))
                nl = end - q + 1
                if ver < 3:
                    q += ((nl + 7) // 8) * 8
                    offsets.append(self.u(q, 4))
                    q += 4
                    if ver == 1:
                        ndim = b[q]
                        dims = [self.u(q + 12 + 4 * i, 4) for i in range(ndim)]
                        q += 28
                    else:
                        dims = []
                else:
                    q += nl
                    ob = 1 if size < 256 else 2 if size < 65536 else 3 if size < 1 << 24 else 4
                    offsets.append(self.u(q, ob))
                    q += ob
                    dims = []
                mt, ml = self.datatype(q)
                q += ml
                if isinstance(mt, tuple):
                    raise HDF5Error("variable-length compound members are not supported")
                formats.append((mt, tuple(dims)) if dims else mt)
            dt = np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": size})
            if (names == ["r", "i"] and offsets == [0, size // 2] and formats[0] == formats[1]
                    and np.dtype(formats[0]).kind == "f"):
                dt = np.dtype(f"{np.dtype(formats[0]).byteorder.replace('=', '<')}c{size}")
            return dt, q - p
        if cls == 8:  # enumeration
            nmem = bits & 0xFFFF
            base, bl = self.datatype(q)
            q += bl
            names = []
            for _ in range(nmem):
                end = b.find(b"\0", q)
                names.append(bytes(b[q: end]))
                nl = end - q + 1
                q += ((nl + 7) // 8) * 8 if ver < 3 else nl
            q += nmem * base.itemsize
            if sorted(names) == [b"FALSE", b"TRUE"] and base.itemsize == 1:
                return np.dtype("?"), q - p
            return base, q - p
        if cls == 9:  # variable length
            is_str = (bits & 0x0F) == 1
            base, bl = self.datatype(q)
            q += bl
            return ("vlen", is_str, base, size), q - p
        if cls == 10:  # array
            ndim = b[q]
            q += 4 if ver < 3 else 1
            dims = tuple(self.u(q + 4 * i, 4) for i in range(ndim))
            q += 4 * ndim * (2 if ver < 3 else 1)
            base, bl = self.datatype(q)
            q += bl
            if isinstance(base, tuple):
                raise HDF5Error("arrays of variable-length elements are not supported")
            return np.dtype((base, dims)), q - p
        if cls == 7:  # reference
            return np.dtype(f"<u{size}"), 8
        raise HDF5Error(f"datatype class {cls} is not supported")

    def dataspace(self, p):
        """Returns the shape tuple, or None for a null dataspace."""
        b = self.buf
        ver, rank, flags = b[p], b[p + 1], b[p + 2]
        if ver == 1:
            pos = p + 8
            kind = 1 if rank else 0
        elif ver == 2:
            kind = b[p + 3]
            pos = p + 4
        else:
            raise HDF5Error(f"dataspace version {ver} is not supported")
        if kind == 2:
            return None
        return tuple(self.length(pos + i * self.sl) for i in range(rank))

    def global_heap_object(self, coll, index):
        objs = self._gheaps.get(coll)
        if objs is None:
            a = self.base + coll
            if self.buf[a: a + 4] != b"GCOL":
                raise HDF5Error("bad global heap collection")
            csize = self.length(a + 8)
            objs = {}
            pos, end = a + 8 + self.sl, a + csize
            while pos + 8 + self.sl <= end:
                idx = self.u(pos, 2)
                osize = self.length(pos + 8)
                if idx == 0:
                    break
                objs[idx] = (pos + 8 + self.sl, osize)
                pos += 8 + self.sl + ((osize + 7) // 8) * 8
            self._gheaps[coll] = objs
        start, osize = objs[index]
        return bytes(self.buf[start: start + osize])

    def decode(self, raw, dtype, shape):
        """Raw bytes of n elements → numpy array (or object array of vlen values)."""
        n = int(np.prod(shape)) if shape else 1
        if isinstance(dtype, tuple):
            _, is_str, base, esize = dtype
            out = np.empty(n, dtype=object)
            for i in range(n):
                e = raw[i * esize: (i + 1) * esize]
                cnt = int.from_bytes(e[:4], "little")
                coll = int.from_bytes(e[4: 4 + self.so], "little")
                idx = int.from_bytes(e[4 + self.so: 8 + self.so], "little")
                data = b"" if coll == 0 or cnt == 0 else self.global_heap_object(coll, idx)
                if is_str:
                    out[i] = data[:cnt].split(b"\0", 1)[0].decode("utf-8")
                else:
                    out[i] = np.frombuffer(data, dtype=base, count=cnt).copy()
            return out.reshape(shape) if shape else out[0]
        arr = np.frombuffer(raw, dtype=dtype, count=n).copy()
        if arr.dtype.byteorder == ">":
            arr = arr.astype(arr.dtype.newbyteorder("="))
        return arr.reshape(shape) if shape else arr[0]

    def attributes(self, addr):
        attrs = {}
        b = self.buf
        for mtype, _, p, _ in self.messages(addr):
            if mtype == 0x15:
                flags = b[p + 1]
                if not self.undefined(self.addr(p + 2 + (8 if flags & 1 else 0))):
                    raise HDF5Error("dense attribute storage (fractal heap) is not supported")
                continue
            if mtype != 0x0C:
                continue
            ver = b[p]
            if ver not in (1, 2, 3):
                raise HDF5Error(f"attribute message version {ver} is not supported")
            if ver > 1 and b[p + 1] & 0x03:
                raise HDF5Error("attributes with shared datatype or dataspace are not supported")
            nsz, tsz, ssz = self.u(p + 2, 2), self.u(p + 4, 2), self.u(p + 6, 2)
            pos = p + 8 + (1 if ver == 3 else 0)
            pad = (lambda x: ((x + 7) // 8) * 8) if ver == 1 else (lambda x: x)
            name = bytes(b[pos: pos + nsz]).split(b"\0", 1)[0].decode("utf-8")
            pos += pad(nsz)
            dtype, _ = self.datatype(pos)
            pos += pad(tsz)
            shape = self.dataspace(pos)
            pos += pad(ssz)
            if shape is None:
                attrs[name] = None
                continue
            n = int(np.prod(shape)) if shape else 1
            esize = dtype[3] if isinstance(dtype, tuple) else dtype.itemsize
            val = self.decode(bytes(b[pos: pos + n * esize]), dtype, shape)
            if isinstance(val, np.bytes_):
                val = bytes(val)
            attrs[name] = val
        return attrs

    def dataset_info(self, addr):
        info = {"filters": []}
        b = self.buf
        for mtype, _, p, _ in self.messages(addr):
            if mtype == 0x01:
                info["shape"] = self.dataspace(p)
            elif mtype == 0x03:
                info["dtype"] = self.datatype(p)[0]
            elif mtype == 0x08:
                info["layout"] = self._layout(p)
            elif mtype == 0x0B:
                info["filters"] = self._filters(p)
        if "layout" not in info:
            return None
        return info

    def _layout(self, p):
        b = self.buf
        ver = b[p]
        if ver == 3:
            cls = b[p + 1]
            if cls == 0:
                size = self.u(p + 2, 2)
                return ("compact", p + 4, size)
            if cls == 1:
                return ("contiguous", self.addr(p + 2), self.length(p + 2 + self.so))
            if cls == 2:
                ndim = b[p + 2]
                btree = self.addr(p + 3)
                dims = [self.u(p + 3 + self.so + 4 * i, 4) for i in range(ndim)]
                return ("chunked", btree, dims)
        elif ver in (1, 2):
            ndim, cls = b[p + 1], b[p + 2]
            pos = p + 8
            if cls == 0:
                dims = [self.u(pos + 4 * i, 4) for i in range(ndim)]
                pos += 4 * ndim
                return ("compact", pos + 4, self.u(pos, 4))
            a = self.addr(pos)
            pos += self.so
            dims = [self.u(pos + 4 * i, 4) for i in range(ndim)]
            if cls == 1:
                return ("contiguous", a, None)
            return ("chunked", a, dims)
        raise HDF5Error(f"data layout version {ver} (class {b[p + 1]}) is not supported")

    def _filters(self, p):
        b = self.buf
        ver, nf = b[p], b[p + 1]
        pos = p + (8 if ver == 1 else 2)
        out = []
        for _ in range(nf):
            fid = self.u(pos, 2)
            if ver == 1 or fid >= 256:
                nlen = self.u(pos + 2, 2)
                pos += 4
            else:
                nlen = 0
                pos += 2
            nval = self.u(pos + 2, 2)
            pos += 4
            pos += ((nlen + 7) // 8) * 8 if ver == 1 else nlen
            vals = [self.u(pos + 4 * i, 4) for i in range(nval)]
            pos += 4 * nval
            if ver == 1 and nval % 2:
                pos += 4
            out.append((fid, vals))
        return out

    def _unfilter(self, raw, filters, mask):
        for i in reversed(range(len(filters))):
            if mask & (1 << i):
                continue
            fid, vals = filters[i]
            if fid == 1:
                raw = zlib.decompress(raw)
            elif fid == 2:
                es = vals[0] if vals else 1
                a = np.frombuffer(raw, np.uint8)
                n = len(a) // es
                body = a[: n * es].reshape(es, n).T.reshape(-1)
                raw = body.tobytes() + bytes(a[n * es:])
            elif fid == 3:
                raw = raw[:-4]
            else:
                raise HDF5Error(f"filter {fid} is not supported")
        return raw

    def read_dataset(self, info):
        shape, dtype = info["shape"], info["dtype"]
        if shape is None:
            return None
        esize = dtype[3] if isinstance(dtype, tuple) else dtype.itemsize
        n = int(np.prod(shape)) if shape else 1
        kind = info["layout"][0]
        if kind == "compact":
            _, pos, size = info["layout"]
            return self.decode(bytes(self.buf[pos: pos + n * esize]), dtype, shape)
        if kind == "contiguous":
            a = info["layout"][1]
            if self.undefined(a):
                raw = bytes(n * esize)
            else:
                raw = bytes(self.buf[self.base + a: self.base + a + n * esize])
            return self.decode(raw, dtype, shape)
        _, btree, cdims = info["layout"]
        rank = len(shape)
        cshape = tuple(cdims[:rank])
        flat = bytearray(n * esize)
        out = np.frombuffer(flat, dtype=np.uint8).reshape(tuple(shape) + (esize,))
        if not self.undefined(btree):
            for offs, raw in self._chunks(btree, rank, info["filters"]):
                c = np.frombuffer(raw, np.uint8)[: int(np.prod(cshape)) * esize].reshape(cshape + (esize,))
                sl_out = tuple(slice(o, min(o + cs, s)) for o, cs, s in zip(offs, cshape, shape))
                sl_in = tuple(slice(0, s.stop - s.start) for s in sl_out)
                out[sl_out] = c[sl_in]
        return self.decode(bytes(flat), dtype, shape)

    def _chunks(self, addr, rank, filters):
        a = self.base + addr
        b = self.buf
        if b[a: a + 4] != b"TREE" or b[a + 4] != 1:
            raise HDF5Error("bad chunk B-tree node")
        level, used = b[a + 5], self.u(a + 6, 2)
        ksize = 8 + 8 * (rank + 1)
        pos = a + 8 + 2 * self.so
        for _ in range(used):
            csize, mask = self.u(pos, 4), self.u(pos + 4, 4)
            offs = [self.u(pos + 8 + 8 * i, 8) for i in range(rank)]
            child = self.addr(pos + ksize)
            pos += ksize + self.so
            if level > 0:
                yield from self._chunks(child, rank, filters)
            else:
                raw = bytes(b[self.base + child: self.base + child + csize])
                yield offs, self._unfilter(raw, filters, mask)


class Dataset:
    def __init__(self, reader, addr, info, name):
        self._r, self._addr, self._info, self.name = reader, addr, info, name
        self._attrs = None

    @property
    def shape(self):
        return self._info["shape"]

    @property
    def dtype(self):
        dt = self._info["dtype"]
        return np.dtype(object) if isinstance(dt, tuple) else dt

    @property
    def attrs(self):
        if self._attrs is None:
            self._attrs = self._r.attributes(self._addr)
        return self._attrs

    def __getitem__(self, key):
        data = self._r.read_dataset(self._info)
        if key == () or key is Ellipsis:
            return data
        return data[key]

    def __array__(self, dtype=None, copy=None):
        a = np.asarray(self[()])
        return a if dtype is None else a.astype(dtype)

    def __len__(self):
        return self.shape[0]


class Group:
    def __init__(self, reader, addr, name="/"):
        self._r, self._addr, self.name = reader, addr, name
        self._links = None
        self._attrs = None

    def _get_links(self):
        if self._links is None:
            self._links = self._r.group_links(self._addr)
        return self._links

    def keys(self):
        return list(self._get_links().keys())

    def __iter__(self):
        return iter(self.keys())

    def items(self):
        return [(k, self[k]) for k in self.keys()]

    def __contains__(self, path):
        try:
            self[path]
        except KeyError:
            return False
        return True

    @property
    def attrs(self):
        if self._attrs is None:
            self._attrs = self._r.attributes(self._addr)
        return self._attrs

    def __getitem__(self, path):
        obj = self
        for part in [p for p in path.split("/") if p]:
            if not isinstance(obj, Group):
                raise KeyError(path)
            links = obj._get_links()
            if part not in links:
                raise KeyError(f"'{path}' not found in '{self._r.path}'")
            addr = links[part]
            sub = obj.name.rstrip("/") + "/" + part
            info = obj._r.dataset_info(addr)
            obj = Dataset(obj._r, addr, info, sub) if info is not None else Group(obj._r, addr, sub)
        return obj


class File(Group):
    """Read-only HDF5 file; use as a context manager or call close()."""

    def __init__(self, path, mode="r"):
        if mode != "r":
            raise ValueError("only mode 'r' is supported")
        r = _Reader(path)
        super().__init__(r, r.root_addr, "/")

    def close(self):
        self._r.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
