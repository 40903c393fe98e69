"""A small reader and writer for the subset of HDF5 that the staged-input cache uses.

The reference caches its staged inputs with h5py (trot/staging.py:1353-1426); h5py and
libhdf5 are not available to this package, so this module implements the parts of the
published HDF5 file format (the "HDF5 File Format Specification", versions 0-3 of the
superblock) that such a cache needs, with an h5py-like surface: ``File``, ``Group``,
``Dataset``, ``.attrs``, ``create_group``, ``create_dataset``, ``keys()``, ``in``.

Writer (what h5py writes with its default, earliest-format settings):
  superblock version 0, version-1 object headers, groups as symbol tables (version-1
  B-tree of symbol-table nodes + local name heap), datasets with contiguous storage,
  little-endian IEEE floats, two's-complement integers, complex numbers as the
  compound {"r", "i"} h5py uses, str attributes as variable-length UTF-8 strings in a
  global heap. No timestamps are written, so equal inputs give equal bytes.
Reader: the above, plus superblock versions 1-3, version-2 object headers and their
  continuation chunks, groups held as link messages, compact and chunked storage
  (version-1 B-tree chunk index; deflate, shuffle and Fletcher-32 filters), fixed-length
  strings, general compounds and big-endian numbers. Dense (fractal-heap) link and
  attribute storage and the version-4 chunk indexes raise ``NotImplementedError``.

Dataset payloads are read with one positioned read (contiguous storage), and
``Dataset.extent()`` exposes the payload's file offset so a caller can stream it into
pinned host buffers without an intermediate copy.
"""
from __future__ import annotations

import os
import struct
import zlib
from typing import Any, Iterator

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
_LEAF_K = 4  # symbol-table node capacity 2 * 4 entries
_NODE_K = 16  # group B-tree node capacity 2 * 16 children
_ENTRY = 40  # symbol-table entry with 8-byte offsets
_SNOD_SIZE = 8 + 2 * _LEAF_K * _ENTRY
_TREE_SIZE = 24 + 2 * _NODE_K * 8 + (2 * _NODE_K + 1) * 8
_GCOL_MIN = 4096

# message types
_M_DATASPACE, _M_LINKINFO, _M_DATATYPE, _M_FILL_OLD, _M_FILL = 0x01, 0x02, 0x03, 0x04, 0x05
_M_LINK, _M_LAYOUT, _M_FILTERS, _M_ATTR, _M_CONT, _M_STAB, _M_ATTRINFO = 0x06, 0x08, 0x0B, 0x0C, 0x10, 0x11, 0x15


def _pad8(n: int) -> int:
    return (n + 7) & ~7


def _pad(b: bytes) -> bytes:
    return b + b"\0" * (_pad8(len(b)) - len(b))


class _VlenStr:
    """Marker dtype: variable-length string (decoded to ``str``)."""


# ------------------------------------------------------------------------- datatypes
def _encode_dtype(dt: np.dtype) -> bytes:
    """Datatype message body for a numpy dtype (little-endian numbers, complex as {r, i})."""
    dt = np.dtype(dt)
    if dt.kind in "iu":
        bits = 0x08 if dt.kind == "i" else 0x00
        return bytes([0x10, bits, 0, 0]) + struct.pack("<IHH", dt.itemsize, 0, 8 * dt.itemsize)
    if dt.kind == "f":
        if dt.itemsize == 8:
            sign, eloc, esz, msz, bias = 63, 52, 11, 52, 1023
        elif dt.itemsize == 4:
            sign, eloc, esz, msz, bias = 31, 23, 8, 23, 127
        else:
            raise TypeError(f"unsupported float size {dt.itemsize}")
        # byte order LE, padding 0, mantissa normalisation 2 (implied leading 1)
        return (bytes([0x11, 0x20, sign, 0]) + struct.pack("<I", dt.itemsize)
                + struct.pack("<HHBBBBI", 0, 8 * dt.itemsize, eloc, esz, 0, msz, bias))
    if dt.kind == "c":
        part = np.dtype(f"<f{dt.itemsize // 2}")
        sub = _encode_dtype(part)
        members = b""
        for name, off in (("r", 0), ("i", part.itemsize)):
            members += _pad(name.encode() + b"\0") + struct.pack("<IB3sI4s4I", off, 0, b"\0" * 3, 0, b"\0" * 4,
                                                                0, 0, 0, 0) + sub
        return bytes([0x16, 2, 0, 0]) + struct.pack("<I", dt.itemsize) + members
    if dt.kind == "S":
        return bytes([0x13, 0x00, 0, 0]) + struct.pack("<I", dt.itemsize)
    raise TypeError(f"unsupported dtype {dt}")


def _encode_vlen_str() -> bytes:
    base = bytes([0x10, 0, 0, 0]) + struct.pack("<IHH", 1, 0, 8)  # unsigned 8-bit characters
    return bytes([0x19, 0x01, 0x01, 0x00]) + struct.pack("<I", 16) + base  # string, null-term, UTF-8


def _decode_dtype(b: bytes, p: int = 0):
    """Parse a datatype message at b[p:]; returns (dtype or _VlenStr, end offset)."""
    cls, ver = b[p] & 0x0F, b[p] >> 4
    bf = b[p + 1] | (b[p + 2] << 8) | (b[p + 3] << 16)
    size = struct.unpack_from("<I", b, p + 4)[0]
    q = p + 8
    if cls == 0:  # fixed point
        order = ">" if bf & 1 else "<"
        kind = "i" if bf & 0x08 else "u"
        return np.dtype(f"{order}{kind}{size}"), q + 4
    if cls == 1:  # floating point (IEEE layouts)
        order = ">" if bf & 1 else "<"
        return np.dtype(f"{order}f{size}"), q + 12
    if cls == 3:  # fixed-length string
        return np.dtype(f"S{size}"), q
    if cls == 6:  # compound
        nmem = bf & 0xFFFF
        names, fmts, offs = [], [], []
        for _ in range(nmem):
            end = b.index(b"\0", q)
            name = b[q:end].decode()
            if ver < 3:
                q += _pad8(end + 1 - q)
                off = struct.unpack_from("<I", b, q)[0]
                q += 4
                if ver == 1:
                    q += 28  # dimensionality, permutation and sizes of the old array members
            else:
                q = end + 1
                nb = max(1, (size.bit_length() + 7) // 8)
                off = int.from_bytes(b[q:q + nb], "little")
                q += nb
            mdt, q = _decode_dtype(b, q)
            names.append(name)
            fmts.append(mdt)
            offs.append(off)
        if (len(names) == 2 and names == ["r", "i"] and fmts[0] == fmts[1] and fmts[0].kind == "f"
                and offs == [0, fmts[0].itemsize] and size == 2 * fmts[0].itemsize):
            return np.dtype(f"{fmts[0].byteorder if fmts[0].byteorder in '<>' else '<'}c{size}"), q
        return np.dtype({"names": names, "formats": fmts, "offsets": offs, "itemsize": size}), q
    if cls == 9:  # variable length
        _, q = _decode_dtype(b, q)
        if bf & 0x0F == 1:
            return _VlenStr, q
        raise NotImplementedError("variable-length sequences")
    if cls == 8:  # enumeration (h5py booleans): values keep the base integer type
        base, q = _decode_dtype(b, q)
        nmem = bf & 0xFFFF
        for _ in range(nmem):
            end = b.index(b"\0", q)
            q = end + 1 if ver >= 3 else q + _pad8(end + 1 - q)
        return base, q + nmem * base.itemsize
    raise NotImplementedError(f"HDF5 datatype class {cls}")


# ------------------------------------------------------------------------- reader
class _FileReader:
    def __init__(self, path: str):
        self.fh = open(path, "rb")
        self.size = os.fstat(self.fh.fileno()).st_size
        self._heaps: dict[int, dict[int, bytes]] = {}
        sb = 0
        while True:
            if self.read(sb, 8) == SIGNATURE:
                break
            sb = 512 if sb == 0 else 2 * sb
            if sb >= self.size:
                raise OSError(f"{path}: not an HDF5 file")
        ver = self.read(sb + 8, 1)[0]
        if ver in (0, 1):
            h = self.read(sb, 96 + 4 * (ver == 1))
            self.so, self.sl = h[13], h[14]
            if (self.so, self.sl) != (8, 8):
                raise NotImplementedError("offset and length sizes other than 8 bytes")
            p = 24 + (4 if ver == 1 else 0)
            self.base = struct.unpack_from("<Q", h, p)[0]
            root = struct.unpack_from("<QQIi", h, p + 32)
            self.root = root[1]
        elif ver in (2, 3):
            h = self.read(sb, 48)
            self.so, self.sl = h[9], h[10]
            if (self.so, self.sl) != (8, 8):
                raise NotImplementedError("offset and length sizes other than 8 bytes")
            self.base, _ext, _eof, self.root = struct.unpack_from("<QQQQ", h, 12)
        else:
            raise NotImplementedError(f"superblock version {ver}")

    def read(self, addr: int, n: int) -> bytes:
        b = os.pread(self.fh.fileno(), n, addr)
        if len(b) != n:
            raise OSError(f"short read at {addr} ({len(b)} of {n} bytes)")
        return b

    def ra(self, addr: int, n: int) -> bytes:  # relative to the base address
        return self.read(self.base + addr, n)

    # object headers -> [(type, flags, data)]
    def messages(self, addr: int) -> list[tuple[int, int, bytes]]:
        first = self.ra(addr, 16)
        out: list[tuple[int, int, bytes]] = []
        if first[:4] == b"OHDR":
            flags = first[5]
            p = 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
            nsz = 1 << (flags & 3)
            hdr = self.ra(addr, p + nsz)
            size0 = int.from_bytes(hdr[p:p + nsz], "little")
            blocks = [(addr + p + nsz, size0)]
            track = bool(flags & 0x04)
            while blocks:
                start, size = blocks.pop(0)
                b = self.ra(start, size)
                q = 0
                hlen = 4 + (2 if track else 0)
                while q + hlen <= size:
                    mtype, msize, mflags = b[q], struct.unpack_from("<H", b, q + 1)[0], b[q + 3]
                    q += hlen
                    data = b[q:q + msize]
                    q += msize
                    if mtype == _M_CONT:
                        caddr, clen = struct.unpack_from("<QQ", data)
                        blocks.append((caddr + 4, clen - 8))  # skip "OCHK" and the checksum
                    elif mtype != 0:
                        out.append((mtype, mflags, data))
            return out
        ver = first[0]
        if ver != 1:
            raise NotImplementedError(f"object header version {ver}")
        size = struct.unpack_from("<I", first, 8)[0]
        blocks = [(addr + 16, size)]
        while blocks:
            start, size = blocks.pop(0)
            b = self.ra(start, size)
            q = 0
            while q + 8 <= size:
                mtype, msize, mflags = struct.unpack_from("<HHB", b, q)
                data = b[q + 8:q + 8 + msize]
                q += 8 + msize
                if mtype == _M_CONT:
                    blocks.append(struct.unpack_from("<QQ", data))
                elif mtype != 0:
                    out.append((mtype, mflags, data))
        return out

    # groups
    def links(self, msgs) -> dict[str, int]:
        links: dict[str, int] = {}
        for mtype, _, data in msgs:
            if mtype == _M_STAB:
                btree, heap = struct.unpack_from("<QQ", data)
                names = self._local_heap(heap)
                for off, obj in self._group_btree(btree):
                    links[_cstr(names, off)] = obj
            elif mtype == _M_LINK:
                name, addr = _parse_link(data)
                if addr is not None:
                    links[name] = addr
            elif mtype == _M_LINKINFO:
                flags = data[1]
                p = 2 + (8 if flags & 1 else 0)
                fheap = struct.unpack_from("<Q", data, p)[0]
                if fheap != UNDEF:
                    raise NotImplementedError("dense link storage (fractal heap)")
        return links

    def _local_heap(self, addr: int) -> bytes:
        h = self.ra(addr, 32)
        if h[:4] != b"HEAP":
            raise OSError("bad local heap")
        size, _free, data = struct.unpack_from("<QQQ", h, 8)
        return self.ra(data, size)

    def _group_btree(self, addr: int) -> Iterator[tuple[int, int]]:
        h = self.ra(addr, 24)
        if h[:4] != b"TREE" or h[4] != 0:
            raise OSError("bad group B-tree node")
        level, used = h[5], struct.unpack_from("<H", h, 6)[0]
        body = self.ra(addr + 24, used * 16 + 8)
        for i in range(used):
            child = struct.unpack_from("<Q", body, 8 + 16 * i)[0]
            if level > 0:
                yield from self._group_btree(child)
            else:
                s = self.ra(child, 8)
                if s[:4] != b"SNOD":
                    raise OSError("bad symbol-table node")
                n = struct.unpack_from("<H", s, 6)[0]
                ents = self.ra(child + 8, n * _ENTRY)
                for k in range(n):
                    off, obj = struct.unpack_from("<QQ", ents, k * _ENTRY)
                    yield off, obj

    def global_heap_object(self, coll: int, index: int) -> bytes:
        objs = self._heaps.get(coll)
        if objs is None:
            h = self.ra(coll, 16)
            if h[:4] != b"GCOL":
                raise OSError("bad global heap collection")
            size = struct.unpack_from("<Q", h, 8)[0]
            b = self.ra(coll, size)
            objs, p = {}, 16
            while p + 16 <= size:
                idx, _ref, _r, osz = struct.unpack_from("<HHIQ", b, p)
                if idx == 0:
                    break
                objs[idx] = b[p + 16:p + 16 + osz]
                p += 16 + _pad8(osz)
            self._heaps[coll] = objs
        return objs[index]

    def decode_values(self, raw: bytes, dt, shape: tuple[int, ...]):
        if dt is _VlenStr:
            n = int(np.prod(shape)) if shape else 1
            vals = []
            for i in range(n):
                ln, coll, idx = struct.unpack_from("<IQI", raw, 16 * i)
                vals.append(self.global_heap_object(coll, idx)[:ln].decode("utf-8") if coll else "")
            if not shape:
                return vals[0]
            return np.array(vals, dtype=object).reshape(shape)
        arr = np.frombuffer(raw, dtype=dt, count=int(np.prod(shape)) if shape else 1)
        return arr.reshape(shape)


def _cstr(b: bytes, off: int) -> str:
    return b[off:b.index(b"\0", off)].decode("utf-8")


def _parse_link(data: bytes):
    flags = data[1]
    p = 2
    ltype = 0
    if flags & 0x08:
        ltype = data[p]
        p += 1
    if flags & 0x04:
        p += 8
    if flags & 0x10:
        p += 1
    nb = 1 << (flags & 3)
    ln = int.from_bytes(data[p:p + nb], "little")
    p += nb
    name = data[p:p + ln].decode("utf-8")
    p += ln
    if ltype != 0:
        return name, None  # soft / external links are not followed
    return name, struct.unpack_from("<Q", data, p)[0]


def _parse_dataspace(data: bytes) -> tuple[int, ...]:
    ver, rank, flags = data[0], data[1], data[2]
    if ver == 1:
        p = 8
    else:
        if data[3] == 2:
            return (0,)  # null dataspace: no elements
        p = 4
    return tuple(struct.unpack_from(f"<{rank}Q", data, p)) if rank else ()


def _parse_attribute(rd: _FileReader, data: bytes):
    ver = data[0]
    nsz, tsz, ssz = struct.unpack_from("<HHH", data, 2)
    p = 8 + (1 if ver == 3 else 0)
    name = data[p:p + nsz].split(b"\0", 1)[0].decode("utf-8")
    p += _pad8(nsz) if ver == 1 else nsz
    dt, _ = _decode_dtype(data, p)
    p += _pad8(tsz) if ver == 1 else tsz
    shape = _parse_dataspace(data[p:p + ssz])
    p += _pad8(ssz) if ver == 1 else ssz
    val = rd.decode_values(data[p:], dt, shape)
    if isinstance(val, np.ndarray) and val.ndim == 0:
        val = val[()]
    return name, val


class AttributeManager:
    """Dict-like attributes of a group or dataset."""

    def __init__(self, owner):
        self._owner = owner
        self._items: dict[str, Any] = {}

    def __getitem__(self, key: str):
        return self._items[key]

    def __setitem__(self, key: str, value):
        if not self._owner._writable:
            raise OSError("file opened read-only")
        if isinstance(value, str):
            self._items[key] = value
        elif isinstance(value, (bool, np.bool_)):
            raise TypeError("boolean attributes are not supported")
        elif isinstance(value, (int, np.integer)):
            self._items[key] = np.int64(value)
        elif isinstance(value, (float, np.floating)):
            self._items[key] = np.float64(value)
        else:
            self._items[key] = np.asarray(value, order="C")

    def __contains__(self, key) -> bool:
        return key in self._items

    def keys(self):
        return self._items.keys()

    def items(self):
        return self._items.items()

    def __iter__(self):
        return iter(self._items)

    def __len__(self):
        return len(self._items)


class Dataset:
    def __init__(self, file: "File", name: str, shape, dtype, *, addr=None, msgs=None):
        self.file, self.name = file, name
        self.shape, self.dtype = tuple(shape), dtype
        self.attrs = AttributeManager(self)
        self._writable = file._writable
        self._layout = None
        self._filters: list[tuple[int, tuple[int, ...]]] = []
        self._wdata: tuple[int, int] | None = None  # (offset, nbytes) of a written payload
        if msgs is not None:
            for mtype, _, data in msgs:
                if mtype == _M_LAYOUT:
                    self._layout = data
                elif mtype == _M_FILTERS:
                    self._filters = _parse_filters(data)
                elif mtype == _M_ATTR:
                    k, v = _parse_attribute(file._rd, data)
                    self.attrs._items[k] = v

    @property
    def ndim(self) -> int:
        return len(self.shape)

    @property
    def size(self) -> int:
        return int(np.prod(self.shape)) if self.shape else 1

    def extent(self) -> tuple[int, int] | None:
        """(absolute file offset, bytes) of a contiguous payload; None for other layouts."""
        lay = self._layout
        if lay is None or lay[0] < 3:
            return None
        if lay[1] == 1:
            addr, nbytes = struct.unpack_from("<QQ", lay, 2)
            if addr == UNDEF:
                return None
            return self.file._rd.base + addr, nbytes
        return None

    def _read_all(self):
        rd = self.file._rd
        dt = self.dtype
        isz = 16 if dt is _VlenStr else dt.itemsize
        n = self.size
        lay = self._layout
        ver = lay[0]
        if ver >= 3:
            cls = lay[1]
        else:
            cls = lay[2]
        if cls == 0:  # compact
            if ver >= 3:
                sz = struct.unpack_from("<H", lay, 2)[0]
                raw = lay[4:4 + sz]
            else:
                rank = lay[1]
                p = 8 + 4 * rank
                sz = struct.unpack_from("<I", lay, p)[0]
                raw = lay[p + 4:p + 4 + sz]
            return rd.decode_values(raw[:n * isz], dt, self.shape)
        if cls == 1:  # contiguous
            addr = struct.unpack_from("<Q", lay, 2 if ver >= 3 else 8)[0]
            if addr == UNDEF or n == 0:
                return rd.decode_values(b"\0" * (n * isz), dt, self.shape)
            if dt is _VlenStr:
                return rd.decode_values(rd.ra(addr, n * isz), dt, self.shape)
            out = np.empty(self.shape, dtype=dt)  # writable, filled by one positioned read
            view = memoryview(out.reshape(-1).view(np.uint8))
            got = os.preadv(rd.fh.fileno(), [view], rd.base + addr)
            if got != n * isz:
                raise OSError(f"{self.name}: short read ({got} of {n * isz} bytes)")
            return out
        if cls == 2:
            if ver >= 4:
                raise NotImplementedError("version-4 chunk indexes")
            if ver == 3:
                rank1 = lay[2]
                btree = struct.unpack_from("<Q", lay, 3)[0]
                cdims = struct.unpack_from(f"<{rank1}I", lay, 11)
            else:
                rank1 = lay[1]
                btree = struct.unpack_from("<Q", lay, 8)[0]
                cdims = struct.unpack_from(f"<{rank1}I", lay, 16)
            return self._read_chunked(btree, tuple(cdims[:-1]), isz)
        raise NotImplementedError(f"layout class {cls}")

    def _read_chunked(self, btree: int, cdims: tuple[int, ...], isz: int):
        rd = self.file._rd
        if self.dtype is _VlenStr:
            raise NotImplementedError("chunked variable-length strings")
        out = np.zeros(self.shape, dtype=self.dtype)
        rank = len(self.shape)
        for nbytes, mask, offs, addr in _chunk_btree(rd, btree, rank + 1):
            raw = rd.ra(addr, nbytes)
            for k in range(len(self._filters) - 1, -1, -1):
                if mask & (1 << k):
                    continue
                fid, cd = self._filters[k]
                if fid == 1:
                    raw = zlib.decompress(raw)
                elif fid == 2:
                    es = cd[0] if cd else isz
                    a = np.frombuffer(raw, np.uint8)
                    m = len(a) // es
                    raw = a[:m * es].reshape(es, m).T.tobytes() + a[m * es:].tobytes()
                elif fid == 3:
                    raw = raw[:-4]
                else:
                    raise NotImplementedError(f"HDF5 filter {fid}")
            chunk = np.frombuffer(raw, dtype=self.dtype, count=int(np.prod(cdims))).reshape(cdims)
            dst = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, self.shape))
            src = tuple(slice(0, d.stop - d.start) for d in dst)
            out[dst] = chunk[src]
        return out

    def __getitem__(self, key):
        if self._wdata is not None:
            raise OSError("reading back datasets of a file opened for writing is not supported")
        v = self._read_all()
        if key is Ellipsis or key == ():
            return v
        return v[key]

    def __array__(self, dtype=None, copy=None):
        v = self[...]
        a = np.asarray(v)
        return a.astype(dtype) if dtype is not None else a

    def read_into(self, out: np.ndarray) -> None:
        """Read a contiguous payload straight into ``out`` (a writable C-contiguous array)."""
        ext = self.extent()
        if ext is None or self.dtype is _VlenStr:
            out[...] = self[...]
            return
        mv = memoryview(out.reshape(-1).view(np.uint8))
        off, n = ext
        got = os.preadv(self.file._rd.fh.fileno(), [mv[:n]], off)
        if got != n:
            raise OSError(f"short read of {self.name}")


def _parse_filters(data: bytes) -> list[tuple[int, tuple[int, ...]]]:
    ver, n = data[0], data[1]
    p = 8 if ver == 1 else 2
    out = []
    for _ in range(n):
        fid = struct.unpack_from("<H", data, p)[0]
        p += 2
        nlen = 0
        if ver == 1 or fid >= 256:
            nlen = struct.unpack_from("<H", data, p)[0]
            p += 2
        _flags, nval = struct.unpack_from("<HH", data, p)
        p += 4
        p += _pad8(nlen) if ver == 1 else nlen
        cd = struct.unpack_from(f"<{nval}I", data, p)
        p += 4 * nval
        if ver == 1 and nval % 2:
            p += 4
        out.append((fid, tuple(cd)))
    return out


def _chunk_btree(rd: _FileReader, addr: int, ndims: int):
    h = rd.ra(addr, 24)
    if h[:4] != b"TREE" or h[4] != 1:
        raise OSError("bad chunk B-tree node")
    level, used = h[5], struct.unpack_from("<H", h, 6)[0]
    ksz = 8 + 8 * ndims
    body = rd.ra(addr + 24, used * (ksz + 8) + ksz)
    for i in range(used):
        p = i * (ksz + 8)
        nbytes, mask = struct.unpack_from("<II", body, p)
        offs = struct.unpack_from(f"<{ndims}Q", body, p + 8)
        child = struct.unpack_from("<Q", body, p + ksz)[0]
        if level > 0:
            yield from _chunk_btree(rd, child, ndims)
        else:
            yield nbytes, mask, offs[:-1], child


class Group:
    def __init__(self, file: "File", name: str, *, msgs=None):
        self.file, self.name = file, name
        self.attrs = AttributeManager(self)
        self._writable = file._writable if file is not None else True
        self._children: dict[str, Any] = {}
        self._links: dict[str, int] = {}
        if msgs is not None:
            self._links = file._rd.links(msgs)
            for mtype, _, data in msgs:
                if mtype == _M_ATTR:
                    k, v = _parse_attribute(file._rd, data)
                    self.attrs._items[k] = v
                elif mtype == _M_ATTRINFO:
                    flags = data[1]
                    p = 2 + (2 if flags & 1 else 0)
                    if struct.unpack_from("<Q", data, p)[0] != UNDEF:
                        raise NotImplementedError("dense attribute storage (fractal heap)")

    def keys(self):
        return list(self._children) if self._writable else list(self._links)

    def __iter__(self):
        return iter(self.keys())

    def __len__(self):
        return len(self.keys())

    def items(self):
        return [(k, self[k]) for k in self.keys()]

    def __contains__(self, path) -> bool:
        try:
            self[path]
        except KeyError:
            return False
        return True

    def __getitem__(self, path: str):
        parts = [p for p in path.split("/") if p]
        node = self
        for part in parts:
            node = node._child(part)
        return node

    def _child(self, name: str):
        if name in self._children:
            return self._children[name]
        if self._writable or name not in self._links:
            raise KeyError(name)
        msgs = self.file._rd.messages(self._links[name])
        full = f"{self.name.rstrip('/')}/{name}"
        types = {m[0] for m in msgs}
        if _M_LAYOUT in types:
            shape, dt = (), None
            for mtype, _, data in msgs:
                if mtype == _M_DATASPACE:
                    shape = _parse_dataspace(data)
                elif mtype == _M_DATATYPE:
                    dt, _ = _decode_dtype(data)
            node = Dataset(self.file, full, shape, dt, msgs=msgs)
        else:
            node = Group(self.file, full, msgs=msgs)
        self._children[name] = node
        return node

    def create_group(self, name: str) -> "Group":
        if not self._writable:
            raise OSError("file opened read-only")
        if "/" in name.strip("/"):
            head, tail = name.strip("/").split("/", 1)
            g = self._children.get(head) or self.create_group(head)
            return g.create_group(tail)
        if name in self._children:
            raise ValueError(f"{name} already exists")
        g = Group(self.file, f"{self.name.rstrip('/')}/{name}")
        self._children[name] = g
        return g

    def create_dataset(self, name: str, data=None, **_unused) -> Dataset:
        """Write ``data`` (array-like) as a contiguous dataset; the payload goes to the file now."""
        if not self._writable:
            raise OSError("file opened read-only")
        if name in self._children:
            raise ValueError(f"{name} already exists")
        arr = np.asarray(data)
        if arr.dtype.kind == "U":
            arr = np.char.encode(arr, "utf-8")
        if arr.dtype.byteorder == ">":
            arr = arr.astype(arr.dtype.newbyteorder("<"))
        arr = np.asarray(arr, order="C")
        _encode_dtype(arr.dtype)  # reject unsupported types before writing
        ds = Dataset(self.file, f"{self.name.rstrip('/')}/{name}", arr.shape, arr.dtype)
        ds._wdata = self.file._w.payload(arr)
        self._children[name] = ds
        return ds


class File(Group):
    """``File(path, "r")`` reads; ``File(path, "w")`` creates (the file is written on close)."""

    def __init__(self, path, mode: str = "r"):
        self.filename = os.fspath(path)
        self._writable = mode in ("w", "w-", "x")
        self._rd = None
        self._w = None
        if self._writable:
            if mode in ("w-", "x") and os.path.exists(self.filename):
                raise FileExistsError(self.filename)
            self._w = _FileWriter(self.filename)
            super().__init__(self, "/")
        elif mode == "r":
            self._rd = _FileReader(self.filename)
            super().__init__(self, "/", msgs=self._rd.messages(self._rd.root))
        else:
            raise ValueError(f"unsupported mode {mode!r}")

    def close(self) -> None:
        if self._w is not None:
            w, self._w = self._w, None
            w.finish(self)
        if self._rd is not None:
            self._rd.fh.close()
            self._rd = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False


# ------------------------------------------------------------------------- writer
class _FileWriter:
    """Appends payloads as datasets are created, then the metadata tree on close."""

    def __init__(self, path: str):
        self.fh = open(path, "wb")
        self.fh.write(b"\0" * 96)  # superblock, patched on close
        self.pos = 96

    def _append(self, b: bytes) -> int:
        addr = self.pos
        self.fh.write(b)
        self.pos += len(b)
        return addr

    def _align(self, a: int = 8) -> None:
        r = (-self.pos) % a
        if r:
            self._append(b"\0" * r)

    def payload(self, arr: np.ndarray) -> tuple[int, int]:
        self._align(64)
        addr = self.pos
        mv = memoryview(arr.reshape(-1).view(np.uint8)) if arr.size else b""
        self.fh.write(mv)
        self.pos += arr.nbytes
        return addr, arr.nbytes

    def _attr_messages(self, attrs: AttributeManager) -> list[tuple[int, int, bytes]]:
        strs = [(k, v) for k, v in attrs.items() if isinstance(v, str)]
        gcol = {}
        if strs:
            body = b""
            for i, (k, v) in enumerate(strs, start=1):
                enc = v.encode("utf-8")
                body += struct.pack("<HHIQ", i, 1, 0, len(enc)) + _pad(enc)
                gcol[k] = (len(enc), i)
            size = max(_GCOL_MIN, 16 + len(body) + 16)
            free = size - 16 - len(body)
            blob = b"GCOL" + bytes([1, 0, 0, 0]) + struct.pack("<Q", size) + body
            blob += struct.pack("<HHIQ", 0, 0, 0, free) + b"\0" * (free - 16)
            self._align()
            coll = self._append(blob)
        msgs = []
        for k, v in attrs.items():
            name = k.encode("utf-8") + b"\0"
            if isinstance(v, str):
                dt = _encode_vlen_str()
                space = _dataspace(())
                ln, idx = gcol[k]
                data = struct.pack("<IQI", ln, coll, idx)
            else:
                a = np.asarray(v, order="C")
                if a.dtype.byteorder == ">":
                    a = a.astype(a.dtype.newbyteorder("<"))
                dt = _encode_dtype(a.dtype)
                space = _dataspace(a.shape)
                data = a.tobytes()
            body = (bytes([1, 0]) + struct.pack("<HHH", len(name), len(dt), len(space))
                    + _pad(name) + _pad(dt) + _pad(space) + data)
            msgs.append((_M_ATTR, 0, body))
        return msgs

    def _object_header(self, msgs: list[tuple[int, int, bytes]]) -> int:
        body = b""
        for mtype, flags, data in msgs:
            d = _pad(data)
            body += struct.pack("<HHB3s", mtype, len(d), flags, b"\0" * 3) + d
        self._align()
        return self._append(struct.pack("<BBHII4s", 1, 0, len(msgs), 1, len(body), b"\0" * 4) + body)

    def _dataset(self, ds: Dataset) -> int:
        addr, nbytes = ds._wdata
        layout = struct.pack("<BBQQ", 3, 1, addr if nbytes else UNDEF, nbytes)
        fill = bytes([2, 2, 2, 0])  # version 2: late allocation, fill on allocation if set, no value
        msgs = [(_M_DATASPACE, 0, _dataspace(ds.shape)), (_M_DATATYPE, 1, _encode_dtype(ds.dtype)),
                (_M_FILL, 1, fill), (_M_LAYOUT, 0, layout)] + self._attr_messages(ds.attrs)
        return self._object_header(msgs)

    def _group(self, g: Group) -> tuple[int, int, int]:
        """Write children, name heap, symbol-table nodes, B-tree and header; returns
        (header address, B-tree address, heap address)."""
        entries = []
        for name, child in g._children.items():
            if isinstance(child, Group):
                hdr, bt, hp = self._group(child)
                entries.append((name, hdr, 1, struct.pack("<QQ", bt, hp)))
            else:
                entries.append((name, self._dataset(child), 0, b"\0" * 16))
        entries.sort(key=lambda e: e[0].encode("utf-8"))
        heap = b"\0" * 8
        offs = {}
        for name, *_ in entries:
            offs[name] = len(heap)
            heap += _pad(name.encode("utf-8") + b"\0")
        self._align()
        data_addr = self._append(heap)
        heap_addr = self._append(b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap), UNDEF, data_addr))
        cap = 2 * _LEAF_K
        nodes = [entries[i:i + cap] for i in range(0, len(entries), cap)] or [[]]
        if len(nodes) > 2 * _NODE_K:
            raise NotImplementedError(f"groups with more than {2 * _NODE_K * cap} members")
        snods = []
        for chunk in nodes:
            b = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(chunk))
            for name, hdr, cache, scratch in chunk:
                b += struct.pack("<QQI4s", offs[name], hdr, cache, b"\0" * 4) + scratch
            snods.append(self._append(b + b"\0" * (_SNOD_SIZE - len(b))))
        used = len(snods) if entries else 0
        tree = b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", used, UNDEF, UNDEF)
        tree += struct.pack("<Q", 0)
        for i in range(used):
            last = nodes[i][-1][0]
            tree += struct.pack("<QQ", snods[i], offs[last])
        btree = self._append(tree + b"\0" * (_TREE_SIZE - len(tree)))
        hdr = self._object_header([(_M_STAB, 0, struct.pack("<QQ", btree, heap_addr))]
                                  + self._attr_messages(g.attrs))
        return hdr, btree, heap_addr

    def finish(self, root: Group) -> None:
        try:
            hdr, bt, hp = self._group(root)
        except BaseException:
            self.fh.close()
            raise
        eof = self.pos
        sb = (SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", _LEAF_K, _NODE_K, 0)
              + struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
              + struct.pack("<QQI4sQQ", 0, hdr, 1, b"\0" * 4, bt, hp))
        assert len(sb) == 96
        self.fh.seek(0)
        self.fh.write(sb)
        self.fh.close()


def _dataspace(shape: tuple[int, ...]) -> bytes:
    return bytes([1, len(shape), 0, 0, 0, 0, 0, 0]) + struct.pack(f"<{len(shape)}Q", *shape)
