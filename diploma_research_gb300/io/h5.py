"""A self-contained subset of HDF5 for the reference's matrix files (no libhdf5 / h5py needed).

The reference stores matrices with libhdf5 (libs/dim/io/h5.cpp, include/dim/io/h5.h):

* a MATLAB-compatible CSR group (``write_matlab_compatible`` / ``read_matlab_compatible``,
  include/dim/io/h5.h:68-97): datasets ``data`` (f64), ``ir`` (u32 column indices), ``jc`` (u32 row
  offsets) and the scalar u32 attribute ``MATLAB_sparse`` = column count;
* a CSR5 group (``store`` / ``load_csr5``, libs/dim/io/h5.cpp:45-74): attribute ``column_count`` and
  datasets ``vals``, ``col_idx``, ``row_ptr``, ``tile_ptr``, ``tile_desc`` (one H5T array of 4 u32 per
  tile), ``tile_desc_offset_ptr``, ``tile_desc_offset``;
* result vectors (f64 datasets, benchmarks/csr5/dim/main.cpp:35-43) compared by ``compare_results``.

Writer: the HDF5 layout libhdf5 produces with its default ("earliest") format -- version-0 superblock,
version-1 object headers, groups as symbol tables (v1 B-tree + local heap + symbol table nodes),
contiguous datasets, version-1 attributes.  Reader: that layout, plus chunked datasets (v1 B-tree chunk
index, optional deflate filter) and object-header continuation blocks, as libhdf5 writes them when the
reference's dataset properties ask for chunking/compression.  Files with version-2 object headers
(libver "latest") are rejected with an error.

The format follows the HDF5 File Format Specification (superblock v0, object header v1, messages
0x0001 dataspace, 0x0003 datatype, 0x0005 fill value, 0x0008 layout v3, 0x000B filter pipeline,
0x000C attribute, 0x0010 continuation, 0x0011 symbol table).  Neither libhdf5 nor h5py is installed
where this was built, so interoperability with them is by construction, not by test.
"""
from __future__ import annotations

import math
import mmap
import os
import struct
import zlib
from dataclasses import dataclass, field

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
_LEAF_K = 4       # group leaf node K: a symbol table node holds up to 2K entries
_INTERNAL_K = 16  # group internal node K: a B-tree node holds up to 2K children
_HEAP_FREE_NULL = 1  # "no free block" in a local heap's free-list field


def is_hdf5(path) -> bool:
    """True when the file starts with the HDF5 signature (libs/dim/io/h5.cpp:76-87)."""
    try:
        with open(path, "rb") as fh:
            return fh.read(8) == SIGNATURE
    except OSError:
        return False


# ------------------------------------------------------------------------------------------------
# datatypes
# ------------------------------------------------------------------------------------------------

def _dt_fixed(size: int, signed: bool) -> bytes:
    bits = 0x08 if signed else 0x00
    return struct.pack("<BBBBIHH", 0x10, bits, 0, 0, size, 0, 8 * size)


def _dt_float(size: int) -> bytes:
    if size == 8:
        return struct.pack("<BBBBIHHBBBBI", 0x11, 0x20, 63, 0, 8, 0, 64, 52, 11, 0, 52, 1023)
    if size == 4:
        return struct.pack("<BBBBIHHBBBBI", 0x11, 0x20, 31, 0, 4, 0, 32, 23, 8, 0, 23, 127)
    raise ValueError("only 4- and 8-byte floats")


def _dt_array(base: bytes, base_size: int, dims) -> bytes:
    n = math.prod(dims)
    props = struct.pack("<B3x", len(dims)) + b"".join(struct.pack("<I", d) for d in dims)
    props += b"".join(struct.pack("<I", i) for i in range(len(dims)))  # permutation (version 2)
    return struct.pack("<BBBBI", 0x2A, 0, 0, 0, base_size * n) + props + base


def _datatype_for(arr: np.ndarray, inner: int = 0) -> bytes:
    """Datatype message for a numpy array's element type; inner > 0 makes an array type of that many
    elements per dataset element (tile_desc: 4 x u32)."""
    dt = arr.dtype
    if dt.byteorder == ">":
        raise ValueError("big-endian data is not supported")
    if dt.kind == "f":
        base = _dt_float(dt.itemsize)
    elif dt.kind in "ui":
        base = _dt_fixed(dt.itemsize, dt.kind == "i")
    else:
        raise ValueError(f"unsupported dtype {dt}")
    return _dt_array(base, dt.itemsize, [inner]) if inner else base


# ------------------------------------------------------------------------------------------------
# writer
# ------------------------------------------------------------------------------------------------

def _pad8(b: bytes) -> bytes:
    return b + b"\0" * (-len(b) % 8)


def _msg(mtype: int, data: bytes, flags: int = 0) -> bytes:
    data = _pad8(data)
    return struct.pack("<HHB3x", mtype, len(data), flags) + data


def _ohdr(messages) -> bytes:
    body = b"".join(messages)
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body


def _dataspace(shape) -> bytes:
    return struct.pack("<BBBB4x", 1, len(shape), 0, 0) + b"".join(struct.pack("<Q", d) for d in shape)


def _attribute(name: str, value) -> bytes:
    arr = np.asarray(value)
    if arr.ndim != 0:
        raise ValueError("attributes are scalars here")
    dt = _datatype_for(arr)
    sp = _dataspace(())
    nm = name.encode() + b"\0"
    head = struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(sp))
    return _msg(0x000C, head + _pad8(nm) + _pad8(dt) + _pad8(sp) + arr.astype(arr.dtype.newbyteorder("<")).tobytes())


@dataclass
class _Dataset:
    data: np.ndarray
    inner: int = 0  # > 0: the trailing axis is an array type of this many elements


@dataclass
class _Group:
    members: dict = field(default_factory=dict)  # name -> _Group | _Dataset
    attrs: dict = field(default_factory=dict)


class _Image:
    def __init__(self):
        self.buf = bytearray()

    def alloc(self, size: int) -> int:
        addr = len(self.buf)
        self.buf += b"\0" * (size + (-size % 8))
        return addr

    def put(self, addr: int, data: bytes):
        self.buf[addr:addr + len(data)] = data


def _write_dataset(img: _Image, ds: _Dataset) -> int:
    arr = np.ascontiguousarray(ds.data)
    arr = arr.astype(arr.dtype.newbyteorder("<"), copy=False)
    shape = arr.shape[:-1] if ds.inner else arr.shape
    raw = arr.tobytes()
    daddr = img.alloc(len(raw)) if raw else UNDEF
    if raw:
        img.put(daddr, raw)
    msgs = [
        _msg(0x0001, _dataspace(shape)),
        _msg(0x0003, _datatype_for(arr, ds.inner), flags=1),  # constant
        _msg(0x0005, struct.pack("<BBBB", 2, 2, 2, 0)),       # fill value: late allocation, none defined
        _msg(0x0008, struct.pack("<BBQQ", 3, 1, daddr, len(raw))),  # contiguous layout
    ]
    hdr = _ohdr(msgs)
    addr = img.alloc(len(hdr))
    img.put(addr, hdr)
    return addr


def _write_group(img: _Image, grp: _Group) -> tuple[int, int, int]:
    """Writes a group; returns (object header address, B-tree address, local heap address)."""
    names = sorted(grp.members)  # symbol table nodes keep their entries in name order
    child = {nm: (_write_group(img, m) if isinstance(m, _Group) else (_write_dataset(img, m), None, None))
             for nm, m in grp.members.items()}
    # local heap: "" at offset 0, then every name
    seg = bytearray(b"\0" * 8)
    offs = {}
    for nm in names:
        offs[nm] = len(seg)
        seg += _pad8(nm.encode() + b"\0")
    seg_addr = img.alloc(len(seg))
    img.put(seg_addr, bytes(seg))
    heap = b"HEAP" + struct.pack("<B3xQQQ", 0, len(seg), _HEAP_FREE_NULL, seg_addr)
    heap_addr = img.alloc(len(heap))
    img.put(heap_addr, heap)
    # symbol table nodes of at most 2K entries
    chunks = [names[i:i + 2 * _LEAF_K] for i in range(0, len(names), 2 * _LEAF_K)] or [[]]
    if len(chunks) > 2 * _INTERNAL_K:
        raise ValueError(f"a group holds at most {2 * _INTERNAL_K * 2 * _LEAF_K} members here")
    snods = []
    for ch in chunks:
        ent = b""
        for nm in ch:
            oh, bt, hp = child[nm]
            if bt is None:
                ent += struct.pack("<QQII16x", offs[nm], oh, 0, 0)
            else:
                ent += struct.pack("<QQII", offs[nm], oh, 1, 0) + struct.pack("<QQ", bt, hp)
        node = b"SNOD" + struct.pack("<BBH", 1, 0, len(ch)) + ent
        node += b"\0" * (8 + 2 * _LEAF_K * 40 - len(node))
        a = img.alloc(len(node))
        img.put(a, node)
        snods.append((a, offs[ch[-1]] if ch else 0))
    # one leaf B-tree node: key0 = "" (offset 0), child i, key i+1 = last name of child i
    tree = b"TREE" + struct.pack("<BBHQQ", 0, 0, len(snods), UNDEF, UNDEF) + struct.pack("<Q", 0)
    for a, last in snods:
        tree += struct.pack("<QQ", a, last)
    size = 24 + (2 * _INTERNAL_K + 1) * 8 + 2 * _INTERNAL_K * 8
    tree += b"\0" * (size - len(tree))
    tree_addr = img.alloc(len(tree))
    img.put(tree_addr, tree)
    msgs = [_msg(0x0011, struct.pack("<QQ", tree_addr, heap_addr))]
    msgs += [_attribute(k, v) for k, v in grp.attrs.items()]
    hdr = _ohdr(msgs)
    oh = img.alloc(len(hdr))
    img.put(oh, hdr)
    return oh, tree_addr, heap_addr


def _write_file(path, root: _Group):
    img = _Image()
    img.alloc(96)  # superblock v0 with 8-byte offsets and lengths
    oh, bt, hp = _write_group(img, root)
    sb = SIGNATURE + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, _LEAF_K, _INTERNAL_K, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, len(img.buf), UNDEF)
    sb += struct.pack("<QQII", 0, oh, 1, 0) + struct.pack("<QQ", bt, hp)
    assert len(sb) == 96
    img.put(0, sb)
    with open(path, "wb") as fh:
        fh.write(bytes(img.buf))


# ------------------------------------------------------------------------------------------------
# reader
# ------------------------------------------------------------------------------------------------

class H5FormatError(ValueError):
    pass


@dataclass
class _Type:
    kind: str        # "u", "i", "f"
    size: int        # bytes of one dataset element
    base_size: int   # bytes of the scalar base type
    inner: int = 0   # elements per dataset element for array types

    def numpy(self) -> np.dtype:
        return np.dtype(f"<{self.kind}{self.base_size}")


def _parse_type(b: bytes, p: int) -> tuple[_Type, int]:
    cv = b[p]
    cls, ver = cv & 0x0F, cv >> 4
    bits = b[p + 1] | (b[p + 2] << 8) | (b[p + 3] << 16)
    size = struct.unpack_from("<I", b, p + 4)[0]
    q = p + 8
    if cls == 0:
        if bits & 1:
            raise H5FormatError("big-endian integers are not supported")
        return _Type("i" if bits & 0x08 else "u", size, size), q + 4
    if cls == 1:
        if bits & 1:
            raise H5FormatError("big-endian floats are not supported")
        return _Type("f", size, size), q + 12
    if cls == 10:
        nd = b[q]
        q += 4
        dims = struct.unpack_from(f"<{nd}I", b, q)
        q += 4 * nd
        if ver < 3:
            q += 4 * nd  # permutation indices
        base, q = _parse_type(b, q)
        n = math.prod(dims)
        return _Type(base.kind, size, base.size, n), q
    raise H5FormatError(f"datatype class {cls} is not supported")


def _host_memory() -> int | None:
    try:
        return os.sysconf("SC_PHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    except (AttributeError, ValueError, OSError):
        return None


def _check_extent(nbytes: int, layout: bytes) -> None:
    """Sizes read from a file are checked before they size an allocation: no dataset larger than the host's
    memory, and a contiguous dataset must store as many bytes as its dataspace holds."""
    mem = _host_memory()
    if mem is not None and nbytes > mem:
        raise H5FormatError(f"dataset of {nbytes} bytes exceeds the host's memory")
    if layout[1] == 1:
        a, sz = struct.unpack_from("<QQ", layout, 2)
        if a != UNDEF and sz < nbytes:
            raise H5FormatError("contiguous dataset stores fewer bytes than its dataspace holds")


def _parse_space(b: bytes, p: int) -> tuple:
    ver, rank, flags = b[p], b[p + 1], b[p + 2]
    if ver == 1:
        q = p + 8
    elif ver == 2:
        if b[p + 3] == 2:  # null dataspace
            return ()
        q = p + 4
    else:
        raise H5FormatError(f"dataspace version {ver}")
    return tuple(struct.unpack_from(f"<{rank}Q", b, q))


class _File:
    def __init__(self, path):
        # mapped, not read: a slab read touches only the pages of its bytes
        with open(path, "rb") as fh:
            self.b = mmap.mmap(fh.fileno(), 0, access=mmap.ACCESS_READ) if os.path.getsize(path) else b""
        b = self.b
        if b[:8] != SIGNATURE:
            raise H5FormatError(f"{path} is not an HDF5 file")
        ver = b[8]
        if ver not in (0, 1):
            raise H5FormatError(f"superblock version {ver} (files written with libver 'latest') is not supported")
        if b[13] != 8 or b[14] != 8:
            raise H5FormatError("only 8-byte offsets and lengths are supported")
        p = 24 + (4 if ver == 1 else 0)
        self.base = struct.unpack_from("<Q", b, p)[0]
        p += 32
        self.root = struct.unpack_from("<Q", b, p + 8)[0] + self.base

    def close(self):
        if isinstance(self.b, mmap.mmap):
            self.b.close()
        self.b = b""

    def u64(self, p):
        return struct.unpack_from("<Q", self.b, p)[0]

    def messages(self, addr: int):
        """(type, payload) of the messages of the v1 object header at addr, continuation blocks included."""
        b = self.b
        if b[addr:addr + 4] == b"OHDR":
            raise H5FormatError("version-2 object headers are not supported")
        if b[addr] != 1:
            raise H5FormatError(f"object header version {b[addr]} at {addr}")
        n, size = struct.unpack_from("<H", b, addr + 2)[0], struct.unpack_from("<I", b, addr + 8)[0]
        blocks = [(addr + 16, size)]
        out = []
        while blocks:
            p, sz = blocks.pop(0)
            end = p + sz
            while p + 8 <= end and len(out) < n:
                mtype, msz = struct.unpack_from("<HH", b, p)
                data = b[p + 8:p + 8 + msz]
                if mtype == 0x0010:
                    blocks.append((self.u64(p + 8) + self.base, self.u64(p + 16)))
                out.append((mtype, data))
                p += 8 + msz
        return out

    def group_members(self, addr: int) -> dict:
        stab = [d for t, d in self.messages(addr) if t == 0x0011]
        if not stab:
            raise H5FormatError("not a group (no symbol table message; link-message groups are not supported)")
        tree, heap = struct.unpack_from("<QQ", stab[0])
        b = self.b
        heap += self.base
        if b[heap:heap + 4] != b"HEAP":
            raise H5FormatError("bad local heap")
        seg = self.u64(heap + 24) + self.base
        members = {}

        def walk(node):
            node += self.base
            if b[node:node + 4] != b"TREE":
                raise H5FormatError("bad group B-tree node")
            level, used = b[node + 5], struct.unpack_from("<H", b, node + 6)[0]
            for i in range(used):
                child = self.u64(node + 24 + 8 + 16 * i)
                if level > 0:
                    walk(child)
                    continue
                sn = child + self.base
                if b[sn:sn + 4] != b"SNOD":
                    raise H5FormatError("bad symbol table node")
                for e in range(struct.unpack_from("<H", b, sn + 6)[0]):
                    q = sn + 8 + 40 * e
                    name_off, oh = self.u64(q), self.u64(q + 8)
                    s = seg + name_off
                    name = b[s:b.find(b"\0", s)].decode()
                    members[name] = oh + self.base

        walk(tree)
        return members

    def attributes(self, addr: int) -> dict:
        out = {}
        for t, d in self.messages(addr):
            if t != 0x000C:
                continue
            ver = d[0]
            nsz, tsz, ssz = struct.unpack_from("<HHH", d, 2)
            p = 8
            if ver == 3:
                p += 1
            name = d[p:p + nsz].split(b"\0")[0].decode()
            rnd = (lambda x: x + (-x % 8)) if ver == 1 else (lambda x: x)
            p += rnd(nsz)
            typ, _ = _parse_type(d, p)
            p += rnd(tsz)
            shape = _parse_space(d, p)
            p += rnd(ssz)
            n = math.prod(shape) if shape else 1
            val = np.frombuffer(d, typ.numpy(), n * max(1, typ.inner), p)
            out[name] = val[0] if n == 1 and not typ.inner else val.copy()
        return out

    def read_slab(self, addr: int, start: int, count: int) -> np.ndarray:
        """Elements [start, start + count) of a 1-D dataset: only those bytes for the contiguous layout
        (the reference's read_slab, h5.h), a slice of the whole for the others."""
        typ = shape = layout = None
        for t, d in self.messages(addr):
            if t == 0x0001:
                shape = _parse_space(d, 0)
            elif t == 0x0003:
                typ, _ = _parse_type(d, 0)
            elif t == 0x0008:
                layout = d
        if typ is None or shape is None or layout is None:
            raise H5FormatError("not a dataset")
        n = int(shape[0]) if shape else 1
        if start < 0 or count < 0 or start + count > n:
            raise ValueError(f"slab [{start}, {start + count}) of a dataset of {n}")
        per = typ.size * max(1, typ.inner) if typ.inner else typ.size
        if len(shape) == 1 and layout[0] == 3 and layout[1] == 1 and not typ.inner:
            _check_extent(n * per, layout)
            a, sz = struct.unpack_from("<QQ", layout, 2)
            if a == UNDEF:
                return np.zeros(count, typ.numpy())
            lo = a + self.base + start * per
            raw = bytes(self.b[lo:lo + count * per]).ljust(count * per, b"\0")
            return np.frombuffer(raw, typ.numpy()).copy()
        return self.read_dataset(addr)[start:start + count].copy()

    def read_dataset(self, addr: int) -> np.ndarray:
        typ = shape = layout = None
        filters = []
        for t, d in self.messages(addr):
            if t == 0x0001:
                shape = _parse_space(d, 0)
            elif t == 0x0003:
                typ, _ = _parse_type(d, 0)
            elif t == 0x0008:
                layout = d
            elif t == 0x000B:
                filters = self._filters(d)
        if typ is None or shape is None or layout is None:
            raise H5FormatError("not a dataset")
        count = math.prod(shape) if shape else 1
        nbytes = count * typ.size
        if layout[0] != 3:
            raise H5FormatError(f"layout message version {layout[0]}")
        _check_extent(nbytes, layout)
        cls = layout[1]
        if cls == 0:  # compact
            sz = struct.unpack_from("<H", layout, 2)[0]
            raw = layout[4:4 + sz]
        elif cls == 1:  # contiguous
            a, sz = struct.unpack_from("<QQ", layout, 2)
            raw = b"" if a == UNDEF else self.b[a + self.base:a + self.base + sz]
            raw = raw.ljust(nbytes, b"\0")
        elif cls == 2:
            raw = self._read_chunked(layout, shape, typ, filters)
        else:
            raise H5FormatError(f"layout class {cls}")
        arr = np.frombuffer(raw[:nbytes], typ.numpy()).copy()
        if typ.inner:
            return arr.reshape(tuple(shape) + (typ.inner,))
        return arr.reshape(shape)

    def _filters(self, d: bytes):
        ver, n = d[0], d[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = struct.unpack_from("<H", d, p)[0]
            if ver == 1 or fid >= 256:
                nlen = struct.unpack_from("<H", d, p + 2)[0]
                flags, nval = struct.unpack_from("<HH", d, p + 4)
                p += 8 + (nlen + (-nlen % 8) if ver == 1 else nlen)
            else:
                flags, nval = struct.unpack_from("<HH", d, p + 2)
                p += 6
            p += 4 * nval + (4 if ver == 1 and nval % 2 else 0)
            out.append(fid)
        return out

    def _read_chunked(self, layout: bytes, shape, typ: _Type, filters) -> bytes:
        nd = layout[2]
        tree = struct.unpack_from("<Q", layout, 3)[0]
        cdims = struct.unpack_from(f"<{nd}I", layout, 11)
        if nd != 2:
            raise H5FormatError("only 1-D chunked datasets are supported")
        chunk_elems = cdims[0]
        count = math.prod(shape)
        out = bytearray(count * typ.size)
        b = self.b
        for f in filters:
            if f not in (1,):
                raise H5FormatError(f"filter {f} is not supported (deflate only)")

        def walk(node):
            node += self.base
            if b[node:node + 4] != b"TREE" or b[node + 4] != 1:
                raise H5FormatError("bad chunk B-tree node")
            level, used = b[node + 5], struct.unpack_from("<H", b, node + 6)[0]
            ksz = 8 + 8 * nd
            p = node + 24
            for _ in range(used):
                csize, fmask = struct.unpack_from("<II", b, p)
                off0 = struct.unpack_from("<Q", b, p + 8)[0]
                child = self.u64(p + ksz)
                p += ksz + 8
                if level > 0:
                    walk(child)
                    continue
                raw = b[child + self.base:child + self.base + csize]
                if 1 in filters and not (fmask & 1):
                    raw = zlib.decompress(raw)
                start = off0 * typ.size
                n = min(chunk_elems, count - off0) * typ.size
                out[start:start + n] = raw[:n]

        if tree != UNDEF:
            walk(tree)
        return bytes(out)


# ------------------------------------------------------------------------------------------------
# public API: the reference's IO functions
# ------------------------------------------------------------------------------------------------

def _split(path: str):
    parts = [p for p in path.split("/") if p]
    return parts


class H5Reader:
    """Read access to a file: groups, datasets and attributes by path ("/" separated)."""

    def __init__(self, path):
        self.f = _File(path)

    def close(self):
        """Unmaps the file (a mapped file that another writer truncates must not be touched again)."""
        self.f.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _resolve(self, path: str) -> int:
        addr = self.f.root
        for part in _split(path):
            members = self.f.group_members(addr)
            if part not in members:
                raise KeyError(f"'{part}' not found in HDF5 file")
            addr = members[part]
        return addr

    def members(self, group: str = "/") -> list:
        return sorted(self.f.group_members(self._resolve(group)))

    def attributes(self, path: str = "/") -> dict:
        return self.f.attributes(self._resolve(path))

    def dataset(self, path: str) -> np.ndarray:
        return self.f.read_dataset(self._resolve(path))

    def dataset_slab(self, path: str, start: int, count: int) -> np.ndarray:
        return self.f.read_slab(self._resolve(path), start, count)

    def dataset_length(self, path: str) -> int:
        for t, d in self.f.messages(self._resolve(path)):
            if t == 0x0001:
                shape = _parse_space(d, 0)
                return int(shape[0]) if shape else 1
        raise H5FormatError("not a dataset")

    def contains(self, path: str) -> bool:
        try:
            self._resolve(path)
            return True
        except KeyError:
            return False


class H5Writer:
    """Builds a file in memory (groups, datasets, scalar attributes) and writes it on close().  With
    ``append=True`` the datasets and attributes of an existing file are read back and rewritten."""

    def __init__(self, path, append: bool = False):
        self.path = path
        self.root = _Group()
        if append and is_hdf5(path):
            with H5Reader(path) as r:  # everything is copied out before the file is rewritten
                self._load(r, "/", self.root)

    def _load(self, r: H5Reader, path: str, grp: _Group):
        grp.attrs.update(r.attributes(path))
        for nm in r.members(path):
            sub = path.rstrip("/") + "/" + nm
            try:
                data = r.dataset(sub)
                # 2-D arrays come back only from array-typed datasets (tile_desc)
                grp.members[nm] = _Dataset(data, data.shape[1] if data.ndim == 2 else 0)
            except H5FormatError:
                g = _Group()
                self._load(r, sub, g)
                grp.members[nm] = g

    def group(self, path: str) -> _Group:
        g = self.root
        for part in _split(path):
            m = g.members.get(part)
            if m is None:
                m = g.members[part] = _Group()
            if not isinstance(m, _Group):
                raise ValueError(f"'{part}' is a dataset")
            g = m
        return g

    def remove(self, path: str):
        parts = _split(path)
        self.group("/".join(parts[:-1])).members.pop(parts[-1], None)

    def dataset(self, path: str, data, inner: int = 0):
        parts = _split(path)
        self.group("/".join(parts[:-1])).members[parts[-1]] = _Dataset(np.asarray(data), inner)

    def attribute(self, path: str, name: str, value):
        self.group(path).attrs[name] = value

    def close(self):
        _write_file(self.path, self.root)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        if exc[0] is None:
            self.close()


def write_matlab_compatible(path, group: str, m, append: bool = False):
    """include/dim/io/h5.h:68-76: data, ir (column indices), jc (row offsets), MATLAB_sparse = cols."""
    with H5Writer(path, append=append) as w:
        w.remove(group)
        w.dataset(f"{group}/data", np.asarray(m.values, np.float64))
        w.dataset(f"{group}/ir", np.asarray(m.col_indices, np.uint32))
        w.dataset(f"{group}/jc", np.asarray(m.row_start_offsets, np.uint32))
        w.attribute(group, "MATLAB_sparse", np.uint32(m.dimensions.cols))


def read_matlab_compatible(path, group: str = "A"):
    """include/dim/io/h5.h:78-97."""
    from ..mat import csr, dimensions_t

    with H5Reader(path) as r:
        jc = r.dataset(f"{group}/jc").astype(np.uint32)
        cols = int(r.attributes(group)["MATLAB_sparse"])
        return csr(dimensions_t(jc.size - 1, cols), r.dataset(f"{group}/data").astype(np.float64), jc,
                   r.dataset(f"{group}/ir").astype(np.uint32))


def store_csr5(path, group: str, arrays, cols: int, append: bool = False):
    """libs/dim/io/h5.cpp:45-55.  ``arrays`` holds the reference-layout CSR5 arrays (sigma 16, omega 4):
    vals, col_idx, row_ptr, tile_ptr, tile_desc (T x 4 u32), tile_desc_offset_ptr, tile_desc_offset."""
    with H5Writer(path, append=append) as w:
        w.remove(group)
        w.attribute(group, "column_count", np.uint32(cols))
        w.dataset(f"{group}/vals", np.asarray(arrays.vals, np.float64))
        w.dataset(f"{group}/col_idx", np.asarray(arrays.col_idx, np.uint32))
        w.dataset(f"{group}/row_ptr", np.asarray(arrays.row_ptr, np.uint32))
        w.dataset(f"{group}/tile_ptr", np.asarray(arrays.tile_ptr, np.uint32))
        w.dataset(f"{group}/tile_desc", np.asarray(arrays.tile_desc, np.uint32).reshape(-1, 4), inner=4)
        w.dataset(f"{group}/tile_desc_offset_ptr", np.asarray(arrays.tile_desc_offset_ptr, np.uint32))
        w.dataset(f"{group}/tile_desc_offset", np.asarray(arrays.tile_desc_offset, np.uint32))


def load_csr5_arrays(path, group: str = "A"):
    """libs/dim/io/h5.cpp:57-74: the stored arrays and the dimensions (rows = len(row_ptr) - 1)."""
    with H5Reader(path) as r:
        return _csr5_arrays(r, group)


def _csr5_arrays(r, group: str):
    from types import SimpleNamespace

    td = r.dataset(f"{group}/tile_desc")
    out = SimpleNamespace(
        vals=r.dataset(f"{group}/vals").astype(np.float64),
        col_idx=r.dataset(f"{group}/col_idx").astype(np.uint32),
        row_ptr=r.dataset(f"{group}/row_ptr").astype(np.uint32),
        tile_ptr=r.dataset(f"{group}/tile_ptr").astype(np.uint32),
        tile_desc=td.reshape(-1).astype(np.uint32),
        tile_desc_offset_ptr=r.dataset(f"{group}/tile_desc_offset_ptr").astype(np.uint32),
        tile_desc_offset=r.dataset(f"{group}/tile_desc_offset").astype(np.uint32),
    )
    out.tile_count = td.shape[0]
    out.rows = out.row_ptr.size - 1
    out.cols = int(r.attributes(group)["column_count"])
    return out


def load_csr5_partial(path, group: str, part):
    """Part `part` (a partial.partial_identifier_t) of a stored CSR5 matrix, reading only its slabs
    (load_csr5_partial, h5.cpp:105-173): the stored tiles (sigma 16 x omega 4) are cut into runs of
    ceil(T / parts), the last part also takes the CSR tail.  The chunk's tiles are put back into CSR order
    (the inverse of csr5::transpose, csr5.h:463-493: a full tile whose rows differ was stored row-major
    over its omega columns) and returned as a partial.partial_layout."""
    with H5Reader(path) as r:
        return _load_csr5_partial(r, group, part)


def _load_csr5_partial(r, group: str, part):
    from ..partial import REF_TILE, partial_layout

    cols = int(r.attributes(group)["column_count"])
    rows = r.dataset_length(f"{group}/row_ptr") - 1
    nnz = r.dataset_length(f"{group}/vals")
    tiles = r.dataset_length(f"{group}/tile_desc")
    if tiles != nnz // REF_TILE:
        raise H5FormatError(f"{tiles} stored tiles for {nnz} elements: not a sigma 16 x omega 4 CSR5 group")
    start, count, e0, e1 = partial_layout.chunk_of(nnz, part)
    tp = r.dataset_slab(f"{group}/tile_ptr", start, count + 1).astype(np.int64) & 0x7FFFFFFF
    vals = r.dataset_slab(f"{group}/vals", e0, e1 - e0).astype(np.float64)
    col = r.dataset_slab(f"{group}/col_idx", e0, e1 - e0).astype(np.uint32)
    sigma, omega = 16, REF_TILE // 16
    for i in range(count):
        if tp[i] != tp[i + 1]:
            blk = slice(i * REF_TILE, (i + 1) * REF_TILE)
            vals[blk] = vals[blk].reshape(sigma, omega).T.reshape(-1)
            col[blk] = col[blk].reshape(sigma, omega).T.reshape(-1)
    # row offsets from the chunk's first row (tile_ptr[start]) to beyond its last row
    r0 = int(tp[0])
    r1 = rows if part.idx == part.total_count - 1 else min(rows, int(tp[-1]) + 1)
    rp = r.dataset_slab(f"{group}/row_ptr", r0, r1 + 1 - r0)
    return partial_layout.from_chunk(part, rows, cols, nnz, rp, r0, vals, col)


def write_vector(path, dataset: str, y, overwrite: bool = False, append: bool = True):
    """The result dump of benchmarks/csr5/dim/main.cpp:35-43 (f64 dataset, refuses to overwrite unless asked)."""
    with H5Writer(path, append=append) as w:
        parts = _split(dataset)
        g = w.group("/".join(parts[:-1]))
        if parts[-1] in g.members and not overwrite:
            raise FileExistsError(f"outfile already contains {dataset}; pass overwrite to replace it")
        w.dataset(dataset, np.asarray(y, np.float64))


def read_vector(path, dataset: str) -> np.ndarray:
    with H5Reader(path) as r:
        return r.dataset(dataset).astype(np.float64)
