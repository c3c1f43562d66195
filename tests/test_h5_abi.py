"""The HDF5 matrix files through the C ABI (dimgpu_h5_*, the reference's dim::io::h5 for C++ callers).

The library's C++ reader and writer are checked against the package's Python implementation of the same
subset (diploma_research_gb300/io/h5.py): the writer must produce the same bytes for the same content,
also when appending to a file, and the reader must return the same arrays, including for files laid out
the way libhdf5 writes chunked, deflate-compressed datasets (deflate streams made by zlib with stored,
fixed-code and dynamic-code blocks), with multi-level chunk B-trees and object-header continuation
blocks.  CPU only (host code); the CSR5 store/load entry points, which convert on the device, are in
test_h5_abi_gpu.py."""
import ctypes
import struct
import zlib

import numpy as np
import pytest

from diploma_research_gb300 import _native as N
from diploma_research_gb300.io import h5
from diploma_research_gb300.mat import csr, dimensions_t
from helpers import random_csr


def _b(p) -> bytes:
    return str(p).encode()


def _c_write_csr(L, path, group, m, append=False):
    rp = np.ascontiguousarray(m.row_start_offsets, np.uint32)
    ci = np.ascontiguousarray(m.col_indices, np.uint32)
    v = np.ascontiguousarray(m.values, np.float64)
    rc = L.dimgpu_h5_write_matlab_compatible(_b(path), group.encode(), m.dimensions.rows, m.dimensions.cols,
                                             v.size, rp.ctypes.data, ci.ctypes.data if v.size else None,
                                             v.ctypes.data if v.size else None, int(append))
    assert rc == N.OK, L.dimgpu_last_error_string()


def _c_read_csr(L, path, group):
    rows, cols, nnz = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint64()
    rc = L.dimgpu_h5_csr_dimensions(_b(path), group.encode(), ctypes.byref(rows), ctypes.byref(cols), ctypes.byref(nnz))
    assert rc == N.OK, L.dimgpu_last_error_string()
    rp = np.zeros(rows.value + 1, np.uint32)
    ci = np.zeros(nnz.value, np.uint32)
    v = np.zeros(nnz.value)
    rc = L.dimgpu_h5_read_matlab_compatible(_b(path), group.encode(), rp.ctypes.data, ci.ctypes.data, v.ctypes.data)
    assert rc == N.OK, L.dimgpu_last_error_string()
    return csr(dimensions_t(rows.value, cols.value), v, rp, ci)


def _c_read_vector(L, path, name):
    n = ctypes.c_uint64()
    assert L.dimgpu_h5_vector_length(_b(path), name.encode(), ctypes.byref(n)) == N.OK, L.dimgpu_last_error_string()
    y = np.zeros(n.value)
    assert L.dimgpu_h5_read_vector(_b(path), name.encode(), y.ctypes.data) == N.OK, L.dimgpu_last_error_string()
    return y


def _c_write_vector(L, path, name, y, overwrite=False):
    y = np.ascontiguousarray(y, np.float64)
    return L.dimgpu_h5_write_vector(_b(path), name.encode(), y.size, y.ctypes.data if y.size else None,
                                    int(overwrite))


def _same(a, b):
    assert a.dimensions == b.dimensions
    assert np.array_equal(a.row_start_offsets, b.row_start_offsets)
    assert np.array_equal(a.col_indices, b.col_indices)
    assert np.array_equal(a.values, b.values)


@pytest.mark.parametrize("shape", [(300, 200, 5.0), (1, 1, 1.0), (17, 40, 0.0)])
def test_matlab_group_bytes_match_the_python_writer(native, tmp_path, shape):
    rows, cols, dens = shape
    m = random_csr(np.random.default_rng(rows), rows, cols, dens, empty_frac=0.2)
    pc, pp = tmp_path / "c.h5", tmp_path / "py.h5"
    _c_write_csr(native, pc, "A", m)
    h5.write_matlab_compatible(pp, "A", m)
    assert pc.read_bytes() == pp.read_bytes()
    _same(_c_read_csr(native, pc, "A"), m)
    _same(h5.read_matlab_compatible(pc, "A"), m)


def test_append_sequence_matches_the_python_writer(native, tmp_path):
    """Groups and vectors added one after another to the same file, each step byte-equal; more than eight
    members in a group (several symbol-table nodes) and nested groups."""
    rng = np.random.default_rng(7)
    a = random_csr(rng, 120, 120, 4.0)
    b = random_csr(rng, 50, 80, 3.0, empty_frac=0.3)
    pc, pp = tmp_path / "c.h5", tmp_path / "py.h5"
    _c_write_csr(native, pc, "A", a)
    h5.write_matlab_compatible(pp, "A", a)
    for i in range(11):
        y = rng.uniform(-1, 1, 10 + i)
        assert _c_write_vector(native, pc, f"runs/y{i:02d}", y) == N.OK, native.dimgpu_last_error_string()
        h5.write_vector(pp, f"runs/y{i:02d}", y)
        assert pc.read_bytes() == pp.read_bytes(), i
    _c_write_csr(native, pc, "B", b, append=True)
    h5.write_matlab_compatible(pp, "B", b, append=True)
    assert pc.read_bytes() == pp.read_bytes()
    _c_write_csr(native, pc, "A", b, append=True)  # replaces A in place
    h5.write_matlab_compatible(pp, "A", b, append=True)
    assert pc.read_bytes() == pp.read_bytes()
    _same(_c_read_csr(native, pc, "A"), b)
    assert np.array_equal(_c_read_vector(native, pc, "runs/y07"), h5.read_vector(pp, "runs/y07"))
    # without append the file holds only the new group
    _c_write_csr(native, pc, "C", a)
    assert h5.H5Reader(pc).members("/") == ["C"]


def test_vectors_and_overwrite(native, tmp_path):
    p = tmp_path / "v.h5"
    y = np.linspace(-2, 3, 1001)
    assert _c_write_vector(native, p, "Y", y) == N.OK
    assert np.array_equal(h5.read_vector(p, "Y"), y)
    assert _c_write_vector(native, p, "Y", y * 2) == N.ERR_INVALID_ARGUMENT
    assert b"overwrite" in native.dimgpu_last_error_string()
    assert np.array_equal(_c_read_vector(native, p, "Y"), y)
    assert _c_write_vector(native, p, "Y", y * 2, overwrite=True) == N.OK
    assert np.array_equal(_c_read_vector(native, p, "Y"), y * 2)
    assert _c_write_vector(native, p, "empty", np.zeros(0)) == N.OK
    assert _c_read_vector(native, p, "empty").size == 0
    # integer and f32 datasets are read converted to f64 (as numpy's astype)
    with h5.H5Writer(p, append=True) as w:
        w.dataset("i32", np.array([-3, 0, 7], np.int32))
        w.dataset("f32", np.array([0.5, -1.25], np.float32))
    assert np.array_equal(_c_read_vector(native, p, "i32"), [-3.0, 0.0, 7.0])
    assert np.array_equal(_c_read_vector(native, p, "f32"), [0.5, -1.25])


def _chunked_writer(chunk, compress=None, levels=1, split_header=False):
    """A replacement for the Python writer's dataset layout: chunked 1-D datasets (a v1 B-tree of chunks,
    `levels` deep), optionally through the deflate filter, optionally with the object header continued in
    a second block -- the forms libhdf5 writes for the reference's chunked or compressed datasets."""

    def write(img, ds):
        arr = np.ascontiguousarray(ds.data)
        n = arr.shape[0]
        per = arr.itemsize * (ds.inner or 1)
        recs = []
        for off in range(0, n, chunk):
            raw = arr[off:off + chunk].tobytes().ljust(chunk * per, b"\0")
            if compress:
                raw = compress(raw)
            a = img.alloc(len(raw))
            img.put(a, raw)
            recs.append((off, a, len(raw)))
        K = 32

        def node(level, entries, last_off):
            b = b"TREE" + struct.pack("<BBHQQ", 1, level, len(entries), h5.UNDEF, h5.UNDEF)
            for off, child, sz in entries:
                b += struct.pack("<IIQQ", sz, 0, off, 0) + struct.pack("<Q", child)
            b += struct.pack("<IIQQ", 0, 0, last_off, 0)
            b += b"\0" * (24 + (2 * K + 1) * 24 + 2 * K * 8 - len(b))
            a = img.alloc(len(b))
            img.put(a, b)
            return a

        if levels == 1:
            tree = node(0, recs, n)
        else:  # leaves of two chunks under one internal node
            leaves = []
            for i in range(0, len(recs), 2):
                part = recs[i:i + 2]
                end = recs[i + 2][0] if i + 2 < len(recs) else n
                leaves.append((part[0][0], node(0, part, end), 0))
            tree = node(1, leaves, n)
        shape = arr.shape[:1]
        msgs = [h5._msg(0x0001, h5._dataspace(shape)), h5._msg(0x0003, h5._datatype_for(arr, ds.inner), flags=1),
                h5._msg(0x0005, struct.pack("<BBBB", 2, 3, 2, 0)),
                h5._msg(0x0008, struct.pack("<BBBQII", 3, 2, 2, tree, chunk, per))]
        if compress:
            msgs.append(h5._msg(0x000B, struct.pack("<BB6x", 1, 1) + struct.pack("<HHHH", 1, 0, 1, 1)
                                + struct.pack("<I4x", 6)))
        if split_header:  # the first two messages in the header, the rest in a continuation block
            rest = b"".join(msgs[2:])
            ca = img.alloc(len(rest))
            img.put(ca, rest)
            body = msgs[:2] + [h5._msg(0x0010, struct.pack("<QQ", ca, len(rest)))]
            hdr = struct.pack("<BBHII4x", 1, 0, len(msgs) + 1, 1, len(b"".join(body))) + b"".join(body)
        else:
            hdr = h5._ohdr(msgs)
        addr = img.alloc(len(hdr))
        img.put(addr, hdr)
        return addr

    return write


def _deflate(level=6, strategy=zlib.Z_DEFAULT_STRATEGY):
    def f(raw):
        c = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
        return c.compress(raw) + c.flush()

    return f


CHUNKED = {
    "plain": dict(chunk=64),
    "stored": dict(chunk=100, compress=_deflate(0)),
    "fixed": dict(chunk=128, compress=_deflate(6, zlib.Z_FIXED)),
    "dynamic": dict(chunk=256, compress=_deflate(9)),
    "two_level": dict(chunk=50, compress=_deflate(6), levels=2),
    "continued_header": dict(chunk=64, compress=_deflate(1), split_header=True),
}


@pytest.mark.parametrize("form", sorted(CHUNKED))
def test_reader_chunked_and_compressed(native, tmp_path, monkeypatch, form):
    rng = np.random.default_rng(11)
    m = random_csr(rng, 700, 650, 6.0, empty_frac=0.1)
    # values that compress (repeats) and values that do not (random)
    m = csr(m.dimensions, np.where(np.arange(m.nnz) % 3 == 0, -1.0, m.values), m.row_start_offsets, m.col_indices)
    y = rng.uniform(-1, 1, 3333)
    p = tmp_path / f"{form}.h5"
    monkeypatch.setattr(h5, "_write_dataset", _chunked_writer(**CHUNKED[form]))
    h5.write_matlab_compatible(p, "A", m)
    h5.write_vector(p, "Y", y)
    monkeypatch.undo()
    _same(h5.read_matlab_compatible(p, "A"), m)  # the Python reader agrees with what was written
    _same(_c_read_csr(native, p, "A"), m)
    assert np.array_equal(_c_read_vector(native, p, "Y"), y)
    # an appending C writer reads the chunked datasets back and rewrites them contiguous
    assert _c_write_vector(native, p, "Z", y[:10]) == N.OK
    _same(h5.read_matlab_compatible(p, "A"), m)
    assert np.array_equal(h5.read_vector(p, "Y"), y)


def test_read_errors(native, tmp_path):
    L = native
    rows, cols, nnz = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint64()

    def dims(path, group="A"):
        return L.dimgpu_h5_csr_dimensions(_b(path), group.encode(), ctypes.byref(rows), ctypes.byref(cols),
                                          ctypes.byref(nnz))

    assert dims(tmp_path / "missing.h5") == N.ERR_IO
    not_h5 = tmp_path / "text.h5"
    not_h5.write_text("not an HDF5 file at all, but long enough to hold a superblock" * 4)
    assert dims(not_h5) == N.ERR_IO
    assert b"not an HDF5 file" in L.dimgpu_last_error_string()
    m = random_csr(np.random.default_rng(3), 200, 200, 5.0)
    p = tmp_path / "m.h5"
    h5.write_matlab_compatible(p, "A", m)
    assert dims(p, "B") == N.ERR_INVALID_ARGUMENT
    assert b"not found" in L.dimgpu_last_error_string()
    assert dims(p, "A/data") == N.ERR_IO  # a dataset, not a group
    # every truncation is an error, never a crash
    raw = p.read_bytes()
    cut = tmp_path / "cut.h5"
    for n in (8, 60, 96, len(raw) // 3, len(raw) // 2, len(raw) - 9):
        cut.write_bytes(raw[:n])
        rc = dims(cut)
        if rc == N.OK:  # the sizes sit early in the file; the arrays are past the cut
            rp = np.zeros(rows.value + 1, np.uint32)
            ci = np.zeros(nnz.value, np.uint32)
            v = np.zeros(nnz.value)
            rc = L.dimgpu_h5_read_matlab_compatible(_b(cut), b"A", rp.ctypes.data, ci.ctypes.data, v.ctypes.data)
        assert rc == N.ERR_IO, n
    # a version-2 superblock (libver "latest") is refused
    v2 = bytearray(raw)
    v2[8] = 2
    (tmp_path / "v2.h5").write_bytes(bytes(v2))
    assert dims(tmp_path / "v2.h5") == N.ERR_IO and b"latest" in L.dimgpu_last_error_string()
    # NULL arguments
    assert L.dimgpu_h5_csr_dimensions(None, b"A", ctypes.byref(rows), ctypes.byref(cols),
                                      ctypes.byref(nnz)) == N.ERR_INVALID_ARGUMENT
    assert L.dimgpu_h5_write_matlab_compatible(_b(p), b"A", 2, 2, 3, None, None, None, 0) == N.ERR_INVALID_ARGUMENT
    assert L.dimgpu_h5_load_csr5(_b(p), b"A", None, None, None) == N.ERR_INVALID_ARGUMENT


def test_wide_indices_are_narrowed_or_refused(native, tmp_path):
    """MATLAB itself stores ir/jc as 64-bit integers; they are read into u32 when they fit."""
    m = random_csr(np.random.default_rng(5), 60, 90, 4.0)
    p = tmp_path / "wide.h5"
    with h5.H5Writer(p) as w:
        w.dataset("A/data", m.values)
        w.dataset("A/ir", m.col_indices.astype(np.uint64))
        w.dataset("A/jc", m.row_start_offsets.astype(np.int64))
        w.attribute("A", "MATLAB_sparse", np.uint64(m.dimensions.cols))
    _same(_c_read_csr(native, p, "A"), m)
    with h5.H5Writer(p) as w:
        w.dataset("A/data", m.values)
        ir = m.col_indices.astype(np.uint64)
        ir[5] = 2**33
        w.dataset("A/ir", ir)
        w.dataset("A/jc", m.row_start_offsets)
        w.attribute("A", "MATLAB_sparse", np.uint32(m.dimensions.cols))
    rp, ci, v = np.zeros(61, np.uint32), np.zeros(m.nnz, np.uint32), np.zeros(m.nnz)
    rc = native.dimgpu_h5_read_matlab_compatible(_b(p), b"A", rp.ctypes.data, ci.ctypes.data, v.ctypes.data)
    assert rc == N.ERR_IO and b"32 bits" in native.dimgpu_last_error_string()


def test_reader_refuses_a_chunk_that_inflates_past_its_size(native, tmp_path, monkeypatch):
    """A deflate stream longer than its chunk (here: the chunk's bytes twice) is an error, not a buffer
    that grows without bound."""
    y = np.arange(300, dtype=np.float64)
    p = tmp_path / "long.h5"
    monkeypatch.setattr(h5, "_write_dataset", _chunked_writer(chunk=64, compress=lambda raw: zlib.compress(raw + raw)))
    h5.write_vector(p, "Y", y)
    monkeypatch.undo()
    n = ctypes.c_uint64()
    assert native.dimgpu_h5_vector_length(_b(p), b"Y", ctypes.byref(n)) == N.OK and n.value == 300
    out = np.zeros(300)
    assert native.dimgpu_h5_read_vector(_b(p), b"Y", out.ctypes.data) == N.ERR_IO
    assert b"expands past" in native.dimgpu_last_error_string()


def test_corrupt_compressed_chunk_is_refused(native, tmp_path, monkeypatch):
    """A byte changed inside a deflate chunk whose stream still decodes (a stored block) is caught by the
    zlib stream's Adler-32 check value, as libhdf5's deflate filter catches it, not returned as data."""
    y = np.random.default_rng(2).uniform(-1, 1, 400)
    p = tmp_path / "stored.h5"
    monkeypatch.setattr(h5, "_write_dataset", _chunked_writer(chunk=100, compress=_deflate(0)))
    h5.write_vector(p, "Y", y)
    monkeypatch.undo()
    assert np.array_equal(_c_read_vector(native, p, "Y"), y)
    raw = bytearray(p.read_bytes())
    at = bytes(raw).find(y[150:152].tobytes())  # chunk 1's stored bytes
    assert at > 0
    raw[at + 3] ^= 0x10
    bad = tmp_path / "bad.h5"
    bad.write_bytes(bytes(raw))
    out = np.zeros(y.size)
    assert native.dimgpu_h5_read_vector(_b(bad), b"Y", out.ctypes.data) == N.ERR_IO
    assert b"Adler-32" in native.dimgpu_last_error_string()


def _patch_u64(raw: bytearray, old: int, new: int, after: int) -> int:
    """Replaces the first little-endian u64 `old` at or after `after`; returns its offset."""
    at = bytes(raw).find(struct.pack("<Q", old), after)
    assert at >= 0
    raw[at:at + 8] = struct.pack("<Q", new)
    return at


def test_oversized_dataspaces_are_refused_before_allocating(native, tmp_path):
    """A dataspace that claims more elements than the group's other datasets, than its stored bytes, or
    than the host's memory is an error found before the dataset's bytes are allocated."""
    m = random_csr(np.random.default_rng(8), 60, 50, 4.0)
    p = tmp_path / "m.h5"
    h5.write_matlab_compatible(p, "A", m)
    h5.write_vector(p, "Y", np.arange(77.0))
    raw = p.read_bytes()
    rows, cols, nnz = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint64()
    rp, ci, v = np.zeros(61, np.uint32), np.zeros(m.nnz, np.uint32), np.zeros(m.nnz)

    # ir (the second dataset of nnz elements) claims 2^39 + nnz elements: refused against data's count
    b = bytearray(raw)
    first = _patch_u64(b, m.nnz, m.nnz, 0)  # data's dataspace stays
    _patch_u64(b, m.nnz, m.nnz + (1 << 39), first + 8)
    f = tmp_path / "ir.h5"
    f.write_bytes(bytes(b))
    rc = native.dimgpu_h5_read_matlab_compatible(_b(f), b"A", rp.ctypes.data, ci.ctypes.data, v.ctypes.data)
    assert rc == N.ERR_IO
    msg = native.dimgpu_last_error_string()
    assert b"expected" in msg or b"fewer bytes" in msg or b"host's memory" in msg, msg

    # the vector claims 2^40 elements: longer than its stored bytes and than the host's memory
    b = bytearray(raw)
    _patch_u64(b, 77, 1 << 40, 0)
    f = tmp_path / "y.h5"
    f.write_bytes(bytes(b))
    n = ctypes.c_uint64()
    assert native.dimgpu_h5_vector_length(_b(f), b"Y", ctypes.byref(n)) == N.ERR_IO
    out = np.zeros(77)
    assert native.dimgpu_h5_read_vector(_b(f), b"Y", out.ctypes.data) == N.ERR_IO

    # a dataspace whose dimensions multiply past 64 bits
    b = bytearray(raw)
    at = _patch_u64(b, 77, 1 << 62, 0)
    f = tmp_path / "ovf.h5"
    f.write_bytes(bytes(b))
    assert native.dimgpu_h5_vector_length(_b(f), b"Y", ctypes.byref(n)) == N.ERR_IO


def test_corrupted_files_return_errors(native, tmp_path, monkeypatch):
    """Truncations and random byte changes of a contiguous and a chunked, compressed file (fixed seed): every
    read returns OK or an error code -- never out of memory, never a crash."""
    import random

    rng = np.random.default_rng(5)
    m = random_csr(rng, 120, 100, 4.0, empty_frac=0.1)
    y = rng.uniform(-1, 1, 300)
    bases = []
    for form in (None, "dynamic"):
        p = tmp_path / f"base_{form}.h5"
        if form:
            monkeypatch.setattr(h5, "_write_dataset", _chunked_writer(**CHUNKED[form]))
        h5.write_matlab_compatible(p, "A", m)
        h5.write_vector(p, "Y", y)
        monkeypatch.undo()
        bases.append(p.read_bytes())
    rnd = random.Random(7)
    cases = []
    for raw in bases:
        cases += [raw[:k] for k in range(0, len(raw), max(1, len(raw) // 60))]
        for _ in range(250):
            b = bytearray(raw)
            lim = min(len(b), 2048) if rnd.random() < 0.7 else len(b)
            for _ in range(rnd.randint(1, 4)):
                i = rnd.randrange(lim)
                b[i] = rnd.randrange(256) if rnd.random() < 0.5 else b[i] ^ (1 << rnd.randrange(8))
            cases.append(bytes(b))
    rows, cols, nnz, n = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint64()
    f = tmp_path / "case.h5"
    allowed = {N.OK, N.ERR_IO, N.ERR_INVALID_ARGUMENT}
    for raw in cases:
        f.write_bytes(raw)
        rc = native.dimgpu_h5_csr_dimensions(_b(f), b"A", ctypes.byref(rows), ctypes.byref(cols), ctypes.byref(nnz))
        assert rc in allowed
        if rc == N.OK:
            assert rows.value < (1 << 20) and nnz.value < (1 << 20)  # the sizes come from intact metadata
            rp = np.zeros(rows.value + 1, np.uint32)
            ci = np.zeros(nnz.value, np.uint32)
            v = np.zeros(nnz.value)
            rc = native.dimgpu_h5_read_matlab_compatible(_b(f), b"A", rp.ctypes.data, ci.ctypes.data, v.ctypes.data)
            assert rc in allowed
        rc = native.dimgpu_h5_vector_length(_b(f), b"Y", ctypes.byref(n))
        assert rc in allowed
        if rc == N.OK and n.value < (1 << 20):
            out = np.zeros(n.value)
            assert native.dimgpu_h5_read_vector(_b(f), b"Y", out.ctypes.data) in allowed
