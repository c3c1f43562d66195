"""The HDF5 subset (the reference's matrix and vector groups) and the CLI's compare-results, on CPU."""
import os
import struct

import numpy as np
import pytest

import oracle
from diploma_research_gb300 import cli
from diploma_research_gb300.io import h5
from diploma_research_gb300.io import matrix_market as mm
from diploma_research_gb300.mat import csr, dimensions_t
from helpers import random_csr

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _mm_fixture():
    """The reference's tests/test_files/mm.mtx matrix (17281 x 17281, 129 entries), from the golden CSR."""
    g = np.load(os.path.join(GOLDEN, "mm_mtx.npz"))
    return csr(dimensions_t(int(g["rows"]), int(g["cols"])), g["vals"], g["row_ptr"], g["col_idx"])


def test_signature_and_superblock(tmp_path):
    p = tmp_path / "v.h5"
    h5.write_vector(p, "Y", np.arange(3.0))
    b = p.read_bytes()
    assert b[:8] == b"\x89HDF\r\n\x1a\n" and h5.is_hdf5(p) and not h5.is_hdf5(__file__)
    assert b[8] == 0 and b[13] == 8 and b[14] == 8               # superblock v0, 8-byte offsets/lengths
    assert struct.unpack_from("<HH", b, 16) == (4, 16)            # group leaf / internal node K
    assert struct.unpack_from("<Q", b, 40)[0] == len(b)           # end-of-file address
    oh, cache = struct.unpack_from("<QI", b, 64)
    btree, heap = struct.unpack_from("<QQ", b, 80)
    assert cache == 1 and b[oh] == 1                              # root: symbol-table cache, v1 header
    assert b[btree:btree + 4] == b"TREE" and b[heap:heap + 4] == b"HEAP"
    snod = struct.unpack_from("<Q", b, btree + 32)[0]
    assert b[snod:snod + 4] == b"SNOD"


def test_matlab_compatible_round_trip(tmp_path):
    m = _mm_fixture()
    p = tmp_path / "m.h5"
    h5.write_matlab_compatible(p, "A", m)
    r = h5.read_matlab_compatible(p, "A")
    assert r.dimensions == m.dimensions
    assert np.array_equal(r.values, m.values)
    assert np.array_equal(r.row_start_offsets, m.row_start_offsets)
    assert np.array_equal(r.col_indices, m.col_indices)
    rd = h5.H5Reader(p)
    assert rd.members("A") == ["data", "ir", "jc"]
    assert rd.dataset("A/ir").dtype == np.uint32 and rd.dataset("A/data").dtype == np.float64
    assert rd.attributes("A")["MATLAB_sparse"] == m.dimensions.cols


def test_csr5_group_round_trip(tmp_path):
    rng = np.random.default_rng(4)
    m = random_csr(rng, 900, 700, 7.0, empty_frac=0.1, long_rows=2, long_len=(100, 600))
    o = oracle.OracleCSR5(900, 700, m.row_start_offsets, m.col_indices, m.values, 16, 4)
    assert int(o.tile_desc.max(initial=0)) < 2**32  # (16, 4) column words fit the reference's u32 storage
    arrays = type("A", (), {})()
    arrays.vals, arrays.col_idx, arrays.row_ptr = o.vals, o.col_idx, m.row_start_offsets
    arrays.tile_ptr, arrays.tile_desc = o.tile_ptr, o.tile_desc.astype(np.uint32)
    arrays.tile_desc_offset_ptr, arrays.tile_desc_offset = o.tile_desc_offset_ptr, o.tile_desc_offset
    p = tmp_path / "c.h5"
    h5.store_csr5(p, "A", arrays, 700)
    a = h5.load_csr5_arrays(p, "A")
    assert a.rows == 900 and a.cols == 700 and a.tile_count == len(o.tile_ptr) - 1
    for name in ("vals", "col_idx", "row_ptr", "tile_ptr", "tile_desc", "tile_desc_offset_ptr", "tile_desc_offset"):
        assert np.array_equal(getattr(a, name), np.asarray(getattr(arrays, name)).reshape(-1)), name
    # the stored tile order maps back to the CSR arrays
    back = cli.csr_from_csr5_arrays(a)
    assert np.array_equal(back.values, m.values) and np.array_equal(back.col_indices, m.col_indices)


def test_many_members_append_and_overwrite(tmp_path):
    p = tmp_path / "v.h5"
    for i in range(20):  # more than one symbol table node
        h5.write_vector(p, f"v{i:02d}", np.full(i + 1, float(i)))
    r = h5.H5Reader(p)
    assert r.members("/") == [f"v{i:02d}" for i in range(20)]
    assert np.array_equal(r.dataset("v13"), np.full(14, 13.0))
    with pytest.raises(FileExistsError):
        h5.write_vector(p, "v03", np.zeros(2))
    h5.write_vector(p, "v03", np.zeros(2), overwrite=True)
    assert np.array_equal(h5.read_vector(p, "v03"), np.zeros(2))
    h5.write_vector(p, "grp/Y", np.ones(4))
    assert np.array_equal(h5.read_vector(p, "/grp/Y"), np.ones(4))


def test_empty_and_scalar_shapes(tmp_path):
    p = tmp_path / "e.h5"
    with h5.H5Writer(p) as w:
        w.dataset("A/empty", np.zeros(0, np.uint32))
        w.attribute("A", "column_count", np.uint32(7))
    r = h5.H5Reader(p)
    assert r.dataset("A/empty").size == 0 and r.attributes("A")["column_count"] == 7


def test_compare_results_rule(tmp_path):
    p = tmp_path / "r.h5"
    y = np.linspace(1, 2, 50)
    h5.write_vector(p, "Y", y)
    h5.write_vector(p, "Z", y * 1.005)  # within 1 %
    h5.write_vector(p, "W", y * 1.02)   # 2 % off
    assert cli.main(["compare-results", str(p), "--rhs-dataset", "Z"]) == 0
    assert cli.main(["compare-results", str(p), "--rhs-dataset", "W"]) == 1
    q = tmp_path / "r2.h5"
    h5.write_vector(q, "Y", y)
    assert cli.main(["compare-results", str(p), "--input-file-2", str(q)]) == 0


def test_store_matrix_csr_from_mtx(tmp_path):
    src = tmp_path / "mm.mtx"
    ref = _mm_fixture()
    mm.save_coo(src, ref)
    assert cli.main(["store-matrix", str(src)]) == 0
    out = tmp_path / "mm.csr.h5"
    m = h5.read_matlab_compatible(out, "A")
    assert np.array_equal(m.values, ref.values) and m.dimensions == ref.dimensions
    # an HDF5 input is read through its MATLAB-compatible group
    assert cli.main(["store-matrix", str(out), "--output", str(tmp_path / "again.h5"), "--group-name", "B"]) == 0
    assert np.array_equal(h5.read_matlab_compatible(tmp_path / "again.h5", "B").col_indices, ref.col_indices)


@pytest.mark.parametrize("deflate", [False, True])
def test_reader_chunked_datasets(tmp_path, monkeypatch, deflate):
    """The reader's chunked path (v1 B-tree chunk index, deflate filter), as libhdf5 writes datasets
    when chunk_size / compression_level are set (libs/dim/io/h5.cpp:34-43); the file is built here."""
    import zlib

    data = np.arange(1000, dtype=np.float64) * 0.5
    chunk = 128

    def chunked_dataset(img, ds):
        n = ds.data.size
        recs = []
        for off in range(0, n, chunk):
            raw = ds.data[off:off + chunk].tobytes().ljust(chunk * 8, b"\0")
            if deflate:
                raw = zlib.compress(raw, 6)
            a = img.alloc(len(raw))
            img.put(a, raw)
            recs.append((off, a, len(raw)))
        K = 32
        node = b"TREE" + struct.pack("<BBHQQ", 1, 0, len(recs), h5.UNDEF, h5.UNDEF)
        for off, a, sz in recs:
            node += struct.pack("<IIQQ", sz, 0, off, 0) + struct.pack("<Q", a)
        node += struct.pack("<IIQQ", 0, 0, n, 0)
        node += b"\0" * (24 + (2 * K + 1) * 24 + 2 * K * 8 - len(node))
        tree = img.alloc(len(node))
        img.put(tree, node)
        msgs = [h5._msg(0x0001, h5._dataspace((n,))), h5._msg(0x0003, h5._datatype_for(ds.data), flags=1),
                h5._msg(0x0005, struct.pack("<BBBB", 2, 3, 2, 0)),
                h5._msg(0x0008, struct.pack("<BBBQII", 3, 2, 2, tree, chunk, 8))]
        if deflate:
            msgs.append(h5._msg(0x000B, struct.pack("<BB6x", 1, 1) + struct.pack("<HHHH", 1, 0, 1, 1)
                                + struct.pack("<I4x", 6)))
        hdr = h5._ohdr(msgs)
        addr = img.alloc(len(hdr))
        img.put(addr, hdr)
        return addr

    monkeypatch.setattr(h5, "_write_dataset", chunked_dataset)
    p = tmp_path / "chunked.h5"
    h5.write_vector(p, "Y", data, append=False)
    monkeypatch.undo()
    assert np.array_equal(h5.read_vector(p, "Y"), data)


def test_reader_refuses_oversized_dataspaces(tmp_path):
    """A dataspace claiming more elements than its contiguous storage holds, or than the host's memory,
    is a format error before anything is allocated; dimensions whose product passes 64 bits as well."""
    p = tmp_path / "y.h5"
    h5.write_vector(p, "Y", np.arange(77.0))
    raw = p.read_bytes()
    for claim in (78, 1 << 40, 1 << 63):
        b = bytearray(raw)
        at = bytes(b).find(struct.pack("<Q", 77))
        b[at:at + 8] = struct.pack("<Q", claim)
        bad = tmp_path / f"bad_{claim}.h5"
        bad.write_bytes(bytes(b))
        with pytest.raises(h5.H5FormatError):
            h5.read_vector(bad, "Y")
