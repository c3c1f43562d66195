"""The oracle (oracle/csr5_oracle.c) pinned against the reference: its own known-answer tests, golden
fixtures generated from the reference, and -- where the reference shim builds -- live bit-for-bit
comparison.  CPU only."""
import os

import numpy as np
import pytest

import oracle
from helpers import csr_from_lengths, random_csr

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def mm():
    return np.load(os.path.join(GOLDEN, "mm_mtx.npz"))


def _oracle_of(rows, cols, rp, ci, v, sigma=16, omega=4):
    return oracle.OracleCSR5(rows, cols, rp, ci, v, sigma, omega)


def test_conversion_known_answers_mm_mtx(mm):
    """tests/test_csr5.cpp:26-57 ("Test conversion from CSR"), restated on the oracle."""
    o = _oracle_of(int(mm["rows"]), int(mm["cols"]), mm["row_ptr"], mm["col_idx"], mm["vals"])
    assert o.rows == 17281 and o.cols == 17281 and o.nnz == 129
    assert not np.array_equal(o.vals, mm["vals"])  # transposed (REQUIRE_FALSE(std::equal(...)))
    assert o.tile_count == 2
    assert o.tail_partition_start == 154
    y, s, f = o.desc_fields()
    expect0 = [(0, 0, 0b1000_0100_0010_0001), (4, 0, 0b1000_1000_1000_1000), (8, 0, 0b1010_1000_1000_1000),
               (13, 0, 0b1010_1010_1010_1010)]
    expect1 = [(0, 3, 0b0000_0000_0000_1110), (4, 0, 0), (4, 0, 0), (4, 0, 0)]
    for c in range(4):
        assert (y[c], s[c], f[c]) == expect0[c]
        assert (y[4 + c], s[4 + c], f[4 + c]) == expect1[c]
    assert o.tile_desc_offset_ptr.size == o.tile_count + 1
    assert o.tile_desc_offset.size == y[4 + 3] + 1
    assert (o.tile_ptr[1] & 0x7FFFFFFF) != 0
    assert o.tile_desc_offset_ptr[1] == 0
    assert o.tile_desc_offset[3] == 154 - (o.tile_ptr[1] & 0x7FFFFFFF)


def test_num_bits_set_semantics():
    """tests/test_csr5.cpp:15-24: column 0 counts an implicit first bit, once."""
    pc = lambda flag, first: bin(flag | int(first)).count("1")
    assert pc(0b1000_1000_1000_1000, False) == 4
    assert pc(0b1000_1000_1000_1000, True) == 5
    assert pc(0b1000_1000_1000_1001, True) == 5


def test_descriptor_decode_known_answers():
    """tests/test_csr5.cpp:68-92 (descriptor vectorization): field extraction and per-row bits, on the
    packed words of the same descriptor."""
    yb, sb = 7, 3  # bit_width(64), bit_width(4)
    cols = [(0, 3, 0b1000_0100_0010_0001), (4, 2, 0b1000_1000_1000_1000), (8, 1, 0b1010_1000_1000_1000),
            (13, 0, 0b1010_1010_1010_1010)]
    words = np.array([y | (s << yb) | (f << (yb + sb)) for y, s, f in cols], np.uint64)
    y = words & np.uint64(0x7F)
    s = (words >> np.uint64(yb)) & np.uint64(7)
    f = (words >> np.uint64(yb + sb)) & np.uint64(0xFFFF)
    assert list(y) == [0, 4, 8, 13] and list(s) == [3, 2, 1, 0]
    assert list(f) == [c[2] for c in cols]
    local_bit = lambda which: [int((int(v) >> which) & 1) for v in f]
    assert local_bit(0) == [1, 0, 0, 0]
    assert local_bit(1) == [0, 0, 0, 1]
    assert local_bit(2) == [0, 0, 0, 0]
    assert local_bit(3) == [0, 1, 1, 1]


def test_raw_word_layout_mm_mtx(mm):
    """The packed words equal the reference's raw bit-field words (GCC layout)."""
    o = _oracle_of(int(mm["rows"]), int(mm["cols"]), mm["row_ptr"], mm["col_idx"], mm["vals"])
    assert [hex(int(w)) for w in o.tile_desc[:4]] == ["0x2108400", "0x2222004", "0x2a22008", "0x2aaa80d"]
    assert np.array_equal(o.tile_desc.astype(np.uint32), mm["ref_tile_desc"])


def test_oracle_matches_reference_fixture_mm(mm):
    o = _oracle_of(int(mm["rows"]), int(mm["cols"]), mm["row_ptr"], mm["col_idx"], mm["vals"])
    assert o.tile_count == int(mm["ref_tile_count"])
    assert o.tail_partition_start == int(mm["ref_tail"])
    assert np.array_equal(o.tile_ptr, mm["ref_tile_ptr"])
    assert np.array_equal(o.tile_desc.astype(np.uint32), mm["ref_tile_desc"])
    assert np.array_equal(o.tile_desc_offset_ptr, mm["ref_tdo_ptr"])
    assert np.array_equal(o.tile_desc_offset, mm["ref_tdo"])
    assert np.array_equal(o.vals, mm["ref_vals"])
    assert np.array_equal(o.col_idx, mm["ref_col_idx"])
    nt = int(mm["ref_threads"])
    assert np.array_equal(o.spmv(np.ones(o.cols), nthreads=nt), mm["ref_y_ones"])
    assert np.array_equal(o.spmv(mm["x_rand"], nthreads=nt), mm["ref_y_rand"])


def test_oracle_matches_reference_fixture_cases():
    g = np.load(os.path.join(GOLDEN, "ref_cases.npz"))
    nt = int(g["ref_threads"])
    for k in g["cases"]:
        p = f"c{k}_"
        o = _oracle_of(int(g[p + "rows"]), int(g[p + "cols"]), g[p + "row_ptr"], g[p + "col_idx"], g[p + "vals"])
        assert np.array_equal(o.tile_ptr, g[p + "tile_ptr"]), k
        assert np.array_equal(o.tile_desc.astype(np.uint32), g[p + "tile_desc"]), k
        assert np.array_equal(o.tile_desc_offset_ptr, g[p + "tdo_ptr"]), k
        assert np.array_equal(o.tile_desc_offset, g[p + "tdo"]), k
        assert np.array_equal(o.vals, g[p + "csr5_vals"]), k
        assert np.array_equal(o.col_idx, g[p + "csr5_col"]), k
        assert o.tail_partition_start == int(g[p + "tail"]), k
        assert np.array_equal(o.spmv(g[p + "x"], nthreads=nt), g[p + "y"]), k


def test_oracle_cg_matches_reference_fixture():
    g = np.load(os.path.join(GOLDEN, "ref_cases.npz"))
    rp = g["cg_row_ptr"]
    n = rp.size - 1
    o = _oracle_of(n, n, rp, g["cg_col_idx"], g["cg_vals"])
    x, it, rel = o.cg(g["cg_b"], tol=1e-10, nthreads=int(g["ref_threads"]))
    assert it == int(g["cg_iters"])
    assert rel <= 1e-10
    np.testing.assert_allclose(x, g["cg_x"], rtol=0, atol=1e-12)


@pytest.mark.skipif(oracle.ref() is None, reason="reference shim not buildable on this host")
@pytest.mark.parametrize("seed", range(12))
def test_oracle_bitexact_vs_live_reference(seed):
    rng = np.random.default_rng(1000 + seed)
    rows, cols = int(rng.integers(50, 4000)), int(rng.integers(50, 4000))
    m = random_csr(rng, rows, cols, float(rng.uniform(0.3, 25)), empty_frac=float(rng.choice([0, 0.2, 0.6])),
                   long_rows=int(rng.integers(0, 4)))
    if m.nnz < 64:
        pytest.skip("the reference cannot run SpMV without a full tile")
    o = _oracle_of(rows, cols, m.row_start_offsets, m.col_indices, m.values)
    R = oracle.RefCSR5(rows, cols, m.row_start_offsets, m.col_indices, m.values)
    e = R.export()
    assert np.array_equal(o.tile_ptr, e["tile_ptr"])
    assert np.array_equal(o.tile_desc.astype(np.uint32), e["tile_desc"])
    assert np.array_equal(o.tile_desc_offset_ptr, e["tile_desc_offset_ptr"])
    assert np.array_equal(o.tile_desc_offset, e["tile_desc_offset"])
    assert np.array_equal(o.vals, e["vals"]) and np.array_equal(o.col_idx, e["col_idx"])
    x = rng.uniform(-1, 1, cols)
    assert np.array_equal(o.spmv(x, nthreads=oracle.RefCSR5.max_threads()), R.spmv(x))


STRUCTURED = {
    # nnz an exact multiple of the 64-element tile: no CSR tail
    "no_tail": [16] * 40,
    # rows of exactly sigma elements, each row one tile column
    "sigma_rows": [16] * 37 + [5],
    # rows of exactly one tile, and a row of one tile plus one element
    "tile_rows": [64] * 9 + [65, 63, 1],
    # one row spanning every thread's chunk, between short rows
    "row_across_threads": [3, 2] + [4000] + [1, 7, 2],
    # empty rows at the edges of tiles and after the last tile (the tail holds only empty rows)
    "empty_at_edges": ([0, 32, 0, 32, 0] * 10) + [0, 0, 0],
    # a lone tail row after full tiles
    "lone_tail_row": [64] * 6 + [3],
    # every row empty but one dense row at the very end
    "dense_last_row": [0] * 300 + [700],
}


@pytest.mark.skipif(oracle.ref() is None, reason="reference shim not buildable on this host")
@pytest.mark.parametrize("case", sorted(STRUCTURED))
def test_oracle_bitexact_vs_live_reference_structured(case):
    """Shapes at the format's boundaries, against the reference's own compiled conversion and SpMV."""
    rng = np.random.default_rng(len(case))
    lens = STRUCTURED[case]
    m = csr_from_lengths(lens, max(5000, max(lens) + 1), rng)
    rows, cols = m.dimensions.rows, m.dimensions.cols
    o = _oracle_of(rows, cols, m.row_start_offsets, m.col_indices, m.values)
    R = oracle.RefCSR5(rows, cols, m.row_start_offsets, m.col_indices, m.values)
    e = R.export()
    assert np.array_equal(o.tile_ptr, e["tile_ptr"])
    assert np.array_equal(o.tile_desc.astype(np.uint32), e["tile_desc"])
    assert np.array_equal(o.tile_desc_offset_ptr, e["tile_desc_offset_ptr"])
    assert np.array_equal(o.tile_desc_offset, e["tile_desc_offset"])
    assert np.array_equal(o.vals, e["vals"]) and np.array_equal(o.col_idx, e["col_idx"])
    x = rng.uniform(-1, 1, cols)
    assert np.array_equal(o.spmv(x, nthreads=oracle.RefCSR5.max_threads()), R.spmv(x))


@pytest.mark.skipif(oracle.ref() is None, reason="reference shim not buildable on this host")
def test_oracle_cg_vs_live_reference():
    from diploma_research_gb300.generators import laplacian_2d_5pt, rhs

    L = laplacian_2d_5pt(40)
    xs, b = rhs(L, 0)
    n = L.dimensions.rows
    o = _oracle_of(n, n, L.row_start_offsets, L.col_indices, L.values)
    R = oracle.RefCSR5(n, n, L.row_start_offsets, L.col_indices, L.values)
    xo, ito, relo = o.cg(b, tol=1e-10)
    xr, itr, relr = R.cg(b, tol=1e-10)
    assert abs(ito - itr) <= 1
    np.testing.assert_allclose(xo, xr, rtol=0, atol=1e-9)


def test_oracle_edge_cases():
    """Edge cases the device code must also handle: no full tile, nnz = 0, empty rows everywhere,
    leading/trailing empty rows, one dense row, rows spanning many tiles."""
    rng = np.random.default_rng(5)
    cases = [
        csr_from_lengths([3, 0, 5, 1], 10, rng),                 # nnz < one tile
        csr_from_lengths([0, 0, 0], 4, rng),                     # nnz = 0
        csr_from_lengths([0] * 50 + [64] + [0] * 50, 100, rng),  # one full row between empty rows
        csr_from_lengths([500], 600, rng),                       # one long row
        csr_from_lengths([0, 70, 0, 0, 200, 1, 0], 300, rng),
    ]
    for m in cases:
        for omega in (4, 32):
            o = _oracle_of(m.dimensions.rows, m.dimensions.cols, m.row_start_offsets, m.col_indices, m.values,
                           omega=omega)
            x = rng.uniform(-1, 1, m.dimensions.cols)
            y = o.spmv(x, nthreads=3)
            y_ref = oracle.csr_spmv(m.dimensions.rows, m.row_start_offsets, m.col_indices, m.values, x)
            ax = oracle.abs_spmv(m.dimensions.rows, m.row_start_offsets, m.col_indices, m.values, x)
            assert np.all(np.abs(y - y_ref) <= 1e-13 * ax + 1e-300)
