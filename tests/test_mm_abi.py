"""Matrix Market files through the C ABI (dimgpu_mm_*, dim::io::matrix_market::load_as_csr for C++ callers):
the library's reader against the package's Python reader (io/matrix_market.py, whose csr::from_coo is
pinned to the reference's own from_coo in tests/test_mat.py) on general, symmetric, pattern and integer
files with comments, blank lines, duplicates and unsorted rows, the reference's mm.mtx when the reference
checkout is present, and the reference's error cases.  CPU only."""
import ctypes
import os

import numpy as np
import pytest

import oracle
from diploma_research_gb300 import _native as N
from diploma_research_gb300.io import matrix_market as mm
from diploma_research_gb300.mat import csr, dimensions_t


def _c_load(L, path):
    rows, cols, nnz = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint64()
    rc = L.dimgpu_mm_csr_dimensions(str(path).encode(), ctypes.byref(rows), ctypes.byref(cols), ctypes.byref(nnz))
    if rc != N.OK:
        return rc
    rp = np.zeros(rows.value + 1, np.uint32)
    ci = np.zeros(nnz.value, np.uint32)
    v = np.zeros(nnz.value)
    rc = L.dimgpu_mm_read_csr(str(path).encode(), rp.ctypes.data, ci.ctypes.data, v.ctypes.data)
    assert rc == N.OK, L.dimgpu_last_error_string()
    return csr(dimensions_t(rows.value, cols.value), v, rp, ci)


def _same(a, b):
    assert a.dimensions == b.dimensions
    assert np.array_equal(a.row_start_offsets, b.row_start_offsets)
    assert np.array_equal(a.col_indices, b.col_indices)
    assert np.array_equal(a.values, b.values)


def _write(path, banner, size, entries, comments=("% a comment", "")):
    with open(path, "w") as fh:
        fh.write(banner + "\n")
        for c in comments:
            fh.write(c + "\n")
        fh.write(size + "\n")
        for e in entries:
            fh.write(e + "\n")


def _random_entries(rng, rows, cols, n, pattern=False, integer=False, lower=False):
    r = rng.integers(1, rows + 1, n)
    c = rng.integers(1, cols + 1, n)
    if lower:
        r, c = np.maximum(r, c), np.minimum(r, c)
    v = rng.integers(-9, 10, n) if integer else rng.uniform(-1, 1, n)
    if pattern:
        return [f"{a} {b}" for a, b in zip(r, c)]
    return [f"{a} {b} {x:.17g}" if not integer else f"{a}  {b}\t{x}" for a, b, x in zip(r, c, v)]


CASES = {
    "general": ("%%MatrixMarket matrix coordinate real general", (300, 250, 2000), {}),
    "symmetric": ("%%MatrixMarket matrix coordinate real symmetric", (400, 400, 3000), {"lower": True}),
    "hermitian_real": ("%%MatrixMarket matrix coordinate real hermitian", (50, 50, 200), {"lower": True}),
    "pattern": ("%%MatrixMarket matrix coordinate pattern general", (120, 90, 700), {"pattern": True}),
    "pattern_symmetric": ("%%MatrixMarket Matrix Coordinate Pattern Symmetric", (80, 80, 300),
                          {"pattern": True, "lower": True}),
    "integer": ("%%MatrixMarket matrix coordinate integer general", (60, 70, 500), {"integer": True}),
    "empty": ("%%MatrixMarket matrix coordinate real general", (5, 7, 0), {}),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_reader_matches_python(native, tmp_path, case):
    banner, (rows, cols, n), kw = CASES[case]
    rng = np.random.default_rng(len(case))
    p = tmp_path / f"{case}.mtx"
    # duplicates and unsorted rows come from the random entries; file order decides equal columns
    _write(p, banner, f"{rows} {cols} {n}", _random_entries(rng, rows, cols, n, **kw))
    _same(_c_load(native, p), mm.load_as_csr(str(p)))


def test_reference_mm_mtx(native):
    path = os.path.join(oracle.ref_root(), "tests", "test_files", "mm.mtx")
    if not os.path.isfile(path):
        pytest.skip("needs the reference checkout")
    _same(_c_load(native, path), mm.load_as_csr(path))


def test_round_trip_of_the_writer(native, tmp_path):
    from helpers import random_csr

    m = random_csr(np.random.default_rng(4), 500, 500, 6.0, empty_frac=0.1)
    p = tmp_path / "w.mtx"
    mm.save_coo(str(p), m)
    _same(_c_load(native, p), m)


@pytest.mark.parametrize("text,code,msg", [
    ("%%MatrixMarket matrix array real general\n3 3\n1\n2\n3\n4\n5\n6\n7\n8\n9\n", N.ERR_INVALID_ARGUMENT,
     b"Only coordinate"),
    ("not a matrix market file\n", N.ERR_INVALID_ARGUMENT, b"banner"),
    ("%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 1 1 0\n", N.ERR_INVALID_ARGUMENT, b"complex"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n", N.ERR_INVALID_ARGUMENT, b"scan failed"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n", N.ERR_INVALID_ARGUMENT, b"out of range"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n0 1 1.0\n", N.ERR_INVALID_ARGUMENT, b"out of range"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 x\n", N.ERR_INVALID_ARGUMENT, b"not a number"),
    # a symmetric matrix that is not square: an entry's mirror would lie outside the rows
    ("%%MatrixMarket matrix coordinate real symmetric\n2 3 1\n1 3 1.0\n", N.ERR_INVALID_ARGUMENT, b"square"),
    ("%%MatrixMarket matrix coordinate real hermitian\n50 90 1\n22 58 1.0\n", N.ERR_INVALID_ARGUMENT, b"square"),
    # a size line that would size the arrays far past what the file can hold is refused before allocating
    ("%%MatrixMarket matrix coordinate real general\n3 3 1000000000000\n1 1 1.0\n", N.ERR_INVALID_ARGUMENT,
     b"more entries than the file holds"),
])
def test_errors(native, tmp_path, text, code, msg):
    p = tmp_path / "bad.mtx"
    p.write_text(text)
    assert _c_load(native, p) == code
    assert msg in native.dimgpu_last_error_string()


def test_python_reader_refuses_a_non_square_symmetric_file(tmp_path):
    p = tmp_path / "ns.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real symmetric\n2 3 1\n1 3 1.0\n")
    with pytest.raises(ValueError, match="square"):
        mm.load_as_csr(str(p))


def test_missing_file(native, tmp_path):
    assert _c_load(native, tmp_path / "missing.mtx") == N.ERR_IO


def test_corrupted_files_return_errors(native, tmp_path):
    """Random byte changes and truncations of a symmetric file (fixed seed): every read returns OK or an
    error code, and a successful read has no more entries than the file can hold."""
    import random

    p = tmp_path / "s.mtx"
    _write(p, CASES["symmetric"][0], "400 400 3000",
           _random_entries(np.random.default_rng(1), 400, 400, 3000, lower=True))
    raw = p.read_bytes()
    rnd = random.Random(3)
    f = tmp_path / "case.mtx"
    allowed = {N.OK, N.ERR_INVALID_ARGUMENT, N.ERR_IO}
    cases = [raw[:k] for k in range(0, len(raw), len(raw) // 40)]
    for _ in range(300):
        b = bytearray(raw)
        lim = 200 if rnd.random() < 0.5 else len(b)
        for _ in range(rnd.randint(1, 4)):
            b[rnd.randrange(lim)] = rnd.choice(b"0123456789 \n%.-eE9")
        cases.append(bytes(b))
    for c in cases:
        f.write_bytes(c)
        r = _c_load(native, f)
        if isinstance(r, int):
            assert r in allowed
        else:
            assert r.nnz <= 2 * len(c)
