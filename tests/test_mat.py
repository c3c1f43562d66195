"""COO -> CSR (csr::from_coo, include/dim/mat/storage_formats/csr.h:42-77, with the symmetric expansion
of coo::iterate, coo.h:33-46) against the reference itself: fixtures made by tests/golden/make_golden.py
from the compiled reference, and -- where the reference shim builds -- live comparisons.  CPU only."""
import os

import numpy as np
import pytest

import oracle
from diploma_research_gb300.mat import coo, csr, dimensions_t

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def cases():
    return np.load(os.path.join(GOLDEN, "coo_cases.npz"))


def _ours(g, name):
    c = coo(dimensions_t(int(g[f"{name}_rows"]), int(g[f"{name}_cols"])), g[f"{name}_v"], g[f"{name}_r"],
            g[f"{name}_c"], symmetric=bool(g[f"{name}_symmetric"]))
    return csr.from_coo(c)


@pytest.mark.parametrize("name", ["mm", "symmetric", "dups_short"])
def test_from_coo_bit_for_bit(cases, name):
    """Row offsets, column indices and values equal the reference's bit for bit.  In rows with
    duplicate coordinates the reference's per-row std::sort keeps their visiting order for short rows
    (insertion sort below 16 elements), which the stable sort here reproduces."""
    m = _ours(cases, name)
    assert np.array_equal(m.row_start_offsets, cases[f"{name}_ref_row_ptr"])
    assert np.array_equal(m.col_indices, cases[f"{name}_ref_col"])
    assert np.array_equal(m.values.view(np.uint64), cases[f"{name}_ref_val"].view(np.uint64))


def test_from_coo_duplicates_in_long_rows(cases):
    """Long rows with duplicate coordinates: the reference's std::sort may order the values of equal
    columns either way, so each row is compared as a set of (column, value) pairs; row offsets and the
    column sequence are exact."""
    m = _ours(cases, "dups_long")
    rp = cases["dups_long_ref_row_ptr"]
    assert np.array_equal(m.row_start_offsets, rp)
    assert np.array_equal(m.col_indices, cases["dups_long_ref_col"])
    for r in range(rp.size - 1):
        a, b = int(rp[r]), int(rp[r + 1])
        ours = sorted(zip(m.col_indices[a:b].tolist(), m.values[a:b].tolist()))
        ref = sorted(zip(cases["dups_long_ref_col"][a:b].tolist(), cases["dups_long_ref_val"][a:b].tolist()))
        assert ours == ref


def test_symmetric_expansion_counts(cases):
    """Every off-diagonal entry of a symmetric COO stands for two CSR entries, the diagonal for one."""
    r, c = cases["symmetric_r"], cases["symmetric_c"]
    m = _ours(cases, "symmetric")
    assert m.nnz == 2 * int((r != c).sum()) + int((r == c).sum())


@pytest.mark.skipif(oracle.ref() is None, reason="the reference shim builds only with the reference checkout on x86-64")
def test_from_coo_live_against_reference():
    rng = np.random.default_rng(3)
    for symmetric in (False, True):
        n = 2000
        r = rng.integers(0, n, 12000)
        c = rng.integers(0, n, 12000)
        if symmetric:
            r, c = np.maximum(r, c), np.minimum(r, c)
            key = np.unique(r * n + c)
            r, c = key // n, key % n
        v = rng.standard_normal(r.size)
        rp, ci, vv = oracle.ref_csr_from_coo(n, n, v, r, c, symmetric=symmetric)
        m = csr.from_coo(coo(dimensions_t(n, n), v, r, c, symmetric=symmetric))
        assert np.array_equal(m.row_start_offsets, rp)
        assert np.array_equal(m.col_indices, ci)
        assert np.array_equal(m.values, vv)
