"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run on an x86-64 host with the reference checkout at REF_ROOT (default: a `reference` directory beside
the repository):

    python tests/golden/make_golden.py

* ``mm_mtx.npz`` -- the reference's own conversion fixture, tests/test_files/mm.mtx (17281 x 17281,
  129 non-zeros, mostly empty rows), as CSR arrays built the way csr::from_coo builds them, plus
  what the reference's csr5<double,16,4,uint32_t> makes of it (tile_ptr, raw tile_desc words,
  tile_desc_offset_ptr, tile_desc_offset, transposed vals/col_idx) and its SpMV for x = 1 and for a
  seeded x (oracle rule: zeroed y, fresh calibrator).
* ``ref_cases.npz`` -- small seeded matrices (random lengths, empty rows, long rows, a dense row,
  rows spanning tiles) with the reference's conversion arrays, SpMV outputs and CG iterates.
* ``coo_cases.npz`` -- COO inputs and what the reference's csr::from_coo (csr.h:42-77) makes of them:
  mm.mtx as read, a symmetric COO (lower triangle, expanded by coo::iterate, coo.h:33-46), short rows
  with duplicate coordinates, and long unsorted rows with duplicates.

The reference runs through oracle/ref_shim.cpp compiled against the reference headers
(``make -C oracle ref``).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from diploma_research_gb300.io.matrix_market import load_as_coo, load_as_csr  # noqa: E402

REF_ROOT = oracle.ref_root()


def ref_arrays(rows, cols, rp, ci, v):
    R = oracle.RefCSR5(rows, cols, rp, ci, v)
    e = R.export()
    return R, e


def random_case(rng, rows, cols, density, empty_frac=0.0, long_rows=0, dense_row=False):
    lens = rng.poisson(density, rows)
    if empty_frac:
        lens[rng.random(rows) < empty_frac] = 0
    for _ in range(long_rows):
        lens[rng.integers(rows)] = rng.integers(64, 700)
    if dense_row:
        lens[rng.integers(rows)] = cols
    lens = np.minimum(lens, cols)
    rp = np.zeros(rows + 1, np.int64)
    rp[1:] = np.cumsum(lens)
    ci = np.concatenate([np.sort(rng.choice(cols, l, replace=False)) for l in lens]) if rp[-1] else np.zeros(0)
    v = rng.standard_normal(int(rp[-1]))
    return rp.astype(np.uint32), ci.astype(np.uint32), v


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "coo":
        if oracle.ref() is None:
            raise SystemExit("the reference shim cannot be built on this host")
        return coo_cases()
    if oracle.ref() is None:
        raise SystemExit("the reference shim cannot be built on this host")
    # ---- mm.mtx ----
    m = load_as_csr(os.path.join(REF_ROOT, "tests", "test_files", "mm.mtx"))
    rows, cols = m.dimensions.rows, m.dimensions.cols
    R, e = ref_arrays(rows, cols, m.row_start_offsets, m.col_indices, m.values)
    x1 = np.ones(cols)
    xr = np.random.default_rng(7).uniform(-1, 1, cols)
    np.savez_compressed(
        os.path.join(HERE, "mm_mtx.npz"), rows=rows, cols=cols, row_ptr=m.row_start_offsets, col_idx=m.col_indices,
        vals=m.values, ref_tile_count=e["tile_count"], ref_tail=e["tail_partition_start"], ref_tile_ptr=e["tile_ptr"],
        ref_tile_desc=e["tile_desc"], ref_tdo_ptr=e["tile_desc_offset_ptr"], ref_tdo=e["tile_desc_offset"],
        ref_vals=e["vals"], ref_col_idx=e["col_idx"], x_rand=xr, ref_y_ones=R.spmv(x1), ref_y_rand=R.spmv(xr),
        ref_threads=oracle.RefCSR5.max_threads())

    # ---- seeded small cases ----
    rng = np.random.default_rng(20261203)
    cases = []
    specs = [
        dict(rows=300, cols=300, density=7.0),
        dict(rows=1000, cols=800, density=3.0, empty_frac=0.3),
        dict(rows=700, cols=700, density=12.0, long_rows=3),
        dict(rows=200, cols=5000, density=1.0, dense_row=True),
        dict(rows=2500, cols=2500, density=0.5, empty_frac=0.5),
        dict(rows=64, cols=64, density=40.0),
        dict(rows=129, cols=97, density=2.0, long_rows=1),
    ]
    out = {}
    for k, sp in enumerate(specs):
        rp, ci, v = random_case(rng, **sp)
        if len(v) < 64:
            continue
        R, e = ref_arrays(sp["rows"], sp["cols"], rp, ci, v)
        x = rng.uniform(-1, 1, sp["cols"])
        y = R.spmv(x)
        pre = f"c{k}_"
        out.update({pre + "rows": sp["rows"], pre + "cols": sp["cols"], pre + "row_ptr": rp, pre + "col_idx": ci,
                    pre + "vals": v, pre + "tile_ptr": e["tile_ptr"], pre + "tile_desc": e["tile_desc"],
                    pre + "tdo_ptr": e["tile_desc_offset_ptr"], pre + "tdo": e["tile_desc_offset"],
                    pre + "csr5_vals": e["vals"], pre + "csr5_col": e["col_idx"], pre + "tail": e["tail_partition_start"],
                    pre + "x": x, pre + "y": y})
        cases.append(k)
    # an SPD case with the reference CG (2-D Laplacian 24x24)
    from diploma_research_gb300.generators import laplacian_2d_5pt, rhs

    L = laplacian_2d_5pt(24)
    xs, b = rhs(L, 0)
    R = oracle.RefCSR5(L.dimensions.rows, L.dimensions.cols, L.row_start_offsets, L.col_indices, L.values)
    xcg, it, rel = R.cg(b, tol=1e-10)
    out.update(dict(cg_row_ptr=L.row_start_offsets, cg_col_idx=L.col_indices, cg_vals=L.values, cg_b=b, cg_x=xcg,
                    cg_iters=it, cg_rel=rel))
    out["cases"] = np.array(cases)
    out["ref_threads"] = oracle.RefCSR5.max_threads()
    np.savez_compressed(os.path.join(HERE, "ref_cases.npz"), **out)
    print("wrote mm_mtx.npz and ref_cases.npz; cases", cases, "cg iters", it)
    coo_cases()


def coo_cases():
    """COO -> CSR through the reference's csr::from_coo, on four inputs (see the module docstring)."""
    rng = np.random.default_rng(20261204)
    cases = {}
    c = load_as_coo(os.path.join(REF_ROOT, "tests", "test_files", "mm.mtx"))
    cases["mm"] = (c.dimensions.rows, c.dimensions.cols, c.values, c.row_indices, c.col_indices, False)
    # symmetric: lower triangle with the diagonal, shuffled entry order
    n = 400
    rows = rng.integers(0, n, 3000)
    cols = rng.integers(0, n, 3000)
    lo = np.minimum(rows, cols), np.maximum(rows, cols)
    key = np.unique(lo[1] * n + lo[0])
    r, cc = key // n, key % n
    perm = rng.permutation(key.size)
    cases["symmetric"] = (n, n, rng.standard_normal(key.size)[perm], r[perm], cc[perm], True)
    # short rows (< 16 elements) with duplicate coordinates
    n = 300
    r = rng.integers(0, n, 1800)
    cc = rng.integers(0, 40, 1800)
    cases["dups_short"] = (n, 40, rng.standard_normal(r.size), r, cc, False)
    # long rows with duplicates, entries in random order
    n = 30
    r = rng.integers(0, n, 4000)
    cc = rng.integers(0, 300, 4000)
    cases["dups_long"] = (n, 300, rng.standard_normal(r.size), r, cc, False)
    out = {}
    for name, (nr, nc, v, r, cc, sym) in cases.items():
        rp, ci, vv = oracle.ref_csr_from_coo(nr, nc, v, r, cc, symmetric=sym)
        out.update({f"{name}_rows": nr, f"{name}_cols": nc, f"{name}_v": np.asarray(v, np.float64),
                    f"{name}_r": np.asarray(r, np.uint32), f"{name}_c": np.asarray(cc, np.uint32),
                    f"{name}_symmetric": sym, f"{name}_ref_row_ptr": rp, f"{name}_ref_col": ci,
                    f"{name}_ref_val": vv})
    out["cases"] = np.array(list(cases))
    np.savez_compressed(os.path.join(HERE, "coo_cases.npz"), **out)
    print("wrote coo_cases.npz:", list(cases))


if __name__ == "__main__":
    main()
