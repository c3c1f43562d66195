"""Shared helpers of the test-suite: matrix builders and tolerance checks."""
import numpy as np

from diploma_research_gb300.mat import csr, dimensions_t


def random_csr(rng, rows, cols, density, empty_frac=0.0, long_rows=0, dense_row=False, long_len=(64, 700)):
    lens = rng.poisson(density, rows)
    if empty_frac:
        lens[rng.random(rows) < empty_frac] = 0
    for _ in range(long_rows):
        lens[rng.integers(rows)] = rng.integers(*long_len)
    if dense_row:
        lens[rng.integers(rows)] = cols
    lens = np.minimum(lens, cols)
    rp = np.zeros(rows + 1, np.int64)
    rp[1:] = np.cumsum(lens)
    ci = (np.concatenate([np.sort(rng.choice(cols, l, replace=False)) for l in lens]) if rp[-1]
          else np.zeros(0, np.int64))
    v = rng.standard_normal(int(rp[-1]))
    return csr(dimensions_t(rows, cols), v, rp.astype(np.uint32), ci.astype(np.uint32))


def csr_from_lengths(lens, cols, rng):
    lens = np.asarray(lens, np.int64)
    rp = np.zeros(len(lens) + 1, np.int64)
    rp[1:] = np.cumsum(lens)
    ci = (np.concatenate([np.sort(rng.choice(cols, l, replace=False)) for l in lens]) if rp[-1]
          else np.zeros(0, np.int64))
    v = rng.standard_normal(int(rp[-1]))
    return csr(dimensions_t(len(lens), cols), v, rp.astype(np.uint32), ci.astype(np.uint32))


# Componentwise SpMV tolerance: |y - y_ref|_i <= RTOL * (|A| |x|)_i (+ a tiny absolute floor for
# rows whose |A||x| is 0).  FP64 parity bar: 1e-12.
SPMV_RTOL_F64 = 1e-12
SPMV_RTOL_F32 = 2e-6


def assert_spmv_close(y, y_ref, absax, rtol):
    y = np.asarray(y)
    y_ref = np.asarray(y_ref)
    err = np.abs(y - y_ref)
    bound = rtol * absax + 1e-300
    bad = np.flatnonzero(err > bound)
    assert bad.size == 0, (f"{bad.size} rows exceed {rtol} * (|A||x|): first {bad[:5]}, "
                           f"err {err[bad[:5]]}, bound {bound[bad[:5]]}")


def record(case: str, **values):
    """Appends one JSON line {case, values} to the file named by DIMGPU_TEST_RECORD (when set), so that a
    run can keep the measured errors and iteration counts of the full-size parity cases."""
    import json
    import os

    path = os.environ.get("DIMGPU_TEST_RECORD")
    if path:
        with open(path, "a") as fh:
            fh.write(json.dumps({"case": case, **values}) + "\n")
