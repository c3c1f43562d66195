"""Matrix Market coordinate reader -> COO -> CSR.

Mirrors ``dim::io::matrix_market`` (include/dim/io/matrix_market.h:25-83):

* only ``coordinate`` matrices are accepted (``std::invalid_argument`` in the reference,
  ``ValueError`` here, matrix_market.h:59-60);
* ``pattern`` matrices get value 1.0 (matrix_market.h:33-34);
* indices are made 0-based (matrix_market.h:44-46);
* ``symmetric`` / ``hermitian`` matrices are expanded when converting to CSR, the mirrored entry
  being emitted right after its source entry (coo.h:33-46);
* ``load_as_csr`` = ``load_as_coo`` + ``csr.from_coo`` (matrix_market.h:68-73).
"""
from __future__ import annotations

import numpy as np

from ..mat import coo, csr, dimensions_t


def _read_banner(fh):
    line = fh.readline()
    if not line.startswith("%%MatrixMarket"):
        raise ValueError("not a Matrix Market file (missing %%MatrixMarket banner)")
    parts = line.split()
    if len(parts) < 5:
        raise ValueError("malformed Matrix Market banner")
    obj, fmt, field, symm = (p.lower() for p in parts[1:5])
    if obj != "matrix":
        raise ValueError(f"unsupported Matrix Market object {obj!r}")
    return fmt, field, symm


def load_as_coo(path) -> coo:
    with open(path, "r") as fh:
        fmt, field, symm = _read_banner(fh)
        if fmt != "coordinate":
            raise ValueError("Only coordinate matrix loading is implemented.")
        if field == "complex":
            raise ValueError("complex Matrix Market matrices are not supported")
        line = fh.readline()
        while line and (line.startswith("%") or not line.strip()):
            line = fh.readline()
        rows, cols, nnz = (int(t) for t in line.split()[:3])
        if symm in ("symmetric", "hermitian") and rows != cols:  # the mirror (col, row) must be a row
            raise ValueError("a symmetric or Hermitian matrix must be square")
        pattern = field == "pattern"
        ncol = 2 if pattern else 3
        data = np.loadtxt(fh, dtype=np.float64, ndmin=2, max_rows=nnz) if nnz else np.zeros((0, ncol))
    if data.shape[0] != nnz or (nnz and data.shape[1] < ncol):
        raise ValueError("scan failed")
    r = data[:, 0].astype(np.int64) - 1
    c = data[:, 1].astype(np.int64) - 1
    v = np.ones(nnz) if pattern else data[:, 2].astype(np.float64)
    if nnz and (r.min() < 0 or c.min() < 0 or r.max() >= rows or c.max() >= cols):
        raise ValueError("Matrix Market entry out of range")
    return coo(dimensions_t(rows, cols), v, r.astype(np.uint32), c.astype(np.uint32),
               symmetric=symm in ("symmetric", "hermitian"))


def load_as_csr(path) -> csr:
    return csr.from_coo(load_as_coo(path))


def save_coo(path, m: csr, symmetric: bool = False) -> None:
    """Writes a CSR matrix as a general (or, given a symmetric matrix, lower-triangle symmetric) file."""
    rows = np.repeat(np.arange(m.dimensions.rows, dtype=np.int64), np.diff(m.row_start_offsets.astype(np.int64)))
    cols = m.col_indices.astype(np.int64)
    vals = m.values
    if symmetric:
        keep = rows >= cols
        rows, cols, vals = rows[keep], cols[keep], vals[keep]
    with open(path, "w") as fh:
        fh.write(f"%%MatrixMarket matrix coordinate real {'symmetric' if symmetric else 'general'}\n")
        fh.write(f"{m.dimensions.rows} {m.dimensions.cols} {len(vals)}\n")
        for a, b, v in zip(rows, cols, vals):
            fh.write(f"{a + 1} {b + 1} {v:.17g}\n")
