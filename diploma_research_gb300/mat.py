"""Host-side sparse containers mirroring ``dim::mat`` (include/dim/mat/storage_formats/).

* ``dimensions_t`` -- base.h:10-17
* ``coo``          -- coo.h:17-47 (with the symmetric expansion of ``coo::iterate``)
* ``csr``          -- csr.h:19-78 (``values``, ``row_start_offsets``, ``col_indices``; u32 indices)

The device CSR5 matrix lives in :mod:`diploma_research_gb300.csr5`.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class dimensions_t:
    rows: int
    cols: int


class coo:
    """Coordinate matrix; ``symmetric`` means every off-diagonal entry also stands for its mirror."""

    def __init__(self, dimensions: dimensions_t, values, row_indices, col_indices, symmetric: bool = False):
        self.dimensions = dimensions
        self.values = np.ascontiguousarray(values, dtype=np.float64)
        self.row_indices = np.ascontiguousarray(row_indices, dtype=np.uint32)
        self.col_indices = np.ascontiguousarray(col_indices, dtype=np.uint32)
        self.symmetric = bool(symmetric)

    def expanded(self):
        """(values, rows, cols) in the order ``coo::iterate`` visits them (coo.h:33-46)."""
        v, r, c = self.values, self.row_indices, self.col_indices
        if not self.symmetric:
            return v, r, c
        off = r != c
        # each entry, immediately followed by its mirror when off-diagonal
        order_v = np.empty(len(v) + int(off.sum()), np.float64)
        order_r = np.empty_like(order_v, dtype=np.uint32)
        order_c = np.empty_like(order_v, dtype=np.uint32)
        pos = np.arange(len(v)) + np.concatenate(([0], np.cumsum(off)[:-1])) if len(v) else np.zeros(0, np.int64)
        order_v[pos], order_r[pos], order_c[pos] = v, r, c
        mpos = pos[off] + 1
        order_v[mpos], order_r[mpos], order_c[mpos] = v[off], c[off], r[off]
        return order_v, order_r, order_c


class csr:
    """Compressed sparse row matrix (csr.h:19-40): f64 values, u32 row offsets and column indices."""

    def __init__(self, dimensions: dimensions_t, values, row_start_offsets, col_indices):
        self.dimensions = dimensions
        self.values = np.ascontiguousarray(values, dtype=np.float64)
        self.row_start_offsets = np.ascontiguousarray(row_start_offsets, dtype=np.uint32)
        self.col_indices = np.ascontiguousarray(col_indices, dtype=np.uint32)
        if self.row_start_offsets.size != dimensions.rows + 1:
            raise ValueError("row_start_offsets must hold rows + 1 entries")
        if self.values.size != self.col_indices.size:
            raise ValueError("values and col_indices differ in length")
        if int(self.row_start_offsets[-1]) != self.values.size:
            raise ValueError("row_start_offsets[-1] must equal the number of non-zeros")

    @property
    def nnz(self) -> int:
        return int(self.values.size)

    @staticmethod
    def from_coo(m: coo) -> "csr":
        """csr::from_coo (csr.h:42-77): count rows, exclusive scan, scatter in iteration order, then
        sort each row by column.  The per-row sort here is stable; the reference's std::sort only
        differs on duplicate column indices within a row."""
        v, r, c = m.expanded()
        rows = m.dimensions.rows
        counts = np.bincount(r.astype(np.int64), minlength=rows + 1)[: rows + 1] if len(r) else np.zeros(rows + 1,
                                                                                                        np.int64)
        row_ptr = np.zeros(rows + 1, np.int64)
        row_ptr[1:] = np.cumsum(counts[:rows])
        order = np.lexsort((c, r)) if len(r) else np.zeros(0, np.int64)
        if row_ptr[-1] > 0xFFFFFFFF:
            raise ValueError("too many non-zeros for u32 row offsets")
        return csr(m.dimensions, v[order], row_ptr.astype(np.uint32), c[order])

    def to_scipy(self):
        import scipy.sparse as sp

        return sp.csr_matrix((self.values, self.col_indices.astype(np.int64), self.row_start_offsets.astype(np.int64)),
                             shape=(self.dimensions.rows, self.dimensions.cols))

    @staticmethod
    def from_scipy(a) -> "csr":
        a = a.tocsr()
        a.sort_indices()
        return csr(dimensions_t(a.shape[0], a.shape[1]), a.data, a.indptr.astype(np.uint32),
                   a.indices.astype(np.uint32))

    def permuted(self, perm) -> "csr":
        """P A P^T for a square matrix: new row/column i is old row/column perm[i] (columns re-sorted per
        row).  CG on the permuted system, with b permuted the same way, gives the permuted solution."""
        import scipy.sparse as sp

        if self.dimensions.rows != self.dimensions.cols:
            raise ValueError("a symmetric permutation needs a square matrix")
        perm = np.asarray(perm, dtype=np.int64)
        P = self.to_scipy()[perm][:, perm].tocsr()
        P.sort_indices()
        return csr.from_scipy(sp.csr_matrix(P))

    def hub_first_order(self) -> np.ndarray:
        """The permutation that numbers rows by decreasing length (stable): for a symmetric matrix the most
        referenced columns then come first and their x entries share cache sectors."""
        return np.argsort(-np.diff(self.row_start_offsets.astype(np.int64)), kind="stable")

    def iterate(self, body) -> None:
        """Calls ``body((row, col), value)`` for every stored element in row order (csr5.h:868-877)."""
        rp = self.row_start_offsets
        for row in range(self.dimensions.rows):
            for i in range(int(rp[row]), int(rp[row + 1])):
                body((row, int(self.col_indices[i])), float(self.values[i]))
