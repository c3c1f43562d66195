"""Seeded synthetic matrices with the shapes, sizes and value distributions of the five workloads.

They stand in for the reference's SuiteSparse inputs (nlpkkt240, GAP-web, GAP-kron), which are not
available here.  All are symmetric positive definite, u32 indices, f64 values, columns sorted per row.

* ``laplacian_2d_5pt(m)``        2-D 5-point Laplacian, Dirichlet, 4 on the diagonal, -1 off it
* ``stencil_3d_27pt(N, shift)``  3-D 27-point stencil, 26 + shift on the diagonal, -1 off it
* ``power_law(n, alpha, kmax)``  Zipf(alpha) off-diagonal row counts clipped to [1, kmax], uniform
                                 columns, symmetrised (duplicates summed), U[-1,0) values, diagonal =
                                 sum |off| + 1
* ``laplacian_3d_7pt(N)``        3-D 7-point Laplacian, 6 on the diagonal, -1 off it
* ``anisotropic_2d(m, ...)``     2-D 5-point diffusion with conductivities exp(g), g a Gaussian random
                                 field (squared-exponential kernel) sampled by FFT circulant embedding,
                                 x-edges scaled by the anisotropy ratio
"""
from __future__ import annotations

import numpy as np

from .mat import csr, dimensions_t


def _stencil(shape, offsets, diag_value, off_value=-1.0):
    """CSR of a constant-coefficient stencil on a row-major grid (last axis fastest).  `offsets` must be
    given in increasing column order."""
    shape = tuple(int(s) for s in shape)
    n = int(np.prod(shape))
    strides = [int(np.prod(shape[i + 1:])) for i in range(len(shape))]
    coords = np.indices(shape, dtype=np.int32).reshape(len(shape), n)
    K = len(offsets)
    mask = np.ones((n, K), dtype=bool)
    colofs = np.zeros(K, np.int64)
    for k, off in enumerate(offsets):
        for d, o in enumerate(off):
            if o:
                v = coords[d] + o
                mask[:, k] &= (v >= 0) & (v < shape[d])
            colofs[k] += o * strides[d]
    counts = mask.sum(axis=1)
    row_ptr = np.zeros(n + 1, np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    rows = np.arange(n, dtype=np.int64)
    cols = (rows[:, None] + colofs[None, :])[mask].astype(np.uint32)
    vals = np.full(cols.size, off_value, np.float64)
    kd = [k for k, off in enumerate(offsets) if not any(off)][0]
    diag_pos = row_ptr[:-1] + mask[:, :kd].sum(axis=1)
    vals[diag_pos] = diag_value
    return csr(dimensions_t(n, n), vals, row_ptr.astype(np.uint32), cols)


def laplacian_2d_5pt(m: int = 512) -> csr:
    offs = [(-1, 0), (0, -1), (0, 0), (0, 1), (1, 0)]
    return _stencil((m, m), offs, 4.0)


def stencil_3d_27pt(N: int = 128, shift: float = 1e-3) -> csr:
    offs = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]
    return _stencil((N, N, N), offs, 26.0 + shift)


def laplacian_3d_7pt(N: int = 192) -> csr:
    offs = [(-1, 0, 0), (0, -1, 0), (0, 0, -1), (0, 0, 0), (0, 0, 1), (0, 1, 0), (1, 0, 0)]
    return _stencil((N, N, N), offs, 6.0)


def power_law(n: int = 4194304, alpha: float = 2.0, kmax: int = 10000, seed: int = 2) -> csr:
    rng = np.random.default_rng(seed)
    k = np.minimum(rng.zipf(alpha, n), kmax).astype(np.int64)  # zipf >= 1
    rows = np.repeat(np.arange(n, dtype=np.int64), k)
    cols = rng.integers(0, n, rows.size, dtype=np.int64)
    vals = rng.uniform(-1.0, 0.0, rows.size)
    keep = rows != cols
    rows, cols, vals = rows[keep], cols[keep], vals[keep]
    # symmetrise: (i, j, v) and (j, i, v); duplicates are summed
    key = np.concatenate([rows * n + cols, cols * n + rows, np.arange(n, dtype=np.int64) * (n + 1)])
    v = np.concatenate([vals, vals, np.zeros(n)])
    del rows, cols, vals
    order = np.argsort(key, kind="stable")
    key = key[order]
    v = v[order]
    del order
    first = np.ones(key.size, dtype=bool)
    first[1:] = key[1:] != key[:-1]
    starts = np.flatnonzero(first)
    v = np.add.reduceat(v, starts)
    key = key[starts]
    r = (key // n).astype(np.int64)
    c = (key % n).astype(np.int64)
    del key
    row_ptr = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=n), out=row_ptr[1:])
    is_diag = r == c
    offabs = np.where(is_diag, 0.0, np.abs(v))
    rowsum = np.add.reduceat(offabs, row_ptr[:-1])  # every row holds its diagonal, so no empty rows
    v[is_diag] = rowsum[r[is_diag]] + 1.0
    return csr(dimensions_t(n, n), v, row_ptr.astype(np.uint32), c.astype(np.uint32))


def gaussian_random_field(m: int, ell: float, variance: float, seed: int) -> np.ndarray:
    """m x m sample of a stationary GRF with covariance variance*exp(-d^2 / (2 ell^2)), by circulant
    embedding on a 2m x 2m torus (negative eigenvalues of the embedding clipped to 0)."""
    M = 2 * m
    d = np.minimum(np.arange(M), M - np.arange(M)).astype(np.float64)
    dist2 = d[:, None] ** 2 + d[None, :] ** 2
    cov = variance * np.exp(-dist2 / (2.0 * ell * ell))
    lam = np.maximum(np.fft.fft2(cov).real, 0.0)
    rng = np.random.default_rng(seed)
    xi = rng.standard_normal((M, M)) + 1j * rng.standard_normal((M, M))
    field = np.fft.fft2(np.sqrt(lam / (M * M)) * xi)
    return field.real[:m, :m].copy()


def anisotropic_2d(m: int = 1024, ell: float = 16.0, variance: float = 1.0, ratio: float = 10.0,
                   seed: int = 4) -> tuple[csr, np.ndarray]:
    """5-point diffusion with edge conductances exp((g_a + g_b)/2) (geometric mean of the two cells),
    x-edges (along the fast axis) multiplied by `ratio`; Dirichlet boundary edges use the cell's own
    conductance.  Returns (matrix, g)."""
    g = gaussian_random_field(m, ell, variance, seed)
    kap = np.exp(g)
    n = m * m
    # conductances of the edges to the four neighbours (boundary: own cell)
    gx_right = np.empty_like(g)
    gx_right[:, :-1] = np.exp(0.5 * (g[:, :-1] + g[:, 1:]))
    gx_right[:, -1] = kap[:, -1]
    gx_left = np.empty_like(g)
    gx_left[:, 1:] = gx_right[:, :-1]
    gx_left[:, 0] = kap[:, 0]
    gy_down = np.empty_like(g)
    gy_down[:-1, :] = np.exp(0.5 * (g[:-1, :] + g[1:, :]))
    gy_down[-1, :] = kap[-1, :]
    gy_up = np.empty_like(g)
    gy_up[1:, :] = gy_down[:-1, :]
    gy_up[0, :] = kap[0, :]
    wl, wr = ratio * gx_left, ratio * gx_right
    wu, wd = gy_up, gy_down
    diag = (wl + wr + wu + wd).ravel()
    base = _stencil((m, m), [(-1, 0), (0, -1), (0, 0), (0, 1), (1, 0)], 1.0)
    # fill the values in the same masked order: (up, left, diag, right, down)
    i, j = np.indices((m, m))
    masks = [(i > 0), (j > 0), np.ones_like(i, bool), (j < m - 1), (i < m - 1)]
    vals_k = [-wu, -wl, diag.reshape(m, m), -wr, -wd]
    stacked_mask = np.stack([mk.ravel() for mk in masks], axis=1)
    stacked_vals = np.stack([vk.ravel() for vk in vals_k], axis=1)
    base.values[:] = stacked_vals[stacked_mask]
    return base, g


def rhs(A: csr, seed: int, k: int | None = None):
    """x* ~ U[-1, 1] (one column, or k columns row-major) and b = A x*."""
    rng = np.random.default_rng(seed)
    n = A.dimensions.cols
    xs = rng.uniform(-1.0, 1.0, n if k is None else (n, k))
    b = A.to_scipy() @ xs
    return xs, np.ascontiguousarray(b)


WORKLOADS = {
    "lap2d_512": dict(build=lambda: laplacian_2d_5pt(512), seed=0, tol=1e-8),
    "stencil27_128": dict(build=lambda: stencil_3d_27pt(128, 1e-3), seed=1, tol=1e-10),
    "powerlaw_4m": dict(build=lambda: power_law(4194304, 2.0, 10000, 2), seed=2, tol=1e-10),
    "lap3d7_192": dict(build=lambda: laplacian_3d_7pt(192), seed=3, tol=1e-10),
    "aniso2d_1024": dict(build=lambda: anisotropic_2d(1024)[0], seed=4, tol=1e-10),
}
