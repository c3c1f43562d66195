"""Element orders inside CSR5 tiles (host side), matching csrc/layout.cuh.

Within every full tile that spans more than one row, element (column c, row r) -- CSR position
``t*sigma*omega + c*sigma + r`` -- is stored at

* ``r*omega + c``                          reference order (csr5.h:463-493)
* ``(r//2)*2*omega + 2*c + r%2``           device order of f64 values (16-byte pairs)
* ``(r//4)*4*omega + 4*c + r%4``           device order of u32 column indices and f32 values (quads)

The reference order leaves single-row (fast-track) tiles in CSR order; the device orders re-order
every full tile.  The tail keeps CSR order.
"""
from __future__ import annotations

import numpy as np

DIRTY = np.uint32(0x80000000)


def positions(sigma: int, omega: int, kind: str) -> np.ndarray:
    k = np.arange(sigma * omega)
    c, r = k // sigma, k % sigma
    if kind == "ref":
        return r * omega + c
    if kind == "f64":
        return (r // 2) * (2 * omega) + 2 * c + (r % 2)
    if kind == "q32":
        return (r // 4) * (4 * omega) + 4 * c + (r % 4)
    raise ValueError(kind)


def multirow_tiles(tile_ptr: np.ndarray) -> np.ndarray:
    tp = np.asarray(tile_ptr, np.uint32) & ~DIRTY
    return tp[:-1] != tp[1:]


def _reordered(tile_ptr, kind):
    mr = multirow_tiles(tile_ptr)
    return mr if kind == "ref" else np.ones_like(mr)


def permute(arr_csr: np.ndarray, tile_ptr: np.ndarray, sigma: int, omega: int, kind: str) -> np.ndarray:
    """CSR order -> tile order."""
    T = len(tile_ptr) - 1
    ts = sigma * omega
    out = np.array(arr_csr, copy=True)
    if T == 0:
        return out
    mr = _reordered(tile_ptr, kind)
    body = out[: T * ts].reshape(T, ts)
    src = np.asarray(arr_csr)[: T * ts].reshape(T, ts)[mr]
    dst = np.empty_like(src)
    dst[:, positions(sigma, omega, kind)] = src
    body[mr] = dst
    return out


def unpermute(arr_tiled: np.ndarray, tile_ptr: np.ndarray, sigma: int, omega: int, kind: str) -> np.ndarray:
    """Tile order -> CSR order."""
    T = len(tile_ptr) - 1
    ts = sigma * omega
    out = np.array(arr_tiled, copy=True)
    if T == 0:
        return out
    mr = _reordered(tile_ptr, kind)
    body = out[: T * ts].reshape(T, ts)
    src = np.asarray(arr_tiled)[: T * ts].reshape(T, ts)[mr]
    body[mr] = src[:, positions(sigma, omega, kind)]
    return out


def csr_order(matrix, vals_tiled, col_tiled):
    """Maps a csr5 handle's exported vals/col_idx back to CSR order."""
    tp = matrix.export().tile_ptr
    if matrix.omega == 32:
        return (unpermute(vals_tiled, tp, matrix.sigma, 32, "f64"),
                unpermute(col_tiled, tp, matrix.sigma, 32, "q32"))
    return (unpermute(vals_tiled, tp, matrix.sigma, matrix.omega, "ref"),
            unpermute(col_tiled, tp, matrix.sigma, matrix.omega, "ref"))
