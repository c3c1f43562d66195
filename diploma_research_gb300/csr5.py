"""Device CSR5 matrix: the host-side mirror of ``dim::mat::csr5<double,16,4,uint32_t>``.

Reference interface (include/dim/mat/storage_formats/csr5.h):

==========================================  ============================================================
reference                                    here
==========================================  ============================================================
``csr5::from_csr(csr)`` (:791-803)           ``csr5.from_csr(m, sigma=16, omega=32)`` -- converts on GPU
``csr5::spmv(spmv_data_t{x, y, cal})``       ``A.spmv(spmv_data_t(x, y, cal))`` or ``A.spmv(x, y, cal)``
(:280-285, 818-829)
``csr5::create_calibrator()`` (:809)         ``A.create_calibrator()``
``csr5::tail_partition_start()`` (:806)      ``A.tail_partition_start()``
``csr5::non_zero_count()`` (:880)            ``A.non_zero_count()``
``csr5::iterate(body)`` (:868-877)           ``A.iterate(body)`` (host copy of the CSR arrays)
``csr5::dimensions`` / ``vals`` /            ``A.dimensions``, ``A.vals``, ``A.col_idx``, ``A.row_ptr``
``col_idx`` / ``row_ptr`` (:450-453)         (host copies, exported on first access)
``csr5::csr5_info`` (:287-447)               ``A.csr5_info`` (tile_count, tile_ptr, tile_desc, ...)
==========================================  ============================================================

Errors follow the reference: a size mismatch in ``spmv`` raises ``ValueError`` (the reference's
``std::invalid_argument``, csr5.h:820-821).  Unlike the reference, ``spmv`` overwrites ``y`` (no
zero-fill needed) and a calibrator can be reused across calls.

``x``/``y`` may be device arrays (anything exposing ``__cuda_array_interface__``, e.g. torch CUDA
tensors; the product runs on ``stream``) or numpy arrays (host; copied in and out).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from types import SimpleNamespace

import numpy as np

from . import _native as N
from .mat import csr, dimensions_t


class calibrator_t:
    """Scratch of one SpMV at a time (the reference's calibrator_t, csr5/calibrator.h:14-31)."""

    def __init__(self, matrix: "csr5"):
        h = ctypes.c_void_p()
        N.check(N.lib().dimgpu_calibrator_create(matrix._h, ctypes.byref(h)))
        self._h = h
        self._matrix = matrix  # keeps the matrix alive

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            N.lib().dimgpu_calibrator_destroy(h)
            self._h = None


@dataclass
class spmv_data_t:
    """csr5::spmv_data_t (csr5.h:280-285)."""
    x: object
    y: object
    calibrator: calibrator_t | None = None


class csr5:
    sigma: int
    omega: int

    def __init__(self, handle, info: N.csr5_info):
        self._h = handle
        self._info = info
        self.sigma = int(info.sigma)
        self.omega = int(info.omega)
        self.dimensions = dimensions_t(int(info.rows), int(info.cols))
        self._export = None

    # ---- construction -------------------------------------------------------------------------
    @staticmethod
    def from_csr(m: csr, sigma: int = 16, omega: int = 32, layout: int | None = None, stream=None) -> "csr5":
        """Converts a host ``csr`` matrix to CSR5 on the device (csr5.h:791-803).

        omega=32 gives the device layout used by the kernels; omega=4 with the default layout gives
        the reference's csr5<double,16,4,uint32_t> arrays (for export and parity checks)."""
        opt = N.csr5_options(sigma, omega, (0 if omega != 32 else 1) if layout is None else layout, 0)
        h = ctypes.c_void_p()
        rp = np.ascontiguousarray(m.row_start_offsets, np.uint32)
        ci = np.ascontiguousarray(m.col_indices, np.uint32)
        v = np.ascontiguousarray(m.values, np.float64)
        N.check(N.lib().dimgpu_csr5_from_csr(m.dimensions.rows, m.dimensions.cols, v.size, rp.ctypes.data,
                                             ci.ctypes.data if v.size else None, v.ctypes.data if v.size else None,
                                             N.MEM_HOST, ctypes.byref(opt), N.stream_ptr(stream), ctypes.byref(h)))
        return csr5._wrap(h)

    @staticmethod
    def from_device_csr(rows, cols, nnz, row_ptr, col_idx, vals, sigma=16, omega=32, stream=None) -> "csr5":
        """Converts CSR arrays already in device memory (u32, u32, f64 device arrays)."""
        opt = N.csr5_options(sigma, omega, 1 if omega == 32 else 0, 0)
        h = ctypes.c_void_p()
        N.check(N.lib().dimgpu_csr5_from_csr(int(rows), int(cols), int(nnz), N.device_ptr(row_ptr, "<u4"),
                                             N.device_ptr(col_idx, "<u4") if nnz else None,
                                             N.device_ptr(vals, "<f8") if nnz else None, N.MEM_DEVICE,
                                             ctypes.byref(opt), N.stream_ptr(stream), ctypes.byref(h)))
        return csr5._wrap(h)

    @staticmethod
    def _wrap(h) -> "csr5":
        info = N.csr5_info()
        N.check(N.lib().dimgpu_csr5_get_info(h, ctypes.byref(info)))
        return csr5(h, info)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            N.lib().dimgpu_csr5_destroy(h)
            self._h = None

    # ---- reference accessors ------------------------------------------------------------------
    def tail_partition_start(self) -> int:
        return int(self._info.tail_partition_start)

    def non_zero_count(self) -> int:
        return int(self._info.nnz)

    def create_calibrator(self) -> calibrator_t:
        return calibrator_t(self)

    @property
    def tile_count(self) -> int:
        return int(self._info.tile_count)

    @property
    def device_bytes(self) -> int:
        return int(self._info.device_bytes)

    @property
    def empty_rows(self) -> int:
        return int(self._info.empty_rows)

    def export(self) -> SimpleNamespace:
        """Host copies of every CSR5 array (csr5_info_t, csr5.h:287-294, plus vals/col_idx/row_ptr)."""
        if self._export is None:
            i = self._info
            T = int(i.tile_count)
            wdt = np.uint32 if i.desc_word_bytes == 4 else np.uint64
            out = SimpleNamespace(
                tile_count=T,
                tile_ptr=np.zeros(T + 1, np.uint32),
                tile_desc=np.zeros(max(1, T * i.omega), wdt),
                tile_desc_offset_ptr=np.zeros(T + 1, np.uint32),
                tile_desc_offset=np.zeros(max(1, int(i.tile_desc_offset_len)), np.uint32),
                vals=np.zeros(max(1, int(i.nnz)), np.float64),
                col_idx=np.zeros(max(1, int(i.nnz)), np.uint32),
                row_ptr=np.zeros(int(i.rows) + 1, np.uint32),
            )
            N.check(N.lib().dimgpu_csr5_export(self._h, out.tile_ptr.ctypes.data, out.tile_desc.ctypes.data,
                                               out.tile_desc_offset_ptr.ctypes.data, out.tile_desc_offset.ctypes.data,
                                               out.vals.ctypes.data, out.col_idx.ctypes.data, out.row_ptr.ctypes.data))
            out.tile_desc = out.tile_desc[: T * i.omega]
            out.tile_desc_offset = out.tile_desc_offset[: int(i.tile_desc_offset_len)]
            out.vals = out.vals[: int(i.nnz)]
            out.col_idx = out.col_idx[: int(i.nnz)]
            self._export = out
        return self._export

    @property
    def csr5_info(self) -> SimpleNamespace:
        return self.export()

    @property
    def vals(self):
        return self.export().vals

    @property
    def col_idx(self):
        return self.export().col_idx

    @property
    def row_ptr(self):
        return self.export().row_ptr

    def iterate(self, body) -> None:
        """Calls body((row, col), value) for every element in CSR order (csr5.h:868-877).  The
        values are mapped back from the tile order of the exported arrays."""
        e = self.export()
        from .layout import csr_order
        v, c = csr_order(self, e.vals, e.col_idx)
        rp = e.row_ptr
        for row in range(self.dimensions.rows):
            for k in range(int(rp[row]), int(rp[row + 1])):
                body((row, int(c[k])), float(v[k]))

    # ---- SpMV -----------------------------------------------------------------------------------
    _GATHER = {"l1": 0, "stream": 1}

    def spmv_launch(self, f32: bool = False) -> tuple[int, str]:
        """(warps per CTA, "l1" | "stream") of this matrix's SpMV launch, as the library chose it by timing
        (f32=True: the f32 product's, making its values first if needed)."""
        w, g = ctypes.c_uint32(), ctypes.c_int()
        N.check(N.lib().dimgpu_csr5_get_spmv_launch(self._h, int(f32), ctypes.byref(w), ctypes.byref(g)))
        return int(w.value), "stream" if g.value == 1 else "l1"

    def set_spmv_launch(self, warps_per_cta: int, gather: str = "l1", f32: bool = False) -> None:
        """Pins the launch (f64: 16 or 12 warps per CTA; f32: 24 or 20; gather "l1" or "stream")."""
        if gather not in self._GATHER:
            raise ValueError(f"gather must be one of {sorted(self._GATHER)}")
        N.check(N.lib().dimgpu_csr5_set_spmv_launch(self._h, int(f32), int(warps_per_cta), self._GATHER[gather]))

    def spmv(self, data, y=None, calibrator: calibrator_t | None = None, stream=None):
        """y := A x (csr5.h:818-829).  ``data`` is an spmv_data_t or x (then pass y)."""
        if isinstance(data, spmv_data_t):
            x, y, calibrator = data.x, data.y, data.calibrator
        else:
            x = data
        if y is None:
            raise ValueError("spmv needs an output vector y")
        L = N.lib()
        if N.is_device_array(x):
            if not N.is_device_array(y):
                raise TypeError("x is a device array but y is not")
            self._check_len(x, self.dimensions.cols, "x")
            self._check_len(y, self.dimensions.rows, "y")
            cal = calibrator._h if calibrator is not None else None
            typ = getattr(x, "__cuda_array_interface__", {}).get("typestr", "<f8")
            if typ == "<f4":
                N.check(L.dimgpu_csr5_spmv_f32(self._h, N.device_ptr(x, "<f4"), N.device_ptr(y, "<f4"), cal,
                                               N.stream_ptr(stream)))
            else:
                N.check(L.dimgpu_csr5_spmv(self._h, N.device_ptr(x, "<f8"), N.device_ptr(y, "<f8"), cal,
                                           N.stream_ptr(stream)))
            return y
        xh = np.ascontiguousarray(x, np.float64)
        if xh.size != self.dimensions.cols:
            raise ValueError("can't multiply, vector size doesn't match column count of the matrix")
        if not isinstance(y, np.ndarray) or y.dtype != np.float64 or not y.flags.c_contiguous:
            raise TypeError("host y must be a contiguous float64 numpy array")
        if y.size != self.dimensions.rows:
            raise ValueError("output vector size doesn't match the row count of the matrix")
        N.check(L.dimgpu_csr5_spmv_host(self._h, xh.ctypes.data if xh.size else None,
                                        y.ctypes.data if y.size else None))
        return y

    @staticmethod
    def _check_len(a, n, name):
        cai = a.__cuda_array_interface__ if hasattr(a, "__cuda_array_interface__") else None
        if cai is not None:
            size = 1
            for d in cai["shape"]:
                size *= d
            if size != n:
                if name == "x":
                    raise ValueError("can't multiply, vector size doesn't match column count of the matrix")
                raise ValueError(f"{name} has {size} elements, expected {n}")


def spmm(A: csr5, X, Y, stream=None):
    """Y := A X for k right-hand sides (device arrays, row-major: X cols x k, Y rows x k).  f64 or f32.

    The first call for a given (k, precision) picks the fastest SpMM launch shape by timing."""
    cx = X.__cuda_array_interface__
    cy = Y.__cuda_array_interface__
    if len(cx["shape"]) != 2 or len(cy["shape"]) != 2:
        raise ValueError("X and Y must be 2-D (rows x k)")
    n_x, k = cx["shape"]
    n_y, k2 = cy["shape"]
    if k != k2 or n_x != A.dimensions.cols or n_y != A.dimensions.rows:
        raise ValueError("shape mismatch: X must be cols x k and Y rows x k")
    typ = cx["typestr"]
    L = N.lib()
    if typ == "<f4":
        N.check(L.dimgpu_csr5_spmm_f32(A._h, k, N.device_ptr(X, "<f4"), k, N.device_ptr(Y, "<f4"), k,
                                       N.stream_ptr(stream)))
    else:
        N.check(L.dimgpu_csr5_spmm(A._h, k, N.device_ptr(X, "<f8"), k, N.device_ptr(Y, "<f8"), k,
                                   N.stream_ptr(stream)))
    return Y


def spmm_shape(A: csr5, k: int, f32: bool = False) -> int:
    """The autotuned SpMM shape for (k, precision), -1 before the first call: bit 0 the launch shape,
    bits 1-2 the lane grouping (see dimgpu_csr5_spmm_shape in include/dimgpu.h)."""
    v = ctypes.c_int()
    N.check(N.lib().dimgpu_csr5_spmm_shape(A._h, k, 1 if f32 else 0, ctypes.byref(v)))
    return int(v.value)


def set_spmm_shape(A: csr5, k: int, shape: int, f32: bool = False) -> None:
    """Pins the SpMM shape for (k, precision) (0..5, or -1 to re-tune on the next call)."""
    N.check(N.lib().dimgpu_csr5_set_spmm_shape(A._h, k, 1 if f32 else 0, int(shape)))
