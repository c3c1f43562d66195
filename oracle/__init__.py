"""The oracle: CPU restatements of the reference's CSR5 hot path.  TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline / reference legs of ``bench.py``
import this package.  Nothing in ``diploma_research_gb300`` does.

Two libraries sit behind it:

* ``_build/libcsr5_oracle.so`` -- ``csr5_oracle.c``, a plain-C restatement of
  ``include/dim/mat/storage_formats/csr5.h`` (conversion, SpMV, calibrator, tail) and of the
  ``dim_sp`` CG loop (``benchmarks/conjugate_gradient/dim_sp/main.cpp:89-127``).  Builds anywhere
  gcc and OpenMP exist (x86-64 and aarch64).
* ``_ref/libdimref.so`` -- ``ref_shim.cpp`` compiled against the reference's own headers
  (``make -C oracle ref``); x86-64 + AVX2 and a reference checkout only.  It pins the restatement.

Parity for the restatement is pinned two ways: against the reference's own known-answer tests
(``tests/test_csr5.cpp:26-57`` on ``tests/test_files/mm.mtx``, restated in ``tests/golden``) and
bit-for-bit against ``libdimref.so`` on generated matrices (``tests/test_oracle_pin.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libcsr5_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libdimref.so")

_lock = threading.Lock()
_lib = None
_ref = None

_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build(ref: bool = False) -> None:
    """Compile the restatement (and, if asked and possible, the reference shim)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref and ref_buildable():
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={os.path.abspath(ref_root())}"], check=True)


def ref_root() -> str:
    """The reference checkout: $REF_ROOT, else a `reference` directory beside the repository."""
    return os.environ.get("REF_ROOT", os.path.join(os.path.dirname(HERE), os.pardir, "reference"))


def ref_buildable() -> bool:
    import platform

    root = ref_root()
    return platform.machine() in ("x86_64", "AMD64") and os.path.isfile(
        os.path.join(root, "include", "dim", "mat", "storage_formats", "csr5.h"))


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.isfile(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(
                    os.path.join(HERE, "csr5_oracle.c")):
                subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
            L = ctypes.CDLL(ORACLE_SO)
            L.oracle_csr5_plan.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, ctypes.c_uint, ctypes.c_uint,
                                           ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
            L.oracle_csr5_plan.restype = ctypes.c_int
            L.oracle_csr5_convert.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p, _f64p, ctypes.c_uint,
                                              ctypes.c_uint, _u32p, _u64p, _u32p, _u32p, _f64p, _u32p]
            L.oracle_csr5_convert.restype = ctypes.c_int
            L.oracle_csr5_spmv.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint, ctypes.c_uint, _u32p,
                                           _u32p, _u64p, _u32p, _u32p, _f64p, _u32p, _f64p, _f64p, ctypes.c_int]
            L.oracle_csr5_spmv.restype = ctypes.c_int
            L.oracle_csr_spmv.argtypes = [ctypes.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, ctypes.c_int]
            L.oracle_csr_spmv.restype = None
            L.oracle_csr_absspmv.argtypes = [ctypes.c_uint32, _u32p, _u32p, _f64p, _f64p, _f64p, ctypes.c_int]
            L.oracle_csr_absspmv.restype = None
            L.oracle_dot.argtypes = [_f64p, _f64p, ctypes.c_uint64, ctypes.c_int]
            L.oracle_dot.restype = ctypes.c_double
            L.oracle_cg.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint, ctypes.c_uint, _u32p, _u32p,
                                    _u64p, _u32p, _u32p, _f64p, _u32p, _f64p, _f64p, ctypes.c_double,
                                    ctypes.c_int64, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
            L.oracle_cg.restype = ctypes.c_int64
            L.oracle_max_threads.restype = ctypes.c_int
            L.oracle_desc_bits.argtypes = [ctypes.c_uint, ctypes.c_uint]
            L.oracle_desc_bits.restype = ctypes.c_int
            _lib = L
    return _lib


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class OracleCSR5:
    """CSR5 arrays as the reference builds them (csr5_info_t, csr5.h:287-447), at any (sigma, omega)."""

    def __init__(self, rows, cols, row_ptr, col_idx, vals, sigma=16, omega=4):
        self.rows, self.cols = int(rows), int(cols)
        self.row_ptr = _u32(row_ptr)
        col_idx, vals = _u32(col_idx), _f64(vals)
        self.nnz = int(vals.size)
        self.sigma, self.omega = int(sigma), int(omega)
        L = lib()
        T, tdo = ctypes.c_uint64(), ctypes.c_uint64()
        rc = L.oracle_csr5_plan(self.rows, self.nnz, self.row_ptr, self.sigma, self.omega, ctypes.byref(T),
                                ctypes.byref(tdo))
        if rc != 0:
            raise ValueError(f"oracle_csr5_plan failed ({rc})")
        self.tile_count, tdo_size = int(T.value), int(tdo.value)
        self.tile_ptr = np.zeros(self.tile_count + 1, np.uint32)
        self.tile_desc = np.zeros(max(1, self.tile_count * self.omega), np.uint64)
        self.tile_desc_offset_ptr = np.zeros(self.tile_count + 1, np.uint32)
        self.tile_desc_offset = np.zeros(max(1, tdo_size), np.uint32)
        self.vals = np.zeros(max(1, self.nnz), np.float64)
        self.col_idx = np.zeros(max(1, self.nnz), np.uint32)
        v_in = vals if vals.size else np.zeros(1)
        c_in = col_idx if col_idx.size else np.zeros(1, np.uint32)
        rc = L.oracle_csr5_convert(self.rows, self.nnz, self.row_ptr, c_in, v_in, self.sigma, self.omega,
                                   self.tile_ptr, self.tile_desc, self.tile_desc_offset_ptr, self.tile_desc_offset,
                                   self.vals, self.col_idx)
        if rc != 0:
            raise ValueError(f"oracle_csr5_convert failed ({rc})")
        self.tile_desc = self.tile_desc[: self.tile_count * self.omega]
        self.tile_desc_offset = self.tile_desc_offset[:tdo_size]
        self.vals = self.vals[: self.nnz]
        self.col_idx = self.col_idx[: self.nnz]

    @property
    def tail_partition_start(self) -> int:
        return int(self.tile_ptr[-1] & 0x7FFFFFFF)

    def spmv(self, x, nthreads=0):
        x = _f64(x)
        assert x.size == self.cols
        y = np.empty(max(1, self.rows), np.float64)
        L = lib()
        pad = lambda a, dt: a if a.size else np.zeros(1, dt)
        L.oracle_csr5_spmv(self.rows, self.nnz, self.sigma, self.omega, self.row_ptr, self.tile_ptr,
                           pad(self.tile_desc, np.uint64), self.tile_desc_offset_ptr,
                           pad(self.tile_desc_offset, np.uint32), pad(self.vals, np.float64),
                           pad(self.col_idx, np.uint32), x if x.size else np.zeros(1), y, int(nthreads))
        return y[: self.rows]

    def cg(self, b, x0=None, tol=1e-10, max_it=100000, nthreads=0):
        b = _f64(b)
        x = np.zeros(self.rows) if x0 is None else _f64(x0).copy()
        rel = ctypes.c_double()
        pad = lambda a, dt: a if a.size else np.zeros(1, dt)
        it = lib().oracle_cg(self.rows, self.nnz, self.sigma, self.omega, self.row_ptr, self.tile_ptr,
                             pad(self.tile_desc, np.uint64), self.tile_desc_offset_ptr,
                             pad(self.tile_desc_offset, np.uint32), pad(self.vals, np.float64),
                             pad(self.col_idx, np.uint32), b, x, float(tol), int(max_it), int(nthreads),
                             ctypes.byref(rel))
        if it < 0:
            raise RuntimeError(f"oracle_cg failed ({it})")
        return x, int(it), float(rel.value)

    def desc_fields(self):
        """Decode the packed column words into (y_offset, scansum_offset, bit_flag) arrays."""
        yb = int(self.sigma * self.omega).bit_length()
        sb = int(self.omega).bit_length()
        w = self.tile_desc.astype(np.uint64)
        y = w & np.uint64((1 << yb) - 1)
        s = (w >> np.uint64(yb)) & np.uint64((1 << sb) - 1)
        f = (w >> np.uint64(yb + sb)) & np.uint64((1 << self.sigma) - 1)
        return y, s, f


def csr_spmv(rows, row_ptr, col_idx, vals, x, nthreads=0):
    y = np.empty(max(1, rows))
    lib().oracle_csr_spmv(int(rows), _u32(row_ptr), _u32(col_idx) if len(col_idx) else np.zeros(1, np.uint32),
                          _f64(vals) if len(vals) else np.zeros(1), _f64(x) if len(x) else np.zeros(1), y,
                          int(nthreads))
    return y[:rows]


def abs_spmv(rows, row_ptr, col_idx, vals, x, nthreads=0):
    """(|A| |x|)_i -- the scale of the componentwise SpMV tolerance."""
    y = np.empty(max(1, rows))
    lib().oracle_csr_absspmv(int(rows), _u32(row_ptr), _u32(col_idx) if len(col_idx) else np.zeros(1, np.uint32),
                             _f64(vals) if len(vals) else np.zeros(1), _f64(x) if len(x) else np.zeros(1), y,
                             int(nthreads))
    return y[:rows]


def dot(a, b, nthreads=0):
    a, b = _f64(a), _f64(b)
    return float(lib().oracle_dot(a, b, a.size, int(nthreads)))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


# ------------------------------------------------------------------------------------------------
# The reference itself (x86-64 only), behind oracle/ref_shim.cpp.
# ------------------------------------------------------------------------------------------------

def ref():
    """ctypes handle to oracle/_ref/libdimref.so, building it when the reference checkout exists."""
    global _ref
    with _lock:
        if _ref is None:
            if not os.path.isfile(REF_SO):
                if not ref_buildable():
                    return None
                subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={os.path.abspath(ref_root())}"],
                               check=True)
            L = ctypes.CDLL(REF_SO)
            L.dimref_csr5_from_csr.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, _u32p, _u32p,
                                               _f64p]
            L.dimref_csr5_from_csr.restype = ctypes.c_void_p
            L.dimref_csr5_free.argtypes = [ctypes.c_void_p]
            L.dimref_csr5_sizes.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
                                            ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32)]
            L.dimref_csr5_export.argtypes = [ctypes.c_void_p, _u32p, _u32p, _u32p, _u32p, _f64p, _u32p]
            L.dimref_csr5_spmv.argtypes = [ctypes.c_void_p, _f64p, _f64p]
            L.dimref_csr5_spmv.restype = ctypes.c_int
            L.dimref_cg.argtypes = [ctypes.c_void_p, _f64p, _f64p, ctypes.c_double, ctypes.c_int64,
                                    ctypes.POINTER(ctypes.c_double)]
            L.dimref_cg.restype = ctypes.c_int64
            L.dimref_max_threads.restype = ctypes.c_int
            L.dimref_csr_from_coo.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, _f64p, _u32p, _u32p,
                                              ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
            L.dimref_csr_from_coo.restype = ctypes.c_void_p
            L.dimref_csr_export.argtypes = [ctypes.c_void_p, _u32p, _u32p, _f64p]
            L.dimref_csr_free.argtypes = [ctypes.c_void_p]
            _ref = L
    return _ref


def ref_csr_from_coo(rows, cols, values, row_indices, col_indices, symmetric=False):
    """The reference's csr<double>::from_coo (csr.h:42-77) of a coo (coo.h:17-47); returns
    (row_start_offsets, col_indices, values)."""
    L = ref()
    if L is None:
        raise RuntimeError("reference shim unavailable on this host")
    v, r, c = _f64(values), _u32(row_indices), _u32(col_indices)
    pad = lambda a, dt: a if a.size else np.zeros(1, dt)
    nnz_out = ctypes.c_uint64()
    h = L.dimref_csr_from_coo(int(rows), int(cols), v.size, pad(v, np.float64), pad(r, np.uint32),
                              pad(c, np.uint32), 1 if symmetric else 0, ctypes.byref(nnz_out))
    try:
        k = int(nnz_out.value)
        rp = np.zeros(int(rows) + 1, np.uint32)
        ci = np.zeros(max(1, k), np.uint32)
        vv = np.zeros(max(1, k), np.float64)
        L.dimref_csr_export(h, rp, ci, vv)
        return rp, ci[:k], vv[:k]
    finally:
        L.dimref_csr_free(h)


class RefCSR5:
    """The reference's csr5<double,16,4,uint32_t> (via oracle/_ref/libdimref.so)."""

    def __init__(self, rows, cols, row_ptr, col_idx, vals):
        L = ref()
        if L is None:
            raise RuntimeError("reference shim unavailable on this host")
        self._L = L
        self.rows, self.cols = int(rows), int(cols)
        self.nnz = len(vals)
        self._keep = (_u32(row_ptr), _u32(col_idx) if len(col_idx) else np.zeros(1, np.uint32),
                      _f64(vals) if len(vals) else np.zeros(1))
        self._h = L.dimref_csr5_from_csr(self.rows, self.cols, self.nnz, *self._keep)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.dimref_csr5_free(h)
            self._h = None

    def export(self):
        T, tdo, tail = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint32()
        self._L.dimref_csr5_sizes(self._h, ctypes.byref(T), ctypes.byref(tdo), ctypes.byref(tail))
        T, tdo = int(T.value), int(tdo.value)
        out = dict(tile_count=T, tail_partition_start=int(tail.value),
                   tile_ptr=np.zeros(T + 1, np.uint32), tile_desc=np.zeros(max(1, 4 * T), np.uint32),
                   tile_desc_offset_ptr=np.zeros(T + 1, np.uint32), tile_desc_offset=np.zeros(max(1, tdo), np.uint32),
                   vals=np.zeros(max(1, self.nnz)), col_idx=np.zeros(max(1, self.nnz), np.uint32))
        self._L.dimref_csr5_export(self._h, out["tile_ptr"], out["tile_desc"], out["tile_desc_offset_ptr"],
                                   out["tile_desc_offset"], out["vals"], out["col_idx"])
        out["tile_desc"] = out["tile_desc"][: 4 * T]
        out["tile_desc_offset"] = out["tile_desc_offset"][:tdo]
        out["vals"] = out["vals"][: self.nnz]
        out["col_idx"] = out["col_idx"][: self.nnz]
        return out

    def spmv(self, x):
        y = np.empty(max(1, self.rows))
        if self._L.dimref_csr5_spmv(self._h, _f64(x), y) != 0:
            raise ValueError("reference spmv cannot run with tile_count == 0")
        return y[: self.rows]

    def cg(self, b, x0=None, tol=1e-10, max_it=100000):
        x = np.zeros(self.rows) if x0 is None else _f64(x0).copy()
        rel = ctypes.c_double()
        it = self._L.dimref_cg(self._h, _f64(b), x, float(tol), int(max_it), ctypes.byref(rel))
        if it < 0:
            raise ValueError("reference cg cannot run with tile_count == 0")
        return x, int(it), float(rel.value)

    @staticmethod
    def max_threads() -> int:
        L = ref()
        return int(L.dimref_max_threads()) if L is not None else 0
