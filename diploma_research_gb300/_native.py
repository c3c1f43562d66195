"""Loads libdimgpu.so (the CUDA kernels behind the C ABI of include/dimgpu.h) and declares its signatures.

There is no fallback: if the library is missing or cannot be loaded, importing anything that needs
it raises.  Build it with ``python -c "import __graft_entry__ as g; g.build()"`` or
``python -m diploma_research_gb300.build``.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libdimgpu.so")

OK = 0
ERR_INVALID_ARGUMENT = -1
ERR_CUDA = -2
ERR_OUT_OF_MEMORY = -3
ERR_TIMEOUT = -4
ERR_BREAKDOWN = -5
ERR_NOT_CONVERGED = -6
ERR_UNSUPPORTED = -7
ERR_BAD_INDEX = -8
ERR_IO = -9

MEM_HOST = 0
MEM_DEVICE = 1

CG_FP64 = 0
CG_MIXED = 1

TEST_LIB_PATH = os.path.join(HERE, "_lib", "libdimgpu_test.so")

_lock = threading.Lock()
_lib = None
_test_lib = None


class csr5_options(ctypes.Structure):
    _fields_ = [("sigma", ctypes.c_uint32), ("omega", ctypes.c_uint32), ("layout", ctypes.c_int32),
                ("flags", ctypes.c_uint32)]


class csr5_info(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_uint32), ("cols", ctypes.c_uint32), ("nnz", ctypes.c_uint64),
                ("sigma", ctypes.c_uint32), ("omega", ctypes.c_uint32), ("layout", ctypes.c_int32),
                ("desc_word_bytes", ctypes.c_uint32), ("tile_count", ctypes.c_uint64),
                ("tile_desc_offset_len", ctypes.c_uint64), ("tail_partition_start", ctypes.c_uint32),
                ("empty_rows", ctypes.c_uint32), ("device_bytes", ctypes.c_uint64)]


class cg_params(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("max_it", ctypes.c_int64), ("precision", ctypes.c_int32),
                ("use_graph", ctypes.c_int32), ("reliable_delta", ctypes.c_double), ("engine", ctypes.c_int32)]


CG_ENGINE_AUTO, CG_ENGINE_GRAPH = 0, 1


class cg_stats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int64), ("reliable_updates", ctypes.c_int64),
                ("rel_residual", ctypes.c_double), ("recurrence_rel_residual", ctypes.c_double),
                ("seconds", ctypes.c_double), ("status", ctypes.c_int32)]


class block_cg_stats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int64), ("reliable_updates", ctypes.c_int64),
                ("max_rel_residual", ctypes.c_double), ("seconds", ctypes.c_double),
                ("converged_columns", ctypes.c_int32), ("status", ctypes.c_int32), ("spmm_shape", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class DimgpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"dimgpu error {code}: {msg}")
        self.code = code


class BreakdownError(DimgpuError):
    pass


class NotConvergedError(DimgpuError):
    pass


class DeviceTimeoutError(DimgpuError):
    pass


_vp = ctypes.c_void_p
_u32 = ctypes.c_uint32
_u64 = ctypes.c_uint64
_i32 = ctypes.c_int32
_f64 = ctypes.c_double

# name -> argtypes (all functions return int unless noted)
_SIGNATURES = {
    "dimgpu_csr5_from_csr": [_u32, _u32, _u64, _vp, _vp, _vp, ctypes.c_int, ctypes.POINTER(csr5_options), _vp,
                             ctypes.POINTER(_vp)],
    "dimgpu_csr5_destroy": [_vp],
    "dimgpu_csr5_get_info": [_vp, ctypes.POINTER(csr5_info)],
    "dimgpu_csr5_export": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "dimgpu_calibrator_create": [_vp, ctypes.POINTER(_vp)],
    "dimgpu_calibrator_destroy": [_vp],
    "dimgpu_csr5_spmv": [_vp, _vp, _vp, _vp, _vp],
    "dimgpu_csr5_spmv_host": [_vp, _vp, _vp],
    "dimgpu_csr5_spmv_dot": [_vp, _vp, _vp, _vp, _vp, _vp],
    "dimgpu_csr5_get_spmv_launch": [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int)],
    "dimgpu_csr5_set_spmv_launch": [_vp, ctypes.c_int, ctypes.c_uint32, ctypes.c_int],
    "dimgpu_csr5_spmv_f32": [_vp, _vp, _vp, _vp, _vp],
    "dimgpu_csr5_spmm": [_vp, _u32, _vp, _u64, _vp, _u64, _vp],
    "dimgpu_csr5_spmm_f32": [_vp, _u32, _vp, _u64, _vp, _u64, _vp],
    "dimgpu_csr5_spmm_shape": [_vp, _u32, ctypes.c_int, ctypes.POINTER(ctypes.c_int)],
    "dimgpu_csr5_set_spmm_shape": [_vp, _u32, ctypes.c_int, ctypes.c_int],
    "dimgpu_vec_axpy": [_u64, _f64, _vp, _vp, _vp],
    "dimgpu_vec_aypx": [_u64, _f64, _vp, _vp, _vp],
    "dimgpu_vec_set": [_u64, _f64, _vp, _vp],
    "dimgpu_vec_dot": [_u64, _vp, _vp, ctypes.POINTER(_f64), _vp],
    "dimgpu_cg_create": [_vp, ctypes.POINTER(cg_params), _vp, ctypes.POINTER(_vp)],
    "dimgpu_cg_destroy": [_vp],
    "dimgpu_cg_solve": [_vp, _vp, _vp, ctypes.POINTER(cg_stats), _vp],
    "dimgpu_cg_solve_host": [_vp, _vp, _vp, ctypes.POINTER(cg_stats)],
    "dimgpu_block_cg_create": [_vp, _u32, ctypes.POINTER(cg_params), _vp, ctypes.POINTER(_vp)],
    "dimgpu_block_cg_destroy": [_vp],
    "dimgpu_block_cg_solve": [_vp, _vp, _u64, _vp, _u64, ctypes.POINTER(block_cg_stats), _vp, _vp, _vp],
    "dimgpu_csr5_transpose": [_vp, _vp, ctypes.POINTER(_vp)],
    "dimgpu_csr5_spmv_transpose": [_vp, _vp, _vp, _vp],
    "dimgpu_csr5_pattern_outer": [_vp, _vp, _vp, _f64, _vp, _vp],
    "dimgpu_cg_adjoint": [_vp, _vp, _vp, _vp, _vp, ctypes.POINTER(cg_params), ctypes.POINTER(cg_stats), _vp],
    "dimgpu_csr5_status": [_vp, _vp, _vp],
    "dimgpu_static_scratch_status": [_vp],
    "dimgpu_csr5_spmv_static_scratch": [_vp, _vp, _vp, _vp],
    "dimgpu_version": [],
    "dimgpu_h5_csr_dimensions": [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_u32), ctypes.POINTER(_u32),
                                 ctypes.POINTER(_u64)],
    "dimgpu_h5_read_matlab_compatible": [ctypes.c_char_p, ctypes.c_char_p, _vp, _vp, _vp],
    "dimgpu_h5_write_matlab_compatible": [ctypes.c_char_p, ctypes.c_char_p, _u32, _u32, _u64, _vp, _vp, _vp,
                                          ctypes.c_int],
    "dimgpu_h5_store_csr5": [ctypes.c_char_p, ctypes.c_char_p, _vp, ctypes.c_int],
    "dimgpu_h5_load_csr5": [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(csr5_options), _vp, ctypes.POINTER(_vp)],
    "dimgpu_h5_vector_length": [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_u64)],
    "dimgpu_h5_read_vector": [ctypes.c_char_p, ctypes.c_char_p, _vp],
    "dimgpu_h5_write_vector": [ctypes.c_char_p, ctypes.c_char_p, _u64, _vp, ctypes.c_int],
    "dimgpu_mm_csr_dimensions": [ctypes.c_char_p, ctypes.POINTER(_u32), ctypes.POINTER(_u32), ctypes.POINTER(_u64)],
    "dimgpu_mm_read_csr": [ctypes.c_char_p, _vp, _vp, _vp],
}


def declared_symbols():
    """Every entry point include/dimgpu.h declares."""
    import re

    hdr = os.path.join(os.path.dirname(HERE), "include", "dimgpu.h")
    with open(hdr) as fh:
        return re.findall(r"DIMGPU_API\s+(?:const\s+)?\w+\*?\s+\*?(dimgpu_\w+)\(", fh.read())


def _load(path):
    L = ctypes.CDLL(path)
    for name, args in _SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.dimgpu_last_error_string.argtypes = []
    L.dimgpu_last_error_string.restype = ctypes.c_char_p
    return L


def lib():
    """The loaded library; raises when it is missing (there is no CPU fallback)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.isfile(LIB_PATH):
                raise ImportError(f"{LIB_PATH} is missing: build it with diploma_research_gb300.build.build()")
            _lib = _load(LIB_PATH)
    return _lib


def test_lib():
    """libdimgpu_test.so: the same library built with test hooks and 20 ms device waits.  Only the
    tests of the device status words load it; its handles must not be passed to lib()'s functions."""
    global _test_lib
    with _lock:
        if _test_lib is None:
            if not os.path.isfile(TEST_LIB_PATH):
                raise ImportError(f"{TEST_LIB_PATH} is missing: build it with build(variant='test')")
            L = _load(TEST_LIB_PATH)
            L.dimgpu_test_withhold_run.argtypes = [_u32]
            L.dimgpu_test_withhold_run.restype = None
            L.dimgpu_test_set_spmv_grid.argtypes = [_vp, ctypes.c_int]
            L.dimgpu_test_set_spmv_grid.restype = ctypes.c_int
            _test_lib = L
    return _test_lib


def check(rc: int) -> int:
    if rc == OK:
        return rc
    msg = lib().dimgpu_last_error_string().decode(errors="replace")
    if rc == ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    if rc == ERR_BREAKDOWN:
        raise BreakdownError(rc, msg)
    if rc == ERR_NOT_CONVERGED:
        raise NotConvergedError(rc, msg)
    if rc == ERR_TIMEOUT:
        raise DeviceTimeoutError(rc, msg)
    raise DimgpuError(rc, msg)


def device_ptr(a, dtype_str: str | None = None, min_len: int | None = None) -> int:
    """Device address of an object with __cuda_array_interface__ (torch CUDA tensors, CuPy, ...).

    Checks the element type (numpy-style typestr, e.g. '<f8') and contiguity."""
    if isinstance(a, int):
        return a
    cai = getattr(a, "__cuda_array_interface__", None)
    if cai is None:
        raise TypeError("expected a device array (an object exposing __cuda_array_interface__)")
    if dtype_str is not None and cai["typestr"] != dtype_str:
        raise TypeError(f"device array has element type {cai['typestr']}, expected {dtype_str}")
    shape = cai["shape"]
    strides = cai.get("strides")
    if strides is not None:
        expect = int(cai["typestr"][2:])
        for dim, st in zip(reversed(shape), reversed(strides)):
            if dim > 1 and st != expect:
                raise ValueError("device array must be C-contiguous")
            expect *= dim
    if min_len is not None:
        n = 1
        for d in shape:
            n *= d
        if n < min_len:
            raise ValueError(f"device array has {n} elements, needs {min_len}")
    return int(cai["data"][0])


def is_device_array(a) -> bool:
    return isinstance(a, int) or hasattr(a, "__cuda_array_interface__")


def stream_ptr(stream) -> int:
    """A cudaStream_t from None, an int, or an object with .cuda_stream (torch.cuda.Stream)."""
    if stream is None:
        return 0
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream"))
