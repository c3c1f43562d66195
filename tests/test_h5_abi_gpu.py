"""The CSR5 group of the reference's HDF5 files through the C ABI: dimgpu_h5_store_csr5 (store,
libs/dim/io/h5.cpp:45-55) and dimgpu_h5_load_csr5 (load_csr5, h5.cpp:57-74).

store: a matrix converted on the device with the reference's layout (sigma 16, omega 4) is written; the
file must be byte-equal to the one the package's Python writer makes from the oracle's CSR5 arrays of
the same matrix (the oracle is pinned bit for bit to the reference's converter).  load: a stored group is
read back, its transposed tiles put back into CSR order and converted to the device layout; its SpMV is
compared with the oracle's.  Both directions run on a matrix with empty rows and long rows (dirty tiles,
tile_desc_offset entries) and on the reference's mm.mtx."""
import ctypes
import os

import numpy as np
import pytest

import oracle
from diploma_research_gb300 import _native as N
from diploma_research_gb300.io import h5
from diploma_research_gb300.mat import csr, dimensions_t
from helpers import SPMV_RTOL_F64, assert_spmv_close, random_csr

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _matrices():
    g = np.load(os.path.join(GOLDEN, "mm_mtx.npz"))
    yield "mm_mtx", csr(dimensions_t(int(g["rows"]), int(g["cols"])), g["vals"], g["row_ptr"], g["col_idx"])
    rng = np.random.default_rng(12)
    yield "ragged", random_csr(rng, 5000, 4200, 9.0, empty_frac=0.1, long_rows=3, long_len=(200, 2000))


def _oracle_arrays(m):
    o = oracle.OracleCSR5(m.dimensions.rows, m.dimensions.cols, m.row_start_offsets, m.col_indices, m.values, 16, 4)
    a = type("arrays", (), {})()
    a.vals, a.col_idx, a.row_ptr = o.vals[:m.nnz], o.col_idx[:m.nnz], m.row_start_offsets
    a.tile_ptr, a.tile_desc = o.tile_ptr, o.tile_desc.astype(np.uint32)
    a.tile_desc_offset_ptr, a.tile_desc_offset = o.tile_desc_offset_ptr, o.tile_desc_offset
    return a


def _from_csr(L, m, opt=None):
    h = ctypes.c_void_p()
    rc = L.dimgpu_csr5_from_csr(m.dimensions.rows, m.dimensions.cols, m.nnz, m.row_start_offsets.ctypes.data,
                                m.col_indices.ctypes.data, m.values.ctypes.data, N.MEM_HOST,
                                ctypes.byref(opt) if opt else None, None, ctypes.byref(h))
    assert rc == N.OK, L.dimgpu_last_error_string()
    return h


@pytest.mark.parametrize("which", ["mm_mtx", "ragged"])
def test_store_csr5_matches_the_python_writer(native, tmp_path, which):
    m = dict(_matrices())[which]
    L = native
    h = _from_csr(L, m, N.csr5_options(16, 4, 0, 0))  # the reference's layout
    try:
        pc, pp = tmp_path / "c.h5", tmp_path / "py.h5"
        assert L.dimgpu_h5_store_csr5(str(pc).encode(), b"A", h, 0) == N.OK, L.dimgpu_last_error_string()
        h5.store_csr5(pp, "A", _oracle_arrays(m), m.dimensions.cols)
        assert pc.read_bytes() == pp.read_bytes()
    finally:
        L.dimgpu_csr5_destroy(h)


def test_store_csr5_refuses_the_device_layout(native, tmp_path):
    m = dict(_matrices())["ragged"]
    h = _from_csr(native, m)
    try:
        rc = native.dimgpu_h5_store_csr5(str(tmp_path / "x.h5").encode(), b"A", h, 0)
        assert rc == N.ERR_INVALID_ARGUMENT and b"omega 4" in native.dimgpu_last_error_string()
    finally:
        native.dimgpu_csr5_destroy(h)


@pytest.mark.parametrize("which", ["mm_mtx", "ragged"])
def test_load_csr5_spmv_matches_the_oracle(native, torch_cuda, tmp_path, which):
    torch = torch_cuda
    m = dict(_matrices())[which]
    p = tmp_path / "m.h5"
    h5.store_csr5(p, "A", _oracle_arrays(m), m.dimensions.cols)
    h5.write_vector(p, "other", np.arange(5.0))  # another member beside the group
    L = native
    h = ctypes.c_void_p()
    assert L.dimgpu_h5_load_csr5(str(p).encode(), b"A", None, None, ctypes.byref(h)) == N.OK, \
        L.dimgpu_last_error_string()
    try:
        info = N.csr5_info()
        assert L.dimgpu_csr5_get_info(h, ctypes.byref(info)) == N.OK
        assert (info.rows, info.cols, info.nnz, info.omega) == (m.dimensions.rows, m.dimensions.cols, m.nnz, 32)
        # the arrays put back into CSR order are the original ones
        rp = np.zeros(m.dimensions.rows + 1, np.uint32)
        assert L.dimgpu_csr5_export(h, None, None, None, None, None, None, rp.ctypes.data) == N.OK
        assert np.array_equal(rp, m.row_start_offsets)
        x_h = np.random.default_rng(1).uniform(-1, 1, m.dimensions.cols)
        x = torch.tensor(x_h, device="cuda", dtype=torch.float64)
        y = torch.full((m.dimensions.rows,), float("nan"), device="cuda", dtype=torch.float64)
        assert L.dimgpu_csr5_spmv(h, x.data_ptr(), y.data_ptr(), None, None) == N.OK
        torch.cuda.synchronize()
        n = m.dimensions.rows
        y_ref = oracle.csr_spmv(n, m.row_start_offsets, m.col_indices, m.values, x_h)
        absax = oracle.abs_spmv(n, m.row_start_offsets, m.col_indices, m.values, x_h)
        assert_spmv_close(y.cpu().numpy(), y_ref, absax, SPMV_RTOL_F64)
    finally:
        L.dimgpu_csr5_destroy(h)


def test_store_then_load_round_trip(native, tmp_path):
    """C store, C load: the reference-layout handle's arrays survive the file and come back in CSR order."""
    m = dict(_matrices())["ragged"]
    L = native
    h = _from_csr(L, m, N.csr5_options(16, 4, 0, 0))
    p = tmp_path / "rt.h5"
    try:
        assert L.dimgpu_h5_store_csr5(str(p).encode(), b"grp/A", h, 0) == N.OK, L.dimgpu_last_error_string()
    finally:
        L.dimgpu_csr5_destroy(h)
    h2 = ctypes.c_void_p()
    opt = N.csr5_options(16, 4, 0, 0)
    assert L.dimgpu_h5_load_csr5(str(p).encode(), b"grp/A", ctypes.byref(opt), None, ctypes.byref(h2)) == N.OK
    try:
        info = N.csr5_info()
        assert L.dimgpu_csr5_get_info(h2, ctypes.byref(info)) == N.OK
        o = oracle.OracleCSR5(m.dimensions.rows, m.dimensions.cols, m.row_start_offsets, m.col_indices, m.values,
                              16, 4)
        tp = np.zeros(info.tile_count + 1, np.uint32)
        vals = np.zeros(m.nnz)
        assert L.dimgpu_csr5_export(h2, tp.ctypes.data, None, None, None, vals.ctypes.data, None, None) == N.OK
        assert np.array_equal(tp, o.tile_ptr) and np.array_equal(vals, o.vals[:m.nnz])
    finally:
        L.dimgpu_csr5_destroy(h2)
