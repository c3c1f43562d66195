"""Device-side failures of asynchronous calls reach the caller through dimgpu_csr5_status.

Every wait inside the kernels is bounded.  These tests make one such wait run out on purpose, without
faulting or hanging anything: they load libdimgpu_test.so, the same sources built with DIMGPU_TEST_HOOKS
and a 20 ms wait limit, and tell it to leave one warp run's look-back flag unwritten.  The run after it,
which needs that run's row fragment, waits 20 ms, records a timeout in the status word of the scratch
it ran on and returns; the launch completes.  The query must then report DIMGPU_ERR_TIMEOUT and clear
the word, and the next product on the same scratch must be correct again.  (The reference reports its
failures by exception, csr5.h:820-821.)"""
import ctypes

import numpy as np
import pytest

import oracle
from diploma_research_gb300 import _native as N
from helpers import SPMV_RTOL_F64, assert_spmv_close, csr_from_lengths

pytestmark = pytest.mark.gpu

NONE = 0xFFFFFFFF


def _long_rows_matrix(rng):
    """Rows of 3000-6000 elements: every warp run (2 tiles = 1024 elements at this size) ends inside a
    row, so each run's successor looks back at it."""
    lens = rng.integers(3000, 6000, 500)
    return csr_from_lengths(lens, 20000, rng)


def _from_csr(L, m):
    h = ctypes.c_void_p()
    rp, ci, v = m.row_start_offsets, m.col_indices, m.values
    rc = L.dimgpu_csr5_from_csr(m.dimensions.rows, m.dimensions.cols, m.nnz, rp.ctypes.data, ci.ctypes.data,
                                v.ctypes.data, N.MEM_HOST, None, None, ctypes.byref(h))
    assert rc == N.OK, L.dimgpu_last_error_string()
    return h


@pytest.mark.parametrize("own_calibrator", [False, True])
def test_expired_lookback_wait_is_reported_then_cleared(native_test, torch_cuda, own_calibrator):
    torch, L = torch_cuda, native_test
    rng = np.random.default_rng(77)
    m = _long_rows_matrix(rng)
    n, c = m.dimensions.rows, m.dimensions.cols
    x_h = rng.uniform(-1, 1, c)
    y_ref = oracle.csr_spmv(n, m.row_start_offsets, m.col_indices, m.values, x_h)
    absax = oracle.abs_spmv(n, m.row_start_offsets, m.col_indices, m.values, x_h)
    h = _from_csr(L, m)
    cal = ctypes.c_void_p()
    if not own_calibrator:
        assert L.dimgpu_calibrator_create(h, ctypes.byref(cal)) == N.OK
    calp = None if own_calibrator else cal
    x = torch.tensor(x_h, device="cuda", dtype=torch.float64)
    y = torch.empty(n, device="cuda", dtype=torch.float64)
    try:
        # a clean product first: the query reports nothing
        assert L.dimgpu_csr5_spmv(h, x.data_ptr(), y.data_ptr(), calp, None) == N.OK
        assert L.dimgpu_csr5_status(h, calp, None) == N.OK
        assert_spmv_close(y.cpu().numpy(), y_ref, absax, SPMV_RTOL_F64)

        L.dimgpu_test_withhold_run(3)
        try:
            assert L.dimgpu_csr5_spmv(h, x.data_ptr(), y.data_ptr(), calp, None) == N.OK  # asynchronous
        finally:
            L.dimgpu_test_withhold_run(NONE)
        rc = L.dimgpu_csr5_status(h, calp, None)
        assert rc == N.ERR_TIMEOUT, (rc, L.dimgpu_last_error_string())
        assert b"bounded device wait" in L.dimgpu_last_error_string()
        # the query cleared the word
        assert L.dimgpu_csr5_status(h, calp, None) == N.OK

        # the same scratch works again
        y.fill_(float("nan"))
        assert L.dimgpu_csr5_spmv(h, x.data_ptr(), y.data_ptr(), calp, None) == N.OK
        assert L.dimgpu_csr5_status(h, calp, None) == N.OK
        assert_spmv_close(y.cpu().numpy(), y_ref, absax, SPMV_RTOL_F64)
    finally:
        if not own_calibrator:
            L.dimgpu_calibrator_destroy(cal)
        L.dimgpu_csr5_destroy(h)


def test_host_entry_point_returns_the_timeout(native_test):
    """dimgpu_csr5_spmv_host reads the status word itself and returns the code."""
    L = native_test
    rng = np.random.default_rng(78)
    m = _long_rows_matrix(rng)
    n, c = m.dimensions.rows, m.dimensions.cols
    x_h = rng.uniform(-1, 1, c)
    y_h = np.empty(n)
    h = _from_csr(L, m)
    try:
        L.dimgpu_test_withhold_run(2)
        try:
            rc = L.dimgpu_csr5_spmv_host(h, x_h.ctypes.data, y_h.ctypes.data)
        finally:
            L.dimgpu_test_withhold_run(NONE)
        assert rc == N.ERR_TIMEOUT, (rc, L.dimgpu_last_error_string())
        assert L.dimgpu_csr5_spmv_host(h, x_h.ctypes.data, y_h.ctypes.data) == N.OK
        y_ref = oracle.csr_spmv(n, m.row_start_offsets, m.col_indices, m.values, x_h)
        absax = oracle.abs_spmv(n, m.row_start_offsets, m.col_indices, m.values, x_h)
        assert_spmv_close(y_h, y_ref, absax, SPMV_RTOL_F64)
    finally:
        L.dimgpu_csr5_destroy(h)


def test_status_of_a_clean_matrix_is_ok(native, torch_cuda):
    """The product library: after ordinary products (own calibrator, SpMM) the query reports nothing."""
    torch = torch_cuda
    from diploma_research_gb300.csr5 import csr5, spmm

    rng = np.random.default_rng(79)
    m = _long_rows_matrix(rng)
    A = csr5.from_csr(m)
    x = torch.tensor(rng.uniform(-1, 1, m.dimensions.cols), device="cuda", dtype=torch.float64)
    y = torch.empty(m.dimensions.rows, device="cuda", dtype=torch.float64)
    A.spmv(x, y)
    X = torch.tensor(rng.uniform(-1, 1, (m.dimensions.cols, 4)), device="cuda", dtype=torch.float64)
    Y = torch.empty((m.dimensions.rows, 4), device="cuda", dtype=torch.float64)
    spmm(A, X, Y)
    assert native.dimgpu_csr5_status(A._h, None, None) == N.OK
    cal = A.create_calibrator()
    A.spmv(x, y, cal)
    assert native.dimgpu_csr5_status(A._h, cal._h, None) == N.OK
