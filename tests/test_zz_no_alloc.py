"""dimgpu_csr5_spmv_static_scratch: the SpMV entry point for callers that cannot allocate device memory
(its scratch is an array compiled into the library instead of a calibrator from cudaMalloc).

Called through the C ABI, twice in a row, and compared with the oracle (the reference's CSR SpMV
restated in C) within the f64 SpMV tolerance of the other tests; the second call must allocate nothing
on the device.  The matrix has rows that cross warp boundaries and empty rows, so the scratch
(calibrator slots, completion ticket) is exercised, and the second call runs on the scratch contents the
first call left behind.  A plan larger than the scratch is refused, and a failure a kernel records in
the scratch's status word survives later calls until dimgpu_static_scratch_status reads it.  This file
is collected last."""
import ctypes

import numpy as np
import pytest

import oracle
from diploma_research_gb300 import _native as N
from diploma_research_gb300.csr5 import csr5
from helpers import SPMV_RTOL_F64, assert_spmv_close, csr_from_lengths

pytestmark = pytest.mark.gpu


def test_static_scratch_spmv_matches_oracle(native, torch_cuda):
    torch = torch_cuda
    fn = native.dimgpu_csr5_spmv_static_scratch

    rng = np.random.default_rng(2024)
    lens = np.concatenate([rng.poisson(9, 40000), [0] * 500, [300000], rng.integers(0, 40, 30000), [0, 0, 70000]])
    m = csr_from_lengths(lens, 400000, rng)
    A = csr5.from_csr(m)
    n_rows, n_cols = m.dimensions.rows, m.dimensions.cols
    x_host = rng.uniform(-1, 1, n_cols)
    x = torch.tensor(x_host, device="cuda", dtype=torch.float64)
    y_ref = oracle.csr_spmv(n_rows, m.row_start_offsets, m.col_indices, m.values, x_host)
    absax = oracle.abs_spmv(n_rows, m.row_start_offsets, m.col_indices, m.values, x_host)

    ys = [torch.full((n_rows,), float("nan"), device="cuda", dtype=torch.float64) for _ in range(2)]
    torch.cuda.synchronize()
    free_before = None
    for call in range(2):
        if call == 1:
            free_before = torch.cuda.mem_get_info()[0]
        rc = fn(A._h, x.data_ptr(), ys[call].data_ptr(), None)
        assert rc == N.OK, native.dimgpu_last_error_string()
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before, "the second call allocated device memory"
        assert_spmv_close(ys[call].cpu().numpy(), y_ref, absax, SPMV_RTOL_F64)
    assert native.dimgpu_static_scratch_status(None) == N.OK


def test_static_scratch_refuses_a_plan_beyond_its_slots(native_test, torch_cuda):
    """A launch needing more than the 4096 warp slots of the array is refused before anything runs (no
    GB300 launch is that large, so the test library gives the matrix's plan 300 CTAs of 16 warps)."""
    torch, L = torch_cuda, native_test
    rng = np.random.default_rng(5)
    m = csr_from_lengths(rng.poisson(20, 50000), 50000, rng)
    h = ctypes.c_void_p()
    rc = L.dimgpu_csr5_from_csr(m.dimensions.rows, m.dimensions.cols, m.nnz, m.row_start_offsets.ctypes.data,
                                m.col_indices.ctypes.data, m.values.ctypes.data, N.MEM_HOST, None, None,
                                ctypes.byref(h))
    assert rc == N.OK, L.dimgpu_last_error_string()
    try:
        x = torch.zeros(m.dimensions.cols, device="cuda", dtype=torch.float64)
        y = torch.zeros(m.dimensions.rows, device="cuda", dtype=torch.float64)
        assert L.dimgpu_test_set_spmv_grid(h, 300) == N.OK
        rc = L.dimgpu_csr5_spmv_static_scratch(h, x.data_ptr(), y.data_ptr(), None)
        assert rc == N.ERR_INVALID_ARGUMENT
        assert b"4096" in L.dimgpu_last_error_string()
    finally:
        L.dimgpu_csr5_destroy(h)


def test_static_scratch_keeps_a_recorded_failure_until_read(native_test, torch_cuda):
    """A bounded look-back wait made to expire (the test library leaves one warp run's flag unwritten)
    is recorded in the array's status word; a later call does not clear it, the query reads and clears it,
    and the next call is correct."""
    torch, L = torch_cuda, native_test
    rng = np.random.default_rng(91)
    m = csr_from_lengths(rng.integers(3000, 6000, 500), 20000, rng)
    n, c = m.dimensions.rows, m.dimensions.cols
    h = ctypes.c_void_p()
    rc = L.dimgpu_csr5_from_csr(n, c, m.nnz, m.row_start_offsets.ctypes.data, m.col_indices.ctypes.data,
                                m.values.ctypes.data, N.MEM_HOST, None, None, ctypes.byref(h))
    assert rc == N.OK, L.dimgpu_last_error_string()
    x_h = rng.uniform(-1, 1, c)
    x = torch.tensor(x_h, device="cuda", dtype=torch.float64)
    y = torch.empty(n, device="cuda", dtype=torch.float64)
    try:
        assert L.dimgpu_static_scratch_status(None) == N.OK
        L.dimgpu_test_withhold_run(4)
        try:
            assert L.dimgpu_csr5_spmv_static_scratch(h, x.data_ptr(), y.data_ptr(), None) == N.OK
        finally:
            L.dimgpu_test_withhold_run(0xFFFFFFFF)
        assert L.dimgpu_csr5_spmv_static_scratch(h, x.data_ptr(), y.data_ptr(), None) == N.OK
        rc = L.dimgpu_static_scratch_status(None)
        assert rc == N.ERR_TIMEOUT, (rc, L.dimgpu_last_error_string())
        assert L.dimgpu_static_scratch_status(None) == N.OK
        y.fill_(float("nan"))
        assert L.dimgpu_csr5_spmv_static_scratch(h, x.data_ptr(), y.data_ptr(), None) == N.OK
        assert L.dimgpu_static_scratch_status(None) == N.OK
        y_ref = oracle.csr_spmv(n, m.row_start_offsets, m.col_indices, m.values, x_h)
        absax = oracle.abs_spmv(n, m.row_start_offsets, m.col_indices, m.values, x_h)
        assert_spmv_close(y.cpu().numpy(), y_ref, absax, SPMV_RTOL_F64)
    finally:
        L.dimgpu_csr5_destroy(h)
