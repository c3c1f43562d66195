"""dimgpu_csr5_spmv_static_scratch: the SpMV entry point for callers that cannot allocate device memory
(its scratch is an array compiled into the library instead of a calibrator from cudaMalloc).

Called through the C ABI, twice in a row, and compared with dimgpu_csr5_spmv on the same matrix and
input, within the f64 SpMV tolerance of the other tests.  The matrix has rows that cross warp
boundaries and empty rows, so the scratch (calibrator slots, completion ticket) is exercised, and the
second call runs on the scratch contents the first call left behind.  This file is collected last."""
import ctypes

import numpy as np
import pytest

import oracle
from diploma_research_gb300 import _native as N
from diploma_research_gb300.csr5 import csr5
from helpers import SPMV_RTOL_F64, assert_spmv_close, csr_from_lengths

pytestmark = pytest.mark.gpu


def test_static_scratch_spmv_matches_calibrator_spmv(native, torch_cuda):
    torch = torch_cuda
    fn = native.dimgpu_csr5_spmv_static_scratch
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int

    rng = np.random.default_rng(2024)
    lens = np.concatenate([rng.poisson(9, 40000), [0] * 500, [300000], rng.integers(0, 40, 30000), [0, 0, 70000]])
    m = csr_from_lengths(lens, 400000, rng)
    A = csr5.from_csr(m)
    n_rows, n_cols = m.dimensions.rows, m.dimensions.cols
    x_host = rng.uniform(-1, 1, n_cols)
    x = torch.tensor(x_host, device="cuda", dtype=torch.float64)

    y_ref = torch.full((n_rows,), float("nan"), device="cuda", dtype=torch.float64)
    A.spmv(x, y_ref)  # the existing entry point, with the matrix's own calibrator
    torch.cuda.synchronize()
    y_ref = y_ref.cpu().numpy()
    absax = oracle.abs_spmv(n_rows, m.row_start_offsets, m.col_indices, m.values, x_host)

    for call in range(2):
        y = torch.full((n_rows,), float("nan"), device="cuda", dtype=torch.float64)
        rc = fn(A._h, x.data_ptr(), y.data_ptr(), None)
        assert rc == N.OK, native.dimgpu_last_error_string()
        torch.cuda.synchronize()
        assert_spmv_close(y.cpu().numpy(), y_ref, absax, SPMV_RTOL_F64)
