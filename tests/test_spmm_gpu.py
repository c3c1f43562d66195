"""CSR5 SpMM (k right-hand sides) through the C ABI against a CSR reference, f64 and f32."""
import numpy as np
import pytest

from diploma_research_gb300.csr5 import csr5, set_spmm_shape, spmm, spmm_shape
from helpers import csr_from_lengths, random_csr

pytestmark = pytest.mark.gpu

U32 = 2.0 ** -24  # unit roundoff of f32


def _f32_bound(m, AX):
    """Componentwise bound of an f32 product of rows of n elements: each of the n products and n - 1 sums
    rounds once, so |y - y_exact| <= gamma_(n+1) (|A||X|) with gamma_j = j u / (1 - j u)."""
    n = np.diff(m.row_start_offsets.astype(np.int64)).astype(np.float64)[:, None] + 1.0
    return n * U32 / (1.0 - n * U32) * AX


def _check(torch, m, k, seed=0, f32=False, A=None, shape=None):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1, 1, (m.dimensions.cols, k))
    S = m.to_scipy()
    Y_ref = S @ X
    AX = abs(S) @ np.abs(X)
    if A is None:
        A = csr5.from_csr(m)
    if shape is not None:
        set_spmm_shape(A, min(k, 32), shape, f32)
    dt = torch.float32 if f32 else torch.float64
    Xd = torch.tensor(X, device="cuda", dtype=dt)
    Yd = torch.full((m.dimensions.rows, k), float("nan"), device="cuda", dtype=dt)
    spmm(A, Xd, Yd)
    torch.cuda.synchronize()
    Y = Yd.cpu().numpy().astype(np.float64)
    if f32:
        # the exact product of the f32-rounded operands (values and X), and the f32 rounding bound
        S32 = S.copy()
        S32.data = S32.data.astype(np.float32).astype(np.float64)
        X32 = X.astype(np.float32).astype(np.float64)
        Y_ref = S32 @ X32
        bound = _f32_bound(m, abs(S32) @ np.abs(X32))
    else:
        bound = 1e-12 * AX
    err = np.abs(Y - Y_ref)
    assert np.all(err <= bound + 1e-300), float(np.max(err / (bound + 1e-300)))
    assert 0 <= spmm_shape(A, min(k, 32), f32) < 6
    return A


@pytest.mark.parametrize("k", [1, 3, 5, 8, 12, 16, 24, 32, 40])
def test_spmm_random(native, torch_cuda, k):
    rng = np.random.default_rng(k)
    m = random_csr(rng, 5000, 4000, 12.0, empty_frac=0.1, long_rows=3, long_len=(700, 3000))
    _check(torch_cuda, m, k, seed=k)


@pytest.mark.parametrize("k", [2, 6, 8, 12, 20, 28, 32])
def test_spmm_f32(native, torch_cuda, k):
    """f32 at widths where the vector lanes leave lanes of a group idle (k = 2, 6: two values per lane;
    12, 20, 28: four) and where they fill it; the autotuned shape, then every shape pinned."""
    rng = np.random.default_rng(100 + k)
    m = random_csr(rng, 3000, 3000, 9.0, empty_frac=0.05, long_rows=2, long_len=(600, 2000))
    A = _check(torch_cuda, m, k, seed=k, f32=True)
    for shape in range(6):
        _check(torch_cuda, m, k, seed=k + shape, f32=True, A=A, shape=shape)


@pytest.mark.parametrize("f32", [False, True])
@pytest.mark.parametrize("k", [5, 8, 16, 24, 32])
def test_spmm_every_shape(native, torch_cuda, k, f32):
    """Every shape the autotuner may choose (launch shape x lane grouping), pinned, against the reference
    product; groupings that do not apply to the operands fall back to grouping 0."""
    rng = np.random.default_rng(200 + k)
    m = random_csr(rng, 4000, 3500, 10.0, empty_frac=0.05, long_rows=3, long_len=(600, 3000))
    A = csr5.from_csr(m)
    for shape in range(6):
        _check(torch_cuda, m, k, seed=shape, f32=f32, A=A, shape=shape)


@pytest.mark.parametrize("lens,cols", [([3, 0, 5, 1], 10), ([0, 0, 0], 4), ([20000], 20000),
                                       ([0] * 50 + [512] + [0] * 50, 600), ([1] * 4096, 3)])
def test_spmm_edge_cases(native, torch_cuda, lens, cols):
    rng = np.random.default_rng(len(lens))
    m = csr_from_lengths(lens, cols, rng)
    _check(torch_cuda, m, 8, seed=1)


def test_spmm_matches_spmv_columns(native, torch_cuda):
    """Column j of A X equals the SpMV of column j (within f64 rounding)."""
    torch = torch_cuda
    from diploma_research_gb300.generators import laplacian_3d_7pt

    m = laplacian_3d_7pt(24)
    A = csr5.from_csr(m)
    rng = np.random.default_rng(3)
    X = torch.tensor(rng.uniform(-1, 1, (m.dimensions.cols, 16)), device="cuda", dtype=torch.float64)
    Y = torch.empty((m.dimensions.rows, 16), device="cuda", dtype=torch.float64)
    spmm(A, X, Y)
    for j in (0, 7, 15):
        y = torch.empty(m.dimensions.rows, device="cuda", dtype=torch.float64)
        A.spmv(X[:, j].contiguous(), y)
        torch.cuda.synchronize()
        assert torch.allclose(Y[:, j], y, rtol=0, atol=1e-13)


@pytest.mark.parametrize("f32", [True, False])
@pytest.mark.parametrize("ldx,ldy,offset", [(10, 11, 0), (9, 8, 0), (8, 8, 1), (12, 16, 2)])
def test_spmm_strided_and_unaligned_operands(native, torch_cuda, f32, ldx, ldy, offset):
    """k = 8 right-hand sides in wider row-major buffers (leading dimensions ldx, ldy) starting `offset`
    elements into them: the lane widths the operands do not allow (vector accesses need k, both leading
    dimensions and both base addresses to fit them) fall back to narrower lanes; every shape, pinned,
    gives the product."""
    import ctypes

    from diploma_research_gb300 import _native as N

    torch = torch_cuda
    k = 8
    rng = np.random.default_rng(ldx * 100 + ldy * 10 + offset)
    m = random_csr(rng, 3000, 2500, 8.0, empty_frac=0.05, long_rows=2, long_len=(600, 2000))
    A = csr5.from_csr(m)
    dt, npdt = (torch.float32, np.float32) if f32 else (torch.float64, np.float64)
    X = rng.uniform(-1, 1, (m.dimensions.cols, k)).astype(npdt)
    Xb = torch.zeros((m.dimensions.cols * ldx + offset + ldx,), device="cuda", dtype=dt)
    Xb[offset:offset + m.dimensions.cols * ldx].view(m.dimensions.cols, ldx)[:, :k] = torch.tensor(X, device="cuda")
    Yb = torch.full((m.dimensions.rows * ldy + offset + ldy,), float("nan"), device="cuda", dtype=dt)
    esz = 4 if f32 else 8
    fn = native.dimgpu_csr5_spmm_f32 if f32 else native.dimgpu_csr5_spmm
    S = m.to_scipy()
    if f32:
        S.data = S.data.astype(np.float32).astype(np.float64)
    Xe = X.astype(np.float64)
    Y_ref = S @ Xe
    bound = (_f32_bound(m, abs(S) @ np.abs(Xe)) if f32 else 1e-12 * (abs(S) @ np.abs(Xe))) + 1e-300
    for shape in range(6):
        set_spmm_shape(A, k, shape, f32)
        Yb.fill_(float("nan"))
        rc = fn(A._h, k, Xb.data_ptr() + offset * esz, ldx, Yb.data_ptr() + offset * esz, ldy, None)
        assert rc == N.OK, native.dimgpu_last_error_string()
        torch.cuda.synchronize()
        Y = Yb[offset:offset + m.dimensions.rows * ldy].view(m.dimensions.rows, ldy)[:, :k].cpu().numpy()
        err = np.abs(Y.astype(np.float64) - Y_ref)
        assert np.all(err <= bound), (shape, float(np.max(err / bound)))
