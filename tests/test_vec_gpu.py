"""The vector helpers of the C ABI, dimgpu_vec_axpy / aypx / set / dot (the reference's vec::axpy,
vec::aypx, vec::set and dot, include/dim/vec.h:49-84), called directly and compared with numpy.

axpy and aypx compute one fused multiply-add per element, as GCC makes of the reference's
`a * x + y` under its default contraction: each result lies within one rounding of the exact value.
The dot product is summed in a fixed order, so it is compared with a tolerance scaled by sum |l r|
and checked to be bitwise repeatable."""
import ctypes

import numpy as np
import pytest

from diploma_research_gb300 import _native as N

pytestmark = pytest.mark.gpu

SIZES = [0, 1, 7, 256, 1000, 65537, 3_000_001]


def _dev(torch, a):
    return torch.tensor(a, device="cuda", dtype=torch.float64)


def _one_rounding(got, exact_parts):
    """|got - exact| <= 2^-53 |exact| + (the rounding of the product): bounded by eps * sum |parts|."""
    scale = sum(np.abs(p) for p in exact_parts)
    return np.all(np.abs(got - sum(exact_parts)) <= 2.3e-16 * scale + 1e-300)


@pytest.mark.parametrize("n", SIZES)
def test_axpy_aypx_set(native, torch_cuda, n):
    torch = torch_cuda
    rng = np.random.default_rng(n)
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    alpha = -0.3711
    xd, yd = _dev(torch, x), _dev(torch, y)
    N.check(native.dimgpu_vec_axpy(n, alpha, xd.data_ptr(), yd.data_ptr(), None))  # y += a x
    torch.cuda.synchronize()
    assert _one_rounding(yd.cpu().numpy(), [y, alpha * x])
    yd = _dev(torch, y)
    N.check(native.dimgpu_vec_aypx(n, alpha, xd.data_ptr(), yd.data_ptr(), None))  # y = x + a y
    torch.cuda.synchronize()
    assert _one_rounding(yd.cpu().numpy(), [x, alpha * y])
    N.check(native.dimgpu_vec_set(n, 2.5, yd.data_ptr(), None))
    torch.cuda.synchronize()
    assert np.all(yd.cpu().numpy() == 2.5)


@pytest.mark.parametrize("n", SIZES)
def test_dot(native, torch_cuda, n):
    torch = torch_cuda
    rng = np.random.default_rng(100 + n)
    l, r = rng.standard_normal(n), rng.standard_normal(n)
    ld, rd = _dev(torch, l), _dev(torch, r)
    out = ctypes.c_double()
    N.check(native.dimgpu_vec_dot(n, ld.data_ptr(), rd.data_ptr(), ctypes.byref(out), None))
    exact = float(np.dot(l.astype(np.longdouble), r.astype(np.longdouble))) if n else 0.0
    assert abs(out.value - exact) <= 1e-14 * float(np.abs(l * r).sum()) + 1e-300
    again = ctypes.c_double()
    N.check(native.dimgpu_vec_dot(n, ld.data_ptr(), rd.data_ptr(), ctypes.byref(again), None))
    assert out.value == again.value  # fixed summation order


def test_vec_argument_errors(native):
    assert native.dimgpu_vec_axpy(5, 1.0, None, None, None) == N.ERR_INVALID_ARGUMENT
    assert native.dimgpu_vec_dot(5, None, None, None, None) == N.ERR_INVALID_ARGUMENT
    assert native.dimgpu_vec_set(0, 1.0, None, None) == N.OK  # n = 0 touches nothing
