"""Differentiation through x = A^{-1} b (the adjoint variant of the solver; the reference has none).

For a loss L(x) with g = dL/dx:  lambda = A^{-T} g,  dL/db = lambda,  dL/dA = -lambda x^T on the pattern.
All arrays are device arrays (``__cuda_array_interface__``, float64); gradients of A come in the CSR
order of the matrix given to ``csr5.from_csr``.
"""
from __future__ import annotations

import ctypes

from . import _native as N
from .cg import _PREC, cg_result
from .csr5 import csr5


def spmv_transpose(A: csr5, x, y, stream=None):
    """y := A^T x (A^T is built inside A on first use)."""
    N.check(N.lib().dimgpu_csr5_spmv_transpose(A._h, N.device_ptr(x, "<f8", A.dimensions.rows),
                                               N.device_ptr(y, "<f8", A.dimensions.cols), N.stream_ptr(stream)))
    return y


def pattern_outer(A: csr5, u, v, scale, out, stream=None):
    """out[e] := scale * u[row(e)] * v[col(e)] over the stored entries (CSR order)."""
    N.check(N.lib().dimgpu_csr5_pattern_outer(A._h, N.device_ptr(u, "<f8"), N.device_ptr(v, "<f8"), float(scale),
                                              N.device_ptr(out, "<f8", A.non_zero_count()), N.stream_ptr(stream)))
    return out


def cg_adjoint(A: csr5, g, x, lam, grad_vals=None, tol: float = 1e-10, max_it: int = 100000,
               precision: str = "fp64", stream=None, raise_on_failure: bool = True, reliable_delta: float = 0.1,
               engine: str = "auto"):
    """lambda := A^{-T} g by CG on A^T (lam holds the initial guess), grad_vals := -lambda x^T on the
    pattern.  Returns cg_result of the adjoint solve.  reliable_delta: mixed precision only (the residual
    drop between f64 residual replacements)."""
    from .cg import _ENGINE

    p = N.cg_params(float(tol), int(max_it), _PREC[precision], 1, float(reliable_delta), _ENGINE[engine])
    st = N.cg_stats()
    rc = N.lib().dimgpu_cg_adjoint(A._h, N.device_ptr(g, "<f8"), N.device_ptr(x, "<f8"), N.device_ptr(lam, "<f8"),
                                   N.device_ptr(grad_vals, "<f8") if grad_vals is not None else None,
                                   ctypes.byref(p), ctypes.byref(st), N.stream_ptr(stream))
    res = cg_result(int(st.iterations), int(st.reliable_updates), float(st.rel_residual),
                    float(st.recurrence_rel_residual), float(st.seconds), rc == N.OK)
    if rc != N.OK and (raise_on_failure or rc != N.ERR_NOT_CONVERGED):
        N.check(rc)
    return res
