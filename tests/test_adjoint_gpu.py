"""Differentiation through the CG solve: transpose SpMV, gradients on the pattern, adjoint CG, checked
against an FP64 CPU reference gradient and central finite differences.  The torch.autograd.Function
below exists only in this test harness."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from diploma_research_gb300.adjoint import cg_adjoint, pattern_outer, spmv_transpose
from diploma_research_gb300.cg import CGSolver
from diploma_research_gb300.csr5 import csr5
from diploma_research_gb300.generators import anisotropic_2d
from diploma_research_gb300.mat import csr
from helpers import random_csr

pytestmark = pytest.mark.gpu


def test_spmv_transpose(native, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(21)
    m = random_csr(rng, 3000, 2000, 11.0, empty_frac=0.1, long_rows=3, long_len=(600, 1900))
    A = csr5.from_csr(m)
    x = rng.uniform(-1, 1, 3000)
    xd = torch.tensor(x, device="cuda", dtype=torch.float64)
    yd = torch.full((2000,), float("nan"), device="cuda", dtype=torch.float64)
    spmv_transpose(A, xd, yd)
    torch.cuda.synchronize()
    S = m.to_scipy()
    ref = S.T @ x
    scale = abs(S.T) @ np.abs(x)
    assert np.all(np.abs(yd.cpu().numpy() - ref) <= 1e-12 * scale + 1e-300)


def test_pattern_outer(native, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(22)
    m = random_csr(rng, 1500, 1700, 9.0, empty_frac=0.2, long_rows=2, long_len=(600, 1600))
    A = csr5.from_csr(m)
    u, v = rng.standard_normal(1500), rng.standard_normal(1700)
    out = torch.empty(m.nnz, device="cuda", dtype=torch.float64)
    pattern_outer(A, torch.tensor(u, device="cuda"), torch.tensor(v, device="cuda"), -1.0, out)
    rows = np.repeat(np.arange(1500), np.diff(m.row_start_offsets.astype(np.int64)))
    ref = -u[rows] * v[m.col_indices]
    assert np.array_equal(out.cpu().numpy(), ref)


def _problem(mgrid=24, seed=4, ell=4.0):
    m, _ = anisotropic_2d(mgrid, ell=ell, variance=1.0, ratio=10.0, seed=seed)
    rng = np.random.default_rng(seed + 100)
    n = m.dimensions.rows
    b = rng.uniform(-1, 1, n)
    xt = rng.uniform(-1, 1, n)
    return m, b, xt


class _Solve:
    """Forward/backward of x = A(vals)^{-1} b through the library (test harness only)."""

    def __init__(self, torch, m: csr, precision: str):
        self.torch, self.m, self.precision = torch, m, precision

    def function(self):
        torch, m, prec = self.torch, self.m, self.precision
        tol = 1e-15 if prec == "fp64" else 1e-13

        class CGSolveFn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, vals, b):
                mm = csr(m.dimensions, vals.detach().cpu().numpy(), m.row_start_offsets, m.col_indices)
                A = csr5.from_csr(mm)
                x = torch.zeros_like(b)
                CGSolver(A, tol=tol, max_it=5000, precision=prec).solve(b.detach().contiguous(), x, raise_on_failure=False)
                ctx.A = A
                ctx.save_for_backward(x)
                return x

            @staticmethod
            def backward(ctx, gx):
                x = ctx.saved_tensors[0].detach()
                lam = torch.zeros_like(x)
                gvals = torch.empty(ctx.A.non_zero_count(), device=x.device, dtype=torch.float64)
                cg_adjoint(ctx.A, gx.detach().contiguous(), x, lam, gvals, tol=tol, max_it=5000, precision=prec,
                           raise_on_failure=False)
                return gvals, lam

        return CGSolveFn


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("mgrid,ell", [(24, 4.0), (64, 16.0)])
def test_adjoint_matches_cpu_reference_and_fd(native, torch_cuda, precision, mgrid, ell):
    """Central differences (h = 1e-6) over 64 random directions to 1e-6 relative, and the FP64 CPU
    adjoint (direct solves) to 1e-8 relative."""
    torch = torch_cuda
    m, b, xt = _problem(mgrid, ell=ell)
    S = m.to_scipy().tocsc()
    n = m.dimensions.rows
    fn = _Solve(torch, m, precision).function()
    vals = torch.tensor(m.values, device="cuda", dtype=torch.float64, requires_grad=True)
    bt = torch.tensor(b, device="cuda", dtype=torch.float64, requires_grad=True)
    xtt = torch.tensor(xt, device="cuda", dtype=torch.float64)
    x = fn.apply(vals, bt)
    loss = ((x - xtt) ** 2).sum()
    loss.backward()
    g_vals, g_b = vals.grad.cpu().numpy(), bt.grad.cpu().numpy()

    # FP64 CPU reference (direct solves)
    xr = spla.spsolve(S, b)
    lam = spla.spsolve(S.T.tocsc(), 2 * (xr - xt))
    rows = np.repeat(np.arange(n), np.diff(m.row_start_offsets.astype(np.int64)))
    g_vals_ref = -lam[rows] * xr[m.col_indices]
    assert np.linalg.norm(g_b - lam) <= 1e-8 * np.linalg.norm(lam)
    assert np.linalg.norm(g_vals - g_vals_ref) <= 1e-8 * np.linalg.norm(g_vals_ref)

    # central finite differences, h = 1e-6, 64 random directions in (b, symmetric pattern perturbations)
    rng = np.random.default_rng(7)
    Sc = m.to_scipy().tocoo()
    key = np.minimum(Sc.row, Sc.col).astype(np.int64) * n + np.maximum(Sc.row, Sc.col)
    order = np.lexsort((Sc.col, Sc.row))  # CSR order of the COO entries
    key = key[order]

    def L(vv, bb):
        A = csr(m.dimensions, vv, m.row_start_offsets, m.col_indices).to_scipy().tocsc()
        xx = spla.spsolve(A, bb)
        return float(((xx - xt) ** 2).sum())

    h = 1e-6
    fd, ad = [], []
    for _ in range(64):
        w = rng.standard_normal(key.max() + 1)
        dv = w[key] * 0.1            # symmetric: (i,j) and (j,i) share a weight
        db = rng.standard_normal(n)
        fd.append((L(m.values + h * dv, b + h * db) - L(m.values - h * dv, b - h * db)) / (2 * h))
        ad.append(float(g_vals @ dv + g_b @ db))
    fd, ad = np.array(fd), np.array(ad)
    rel = np.linalg.norm(fd - ad) / np.linalg.norm(fd)
    assert rel <= 1e-6, rel


def test_mixed_adjoint(native, torch_cuda):
    torch = torch_cuda
    m, b, xt = _problem(32, seed=9)
    A = csr5.from_csr(m)
    n = m.dimensions.rows
    bd = torch.tensor(b, device="cuda")
    x = torch.zeros(n, device="cuda", dtype=torch.float64)
    CGSolver(A, tol=1e-12).solve(bd, x)
    g = 2 * (x - torch.tensor(xt, device="cuda"))
    lam64 = torch.zeros(n, device="cuda", dtype=torch.float64)
    lam_mx = torch.zeros(n, device="cuda", dtype=torch.float64)
    r64 = cg_adjoint(A, g, x, lam64, tol=1e-10)
    rmx = cg_adjoint(A, g, x, lam_mx, tol=1e-10, precision="mixed")
    assert r64.converged and rmx.converged and rmx.rel_residual <= 1.01e-10
    err = float(torch.linalg.norm(lam_mx - lam64) / torch.linalg.norm(lam64))
    assert err < 1e-5  # cond(A) ~ 4e3, both solves stop at 1e-10 relative residual
