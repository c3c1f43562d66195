"""Device CG (FP64 and mixed precision) against the oracle's CG (the reference's dim_sp loop)."""
import os

import numpy as np
import pytest

import oracle
from diploma_research_gb300 import _native as N
from diploma_research_gb300.cg import CGSolver, cg
from diploma_research_gb300.csr5 import csr5
from diploma_research_gb300.generators import laplacian_2d_5pt, rhs, stencil_3d_27pt
from diploma_research_gb300.mat import csr, dimensions_t

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
pytestmark = pytest.mark.gpu


def _oracle_cg(m, b, tol):
    n = m.dimensions.rows
    o = oracle.OracleCSR5(n, n, m.row_start_offsets, m.col_indices, m.values)
    return o.cg(b, tol=tol)


def test_reference_fixture_cg(native):
    g = np.load(os.path.join(GOLDEN, "ref_cases.npz"))
    rp = g["cg_row_ptr"]
    n = rp.size - 1
    m = csr(dimensions_t(n, n), g["cg_vals"], rp, g["cg_col_idx"])
    A = csr5.from_csr(m)
    x, res = cg(A, g["cg_b"], tol=1e-10)
    assert res.converged
    assert abs(res.iterations - int(g["cg_iters"])) <= 1
    assert res.rel_residual <= 1.5e-10
    np.testing.assert_allclose(x, g["cg_x"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("use_graph", [True, False])
def test_fp64_cg_vs_oracle(native, use_graph):
    m = laplacian_2d_5pt(64)
    xs, b = rhs(m, 0)
    xo, ito, relo = _oracle_cg(m, b, 1e-10)
    A = csr5.from_csr(m)
    x, res = cg(A, b, tol=1e-10, use_graph=use_graph)
    assert res.converged and res.rel_residual <= 1.5e-10
    assert abs(res.iterations - ito) <= 2
    np.testing.assert_allclose(x, xo, rtol=0, atol=1e-8)
    np.testing.assert_allclose(x, xs, rtol=0, atol=1e-6)


def test_graph_and_host_loop_agree_bitwise(native):
    m = laplacian_2d_5pt(48)
    _, b = rhs(m, 1)
    A = csr5.from_csr(m)
    x1, r1 = cg(A, b, tol=1e-9, use_graph=True)
    x2, r2 = cg(A, b, tol=1e-9, use_graph=False)
    assert r1.iterations == r2.iterations
    assert np.array_equal(x1, x2)


def test_device_buffers_and_nonzero_x0(native, torch_cuda):
    m = laplacian_2d_5pt(40)
    xs, b = rhs(m, 2)
    A = csr5.from_csr(m)
    s = CGSolver(A, tol=1e-10)
    bd = torch_cuda.tensor(b, device="cuda", dtype=torch_cuda.float64)
    xd = torch_cuda.tensor(xs + 0.01, device="cuda", dtype=torch_cuda.float64)
    s.solve(bd, xd)
    torch_cuda.cuda.synchronize()
    np.testing.assert_allclose(xd.cpu().numpy(), xs, atol=1e-7)
    # solving again with the same solver and x0 = solution converges at once
    _, res = s.solve(bd, xd)
    assert res.iterations <= 1


def test_mixed_precision_reaches_fp64_residual(native):
    m = laplacian_2d_5pt(96)
    xs, b = rhs(m, 3)
    A = csr5.from_csr(m)
    x, res = cg(A, b, tol=1e-10, precision="mixed")
    assert res.converged
    assert res.rel_residual <= 1e-10 * 1.01
    assert res.reliable_updates >= 1
    xo, ito, _ = _oracle_cg(m, b, 1e-10)
    err = np.linalg.norm(x - xo) / np.linalg.norm(xo)
    assert err < 1e-6
    assert res.iterations <= 2 * ito


def test_not_converged_and_breakdown(native):
    m = laplacian_2d_5pt(64)
    _, b = rhs(m, 4)
    A = csr5.from_csr(m)
    x, res = CGSolver(A, tol=1e-14, max_it=5).solve(b, raise_on_failure=False)
    assert not res.converged and res.iterations == 5
    with pytest.raises(N.NotConvergedError):
        CGSolver(A, tol=1e-14, max_it=5).solve(b)
    neg = csr(m.dimensions, -m.values, m.row_start_offsets, m.col_indices)  # negative definite
    An = csr5.from_csr(neg)
    with pytest.raises(N.BreakdownError):
        cg(An, b, tol=1e-10)


def test_zero_rhs(native):
    m = laplacian_2d_5pt(16)
    A = csr5.from_csr(m)
    x, res = cg(A, np.zeros(256), tol=1e-10)
    assert res.converged and res.iterations == 0 and np.all(x == 0)


@pytest.mark.slow
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_stencil27_128_cg(native, precision):
    m = stencil_3d_27pt(128)
    xs, b = rhs(m, 1)
    A = csr5.from_csr(m)
    x, res = cg(A, b, tol=1e-10, precision=precision)
    assert res.converged and res.rel_residual <= 1e-10 * 1.01
    if precision == "fp64":
        xo, ito, _ = _oracle_cg(m, b, 1e-10)  # the reference's CG loop on the same system
        assert abs(res.iterations - ito) <= 2
        assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-9
    assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-6
