"""Block CG (k simultaneous solves, one SpMM per iteration, per-column masks) against the oracle's CG
(the reference's dim_sp loop, benchmarks/conjugate_gradient/dim_sp/main.cpp:102-127) on every column."""
import numpy as np
import pytest

import oracle
from diploma_research_gb300.cg import BlockCGSolver
from diploma_research_gb300.csr5 import csr5
from diploma_research_gb300.generators import laplacian_2d_5pt, laplacian_3d_7pt, rhs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", [1, 5, 8, 16])
@pytest.mark.parametrize("use_graph", [True, False])
def test_block_cg_fp64_matches_oracle(native, torch_cuda, k, use_graph):
    torch = torch_cuda
    m = laplacian_2d_5pt(40)
    n = m.dimensions.rows
    xs, B = rhs(m, 7, k=k)
    A = csr5.from_csr(m)
    s = BlockCGSolver(A, k, tol=1e-10, use_graph=use_graph)
    Bd = torch.tensor(B, device="cuda", dtype=torch.float64)
    Xd = torch.zeros((n, k), device="cuda", dtype=torch.float64)
    _, res = s.solve(Bd, Xd)
    assert res.converged_columns == k and res.max_rel_residual <= 1.5e-10
    X = Xd.cpu().numpy()
    o = oracle.OracleCSR5(n, n, m.row_start_offsets, m.col_indices, m.values)
    for j in range(k):
        xo, ito, _ = o.cg(np.ascontiguousarray(B[:, j]), tol=1e-10)
        assert abs(res.col_iterations[j] - ito) <= 2, (j, res.col_iterations[j], ito)
        np.testing.assert_allclose(X[:, j], xo, rtol=0, atol=1e-9)


def test_block_cg_masks(native, torch_cuda):
    """A zero column converges at once; a column started at its solution too; the others keep going."""
    torch = torch_cuda
    m = laplacian_2d_5pt(32)
    n = m.dimensions.rows
    xs, B = rhs(m, 3, k=4)
    B[:, 1] = 0.0
    A = csr5.from_csr(m)
    X0 = np.zeros((n, 4))
    X0[:, 2] = xs[:, 2]
    s = BlockCGSolver(A, 4, tol=1e-10)
    Bd = torch.tensor(B, device="cuda", dtype=torch.float64)
    Xd = torch.tensor(X0, device="cuda", dtype=torch.float64)
    _, res = s.solve(Bd, Xd)
    assert res.converged_columns == 4
    assert res.col_iterations[1] == 0 and res.col_iterations[2] <= 1
    assert res.col_iterations[0] > 10 and res.col_iterations[3] > 10
    np.testing.assert_allclose(Xd.cpu().numpy()[:, [0, 3]], xs[:, [0, 3]], atol=1e-7)


@pytest.mark.parametrize("k", [3, 8, 16, 32])
def test_block_cg_mixed(native, torch_cuda, k):
    """Mixed block CG at widths whose f32 SpMM holds four right-hand sides per lane with idle lanes
    (k = 3: padded to 4) and without (8, 16, 32)."""
    torch = torch_cuda
    m = laplacian_3d_7pt(20)
    n = m.dimensions.rows
    xs, B = rhs(m, 11, k=k)
    A = csr5.from_csr(m)
    s = BlockCGSolver(A, k, tol=1e-10, precision="mixed")
    Bd = torch.tensor(B, device="cuda", dtype=torch.float64)
    Xd = torch.zeros((n, k), device="cuda", dtype=torch.float64)
    _, res = s.solve(Bd, Xd)
    assert res.converged_columns == k
    assert res.max_rel_residual <= 1.01e-10
    assert res.reliable_updates >= 1
    err = np.linalg.norm(Xd.cpu().numpy() - xs) / np.linalg.norm(xs)
    assert err < 1e-7


def test_block_cg_not_converged(native, torch_cuda):
    torch = torch_cuda
    m = laplacian_2d_5pt(32)
    n = m.dimensions.rows
    _, B = rhs(m, 5, k=2)
    A = csr5.from_csr(m)
    s = BlockCGSolver(A, 2, tol=1e-14, max_it=7)
    Xd = torch.zeros((n, 2), device="cuda", dtype=torch.float64)
    _, res = s.solve(torch.tensor(B, device="cuda", dtype=torch.float64), Xd, raise_on_failure=False)
    assert res.converged_columns == 0 and res.iterations == 7
