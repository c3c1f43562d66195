"""Device CG (FP64 and mixed precision) against the oracle's CG (the reference's dim_sp loop)."""
import os

import numpy as np
import pytest

import oracle
from diploma_research_gb300 import _native as N
from diploma_research_gb300.cg import CGSolver, cg
from diploma_research_gb300.csr5 import csr5
from diploma_research_gb300.generators import laplacian_2d_5pt, power_law, rhs, stencil_3d_27pt
from diploma_research_gb300.mat import csr, dimensions_t
from helpers import random_csr

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


# (engine, use_graph): use_graph=False runs the same kernels from a host-driven loop
ENGINES = [("graph", True), ("graph", False)]


@pytest.mark.parametrize("engine,use_graph", ENGINES)
def test_fp64_cg_vs_oracle(native, engine, use_graph):
    m = laplacian_2d_5pt(64)
    xs, b = rhs(m, 0)
    xo, ito, relo = _oracle_cg(m, b, 1e-10)
    A = csr5.from_csr(m)
    x, res = cg(A, b, tol=1e-10, use_graph=use_graph, engine=engine)
    assert res.converged and res.rel_residual <= 1.5e-10
    assert abs(res.iterations - ito) <= 2
    np.testing.assert_allclose(x, xo, rtol=0, atol=1e-8)
    np.testing.assert_allclose(x, xs, rtol=0, atol=1e-6)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_and_host_loop_agree_bitwise(native, precision):
    """The graph (device-side WHILE loop; for mixed, the reliable update as an IF node beside the s
    update) and the host-driven loop launch the same kernels: same bits."""
    m = laplacian_2d_5pt(48)
    _, b = rhs(m, 1)
    A = csr5.from_csr(m)
    x1, r1 = cg(A, b, tol=1e-9, use_graph=True, engine="graph", precision=precision)
    x2, r2 = cg(A, b, tol=1e-9, use_graph=False, precision=precision)
    assert r1.iterations == r2.iterations and r1.reliable_updates == r2.reliable_updates
    assert np.array_equal(x1, x2)


def test_graph_is_reproducible(native):
    """Fixed-order reductions: two solves give the same bits, FP64 and mixed."""
    m = laplacian_2d_5pt(80)
    _, b = rhs(m, 5)
    A = csr5.from_csr(m)
    for prec in ("fp64", "mixed"):
        x1, r1 = cg(A, b, tol=1e-10, precision=prec)
        x2, r2 = cg(A, b, tol=1e-10, precision=prec)
        assert r1.iterations == r2.iterations and np.array_equal(x1, x2)


def test_retired_engine_value_is_rejected(native):
    A = csr5.from_csr(laplacian_2d_5pt(16))
    import ctypes

    p = N.cg_params(1e-10, 100, N.CG_FP64, 1, 0.03, 2)  # 2 named the persistent engine, since removed
    h = ctypes.c_void_p()
    assert N.lib().dimgpu_cg_create(A._h, ctypes.byref(p), None, ctypes.byref(h)) == N.ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("n,density,long_rows,long_len,empty", [
    (300, 3.0, 0, (64, 700), 0.0),          # tail only: no full tile
    (700, 1.0, 0, (64, 700), 0.2),          # about one tile, empty rows
    (20000, 6.0, 6, (600, 5000), 0.1),      # rows spanning many warps' runs, empty rows
    (60000, 12.0, 20, (2000, 9000), 0.05),  # many long rows
])
def test_initial_residual_on_general_matrices(native, n, density, long_rows, long_len, empty):
    """With max_it = 0 a solve stops after r0 = b - A x0, whose norm it reports: the SpMV inside the
    solver on general matrices (look-back over warp runs, CSR tail, empty rows)."""
    rng = np.random.default_rng(n)
    m = random_csr(rng, n, n, density, empty_frac=empty, long_rows=long_rows, long_len=long_len)
    A = csr5.from_csr(m)
    x0 = rng.uniform(-1, 1, n)
    b = rng.uniform(-1, 1, n)
    ref = np.linalg.norm(b - m.to_scipy() @ x0)
    for prec in ("fp64", "mixed"):
        _, res = CGSolver(A, tol=0.0, max_it=0, precision=prec).solve(b, x0, raise_on_failure=False)
        got = res.recurrence_rel_residual * np.linalg.norm(b)
        assert abs(got - ref) <= 1e-12 * ref, (prec, got, ref)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_power_law_cg(native, precision):
    """A power-law system whose CG iteration count moves with the summation order: the reference's loop
    takes 282 iterations with 16 OpenMP threads and 285 with 8 (the calibrator chunks differ), a scipy CG
    285, and shuffling the order of every row's sum alone gives 283-287.  Bar: 3 % of the oracle's
    count, and the solution against the oracle's."""
    m = power_law(30000, 2.0, 3000, 7)
    xs, b = rhs(m, 7)
    A = csr5.from_csr(m)
    x, res = cg(A, b, tol=1e-10, precision=precision)
    assert res.converged and res.rel_residual <= 1e-10 * 1.01
    xo, ito, _ = _oracle_cg(m, b, 1e-10)
    if precision == "fp64":
        assert abs(res.iterations - ito) <= max(2, int(np.ceil(0.03 * ito))), (res.iterations, ito)
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-7


@pytest.mark.parametrize("engine", ["auto", "graph"])
def test_device_buffers_and_nonzero_x0(native, torch_cuda, engine):
    m = laplacian_2d_5pt(40)
    xs, b = rhs(m, 2)
    A = csr5.from_csr(m)
    s = CGSolver(A, tol=1e-10, engine=engine)
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


@pytest.mark.parametrize("engine", ["auto", "graph"])
def test_not_converged_and_breakdown(native, engine):
    m = laplacian_2d_5pt(64)
    _, b = rhs(m, 4)
    A = csr5.from_csr(m)
    x, res = CGSolver(A, tol=1e-14, max_it=5, engine=engine).solve(b, raise_on_failure=False)
    assert not res.converged and res.iterations == 5
    with pytest.raises(N.NotConvergedError):
        CGSolver(A, tol=1e-14, max_it=5, engine=engine).solve(b)
    neg = csr(m.dimensions, -m.values, m.row_start_offsets, m.col_indices)  # negative definite
    An = csr5.from_csr(neg)
    with pytest.raises(N.BreakdownError):
        cg(An, b, tol=1e-10, engine=engine)
    # the solver stays usable after a breakdown
    x, res = cg(A, b, tol=1e-10, engine=engine)
    assert res.converged


@pytest.mark.parametrize("engine", ["auto", "graph"])
def test_zero_rhs(native, engine):
    m = laplacian_2d_5pt(16)
    A = csr5.from_csr(m)
    x, res = cg(A, np.zeros(256), tol=1e-10, engine=engine)
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
