"""The five benchmark systems at their full sizes, each against the oracle (the reference's CSR5 SpMV and
its dim_sp CG loop, benchmarks/conjugate_gradient/dim_sp/main.cpp:102-127, restated in C).

* 2-D 5-point Laplacian 512^2, CG to 1e-8 (FP64 and mixed precision);
* power-law n = 4,194,304 (Zipf 2, up to 10,000 off-diagonals, symmetrised), CG to 1e-10 in FP64 and
  mixed precision, each with its error against the oracle's FP64 x;
* 3-D 7-point Laplacian 192^3, block CG with k = 8 right-hand sides (FP64 and mixed), two columns
  against the oracle's CG on that column;
* 2-D anisotropic diffusion 1024^2: the adjoint gradients (FP64 and mixed) against central finite
  differences (h = 1e-6, 64 random directions in (values, b)) and against an FP64 CPU adjoint (sparse
  LU solves).
The 27-point 128^3 system is covered in test_cg_gpu.py.  Set DIMGPU_TEST_RECORD=<file> to keep the
measured errors and iteration counts."""
import numpy as np
import pytest

import oracle
from diploma_research_gb300.cg import BlockCGSolver, cg
from diploma_research_gb300.csr5 import csr5
from diploma_research_gb300.generators import WORKLOADS, rhs
from helpers import record

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def _oracle(m):
    n = m.dimensions.rows
    return oracle.OracleCSR5(n, n, m.row_start_offsets, m.col_indices, m.values)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# ---- 2-D 5-point 512^2 to 1e-8 ----------------------------------------------------------------------

@pytest.fixture(scope="module")
def lap2d():
    w = WORKLOADS["lap2d_512"]
    m = w["build"]()
    xs, b = rhs(m, w["seed"])
    xo, ito, relo = _oracle(m).cg(b, tol=w["tol"])
    return m, xs, b, xo, ito, relo, w["tol"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lap2d_512_cg(native, lap2d, precision):
    m, xs, b, xo, ito, relo, tol = lap2d
    A = csr5.from_csr(m)
    x, res = cg(A, b, tol=tol, precision=precision)
    err = _rel(x, xo)
    record(f"lap2d_512/{precision}", iterations=res.iterations, oracle_iterations=ito,
           rel_residual=res.rel_residual, rel_error_vs_oracle=err)
    assert res.converged and res.rel_residual <= tol * 1.01
    assert relo <= tol
    if precision == "fp64":
        assert abs(res.iterations - ito) <= 2, (res.iterations, ito)
        assert err < 1e-6, err
    else:
        assert err < 1e-5, err


# ---- power law n = 4,194,304 to 1e-10 ---------------------------------------------------------------

@pytest.fixture(scope="module")
def powerlaw():
    w = WORKLOADS["powerlaw_4m"]
    m = w["build"]()
    xs, b = rhs(m, w["seed"])
    xo, ito, relo = _oracle(m).cg(b, tol=w["tol"])
    return m, xs, b, xo, ito, relo, w["tol"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_powerlaw_4m_cg(native, powerlaw, precision):
    m, xs, b, xo, ito, relo, tol = powerlaw
    A = csr5.from_csr(m)
    x, res = cg(A, b, tol=tol, precision=precision)
    err = _rel(x, xo)
    record(f"powerlaw_4m/{precision}", iterations=res.iterations, oracle_iterations=ito,
           rel_residual=res.rel_residual, rel_error_vs_oracle=err, rel_error_vs_xstar=_rel(x, xs),
           reliable_updates=res.reliable_updates)
    assert res.converged and res.rel_residual <= tol * 1.01
    assert relo <= tol
    if precision == "fp64":
        # CG's iteration count on this matrix moves with the summation order by a few iterations near the
        # tolerance: the reference's loop needs 728, the same loop on the 32-lane layout (the oracle at
        # omega = 32) 729, a numpy/scipy CG (CSR-order products, pairwise dots) 731.  Bar: 0.5 %.
        assert abs(res.iterations - ito) <= max(2, int(np.ceil(0.005 * ito))), (res.iterations, ito)
        assert err < 1e-9, err
    else:
        assert err < 1e-8, err


# ---- 3-D 7-point 192^3, block CG with 8 right-hand sides ----------------------------------------------

@pytest.fixture(scope="module")
def lap3d():
    w = WORKLOADS["lap3d7_192"]
    m = w["build"]()
    k = 8
    xs, B = rhs(m, w["seed"], k=k)
    o = _oracle(m)
    cols = (0, k - 1)
    ref = {j: o.cg(np.ascontiguousarray(B[:, j]), tol=w["tol"]) for j in cols}
    return m, xs, B, ref, w["tol"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lap3d7_192_block_cg(native, torch_cuda, lap3d, precision):
    torch = torch_cuda
    m, xs, B, ref, tol = lap3d
    n, k = B.shape
    A = csr5.from_csr(m)
    s = BlockCGSolver(A, k, tol=tol, precision=precision)
    Bd = torch.tensor(B, device="cuda", dtype=torch.float64)
    Xd = torch.zeros((n, k), device="cuda", dtype=torch.float64)
    _, res = s.solve(Bd, Xd)
    X = Xd.cpu().numpy()
    assert res.converged_columns == k and res.max_rel_residual <= tol * 1.01
    for j, (xo, ito, relo) in ref.items():
        err = _rel(X[:, j], xo)
        record(f"lap3d7_192/k{k}/{precision}/col{j}", iterations=int(res.col_iterations[j]), oracle_iterations=ito,
               rel_residual=float(res.col_rel_residual[j]), rel_error_vs_oracle=err)
        assert relo <= tol
        if precision == "fp64":
            assert abs(int(res.col_iterations[j]) - ito) <= 2, (j, res.col_iterations[j], ito)
            assert err < 1e-9, (j, err)
        else:
            assert err < 1e-8, (j, err)


# ---- 2-D anisotropic 1024^2: adjoint gradients ------------------------------------------------------

@pytest.fixture(scope="module")
def aniso():
    """The system, b = A x* (seed 4), the target x_t ~ U[-1,1] (seed 5), the FP64 CPU reference (one sparse
    LU factorisation of A gives x = A^-1 b and lambda = A^-T 2 (x - x_t)), and the central finite
    differences of L = ||x - x_t||^2 along 64 random directions (h = 1e-6)."""
    import scipy.sparse.linalg as spla

    w = WORKLOADS["aniso2d_1024"]
    m = w["build"]()
    n = m.dimensions.rows
    _, b = rhs(m, w["seed"])
    xt = np.random.default_rng(w["seed"] + 1).uniform(-1.0, 1.0, n)
    S = m.to_scipy().tocsc()
    lu = spla.splu(S, permc_spec="MMD_AT_PLUS_A")
    x_ref = lu.solve(b)
    lam_ref = lu.solve(2.0 * (x_ref - xt), trans="T")
    # directions: symmetric value perturbations ((i,j) and (j,i) share a weight) and b perturbations
    rng = np.random.default_rng(7)
    Sc = m.to_scipy().tocoo()
    key = np.minimum(Sc.row, Sc.col).astype(np.int64) * n + np.maximum(Sc.row, Sc.col)
    key = key[np.lexsort((Sc.col, Sc.row))]  # CSR order
    _, key = np.unique(key, return_inverse=True)
    dvs, dbs = [], []
    for _ in range(64):
        dvs.append(rng.standard_normal(key.max() + 1)[key] * 0.1)
        dbs.append(rng.standard_normal(n))
    fd = _central_differences(m, S, lu, b, xt, x_ref, dvs, dbs, 1e-6)
    return m, S, b, xt, x_ref, lam_ref, dvs, dbs, fd


def _central_differences(m, S, lu, b, xt, x, dvs, dbs, h):
    """[L(v + h dv, b + h db) - L(v - h dv, b - h db)] / (2h) for L = ||x - x_t||^2, per direction.

    Each perturbed system A(v +- h dv) x+- = b +- h db is solved to rounding level by iterative refinement
    with the LU factors of A, written as a correction e+- = x+- - x, so that the difference of the two
    losses is formed without cancellation:
        L(+) - L(-) = 2 (x - x_t).(e+ - e-) + e+.e+ - e-.e-.
    The directions run on a few threads (the LU solves release the interpreter lock for part of their
    time)."""
    import concurrent.futures as cf

    r0 = b - S @ x
    z0 = lu.solve(r0)

    def one(dv, db):
        dA = _with_values(m, dv).to_scipy().tocsc()
        q = db - dA @ x
        z1 = lu.solve(q)
        es = []
        for sgn in (1.0, -1.0):
            Ap = S + (sgn * h) * dA
            rhs_v = r0 + (sgn * h) * q
            e = z0 + (sgn * h) * z1  # first refinement step, shared by both signs
            for _ in range(8):
                de = lu.solve(rhs_v - Ap @ e)
                e = e + de
                if np.linalg.norm(de) <= 1e-12 * np.linalg.norm(e):
                    break
            es.append(e)
        ep, em = es
        dl = 2.0 * float((x - xt) @ (ep - em)) + float(ep @ ep - em @ em)
        return dl / (2.0 * h)

    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        return np.array(list(ex.map(one, dvs, dbs)))


def _with_values(m, v):
    from diploma_research_gb300.mat import csr

    return csr(m.dimensions, v, m.row_start_offsets, m.col_indices)


# Solve tolerances of the differentiable solve.  The 1e-6 agreement of the gradients needs tight solves on
# this system: at 1e-10 the adjoint's lambda is off the CPU adjoint's by 1.3e-4, at 1e-12 by 7.8e-7 (FP64)
# and 6.1e-6 (mixed), at 1e-13 by 4.7e-8 (FP64).  The mixed adjoint's f32 recurrence stalls near 1e-13
# (1.1e-13 after 100,000 iterations), so it stops at 1.5e-13.
ADJOINT_TOL = {"fp64": (1e-13, 1e-13), "mixed": (1e-13, 1.5e-13)}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_aniso2d_1024_adjoint(native, torch_cuda, aniso, precision):
    from diploma_research_gb300.adjoint import cg_adjoint
    from diploma_research_gb300.cg import CGSolver

    torch = torch_cuda
    m, S, b, xt, x_ref, lam_ref, dvs, dbs, fd = aniso
    n, nnz = m.dimensions.rows, m.nnz
    tol_fwd, tol_adj = ADJOINT_TOL[precision]
    A = csr5.from_csr(m)
    bd = torch.tensor(b, device="cuda", dtype=torch.float64)
    xd = torch.zeros(n, device="cuda", dtype=torch.float64)
    _, rf = CGSolver(A, tol=tol_fwd, precision=precision, max_it=150000).solve(bd, xd)
    assert rf.converged
    g = 2.0 * (xd - torch.tensor(xt, device="cuda", dtype=torch.float64))
    lam = torch.zeros(n, device="cuda", dtype=torch.float64)
    gv = torch.empty(nnz, device="cuda", dtype=torch.float64)
    ra = cg_adjoint(A, g, xd, lam, gv, tol=tol_adj, precision=precision, max_it=150000, reliable_delta=0.1)
    assert ra.converged
    lam_h, gv_h, x_h = lam.cpu().numpy(), gv.cpu().numpy(), xd.cpu().numpy()

    # FP64 CPU adjoint
    rows = np.repeat(np.arange(n), np.diff(m.row_start_offsets.astype(np.int64)))
    gv_ref = -lam_ref[rows] * x_ref[m.col_indices]
    err_lam, err_gv = _rel(lam_h, lam_ref), _rel(gv_h, gv_ref)

    # the directional derivatives against the central finite differences
    ad = np.array([float(gv_h @ dv + lam_h @ db) for dv, db in zip(dvs, dbs)])
    ad_ref = np.array([float(gv_ref @ dv + lam_ref @ db) for dv, db in zip(dvs, dbs)])
    err_fd = float(np.linalg.norm(ad - fd) / np.linalg.norm(fd))
    err_fd_ref = float(np.linalg.norm(ad_ref - fd) / np.linalg.norm(fd))
    record(f"aniso2d_1024/{precision}", tol_forward=tol_fwd, tol_adjoint=tol_adj,
           forward_iterations=rf.iterations, adjoint_iterations=ra.iterations,
           adjoint_rel_residual=ra.rel_residual,
           rel_error_lambda_vs_cpu=err_lam, rel_error_grad_vals_vs_cpu=err_gv, rel_error_vs_fd=err_fd,
           cpu_adjoint_rel_error_vs_fd=err_fd_ref, rel_error_x_vs_cpu=_rel(x_h, x_ref))
    # h = 1e-6 leaves a truncation error of a few 1e-7 in the differences on this system (it falls as h^2);
    # the CPU adjoint shows it
    assert err_fd_ref <= 1e-6, err_fd_ref
    assert err_fd <= 1e-6, err_fd
    assert err_lam <= 1e-6 and err_gv <= 1e-6, (err_lam, err_gv)
