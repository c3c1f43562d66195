"""Device SpMV through the C ABI against the oracle (componentwise |y - y_ref| <= 1e-12 (|A||x|) in f64)."""
import os

import numpy as np
import pytest

import oracle
from diploma_research_gb300.csr5 import csr5, spmv_data_t
from diploma_research_gb300.mat import csr, dimensions_t
from helpers import SPMV_RTOL_F32, SPMV_RTOL_F64, assert_spmv_close, csr_from_lengths, random_csr

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
pytestmark = pytest.mark.gpu


def _refs(m: csr, x):
    rows = m.dimensions.rows
    y_ref = oracle.csr_spmv(rows, m.row_start_offsets, m.col_indices, m.values, x)
    ax = oracle.abs_spmv(rows, m.row_start_offsets, m.col_indices, m.values, x)
    return y_ref, ax


def _gpu_spmv(torch, A: csr5, x, fill=np.nan, cal=None):
    xd = torch.tensor(x, device="cuda", dtype=torch.float64)
    yd = torch.full((A.dimensions.rows,), fill, device="cuda", dtype=torch.float64)
    A.spmv(spmv_data_t(xd, yd, cal))
    torch.cuda.synchronize()
    return yd.cpu().numpy()


def _check(torch, m: csr, x, sigma=16):
    A = csr5.from_csr(m, sigma=sigma)
    y = _gpu_spmv(torch, A, x)
    y_ref, ax = _refs(m, x)
    assert_spmv_close(y, y_ref, ax, SPMV_RTOL_F64)
    return A, y


def test_reference_fixture_cases(native, torch_cuda):
    g = np.load(os.path.join(GOLDEN, "ref_cases.npz"))
    for k in g["cases"]:
        p = f"c{k}_"
        m = csr(dimensions_t(int(g[p + "rows"]), int(g[p + "cols"])), g[p + "vals"], g[p + "row_ptr"],
                g[p + "col_idx"])
        A = csr5.from_csr(m)
        y = _gpu_spmv(torch_cuda, A, g[p + "x"])
        _, ax = _refs(m, g[p + "x"])
        assert_spmv_close(y, g[p + "y"], ax, SPMV_RTOL_F64)  # the reference's own SpMV output


def test_mm_mtx(native, torch_cuda):
    g = np.load(os.path.join(GOLDEN, "mm_mtx.npz"))
    m = csr(dimensions_t(int(g["rows"]), int(g["cols"])), g["vals"], g["row_ptr"], g["col_idx"])
    A = csr5.from_csr(m)
    for x, yr in ((np.ones(m.dimensions.cols), g["ref_y_ones"]), (g["x_rand"], g["ref_y_rand"])):
        y = _gpu_spmv(torch_cuda, A, x)
        _, ax = _refs(m, x)
        assert_spmv_close(y, yr, ax, SPMV_RTOL_F64)


@pytest.mark.parametrize("seed", range(16))
def test_random(native, torch_cuda, seed):
    rng = np.random.default_rng(seed)
    m = random_csr(rng, int(rng.integers(1, 8000)), int(rng.integers(1, 8000)), float(rng.uniform(0.1, 60)),
                   empty_frac=float(rng.choice([0, 0.05, 0.5, 0.9])), long_rows=int(rng.integers(0, 6)),
                   long_len=(100, 6000))
    _check(torch_cuda, m, rng.uniform(-1, 1, m.dimensions.cols))


@pytest.mark.parametrize("lens,cols", [
    ([3, 0, 5, 1], 10),                         # no full tile: tail only
    ([0, 0, 0], 4),                             # nnz = 0: every row is empty
    ([512], 600),                               # exactly one tile, one row
    ([513], 600),                               # one tile + one tail element of the same row
    ([0] * 50 + [512] + [0] * 50, 600),         # leading and trailing empty rows
    ([20000], 20000),                           # one row spanning 39 tiles
    ([0, 700, 0, 0, 2000, 1, 0], 3000),
    ([1] * 4096, 3),                            # one-element rows
    ([7] * 1000 + [0] * 1000, 100),             # empty rows at the end, below the tail
    ([0] * 3000 + [5000] + [2] * 10, 5000),
    ([511, 1, 511, 1, 1024], 2000),             # rows ending exactly at tile boundaries
])
def test_edge_cases(native, torch_cuda, lens, cols):
    rng = np.random.default_rng(len(lens) * 7 + cols)
    m = csr_from_lengths(lens, cols, rng)
    _check(torch_cuda, m, rng.uniform(-1, 1, cols))


def _single_start_matrices(rng):
    """Matrices whose tiles take the single-row-start segment loop (no 16-element column holds two row
    starts), with the cases that loop treats apart: a row start at every position of a column, columns
    without one, lane 0 with and without a row start at r = 0, empty rows (several rows starting at one
    element, dirty tiles), and one short row that sends its tile down the general loop."""
    yield csr_from_lengths(rng.integers(16, 48, 4000), 5000, rng)
    yield csr_from_lengths([16] * 3000, 3000, rng)  # every column begins a row at r = 0
    yield csr_from_lengths([17] * 3000, 3000, rng)  # the row start walks through every r
    lens = rng.integers(16, 40, 3000)
    lens[rng.choice(3000, 300, replace=False)] = 0
    yield csr_from_lengths(lens, 4000, rng)
    lens = rng.integers(16, 40, 3000)
    lens[1500] = 3
    yield csr_from_lengths(lens, 4000, rng)


def test_single_row_start_columns(native, torch_cuda):
    """The segment loop for tiles whose columns hold at most one row start, in f64 and f32, against the
    oracle."""
    torch = torch_cuda
    rng = np.random.default_rng(91)
    for m in _single_start_matrices(rng):
        x = rng.uniform(-1, 1, m.dimensions.cols)
        A, _ = _check(torch, m, x)
        xd = torch.tensor(x, device="cuda", dtype=torch.float32)
        yd = torch.full((m.dimensions.rows,), float("nan"), device="cuda", dtype=torch.float32)
        A.spmv(xd, yd)
        torch.cuda.synchronize()
        y_ref, ax = _refs(m, x.astype(np.float32).astype(np.float64))
        assert_spmv_close(yd.cpu().numpy().astype(np.float64), y_ref, ax, SPMV_RTOL_F32 * 50)


def test_many_warps_share_a_row(native, torch_cuda):
    """A row long enough to cover several warps' tile runs exercises chained calibrator slots."""
    rng = np.random.default_rng(77)
    lens = [3] * 10000 + [2_000_000] + [5] * 10000
    m = csr_from_lengths(lens, 2_100_000, rng)
    _check(torch_cuda, m, rng.uniform(-1, 1, m.dimensions.cols))


def test_repeat_calls_deterministic_and_calibrator_reuse(native, torch_cuda):
    rng = np.random.default_rng(3)
    m = random_csr(rng, 20000, 20000, 30.0, empty_frac=0.1, long_rows=20, long_len=(1000, 9000))
    A = csr5.from_csr(m)
    cal = A.create_calibrator()
    x = rng.uniform(-1, 1, 20000)
    ys = [_gpu_spmv(torch_cuda, A, x, fill=f, cal=cal) for f in (np.nan, 1e300, 0.0)]
    assert np.array_equal(ys[0], ys[1]) and np.array_equal(ys[1], ys[2])  # bit-identical, y overwritten
    y2 = _gpu_spmv(torch_cuda, A, x)  # matrix's own calibrator
    assert np.array_equal(ys[0], y2)


def test_host_buffers(native):
    rng = np.random.default_rng(4)
    m = random_csr(rng, 3000, 2000, 10.0, empty_frac=0.2)
    A = csr5.from_csr(m)
    x = rng.uniform(-1, 1, 2000)
    y = np.empty(3000)
    A.spmv(x, y)
    y_ref, ax = _refs(m, x)
    assert_spmv_close(y, y_ref, ax, SPMV_RTOL_F64)
    with pytest.raises(ValueError):
        A.spmv(np.ones(1999), y)  # csr5.h:820-821


def test_f32_spmv(native, torch_cuda):
    rng = np.random.default_rng(6)
    m = random_csr(rng, 5000, 5000, 20.0, empty_frac=0.1, long_rows=4, long_len=(600, 3000))
    A = csr5.from_csr(m)
    x = rng.uniform(-1, 1, 5000)
    xd = torch_cuda.tensor(x, device="cuda", dtype=torch_cuda.float32)
    yd = torch_cuda.full((5000,), float("nan"), device="cuda", dtype=torch_cuda.float32)
    A.spmv(xd, yd)
    torch_cuda.cuda.synchronize()
    x32 = x.astype(np.float32).astype(np.float64)
    y_ref, ax = _refs(m, x32)
    # values rounded to f32 too: relative error per term <= 2^-24 (values) + accumulation in f32
    assert_spmv_close(yd.cpu().numpy().astype(np.float64), y_ref, ax, SPMV_RTOL_F32 * 50)


@pytest.mark.parametrize("seed", range(3))
def test_spmv_dot_fused(native, torch_cuda, seed):
    """y = A x with x.y from the same pass (the CG energy product), against numpy."""
    import ctypes

    from diploma_research_gb300 import _native as N

    torch = torch_cuda
    rng = np.random.default_rng(40 + seed)
    n = int(rng.integers(1000, 60000))
    m = random_csr(rng, n, n, float(rng.uniform(2, 40)), empty_frac=0.05, long_rows=3, long_len=(2000, 20000))
    A = csr5.from_csr(m)
    x = rng.uniform(-1, 1, n)
    xd = torch.tensor(x, device="cuda", dtype=torch.float64)
    yd = torch.full((n,), float("nan"), device="cuda", dtype=torch.float64)
    dot = torch.zeros(1, device="cuda", dtype=torch.float64)
    N.check(native.dimgpu_csr5_spmv_dot(A._h, xd.data_ptr(), yd.data_ptr(), dot.data_ptr(), None, None))
    torch.cuda.synchronize()
    y_ref, ax = _refs(m, x)
    assert_spmv_close(yd.cpu().numpy(), y_ref, ax, SPMV_RTOL_F64)
    ref = float(np.dot(x, y_ref))
    scale = float(np.dot(np.abs(x), ax))
    assert abs(float(dot.item()) - ref) <= 1e-12 * scale


def test_linearity(native, torch_cuda):
    rng = np.random.default_rng(8)
    m = random_csr(rng, 6000, 6000, 15.0, long_rows=3, long_len=(1000, 5000))
    A = csr5.from_csr(m)
    x1, x2 = rng.uniform(-1, 1, 6000), rng.uniform(-1, 1, 6000)
    y1, y2 = _gpu_spmv(torch_cuda, A, x1), _gpu_spmv(torch_cuda, A, x2)
    y12 = _gpu_spmv(torch_cuda, A, 2.0 * x1 - 3.0 * x2)
    ax = oracle.abs_spmv(6000, m.row_start_offsets, m.col_indices, m.values, np.abs(2 * x1) + np.abs(3 * x2))
    assert_spmv_close(y12, 2.0 * y1 - 3.0 * y2, ax, 4 * SPMV_RTOL_F64)


@pytest.mark.slow
@pytest.mark.parametrize("name", ["stencil27_128", "lap2d_512", "aniso2d_1024"])
def test_full_size_workloads(native, torch_cuda, name):
    from diploma_research_gb300.generators import WORKLOADS

    m = WORKLOADS[name]["build"]()
    rng = np.random.default_rng(11)
    _check(torch_cuda, m, rng.uniform(-1, 1, m.dimensions.cols))


@pytest.mark.slow
def test_power_law_full_size(native, torch_cuda):
    from diploma_research_gb300.generators import power_law

    m = power_law()
    rng = np.random.default_rng(12)
    _check(torch_cuda, m, rng.uniform(-1, 1, m.dimensions.cols))


def _launch_matrices(rng):
    """Matrices whose tiles fit 16-bit column offsets, and one whose random columns do not (32-bit)."""
    yield random_csr(rng, 9000, 9000, 12.0, empty_frac=0.1, long_rows=4, long_len=(600, 6000))
    yield random_csr(rng, 100000, 100000, 3.0, empty_frac=0.05, long_rows=3, long_len=(2000, 9000))
    yield csr_from_lengths([3] * 10000 + [20000] + [5] * 13999, 24000, rng)  # one row across many warp runs
    yield random_csr(rng, 3000, 3000, 2.0)


@pytest.mark.parametrize("warps,gather", [(16, "l1"), (16, "stream"), (12, "l1"), (12, "stream")])
def test_every_f64_launch_configuration(native, torch_cuda, warps, gather):
    """Each f64 launch the per-matrix timing may choose, pinned: the product, the product with the fused
    dot, and a CG solve."""
    import ctypes

    from diploma_research_gb300 import _native as N
    from diploma_research_gb300.cg import cg

    torch = torch_cuda
    rng = np.random.default_rng(70 + warps)
    for m in _launch_matrices(rng):
        n = m.dimensions.rows
        A = csr5.from_csr(m)
        A.set_spmv_launch(warps, gather)
        assert A.spmv_launch() == (warps, gather)
        x = rng.uniform(-1, 1, n)
        xd = torch.tensor(x, device="cuda", dtype=torch.float64)
        yd = torch.full((n,), float("nan"), device="cuda", dtype=torch.float64)
        dot = torch.zeros(1, device="cuda", dtype=torch.float64)
        N.check(native.dimgpu_csr5_spmv_dot(A._h, xd.data_ptr(), yd.data_ptr(), dot.data_ptr(), None, None))
        torch.cuda.synchronize()
        y_ref, ax = _refs(m, x)
        assert_spmv_close(yd.cpu().numpy(), y_ref, ax, SPMV_RTOL_F64)
        assert abs(float(dot.item()) - float(np.dot(x, y_ref))) <= 1e-12 * float(np.dot(np.abs(x), ax))
        yp = _gpu_spmv(torch, A, x)
        assert_spmv_close(yp, y_ref, ax, SPMV_RTOL_F64)
    # a CG solve on this launch (its SpMV with the fused dot inside the graph)
    from diploma_research_gb300.generators import laplacian_2d_5pt

    L = laplacian_2d_5pt(64)
    A = csr5.from_csr(L)
    A.set_spmv_launch(warps, gather)
    b = oracle.csr_spmv(L.dimensions.rows, L.row_start_offsets, L.col_indices, L.values,
                        rng.uniform(-1, 1, L.dimensions.rows))
    _, res = cg(A, b, tol=1e-10)
    assert res.converged and res.rel_residual <= 1e-10


@pytest.mark.parametrize("warps,gather", [(24, "l1"), (24, "stream"), (20, "l1"), (20, "stream")])
def test_every_f32_launch_configuration(native, torch_cuda, warps, gather):
    """Each f32 launch, pinned: the f32 product, and a mixed-precision CG solve (its f32 product with the
    fused dot)."""
    from diploma_research_gb300.cg import cg

    torch = torch_cuda
    rng = np.random.default_rng(80 + warps)
    for m in _launch_matrices(rng):
        n = m.dimensions.rows
        A = csr5.from_csr(m)
        A.set_spmv_launch(warps, gather, f32=True)
        assert A.spmv_launch(f32=True) == (warps, gather)
        x = rng.uniform(-1, 1, n)
        xd = torch.tensor(x, device="cuda", dtype=torch.float32)
        yd = torch.full((n,), float("nan"), device="cuda", dtype=torch.float32)
        A.spmv(xd, yd)
        torch.cuda.synchronize()
        y_ref, ax = _refs(m, x.astype(np.float32).astype(np.float64))
        assert_spmv_close(yd.cpu().numpy().astype(np.float64), y_ref, ax, SPMV_RTOL_F32 * 50)
    from diploma_research_gb300.generators import laplacian_2d_5pt

    L = laplacian_2d_5pt(64)
    A = csr5.from_csr(L)
    A.set_spmv_launch(warps, gather, f32=True)
    b = oracle.csr_spmv(L.dimensions.rows, L.row_start_offsets, L.col_indices, L.values,
                        rng.uniform(-1, 1, L.dimensions.rows))
    _, res = cg(A, b, tol=1e-10, precision="mixed")
    assert res.converged and res.rel_residual <= 1e-10


def test_launch_configuration_errors(native, torch_cuda):
    A = csr5.from_csr(random_csr(np.random.default_rng(1), 500, 500, 5.0))
    with pytest.raises(ValueError):
        A.set_spmv_launch(20)  # an f32 launch, not an f64 one
    with pytest.raises(ValueError):
        A.set_spmv_launch(16, f32=True)
    with pytest.raises(ValueError):
        A.set_spmv_launch(16, gather="texture")
    assert A.spmv_launch() == (16, "l1")  # small matrices keep the default


def test_16_bit_column_offsets(native, torch_cuda):
    """The converter keeps 16-bit column offsets exactly when every full tile's columns span less than
    2^16 (device_bytes counts them), and the product is the oracle's either way."""
    rng = np.random.default_rng(90)
    narrow = random_csr(rng, 20000, 60000, 8.0)  # columns < 2^16: every tile fits
    wide = random_csr(rng, 20000, 200000, 8.0)  # random columns over 200k: tiles span more
    for m, has16 in ((narrow, True), (wide, False)):
        A = csr5.from_csr(m)
        T = A.tile_count
        # everything but the offsets: values + indices, row_ptr, tile_ptr + tdo_ptr, descriptors (a few
        # dirty tiles' tile_desc_offset entries stay far below the 2 bytes per element of the offsets)
        base = 12 * m.nnz + 4 * (m.dimensions.rows + 1) + 8 * (T + 1) + 4 * T * 32
        assert (A.device_bytes - base >= 2 * T * 512) == has16, (A.device_bytes - base, has16)
        x = rng.uniform(-1, 1, m.dimensions.cols)
        y_ref, ax = _refs(m, x)
        assert_spmv_close(_gpu_spmv(torch_cuda, A, x), y_ref, ax, SPMV_RTOL_F64)
