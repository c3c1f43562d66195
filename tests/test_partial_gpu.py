"""Tile-chunk partitions on the device (diploma_research_gb300.partial): every part's partial product by
the CUDA SpMV, assembled, against the oracle's product of the whole matrix; and the multi-rank CG of the
reference's MPI benchmark (benchmarks/conjugate_gradient/dim/main.cpp:100-180) as two or three gloo ranks that
share one GPU (their kernels never wait on each other: the ranks meet only in host-side collectives)."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

import oracle
from diploma_research_gb300.generators import laplacian_2d_5pt, stencil_3d_27pt
from diploma_research_gb300.partial import REF_TILE, assemble, csr5_partial, partial_identifier_t
from helpers import SPMV_RTOL_F64, assert_spmv_close, csr_from_lengths, random_csr

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _matrices():
    rng = np.random.default_rng(43)
    yield "random", random_csr(rng, 20000, 15000, 7.0)
    yield "empty rows", random_csr(rng, 20000, 20000, 6.0, empty_frac=0.3)
    yield "long rows", random_csr(rng, 8000, 20000, 5.0, long_rows=10, long_len=(2000, 9000))
    yield "dense row", csr_from_lengths([5] * 3000 + [40000] + [4] * 3000, 50000, rng)
    yield "27-point 24^3", stencil_3d_27pt(24)


@pytest.mark.parametrize("parts", [1, 2, 3, 5])
def test_device_partial_products(native, torch_cuda, parts):
    torch = torch_cuda
    rng = np.random.default_rng(7)
    for name, m in _matrices():
        if parts > m.nnz // REF_TILE:
            continue
        x = rng.uniform(-1, 1, m.dimensions.cols)
        xd = torch.tensor(x, device="cuda", dtype=torch.float64)
        ranges, ys = [], []
        for i in range(parts):
            part = csr5_partial.from_csr(m, partial_identifier_t(i, parts))
            y = torch.full((part.output_range().count(),), float("nan"), device="cuda", dtype=torch.float64)
            part.spmv_partial(xd, y)
            ranges.append(part.output_range())
            ys.append(y.cpu().numpy())
        got = assemble(ranges, ys, m.dimensions.rows)
        ref = oracle.csr_spmv(m.dimensions.rows, m.row_start_offsets, m.col_indices, m.values, x)
        ax = oracle.abs_spmv(m.dimensions.rows, m.row_start_offsets, m.col_indices, m.values, x)
        assert_spmv_close(got, ref, ax, SPMV_RTOL_F64)


@pytest.mark.parametrize("parts", [2, 3])
def test_partial_load_then_device_product(native, torch_cuda, tmp_path, parts):
    """The device converter's reference-layout export, stored, loaded part by part from its slabs, each
    part multiplied on the device: the assembled product is the oracle's."""
    from diploma_research_gb300.csr5 import csr5
    from diploma_research_gb300.io import h5

    torch = torch_cuda
    m = dict(_matrices())["empty rows"]
    h5.store_csr5(tmp_path / "m.h5", "A", csr5.from_csr(m, omega=4).export(), m.dimensions.cols)
    x = np.random.default_rng(11).uniform(-1, 1, m.dimensions.cols)
    xd = torch.tensor(x, device="cuda", dtype=torch.float64)
    ranges, ys = [], []
    for i in range(parts):
        part = csr5_partial.from_layout(h5.load_csr5_partial(tmp_path / "m.h5", "A", partial_identifier_t(i, parts)))
        y = torch.empty(part.output_range().count(), device="cuda", dtype=torch.float64)
        part.spmv_partial(xd, y)
        ranges.append(part.output_range())
        ys.append(y.cpu().numpy())
    ref = oracle.csr_spmv(m.dimensions.rows, m.row_start_offsets, m.col_indices, m.values, x)
    ax = oracle.abs_spmv(m.dimensions.rows, m.row_start_offsets, m.col_indices, m.values, x)
    assert_spmv_close(assemble(ranges, ys, m.dimensions.rows), ref, ax, SPMV_RTOL_F64)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _cg_rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    from diploma_research_gb300 import partial as P
    from diploma_research_gb300.generators import laplacian_2d_5pt

    torch.cuda.set_device(0)
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        m = laplacian_2d_5pt(96)
        n = m.dimensions.rows
        xs = np.random.default_rng(3).uniform(-1, 1, n)
        b = np.zeros(n)
        rp = m.row_start_offsets.astype(np.int64)
        for i in range(n):  # b = A x* on the host (small)
            b[i] = float(m.values[rp[i]:rp[i + 1]] @ xs[m.col_indices[rp[i]:rp[i + 1]]])
        part = P.csr5_partial.from_csr(m, P.partial_identifier_t(rank, world))
        own = part.owning_range()
        b_own = torch.tensor(b[own.first_row:own.first_row + own.count()], device="cuda", dtype=torch.float64)
        x_own = torch.zeros_like(b_own)
        _, res = P.cg_partial(part, b_own, x_own, tol=1e-12, max_it=5000)
        out[rank] = (own.first_row, x_own.cpu().numpy(), res.iterations, res.converged)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_multi_rank_cg(native, torch_cuda, world):
    from diploma_research_gb300.cg import cg
    from diploma_research_gb300.csr5 import csr5

    m = laplacian_2d_5pt(96)
    n = m.dimensions.rows
    xs = np.random.default_rng(3).uniform(-1, 1, n)
    port = _free_port()
    # the manager process is started with spawn as well: this process has already initialised CUDA
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_cg_rank, args=(world, port, out), nprocs=world, join=True)
        res = [out[r] for r in range(world)]
    x = np.zeros(n)
    for first, xo, _, conv in res:
        assert conv
        x[first:first + len(xo)] = xo
    its = {r[2] for r in res}
    assert len(its) == 1  # every rank stops on the same all-reduced residual
    # the single-process solver on the same system
    b = oracle.csr_spmv(n, m.row_start_offsets, m.col_indices, m.values, xs)
    A = csr5.from_csr(m)
    x1, r1 = cg(A, b, tol=1e-12)
    # the dots are summed over ranks in another order: the iteration counts may differ by a few
    assert abs(its.pop() - r1.iterations) <= max(5, r1.iterations // 50)
    # cond(A) ~ 4e3 for the 96^2 Laplacian: a 1e-12 residual bounds the error by ~4e-9
    assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-7
    assert np.linalg.norm(x - x1) / np.linalg.norm(x1) < 1e-7
