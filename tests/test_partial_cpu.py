"""Tile-chunk partitions of one matrix across ranks (diploma_research_gb300.partial) on CPU: the partition
and range logic of the reference's partial load (h5.cpp:95-173) and MPI sync (output_range.cpp,
edge_sync.cpp, result_sync.cpp), the per-part products computed by the oracle, and the edge and result
sync over gloo with world sizes 2 and 3."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

import oracle
from diploma_research_gb300.partial import (REF_TILE, assemble, calculate_partition, output_range_t,
                                            owned_slices, partial_identifier_t, partial_layout)
from helpers import SPMV_RTOL_F64, assert_spmv_close, csr_from_lengths, random_csr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _oracle_y(m, x):
    return oracle.csr_spmv(m.dimensions.rows, m.row_start_offsets, m.col_indices, m.values, x)


def _abs_y(m, x):
    return oracle.abs_spmv(m.dimensions.rows, m.row_start_offsets, m.col_indices, m.values, x)


def _matrices():
    rng = np.random.default_rng(41)
    yield "random", random_csr(rng, 3000, 2500, 6.0)
    yield "empty rows", random_csr(rng, 3000, 3000, 5.0, empty_frac=0.3)
    yield "long rows", random_csr(rng, 2000, 4000, 4.0, long_rows=6, long_len=(300, 1500))
    # one row holding most of the matrix: it spans several parts
    yield "dense row", csr_from_lengths([3] * 200 + [3000] + [2] * 300, 4000, rng)
    # rows that start exactly at a tile boundary, with empty rows around the boundaries
    yield "aligned", csr_from_lengths([64, 0, 64, 0, 0, 128, 64] * 20, 500, rng)


def test_calculate_partition():
    p = partial_identifier_t
    assert [calculate_partition(10, p(i, 3)) for i in range(3)] == [(0, 4), (4, 4), (8, 2)]
    assert [calculate_partition(10, p(i, 4)) for i in range(4)] == [(0, 3), (3, 3), (6, 3), (9, 1)]
    assert calculate_partition(7, p(0, 1)) == (0, 7)
    with pytest.raises(ValueError):
        calculate_partition(7, p(3, 3))


def test_syncs_downto():
    rs = [output_range_t(0, 5), output_range_t(5, 5), output_range_t(5, 9), output_range_t(10, 12),
          output_range_t(12, 20)]
    assert [output_range_t.syncs_downto(rs, i) for i in range(5)] == [0, 0, 0, 3, 3]
    assert rs[2].is_continuation_of(rs[1]) and not rs[3].is_continuation_of(rs[2])
    assert rs[1].count() == 1 and rs[2].count() == 5


@pytest.mark.parametrize("parts", [1, 2, 3, 5])
def test_layout_covers_the_matrix(parts):
    for name, m in _matrices():
        rp = m.row_start_offsets.astype(np.int64)
        lays = [partial_layout.of(m, partial_identifier_t(i, parts)) for i in range(parts)]
        # the chunks tile [0, nnz) in order, at the reference's tile granularity
        assert lays[0].element_begin == 0 and lays[-1].element_end == m.nnz, name
        for a, b in zip(lays, lays[1:]):
            assert a.element_end == b.element_begin and a.element_end % REF_TILE == 0, name
        assert sum(l.local.nnz for l in lays) == m.nnz
        for l in lays:
            e0, e1 = l.element_begin, l.element_end
            assert rp[l.first_row] <= e0 < rp[l.first_row + 1], name  # first row holds the first element
            if l.part.idx < parts - 1:
                assert rp[l.last_row] <= e1 - 1 < rp[l.last_row + 1], name
            else:
                assert l.last_row == m.dimensions.rows - 1
            assert l.owns_first_row == (rp[l.first_row] == e0)
            np.testing.assert_array_equal(l.local.values, m.values[e0:e1])
        # owned slices: disjoint, increasing, the skipped first rows are exactly the continued ones
        sl = owned_slices([l.output_range() for l in lays])
        for (s0, c0), (s1, _) in zip(sl, sl[1:]):
            assert s0 + c0 <= s1
        for l, (s, c) in zip(lays, sl):
            assert (s, c) == (l.owning_range().first_row, l.owning_range().count()), name


@pytest.mark.parametrize("parts", [2, 3, 4, 7])
def test_assembled_partial_products_equal_the_product(parts):
    rng = np.random.default_rng(5)
    for name, m in _matrices():
        if parts > m.nnz // REF_TILE:
            continue
        x = rng.uniform(-1, 1, m.dimensions.cols)
        lays = [partial_layout.of(m, partial_identifier_t(i, parts)) for i in range(parts)]
        ys = [_oracle_y(l.local, x) for l in lays]
        y = assemble([l.output_range() for l in lays], ys, m.dimensions.rows)
        assert_spmv_close(y, _oracle_y(m, x), _abs_y(m, x), SPMV_RTOL_F64)


def test_more_parts_than_tiles_is_an_error():
    m = csr_from_lengths([10] * 10, 20, np.random.default_rng(0))  # 100 elements: one tile
    with pytest.raises(ValueError):
        partial_layout.of(m, partial_identifier_t(0, 2))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, case, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch
    import torch.distributed as dist

    from diploma_research_gb300 import partial as P

    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        m = dict(_matrices())[case]
        x = np.random.default_rng(9).uniform(-1, 1, m.dimensions.cols)
        lay = P.partial_layout.of(m, P.partial_identifier_t(rank, world))
        ranges = P.all_output_ranges(lay.output_range())
        y = torch.tensor(_oracle_y(lay.local, x))  # this rank's partial product
        P.edge_sync_t(ranges, rank).sync(y)
        full = torch.zeros(m.dimensions.rows, dtype=torch.float64)
        P.result_sync_t(ranges, rank).sync(full, y)
        out[rank] = full.numpy().copy()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,case", [(2, "empty rows"), (3, "dense row"), (3, "aligned")])
def test_edge_and_result_sync_over_gloo(world, case):
    m = dict(_matrices())[case]
    x = np.random.default_rng(9).uniform(-1, 1, m.dimensions.cols)
    ref, ax = _oracle_y(m, x), _abs_y(m, x)
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, case, out), nprocs=world, join=True)
        fulls = [out[r] for r in range(world)]
    for f in fulls:
        assert_spmv_close(f, ref, ax, SPMV_RTOL_F64)
    for f in fulls[1:]:
        np.testing.assert_array_equal(f, fulls[0])  # every rank holds the same bits


@pytest.mark.parametrize("parts", [1, 2, 3, 4])
def test_partial_load_from_a_stored_csr5_group(tmp_path, parts):
    """A stored CSR5 group (the reference's arrays, written by store_csr5) read part by part gives the same
    chunks as partitioning the CSR; only the part's slabs are read."""
    from types import SimpleNamespace

    from diploma_research_gb300.io import h5

    for name, m in _matrices():
        if parts > m.nnz // REF_TILE:
            continue
        o = oracle.OracleCSR5(m.dimensions.rows, m.dimensions.cols, m.row_start_offsets, m.col_indices, m.values)
        arrays = SimpleNamespace(vals=o.vals, col_idx=o.col_idx, row_ptr=o.row_ptr, tile_ptr=o.tile_ptr,
                                 tile_desc=o.tile_desc.astype(np.uint32), tile_desc_offset_ptr=o.tile_desc_offset_ptr,
                                 tile_desc_offset=o.tile_desc_offset)
        path = tmp_path / f"{name.replace(' ', '_')}_{parts}.h5"
        h5.store_csr5(path, "A", arrays, m.dimensions.cols)
        for i in range(parts):
            pid = partial_identifier_t(i, parts)
            got, want = h5.load_csr5_partial(path, "A", pid), partial_layout.of(m, pid)
            assert (got.first_row, got.last_row, got.owns_first_row) == (want.first_row, want.last_row,
                                                                          want.owns_first_row), name
            assert (got.element_begin, got.element_end) == (want.element_begin, want.element_end)
            np.testing.assert_array_equal(got.local.row_start_offsets, want.local.row_start_offsets)
            np.testing.assert_array_equal(got.local.col_indices, want.local.col_indices)
            np.testing.assert_array_equal(got.local.values, want.local.values)
