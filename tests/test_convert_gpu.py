"""Device CSR -> CSR5 conversion: bit-exact against the reference's arrays at (sigma=16, omega=4) and
against the oracle's construction for the 32-lane device layout."""
import os

import numpy as np
import pytest

import oracle
from diploma_research_gb300.csr5 import csr5
from diploma_research_gb300.layout import permute
from diploma_research_gb300.mat import csr, dimensions_t
from helpers import csr_from_lengths, random_csr

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
pytestmark = pytest.mark.gpu


def _dev_vs_oracle(m: csr, sigma: int):
    A = csr5.from_csr(m, sigma=sigma, omega=32)
    e = A.export()
    o = oracle.OracleCSR5(m.dimensions.rows, m.dimensions.cols, m.row_start_offsets, m.col_indices, m.values,
                          sigma, 32)
    assert e.tile_count == o.tile_count
    assert A.tail_partition_start() == o.tail_partition_start
    assert np.array_equal(e.tile_ptr, o.tile_ptr)
    assert np.array_equal(e.tile_desc.astype(np.uint64), o.tile_desc)
    assert np.array_equal(e.tile_desc_offset_ptr, o.tile_desc_offset_ptr)
    assert np.array_equal(e.tile_desc_offset, o.tile_desc_offset)
    assert np.array_equal(e.vals, permute(m.values, o.tile_ptr, sigma, 32, "f64"))
    assert np.array_equal(e.col_idx, permute(m.col_indices, o.tile_ptr, sigma, 32, "q32"))
    assert np.array_equal(e.row_ptr, m.row_start_offsets)
    return A


def _ref_layout_vs_arrays(m: csr, tile_ptr, tile_desc, tdo_ptr, tdo, vals, col, tail):
    A = csr5.from_csr(m, sigma=16, omega=4)
    e = A.export()
    assert np.array_equal(e.tile_ptr, tile_ptr)
    assert np.array_equal(e.tile_desc, tile_desc)
    assert np.array_equal(e.tile_desc_offset_ptr, tdo_ptr)
    assert np.array_equal(e.tile_desc_offset, tdo)
    assert np.array_equal(e.vals, vals)
    assert np.array_equal(e.col_idx, col)
    assert A.tail_partition_start() == tail


def test_mm_mtx_reference_layout_bitexact(native):
    g = np.load(os.path.join(GOLDEN, "mm_mtx.npz"))
    m = csr(dimensions_t(int(g["rows"]), int(g["cols"])), g["vals"], g["row_ptr"], g["col_idx"])
    _ref_layout_vs_arrays(m, g["ref_tile_ptr"], g["ref_tile_desc"], g["ref_tdo_ptr"], g["ref_tdo"], g["ref_vals"],
                          g["ref_col_idx"], int(g["ref_tail"]))
    A = csr5.from_csr(m, sigma=16, omega=4)
    assert A.csr5_info.tile_count == 2 and A.tail_partition_start() == 154  # test_csr5.cpp:37-38


def test_fixture_cases_reference_layout_bitexact(native):
    g = np.load(os.path.join(GOLDEN, "ref_cases.npz"))
    for k in g["cases"]:
        p = f"c{k}_"
        m = csr(dimensions_t(int(g[p + "rows"]), int(g[p + "cols"])), g[p + "vals"], g[p + "row_ptr"],
                g[p + "col_idx"])
        _ref_layout_vs_arrays(m, g[p + "tile_ptr"], g[p + "tile_desc"], g[p + "tdo_ptr"], g[p + "tdo"],
                              g[p + "csr5_vals"], g[p + "csr5_col"], int(g[p + "tail"]))


def test_mm_mtx_device_layout(native):
    g = np.load(os.path.join(GOLDEN, "mm_mtx.npz"))
    m = csr(dimensions_t(int(g["rows"]), int(g["cols"])), g["vals"], g["row_ptr"], g["col_idx"])
    _dev_vs_oracle(m, 16)


@pytest.mark.parametrize("sigma", [16, 32])
@pytest.mark.parametrize("seed", range(10))
def test_random_device_layout(native, seed, sigma):
    rng = np.random.default_rng(seed)
    m = random_csr(rng, int(rng.integers(10, 6000)), int(rng.integers(10, 6000)), float(rng.uniform(0.2, 40)),
                   empty_frac=float(rng.choice([0, 0.1, 0.7])), long_rows=int(rng.integers(0, 5)),
                   long_len=(500, 3000))
    _dev_vs_oracle(m, sigma)


@pytest.mark.parametrize("seed", range(4))
def test_random_reference_layout_vs_oracle(native, seed):
    rng = np.random.default_rng(100 + seed)
    m = random_csr(rng, int(rng.integers(10, 3000)), int(rng.integers(10, 3000)), float(rng.uniform(0.2, 30)),
                   empty_frac=float(rng.choice([0, 0.3])), long_rows=2)
    o = oracle.OracleCSR5(m.dimensions.rows, m.dimensions.cols, m.row_start_offsets, m.col_indices, m.values, 16, 4)
    _ref_layout_vs_arrays(m, o.tile_ptr, o.tile_desc.astype(np.uint32), o.tile_desc_offset_ptr, o.tile_desc_offset,
                          o.vals, o.col_idx, o.tail_partition_start)


def test_edge_cases_device_layout(native):
    rng = np.random.default_rng(9)
    for lens, cols in [([3, 0, 5, 1], 10), ([0, 0, 0], 4), ([0] * 50 + [512] + [0] * 50, 600), ([5000], 6000),
                       ([0, 700, 0, 0, 2000, 1, 0], 3000), ([512] * 4, 512), ([1] * 2048, 7), ([0] * 1000 + [1], 2)]:
        m = csr_from_lengths(lens, cols, rng)
        _dev_vs_oracle(m, 16)
        _dev_vs_oracle(m, 32)


def test_rejects_malformed_csr(native):
    m = csr(dimensions_t(3, 3), np.ones(3), np.array([0, 1, 2, 3], np.uint32), np.array([0, 1, 7], np.uint32))
    with pytest.raises(ValueError):
        csr5.from_csr(m)
    with pytest.raises(ValueError):
        csr5.from_csr(m, omega=5)


@pytest.mark.slow
def test_stencil27_128_device_layout(native):
    from diploma_research_gb300.generators import stencil_3d_27pt

    _dev_vs_oracle(stencil_3d_27pt(128), 16)
