"""The CLI workflow on the GPU: store-matrix --format csr5 (conversion on the device, the reference's
CSR5 arrays bit for bit), csr5-spmv with --output-file, and compare-results against the oracle's y."""
import numpy as np
import pytest

import oracle
from diploma_research_gb300 import cli
from diploma_research_gb300.io import h5
from diploma_research_gb300.io import matrix_market as mm
from helpers import random_csr

pytestmark = pytest.mark.gpu


def test_store_spmv_compare(native, tmp_path):
    rng = np.random.default_rng(12)
    m = random_csr(rng, 3000, 3000, 8.0, empty_frac=0.05, long_rows=2, long_len=(300, 1500))
    src = tmp_path / "m.mtx"
    mm.save_coo(src, m)
    assert cli.main(["store-matrix", str(src), "--format", "csr5"]) == 0
    out = tmp_path / "m.csr5.h5"
    a = h5.load_csr5_arrays(out, "A")
    o = oracle.OracleCSR5(3000, 3000, m.row_start_offsets, m.col_indices, m.values, 16, 4)
    assert np.array_equal(a.tile_ptr, o.tile_ptr)
    assert np.array_equal(a.tile_desc, o.tile_desc.astype(np.uint32))
    assert np.array_equal(a.tile_desc_offset_ptr, o.tile_desc_offset_ptr)
    assert np.array_equal(a.tile_desc_offset, o.tile_desc_offset)
    assert np.array_equal(a.vals, o.vals) and np.array_equal(a.col_idx, o.col_idx)

    res = tmp_path / "y.h5"
    assert cli.main(["csr5-spmv", str(out), "--num-runs", "2", "--output-file", str(res)]) == 0
    y = h5.read_vector(res, "Y")
    S = m.to_scipy()
    ones = np.ones(3000)
    assert np.all(np.abs(y - S @ ones) <= 1e-12 * (abs(S) @ ones) + 1e-300)
    # the reference's y (oracle) in a second file, compared with the reference's 1 % rule
    ref = tmp_path / "ref.h5"
    h5.write_vector(ref, "Y", o.spmv(ones))
    assert cli.main(["compare-results", str(res), "--input-file-2", str(ref)]) == 0
    with pytest.raises(FileExistsError):
        cli.main(["csr5-spmv", str(out), "--num-runs", "1", "--output-file", str(res)])
    assert cli.main(["csr5-spmv", str(out), "--num-runs", "1", "--output-file", str(res), "--overwrite"]) == 0
