"""Command line of the matrix workflow (the reference's dim_cli and csr5_single_node benchmark).

  python -m diploma_research_gb300.cli store-matrix INPUT [--output O] [--in-group-name A]
                                                   [--group-name A] [--append] [--format csr|csr5]
  python -m diploma_research_gb300.cli csr5-spmv INPUT [--matrix-group A] [--num-runs N]
                                                [--output-file F] [--vector-dataset Y] [--overwrite]
  python -m diploma_research_gb300.cli compare-results INPUT [--input-file-2 F2] [--lhs-group /]
                                                      [--lhs-dataset Y] [--rhs-group /] [--rhs-dataset Y]

store-matrix (apps/dim_cli/subcommands/store_matrix.cpp:82-140): reads a Matrix Market file or the
MATLAB-compatible CSR group of an HDF5 file and writes it as a MATLAB-compatible CSR group or, with
--format csr5, as the reference's CSR5 group (sigma 16, omega 4, converted on the GPU).  The output
name defaults to INPUT with its extensions replaced by ".<format>.h5".
csr5-spmv (benchmarks/csr5/dim/main.cpp:47-79): loads a CSR5 group, runs y = A x with x = 1 on the GPU
(5 warm-up products, then --num-runs timed ones) and optionally stores y as an f64 dataset.
compare-results (apps/dim_cli/subcommands/compare_results.cpp:9-39): compares two stored vectors
element by element with the reference's rule |l - r| <= 0.01 |r|; exit status 0 when equal, 1 if not.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

from .io import h5
from .io import matrix_market as mm


def _log(msg: str):
    print(f"[dim] {msg}", flush=True)


def _deduce_output(inp: str, fmt: str) -> str:
    base = inp
    while os.path.splitext(base)[1]:
        base = os.path.splitext(base)[0]
    return f"{base}.{fmt}.h5"


def load_as_csr(path: str, in_group: str = "A"):
    """A Matrix Market file, or the MATLAB-compatible CSR group of an HDF5 file (store_matrix.cpp:72-80)."""
    if h5.is_hdf5(path):
        return h5.read_matlab_compatible(path, in_group)
    return mm.load_as_csr(path)


def reference_csr5_arrays(m):
    """The reference-layout CSR5 arrays (csr5<double,16,4,uint32_t>) of a host CSR matrix, converted on
    the GPU."""
    from .csr5 import csr5

    A = csr5.from_csr(m, sigma=16, omega=4)
    return A.export()


def store_matrix(args) -> int:
    t0 = time.perf_counter()
    m = load_as_csr(args.input, args.in_group_name)
    _log(f"load and conversion to CSR took: {time.perf_counter() - t0:.3f}s "
         f"({m.dimensions.rows} x {m.dimensions.cols}, {m.nnz} non-zeros)")
    out = args.output or _deduce_output(args.input, args.format)
    _log(f"storing matrix as group '{args.group_name}' to {out}")
    t0 = time.perf_counter()
    if args.format == "csr":
        h5.write_matlab_compatible(out, args.group_name, m, append=args.append)
    else:
        e = reference_csr5_arrays(m)
        h5.store_csr5(out, args.group_name, e, m.dimensions.cols, append=args.append)
    _log(f"storing as HDF5 took: {time.perf_counter() - t0:.3f}s")
    return 0


def csr_from_csr5_arrays(a):
    """CSR (values and indices back in row order) from stored reference-layout CSR5 arrays."""
    from .layout import unpermute
    from .mat import csr, dimensions_t

    vals = unpermute(a.vals, a.tile_ptr, 16, 4, "ref")
    cols = unpermute(a.col_idx, a.tile_ptr, 16, 4, "ref")
    return csr(dimensions_t(a.rows, a.cols), vals, a.row_ptr, cols)


def csr5_spmv(args) -> int:
    import torch

    from .csr5 import csr5

    t0 = time.perf_counter()
    a = h5.load_csr5_arrays(args.input, args.matrix_group)
    A = csr5.from_csr(csr_from_csr5_arrays(a))
    _log(f"CSR5 loading took {time.perf_counter() - t0:.3f}s")
    x = torch.ones(a.cols, device="cuda", dtype=torch.float64)
    y = torch.zeros(a.rows, device="cuda", dtype=torch.float64)
    cal = A.create_calibrator()
    for _ in range(5):
        A.spmv(x, y, cal)
    total = 0.0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for i in range(args.num_runs):
        ev0.record()
        A.spmv(x, y, cal)
        ev1.record()
        torch.cuda.synchronize()
        dt = ev0.elapsed_time(ev1) * 1e-3
        total += dt
        _log(f"iteration {i} took {dt * 1e6:.1f}us")
    _log(f"CSR5 SpMV took {total / max(1, args.num_runs) * 1e6:.1f}us on average")
    if args.output_file:
        h5.write_vector(args.output_file, args.vector_dataset, y.cpu().numpy(), overwrite=args.overwrite)
    return 0


def compare_results(args) -> int:
    def load(path, group, dataset):
        name = f"{os.path.basename(path)}:{group}{dataset}"
        return name, h5.read_vector(path, group.rstrip("/") + "/" + dataset)

    lid, lhs = load(args.input_file, args.lhs_group, args.lhs_dataset)
    rid, rhs = load(args.input_file_2 or args.input_file, args.rhs_group, args.rhs_dataset)
    n = lhs.size
    if rhs.size < n:
        _log(f"vector {rid} has {rhs.size} elements, {lid} has {n}")
        return 1
    bad = np.flatnonzero(~(np.abs(lhs - rhs[:n]) <= 0.01 * np.abs(rhs[:n])))
    for i in bad[:100]:
        _log(f"at {i}: expected {lhs[i]!r}, got {rhs[i]!r}")
    if bad.size:
        _log(f"vectors {lid} and {rid} are not equal")
        return 1
    _log(f"vectors {lid} and {rid} are equal")
    return 0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="dim")
    sub = ap.add_subparsers(dest="cmd", required=True)
    s = sub.add_parser("store-matrix")
    s.add_argument("input")
    s.add_argument("--output")
    s.add_argument("--in-group-name", default="A")
    s.add_argument("--group-name", default="A")
    s.add_argument("--append", action="store_true")
    s.add_argument("--format", choices=["csr", "csr5"], default="csr")
    s.set_defaults(func=store_matrix)
    b = sub.add_parser("csr5-spmv")
    b.add_argument("input")
    b.add_argument("--matrix-group", default="A")
    b.add_argument("--num-runs", type=int, default=10)
    b.add_argument("--output-file")
    b.add_argument("--vector-dataset", default="Y")
    b.add_argument("--overwrite", action="store_true")
    b.set_defaults(func=csr5_spmv)
    c = sub.add_parser("compare-results")
    c.add_argument("input_file")
    c.add_argument("--input-file-2")
    c.add_argument("--lhs-group", default="/")
    c.add_argument("--lhs-dataset", default="Y")
    c.add_argument("--rhs-group", default="/")
    c.add_argument("--rhs-dataset", default="Y")
    c.set_defaults(func=compare_results)
    args = ap.parse_args(argv)
    return args.func(args)


if __name__ == "__main__":
    sys.exit(main())
