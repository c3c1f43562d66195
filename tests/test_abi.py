"""The C-ABI library builds for sm_103a, loads, and exports every entry point include/dimgpu.h declares.
CPU only: argument checks that return before touching the device are exercised, nothing else."""
import ctypes
import subprocess

import numpy as np

from diploma_research_gb300 import _native as N


def test_builds_and_exports_every_declared_symbol(native):
    declared = N.declared_symbols()
    assert len(declared) >= 15
    for name in declared:
        assert hasattr(native, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", N.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert set(declared) <= exported
    # nothing else leaks from the library's C++ internals, and the test hooks are not in the product
    assert all(s.startswith("dimgpu_") for s in exported if not s.startswith("_"))
    assert not any(s.startswith("dimgpu_test_") for s in exported)


def test_test_library_adds_only_the_hooks(native_test):
    """libdimgpu_test.so exports the product's entry points plus the two test hooks."""
    declared = set(N.declared_symbols())
    out = subprocess.run(["nm", "-D", "--defined-only", N.TEST_LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert declared <= exported
    assert {s for s in exported if s.startswith("dimgpu_test_")} == {"dimgpu_test_withhold_run",
                                                                    "dimgpu_test_set_spmv_grid"}


def test_argument_errors_without_device(native):
    h = ctypes.c_void_p()
    rp = np.array([0, 1], np.uint32)
    ci = np.array([0], np.uint32)
    v = np.ones(1)
    # NULL output
    assert native.dimgpu_csr5_from_csr(1, 1, 1, rp.ctypes.data, ci.ctypes.data, v.ctypes.data, 0, None, None,
                                       None) == N.ERR_INVALID_ARGUMENT
    # omega 5
    opt = N.csr5_options(16, 5, 0, 0)
    rc = native.dimgpu_csr5_from_csr(1, 1, 1, rp.ctypes.data, ci.ctypes.data, v.ctypes.data, 0, ctypes.byref(opt),
                                     None, ctypes.byref(h))
    assert rc == N.ERR_INVALID_ARGUMENT
    assert b"omega" in native.dimgpu_last_error_string()
    # device layout with sigma not a multiple of 4
    opt = N.csr5_options(6, 32, 1, 0)
    assert native.dimgpu_csr5_from_csr(1, 1, 1, rp.ctypes.data, ci.ctypes.data, v.ctypes.data, 0, ctypes.byref(opt),
                                       None, ctypes.byref(h)) == N.ERR_INVALID_ARGUMENT
    # NULL matrix
    assert native.dimgpu_csr5_spmv(None, None, None, None, None) == N.ERR_INVALID_ARGUMENT
    assert native.dimgpu_cg_create(None, None, None, None) == N.ERR_INVALID_ARGUMENT
    assert native.dimgpu_csr5_status(None, None, None) == N.ERR_INVALID_ARGUMENT
    assert native.dimgpu_version() == 2


def test_product_does_not_import_oracle():
    """The product package never imports the oracle (test infrastructure)."""
    import os
    import re

    pkg = os.path.dirname(N.__file__)
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".hpp")):
                src = open(os.path.join(dirpath, f)).read()
                assert not re.search(r"^\s*(import|from)\s+oracle", src, re.M), f
                assert "csr5_oracle" not in src, f


def test_probe_library_builds_apart_from_the_product(native):
    """libdimgpu_probe.so (the gather-only kernels bench.py --spmv-only --gather-ceiling times) builds from
    probe/*.cu alone and exports only its measurement entry points; the product library contains none."""
    from diploma_research_gb300 import build as B

    path = B.build(variant="probe")
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert {s for s in exported if s.startswith("dimgpu_")} == {
        "dimgpu_probe_words_per_cta", "dimgpu_probe_gather", "dimgpu_probe_cluster_gather"}
    prod = subprocess.run(["nm", "-D", "--defined-only", N.LIB_PATH], capture_output=True, text=True).stdout
    assert "dimgpu_probe_" not in prod
