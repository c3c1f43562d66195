"""include/dimgpu.hpp, the C++ binding a dim user includes in place of dim::mat::csr5: it compiles
against the reference's own dim::mat::csr<double> (include/dim/mat/storage_formats/csr.h, where the
reference checkout exists) and against a stand-in with the same members, and on the GPU the compiled
program's products and CG solution agree with the oracle (the reference's SpMV and CG restated in C)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dimgpu_cpp_check.cpp")
LIBDIR = os.path.join(ROOT, "diploma_research_gb300", "_lib")
OUT = os.path.join(ROOT, "_build", "cpp")


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _compile(exe, with_reference):
    os.makedirs(OUT, exist_ok=True)
    cuda = _cuda_home()
    cmd = ["g++", "-std=gnu++20", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), SRC, "-o", exe, "-L", LIBDIR, "-ldimgpu",
           f"-Wl,-rpath,{LIBDIR}", "-L", os.path.join(cuda, "lib64"), "-lcudart", f"-Wl,-rpath,{cuda}/lib64"]
    if with_reference:
        cmd[1:1] = ["-fopenmp", "-Wno-interference-size", "-Wno-unused-parameter", "-DDIMGPU_WITH_REFERENCE_CSR",
                    "-I", os.path.join(oracle.ref_root(), "include")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


def _reference_available():
    return os.path.isfile(os.path.join(oracle.ref_root(), "include", "dim", "mat", "storage_formats", "csr.h"))


def test_binding_compiles_with_standin(native):
    _compile(os.path.join(OUT, "check_standin"), False)


@pytest.mark.skipif(not _reference_available(), reason="needs the reference checkout")
def test_binding_compiles_against_reference_csr(native):
    _compile(os.path.join(OUT, "check_reference"), True)


@pytest.mark.gpu
def test_cpp_program_against_oracle(native, tmp_path):
    variants = [False] + ([True] if _reference_available() else [])
    for with_ref in variants:
        exe = _compile(os.path.join(OUT, "check_reference" if with_ref else "check_standin"), with_ref)
        out = str(tmp_path / f"out_{int(with_ref)}.bin")
        r = subprocess.run([exe, out], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        raw = np.fromfile(out, dtype=np.uint8)
        n = int(raw[:8].view(np.uint64)[0])
        x, y, z = raw[8:].view(np.float64).reshape(3, n)
        from diploma_research_gb300.generators import laplacian_2d_5pt

        m = laplacian_2d_5pt(64)
        assert m.dimensions.rows == n
        y_ref = oracle.csr_spmv(n, m.row_start_offsets, m.col_indices, m.values, x)
        absax = oracle.abs_spmv(n, m.row_start_offsets, m.col_indices, m.values, x)
        assert np.all(np.abs(y - y_ref) <= 1e-12 * absax)
        o = oracle.OracleCSR5(n, n, m.row_start_offsets, m.col_indices, m.values)
        zo, _, _ = o.cg(y, tol=1e-10)
        assert np.linalg.norm(z - zo) <= 1e-9 * np.linalg.norm(zo)
        assert np.linalg.norm(z - x) <= 1e-6 * np.linalg.norm(x)
