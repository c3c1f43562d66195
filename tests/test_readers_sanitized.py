"""The host file readers (csrc/h5.cpp, csrc/mm.cpp) built with AddressSanitizer and UBSan and run over a
fixed-seed corpus of truncated and byte-corrupted HDF5 and Matrix Market files: no out-of-bounds access
and no undefined behaviour on any of them (a report stops the driver).  The device entry points the
readers could reach are stubbed (tests/cpp/readers_sanitized_stubs.cpp).  CPU only; skipped where the
compiler has no sanitizer runtime or the CUDA headers are absent."""
import os
import random
import shutil
import struct
import subprocess

import numpy as np
import pytest

from diploma_research_gb300.io import h5
from helpers import random_csr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
CSRC = os.path.join(ROOT, "diploma_research_gb300", "csrc")
OUT = os.path.join(ROOT, "_build", "cpp")


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    return inc if os.path.isfile(os.path.join(inc, "cuda_runtime.h")) else None


@pytest.fixture(scope="module")
def driver():
    inc = _cuda_include()
    if inc is None:
        pytest.skip("CUDA headers not found")
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "readers_sanitized")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
           "-fno-omit-frame-pointer", "-I", os.path.join(ROOT, "include"), "-I", inc, "-I", CSRC,
           os.path.join(CSRC, "h5.cpp"), os.path.join(CSRC, "mm.cpp"),
           os.path.join(CPP, "readers_sanitized_stubs.cpp"), os.path.join(CPP, "readers_sanitized_driver.cpp"),
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("no sanitizer build here: " + r.stderr[-300:])
    return exe


def _corrupt(raw: bytes, rnd: random.Random, n: int, head: int, alphabet=None):
    out = [raw[:k] for k in range(0, len(raw), max(1, len(raw) // 40))]
    for _ in range(n):
        b = bytearray(raw)
        lim = min(len(b), head) if rnd.random() < 0.6 else len(b)
        for _ in range(rnd.randint(1, 5)):
            i = rnd.randrange(lim)
            b[i] = rnd.choice(alphabet) if alphabet else (rnd.randrange(256) if rnd.random() < 0.5
                                                          else b[i] ^ (1 << rnd.randrange(8)))
        out.append(bytes(b))
    return out


def _run(exe, d, *args):
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([exe, str(d), *args], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0 and "runtime error" not in r.stderr and "Sanitizer" not in r.stderr, \
        r.stdout[-500:] + r.stderr[-3000:]
    return r.stdout


def test_hdf5_reader_on_corrupted_files(driver, tmp_path, monkeypatch):
    import test_h5_abi as T

    rng = np.random.default_rng(9)
    m = random_csr(rng, 150, 120, 4.0, empty_frac=0.1)
    y = rng.uniform(-1, 1, 200)
    rnd = random.Random(11)
    d = tmp_path / "h5"
    d.mkdir()
    k = 0
    for form in (None, "dynamic", "two_level", "continued_header"):
        p = tmp_path / f"base_{form}.h5"
        if form:
            monkeypatch.setattr(h5, "_write_dataset", T._chunked_writer(**T.CHUNKED[form]))
        h5.write_matlab_compatible(p, "A", m)
        h5.write_vector(p, "Y", y)
        monkeypatch.undo()
        for c in _corrupt(p.read_bytes(), rnd, 150, 2048):
            (d / f"{k:05d}.h5").write_bytes(c)
            k += 1
    # the corruption the fuzzing found: `ir` claiming 2^39 more elements than `data` (a 2 TB allocation
    # unless the count is checked first)
    raw = bytearray((tmp_path / "base_None.h5").read_bytes())
    first = bytes(raw).find(struct.pack("<Q", m.nnz))
    at = bytes(raw).find(struct.pack("<Q", m.nnz), first + 8)
    raw[at:at + 8] = struct.pack("<Q", m.nnz + (1 << 39))
    (d / "crafted_ir.h5").write_bytes(bytes(raw))
    assert f"files {k + 1} " in _run(driver, d)


def test_matrix_market_reader_on_corrupted_files(driver, tmp_path):
    import test_mm_abi as T

    rnd = random.Random(12)
    d = tmp_path / "mm"
    d.mkdir()
    k = 0
    for case in ("general", "symmetric", "pattern_symmetric", "integer"):
        banner, (r, c, n), kw = T.CASES[case]
        p = tmp_path / f"{case}.mtx"
        T._write(p, banner, f"{r} {c} {n}", T._random_entries(np.random.default_rng(len(case)), r, c, n, **kw))
        for cc in _corrupt(p.read_bytes(), rnd, 150, 120, alphabet=b"0123456789 \n\t%.-+eE"):
            (d / f"{k:05d}.mtx").write_bytes(cc)
            k += 1
    # the corruption the fuzzing found: a symmetric file that is not square, whose mirrored entry (58, 22)
    # would lie past the 50 rows
    (d / "crafted_nonsquare.mtx").write_text(
        "%%MatrixMarket matrix coordinate real hermitian\n50 90 2\n22 58 1.5\n3 3 2.0\n")
    assert f"files {k + 1} " in _run(driver, d, "mm")
