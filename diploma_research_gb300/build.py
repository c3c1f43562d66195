"""Builds libdimgpu.so in-tree from csrc/*.cu with nvcc for sm_103a (GB300).

One nvcc process per translation unit, run in parallel, then one link step.  The library links the
CUDA runtime statically and depends on nothing from PyTorch.

``build(variant="test")`` builds a second library, libdimgpu_test.so, from the same sources with
DIMGPU_TEST_HOOKS defined and a 20 ms limit on every bounded device wait (DIMGPU_WAIT_NS): it adds
hooks that make a wait run out on purpose, for the tests of the device status words.  The product
never loads it.

``build(variant="probe")`` builds libdimgpu_probe.so from probe/*.cu: gather-only kernels that bench.py
times to measure the random-gather ceiling of an SpMV (``bench.py --spmv-only --gather-ceiling``).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(ROOT, "_build", "dimgpu")
LIB = os.path.join(OUT_DIR, "libdimgpu.so")
TEST_LIB = os.path.join(OUT_DIR, "libdimgpu_test.so")
PROBE_LIB = os.path.join(OUT_DIR, "libdimgpu_probe.so")
PROBE_SRC = os.path.join(HERE, "probe")
TEST_FLAGS = ["-DDIMGPU_TEST_HOOKS", "-DDIMGPU_WAIT_NS=20000000ull"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdimgpu")


def sources(variant: str = "product"):
    d = PROBE_SRC if variant == "probe" else CSRC
    return sorted(os.path.join(d, f) for f in os.listdir(d) if f.endswith((".cu", ".cpp")))


def headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))] + [
        os.path.join(ROOT, "include", "dimgpu.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout, r.stderr, file=sys.stderr)


def build(verbose: bool = False, force: bool = False, extra_flags=(), variant: str = "product") -> str:
    """Builds one variant ("product": libdimgpu.so, "test": libdimgpu_test.so, "probe":
    libdimgpu_probe.so); returns its path."""
    return build_variants((variant,), verbose=verbose, force=force, extra_flags=extra_flags)[0]


def build_variants(variants=("product", "test"), verbose: bool = False, force: bool = False, extra_flags=()):
    """Builds the given variants, all translation units of all of them in one parallel pool."""
    nv = nvcc()
    hdrs = headers()
    os.makedirs(OUT_DIR, exist_ok=True)
    jobs, links = [], []
    for variant in variants:
        if variant not in ("product", "test", "probe"):
            raise ValueError(f"unknown variant {variant!r}")
        lib_path = {"product": LIB, "test": TEST_LIB, "probe": PROBE_LIB}[variant]
        build_dir = BUILD_DIR + ("" if variant == "product" else "_" + variant)
        flags = list(extra_flags) + (TEST_FLAGS if variant == "test" else [])
        os.makedirs(build_dir, exist_ok=True)
        objs, fresh = [], False
        for src in sources(variant):
            obj = os.path.join(build_dir, os.path.splitext(os.path.basename(src))[0] + ".o")
            objs.append(obj)
            if force or _stale(obj, [src] + hdrs):
                jobs.append([nv, *ARCH, *NVCC_FLAGS, *flags, "-c", src, "-o", obj])
                fresh = True
        links.append((lib_path, objs, fresh))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs))
    for lib_path, objs, fresh in links:
        if force or fresh or _stale(lib_path, objs):
            _run([nv, *ARCH, "-shared", "-o", lib_path, *objs], verbose)
    return [lp for lp, _, _ in links]


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv,
                variant="test" if "--test" in sys.argv else "product"))
