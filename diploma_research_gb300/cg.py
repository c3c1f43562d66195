"""Conjugate gradients on the device (the reference's dim_sp CG loop,
benchmarks/conjugate_gradient/dim_sp/main.cpp:78-141, with the threshold of docs/paper/thesis.tex:2127-2160).

``CGSolver`` keeps the workspace and the captured CUDA graph of one matrix; ``solve`` takes ``b`` and
an initial guess ``x`` either as device arrays (``__cuda_array_interface__``, e.g. torch CUDA float64
tensors; x is overwritten) or as numpy arrays (copied in and out).  ``precision="fp64"`` runs the
reference algorithm in f64; ``precision="mixed"`` runs it on f32 values/vectors with f64 dots, f64 x
and reliable f64 residual updates, and stops on the same true-residual criterion.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .csr5 import csr5


@dataclass
class cg_result:
    iterations: int
    reliable_updates: int
    rel_residual: float            # ||b - A x|| / ||b|| recomputed in f64
    recurrence_rel_residual: float
    seconds: float                 # device time of the solve
    converged: bool


_PREC = {"fp64": N.CG_FP64, "mixed": N.CG_MIXED}
_ENGINE = {"auto": N.CG_ENGINE_AUTO, "graph": N.CG_ENGINE_GRAPH}


class CGSolver:
    """engine: "auto" or "graph" (one CUDA graph, three kernels per iteration, the reference's
    recurrence); use_graph=False runs the same kernels from a host-driven loop."""

    def __init__(self, A: csr5, tol: float = 1e-10, max_it: int = 100000, precision: str = "fp64",
                 use_graph: bool = True, reliable_delta: float = 0.03, stream=None, engine: str = "auto"):
        if precision not in _PREC:
            raise ValueError(f"precision must be one of {sorted(_PREC)}")
        if engine not in _ENGINE:
            raise ValueError(f"engine must be one of {sorted(_ENGINE)}")
        self.A = A
        self.params = N.cg_params(float(tol), int(max_it), _PREC[precision], 1 if use_graph else 0,
                                  float(reliable_delta), _ENGINE[engine])
        h = ctypes.c_void_p()
        N.check(N.lib().dimgpu_cg_create(A._h, ctypes.byref(self.params), N.stream_ptr(stream), ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            N.lib().dimgpu_cg_destroy(h)
            self._h = None

    def solve(self, b, x=None, stream=None, raise_on_failure: bool = True):
        """Solves A x = b; returns (x, cg_result).  Host inputs give a new numpy x."""
        n = self.A.dimensions.rows
        st = N.cg_stats()
        L = N.lib()
        if N.is_device_array(b):
            if x is None or not N.is_device_array(x):
                raise ValueError("device b needs a device x (initial guess, overwritten)")
            rc = L.dimgpu_cg_solve(self._h, N.device_ptr(b, "<f8", n), N.device_ptr(x, "<f8", n), ctypes.byref(st),
                                   N.stream_ptr(stream))
            out = x
        else:
            bh = np.ascontiguousarray(b, np.float64)
            if bh.size != n:
                raise ValueError("b has the wrong length")
            out = np.zeros(n) if x is None else np.array(x, np.float64, copy=True)
            rc = L.dimgpu_cg_solve_host(self._h, bh.ctypes.data, out.ctypes.data, ctypes.byref(st))
        res = cg_result(int(st.iterations), int(st.reliable_updates), float(st.rel_residual),
                        float(st.recurrence_rel_residual), float(st.seconds), rc == N.OK)
        if rc != N.OK and (raise_on_failure or rc not in (N.ERR_NOT_CONVERGED, N.ERR_BREAKDOWN)):
            N.check(rc)
        return out, res


def cg(A: csr5, b, x0=None, tol: float = 1e-10, max_it: int = 100000, precision: str = "fp64",
       use_graph: bool = True, engine: str = "auto"):
    """One-shot solve: returns (x, cg_result)."""
    return CGSolver(A, tol=tol, max_it=max_it, precision=precision, use_graph=use_graph,
                    engine=engine).solve(b, x0)


@dataclass
class block_cg_result:
    iterations: int               # iterations of the slowest column
    reliable_updates: int
    max_rel_residual: float
    seconds: float
    converged_columns: int
    col_iterations: list
    col_rel_residual: list
    spmm_shape: int = -1           # the autotuned shape of the iteration's SpMM

class BlockCGSolver:
    """k <= 32 simultaneous CG solves sharing one CSR5 SpMM per iteration, per-column convergence masks.

    solve(B, X) takes device arrays of shape (n, k) (float64, row-major); X holds the initial guesses and
    receives the solutions."""

    def __init__(self, A: csr5, k: int, tol: float = 1e-10, max_it: int = 100000, precision: str = "fp64",
                 use_graph: bool = True, reliable_delta: float = 0.1, stream=None):
        if precision not in _PREC:
            raise ValueError(f"precision must be one of {sorted(_PREC)}")
        self.A, self.k = A, int(k)
        self.params = N.cg_params(float(tol), int(max_it), _PREC[precision], 1 if use_graph else 0,
                                  float(reliable_delta), N.CG_ENGINE_GRAPH)
        h = ctypes.c_void_p()
        N.check(N.lib().dimgpu_block_cg_create(A._h, self.k, ctypes.byref(self.params), N.stream_ptr(stream),
                                               ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            N.lib().dimgpu_block_cg_destroy(h)
            self._h = None

    def solve(self, B, X, stream=None, raise_on_failure: bool = True):
        n = self.A.dimensions.rows
        for name, a in (("B", B), ("X", X)):
            shp = a.__cuda_array_interface__["shape"]
            if tuple(shp) != (n, self.k):
                raise ValueError(f"{name} must have shape ({n}, {self.k}), got {tuple(shp)}")
        st = N.block_cg_stats()
        its = (ctypes.c_int64 * self.k)()
        rel = (ctypes.c_double * self.k)()
        rc = N.lib().dimgpu_block_cg_solve(self._h, N.device_ptr(B, "<f8"), self.k, N.device_ptr(X, "<f8"), self.k,
                                           ctypes.byref(st), its, rel, N.stream_ptr(stream))
        res = block_cg_result(int(st.iterations), int(st.reliable_updates), float(st.max_rel_residual),
                              float(st.seconds), int(st.converged_columns), list(its), list(rel), int(st.spmm_shape))
        if rc != N.OK and (raise_on_failure or rc not in (N.ERR_NOT_CONVERGED, N.ERR_BREAKDOWN)):
            N.check(rc)
        return X, res
