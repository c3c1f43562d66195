#!/usr/bin/env python3
"""Benchmark: CG to 1e-10 relative residual on the 3-D 27-point 128^3 stencil (n = 2,097,152,
nnz = 55,742,968, FP64, diagonal 26 + 1e-3, b = A x*, x* ~ U[-1,1] seed 1), with the FP64 CSR5 SpMV
roofline beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

One step = one complete CG solve from x0 = 0 on device-resident inputs (the matrix, 702 MB of CSR5
data, is larger than the 129 MB L2, so no flush is needed between steps).  `value` is FP64 seconds per
solve; the mixed-precision solve (f32 inner recurrence, f64 reliable updates, same f64 residual
criterion) is reported beside it.  `e2e` runs the same FP64 solve through the C ABI with host
buffers (pinned), host<->device copies included.  `roofline` is the FP64 SpMV kernel timed alone
with CUDA events: algorithmic bytes 12*nnz + 16*n per launch.

--impl reference times the reference's CPU CG (the C restatement of its CSR5 AVX2/OpenMP path,
oracle/csr5_oracle.c, with all host threads) on the same workload.
Multi-GPU: replicas only (each rank solves its own copy); max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "CG s to 1e-10 rel. residual, mixed vs FP64 on 1 GB300; SpMV GB/s vs HBM peak"
WORKLOAD = "stencil27_128"
TOL = 1e-10
DESCR = {
    "lap2d_512": "2-D 5-point Laplacian 512^2",
    "stencil27_128": "3-D 27-point stencil 128^3",
    "powerlaw_4m": "power-law rows (Zipf 2.0, up to 10,000 off-diagonals, symmetrised, diagonally dominant)",
    "lap3d7_192": "3-D 7-point Laplacian 192^3",
    "aniso2d_1024": "2-D anisotropic diffusion 1024^2 (kappa = exp(Gaussian random field), 10:1)",
}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _profile_traffic():
    """Per-launch DRAM bytes of the FP64 SpMV from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "spmv_f64_stencil27_128.md")
    if not os.path.isfile(p):
        return None
    with open(p) as fh:
        for line in fh:
            if line.strip().startswith("traffic_bytes_per_launch:"):
                try:
                    return int(float(line.split(":", 1)[1].strip()))
                except ValueError:
                    return None
    return None


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons every 100 ms while alive."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _barrier_max(value: float, ws: int):
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _workload():
    from diploma_research_gb300.generators import WORKLOADS, rhs

    m = WORKLOADS[WORKLOAD]["build"]()
    xs, b = rhs(m, WORKLOADS[WORKLOAD]["seed"])
    return m, xs, b


def _config(m):
    """The workload description both arms print (identical strings for one and the same system)."""
    n, nnz = m.dimensions.rows, m.nnz
    mb = (12 * nnz + 4 * (n + 1)) / 1e6
    return {"workload": f"{WORKLOAD}: {DESCR[WORKLOAD]}, n={n}, nnz={nnz}, CG to {TOL:g} from x0 = 0, FP64",
            "global_batch": 1, "seq_len": n,
            "l2": f"{mb:.0f} MB of CSR data vs 129 MB L2" + ("; no flush" if mb > 135 else
                                                             "; L2-resident, no flush (solve-level timing)")}


def run_reference(args):
    """The reference's CPU CG (oracle/csr5_oracle.c restating csr5.h + dim_sp) on all host threads: one
    full solve to the tolerance per step."""
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    import oracle

    m, xs, b = _workload()
    n = m.dimensions.rows
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    o = oracle.OracleCSR5(n, n, m.row_start_offsets, m.col_indices, m.values, 16, 4)
    convert_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        _, iters, rel = o.cg(b, tol=TOL, nthreads=threads)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        _, iters, rel = o.cg(b, tol=TOL, nthreads=threads)
        times.append(time.perf_counter() - t)
    value = statistics.mean(times)
    sample = (f"full CPU CG solves of {WORKLOAD} to {TOL:g} ({iters} iterations, rel. residual {rel:.2e}), "
              f"one per step, oracle/csr5_oracle.c on {threads} host threads")
    out = {"metric": METRIC, "value": value, "unit": "s", "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3,
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": _config(m), "execution": f"CPU, OpenMP on {threads} threads",
           "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "iterations": iters, "convert_s": convert_s}
    print(json.dumps(out))
    return 0


def run_gpu(args):
    import numpy as np
    import torch

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo", init_method="env://")
    torch.cuda.set_device(local)
    from diploma_research_gb300 import build as B

    B.build()
    from diploma_research_gb300.cg import CGSolver
    from diploma_research_gb300.csr5 import csr5

    m, xs, b = _workload()
    n, nnz = m.dimensions.rows, m.nnz
    t0 = time.perf_counter()
    A = csr5.from_csr(m)
    torch.cuda.synchronize()
    convert_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    bd = torch.tensor(b, device="cuda", dtype=torch.float64)
    xd = torch.zeros(n, device="cuda", dtype=torch.float64)
    s64 = CGSolver(A, tol=TOL, precision="fp64", stream=stream, use_graph=not args.no_graph)
    smx = CGSolver(A, tol=TOL, precision="mixed", stream=stream, use_graph=not args.no_graph)

    def solve(solver):
        xd.zero_()
        return solver.solve(bd, xd, stream=stream)[1]

    # ---- FP64 CG: the headline ----
    for _ in range(args.warmup):
        res64 = solve(s64)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(local).__enter__()  # sampled across every timed region below
    ev0.record(stream)
    iters64 = []
    for _ in range(args.steps):
        r = solve(s64)
        iters64.append(r.iterations)
    ev1.record(stream)
    torch.cuda.synchronize()
    sec64 = ev0.elapsed_time(ev1) * 1e-3 / args.steps
    sec64 = _barrier_max(sec64, ws)
    x64 = xd.cpu().numpy()
    err64 = float(np.linalg.norm(x64 - xs) / np.linalg.norm(xs))
    res64 = r

    # ---- mixed-precision CG ----
    for _ in range(max(1, args.warmup)):
        resm = solve(smx)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        resm = solve(smx)
    ev1.record(stream)
    torch.cuda.synchronize()
    secm = _barrier_max(ev0.elapsed_time(ev1) * 1e-3 / args.steps, ws)
    xmx = xd.cpu().numpy()
    errm = float(np.linalg.norm(xmx - xs) / np.linalg.norm(xs))

    # ---- FP64 SpMV alone: the dominant kernel, for the roofline ----
    x1 = torch.tensor(np.random.default_rng(5).uniform(-1, 1, n), device="cuda", dtype=torch.float64)
    y1 = torch.empty(n, device="cuda", dtype=torch.float64)
    cal = A.create_calibrator()
    for _ in range(5):
        A.spmv(x1, y1, cal, stream=stream)
    spmv_reps = 50
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(spmv_reps):
        A.spmv(x1, y1, cal, stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    spmv_s = ev0.elapsed_time(ev1) * 1e-3 / spmv_reps
    spmv_bytes = 12 * nnz + 16 * n
    spmv_gbs = spmv_bytes / spmv_s / 1e9
    peak, peak_kind = _peaks()

    # the CG variants of the kernel, alone: y = A x with x.y fused (f64), and the f32 product
    from diploma_research_gb300 import _native as N

    dot_d = torch.zeros(1, device="cuda", dtype=torch.float64)
    Lb = N.lib()

    def spmv_dot():
        N.check(Lb.dimgpu_csr5_spmv_dot(A._h, x1.data_ptr(), y1.data_ptr(), dot_d.data_ptr(), cal._h,
                                        stream.cuda_stream))

    x32 = x1.float()
    y32 = torch.empty(n, device="cuda", dtype=torch.float32)

    def spmv32():
        A.spmv(x32, y32, cal, stream=stream)

    def _time(fn, reps=50):
        for _ in range(5):
            fn()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(reps):
            fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) * 1e-3 / reps

    spmv_dot_s = _time(spmv_dot)
    spmv32_s = _time(spmv32)

    # ---- e2e: the same FP64 solve through the C ABI with pinned host buffers ----
    bh = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    bh[:] = b
    xh = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    import ctypes

    from diploma_research_gb300 import _native as N

    st = N.cg_stats()
    L = N.lib()
    for _ in range(max(1, args.warmup)):
        xh[:] = 0
        N.check(L.dimgpu_cg_solve_host(s64._h, bh.ctypes.data, xh.ctypes.data, ctypes.byref(st)))
    e2e_t = []
    for _ in range(args.steps):
        xh[:] = 0
        t = time.perf_counter()
        N.check(L.dimgpu_cg_solve_host(s64._h, bh.ctypes.data, xh.ctypes.data, ctypes.byref(st)))
        e2e_t.append(time.perf_counter() - t)
    e2e_s = _barrier_max(statistics.mean(e2e_t), ws)
    clk.__exit__(None, None, None)

    # ---- CPU baseline: the reference's CPU CG (C restatement), full solve, rank 0 only ----
    cpu = None
    oracle_err = {"fp64": None, "mixed": None, "oracle_iterations": None}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        import oracle

        o = oracle.OracleCSR5(n, n, m.row_start_offsets, m.col_indices, m.values, 16, 4)
        threads = os.cpu_count() or 1
        t = time.perf_counter()
        x_oracle, it_cpu, _ = o.cg(b, tol=TOL, nthreads=threads)
        cpu_s = time.perf_counter() - t
        cpu = {"value": cpu_s, "unit": "s", "cores": threads, "kind": "port",
               "sample": f"one full CPU CG solve of {WORKLOAD} to {TOL:g} ({it_cpu} iterations), "
                         f"oracle/csr5_oracle.c on {threads} host threads"}
        xo_norm = float(np.linalg.norm(x_oracle))
        oracle_err = {"fp64": float(np.linalg.norm(x64 - x_oracle) / xo_norm),
                      "mixed": float(np.linalg.norm(xmx - x_oracle) / xo_norm), "oracle_iterations": it_cpu}

    launches_per_solve = 4 + 3 * statistics.mean(iters64)  # init SpMV + init, 3 per iteration, final SpMV + norms
    clocks = clk.summary()
    if rank == 0:
        out = {
            "metric": METRIC, "value": sec64, "unit": "s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sec64 * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": f"synthetic (seeded {WORKLOAD}, b = A x*, x* ~ U[-1,1])",
            "config": _config(m),
            "execution": (f"{ws} replicas, one GPU each" if ws > 1 else "one GPU")
                         + f", {A.device_bytes / 1e6:.0f} MB of CSR5 data on the device",
            "iterations": res64.iterations, "rel_residual": res64.rel_residual, "rel_error_vs_xstar": err64,
            "rel_error_vs_oracle": oracle_err["fp64"], "oracle_iterations": oracle_err["oracle_iterations"],
            "mixed": {"value": secm, "unit": "s", "iterations": resm.iterations,
                      "reliable_updates": resm.reliable_updates, "rel_residual": resm.rel_residual,
                      "rel_error_vs_xstar": errm, "rel_error_vs_oracle": oracle_err["mixed"],
                      "speedup_vs_fp64": sec64 / secm, "dtype": "f32 inner / f64"},
            "spmv": {"seconds": spmv_s, "gbps": spmv_gbs, "bytes_per_launch": spmv_bytes,
                     "fp64_tflops": 2 * nnz / spmv_s / 1e12, "dot_fused_seconds": spmv_dot_s,
                     "f32_seconds": spmv32_s, "f32_gbps": (8 * nnz + 8 * n) / spmv32_s / 1e9},
            "roofline": {"bound": "hbm", "achieved": spmv_gbs, "peak": peak, "unit": "GB/s",
                         "frac": spmv_gbs / peak,
                         "traffic": _profile_traffic() if WORKLOAD == "stencil27_128" else None, "kernel": "k_spmv<double,16>",
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s"},
            "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n},
            "gpu_launches": int(round(launches_per_solve * args.steps)),
            "cpu_baseline": cpu,
            "clocks": clocks,
            "convert_s": convert_s,
        }
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_spmv_only(args):
    """A short SpMV-only run (few launches) for profiler captures: 5 warm-up + `steps` launches.
    --layout hub_first runs it on the matrix renumbered by decreasing row length (csr.hub_first_order);
    --all-launches times every launch configuration instead (30 launches each)."""
    import numpy as np
    import torch

    from diploma_research_gb300 import build as B

    B.build()
    from diploma_research_gb300.csr5 import csr5

    m, _, _ = _workload()
    if args.layout == "hub_first":
        m = m.permuted(m.hub_first_order())
    n, nnz = m.dimensions.rows, m.nnz
    A = csr5.from_csr(m)
    if args.gather_ceiling:
        return _gather_ceiling(A, m)
    if args.all_launches:
        return _time_all_launches(A, n)
    stream = torch.cuda.current_stream()
    dt = torch.float32 if args.f32 else torch.float64
    x = torch.tensor(np.random.default_rng(5).uniform(-1, 1, n), device="cuda", dtype=dt)
    y = torch.empty(n, device="cuda", dtype=dt)
    cal = A.create_calibrator()
    for _ in range(5):
        A.spmv(x, y, cal, stream=stream)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        A.spmv(x, y, cal, stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    s = ev0.elapsed_time(ev1) * 1e-3 / args.steps
    nbytes = (8 * nnz + 8 * n) if args.f32 else (12 * nnz + 16 * n)
    print(json.dumps({"spmv_seconds": s, "gbps": nbytes / s / 1e9, "nnz": nnz, "n": n, "f32": bool(args.f32),
                      "launch": A.spmv_launch(bool(args.f32))}))
    return 0


def _time_all_launches(A, n):
    """CUDA-event time of the f64 and f32 SpMV in every launch configuration (warps per CTA x gathers)."""
    import numpy as np
    import torch

    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    x = torch.tensor(np.random.default_rng(5).uniform(-1, 1, n), device="cuda", dtype=torch.float64)
    y = torch.empty(n, device="cuda", dtype=torch.float64)
    x32, y32 = x.float(), torch.empty(n, device="cuda", dtype=torch.float32)
    out = {"chosen_f64": A.spmv_launch(False), "chosen_f32": A.spmv_launch(True)}
    for f32, wpcs in ((False, (16, 12)), (True, (24, 20))):
        xx, yy = (x32, y32) if f32 else (x, y)
        for w in wpcs:
            for g in ("l1", "stream"):
                A.set_spmv_launch(w, g, f32=f32)
                for _ in range(5):
                    A.spmv(xx, yy)
                torch.cuda.synchronize()
                ev0.record(stream)
                for _ in range(30):
                    A.spmv(xx, yy)
                ev1.record(stream)
                torch.cuda.synchronize()
                out[f"{'f32' if f32 else 'f64'}_{w}_{g}_us"] = ev0.elapsed_time(ev1) / 30 * 1e3
    print(json.dumps(out))
    return 0


def _gather_ceiling(A, m):
    """The SpMV against the gather-only kernels of libdimgpu_probe.so (CUDA events, 30 launches each):
    x[col] summed over the matrix's own column indices in CSR order, f64 and f32 x, L1-allocating and
    L1-bypassing loads -- the rate at which the random gathers alone can run -- and, over the same number
    of uniform random indices, f32 gathers from all of x, from the distributed shared memory of
    thread-block clusters of 2-16 CTAs and from each CTA's own shared memory."""
    import ctypes

    import numpy as np
    import torch

    from diploma_research_gb300 import build as B

    P = ctypes.CDLL(B.build(variant="probe"))
    P.dimgpu_probe_words_per_cta.restype = ctypes.c_uint32
    P.dimgpu_probe_gather.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint32,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                      ctypes.POINTER(ctypes.c_float)]
    P.dimgpu_probe_cluster_gather.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_float),
                                              ctypes.POINTER(ctypes.c_int)]
    n, nnz = m.dimensions.rows, m.nnz
    stream = torch.cuda.current_stream()
    reps = 30
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    x = torch.tensor(np.random.default_rng(5).uniform(-1, 1, n), device="cuda", dtype=torch.float64)
    y = torch.empty(n, device="cuda", dtype=torch.float64)
    x32, y32 = x.float(), torch.empty(n, device="cuda", dtype=torch.float32)
    out = {"n": n, "nnz": nnz, "reps": reps, "launch_f64": A.spmv_launch(False), "launch_f32": A.spmv_launch(True)}
    for name, xx, yy in (("spmv_f64_us", x, y), ("spmv_f32_us", x32, y32)):
        for _ in range(5):
            A.spmv(xx, yy)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(reps):
            A.spmv(xx, yy)
        ev1.record(stream)
        torch.cuda.synchronize()
        out[name] = ev0.elapsed_time(ev1) / reps * 1e3
    col = torch.from_numpy(m.col_indices.astype(np.int32)).to("cuda")
    us, ctas = ctypes.c_float(), ctypes.c_int()
    for tag, xx in (("f64", x), ("f32", x32)):
        for bypass in (0, 1):
            rc = P.dimgpu_probe_gather(col.data_ptr(), nnz, xx.data_ptr(), n, xx.element_size(), bypass, reps,
                                       stream.cuda_stream, ctypes.byref(us))
            if rc:
                raise RuntimeError(f"dimgpu_probe_gather: CUDA error {rc}")
            out[f"gather_{tag}_{'l1_bypass' if bypass else 'l1'}_us"] = us.value
    gen = torch.Generator(device="cuda").manual_seed(7)
    q = torch.randint(0, n, (nnz,), device="cuda", dtype=torch.int32, generator=gen)
    rc = P.dimgpu_probe_gather(q.data_ptr(), nnz, x32.data_ptr(), n, 4, 0, reps, stream.cuda_stream,
                               ctypes.byref(us))
    if rc:
        raise RuntimeError(f"dimgpu_probe_gather: CUDA error {rc}")
    out["gather_f32_uniform_random_us"] = us.value  # as many indices, uniform over all of x
    del q
    w = int(P.dimgpu_probe_words_per_cta())
    out["cluster_words_per_cta"] = w
    for cl in (2, 4, 8, 16):
        for local in (0, 1):
            span = w if local else cl * w
            q = torch.randint(0, span, (nnz,), device="cuda", dtype=torch.int32, generator=gen)
            rc = P.dimgpu_probe_cluster_gather(q.data_ptr(), nnz, cl, local, reps, stream.cuda_stream,
                                               ctypes.byref(us), ctypes.byref(ctas))
            key = f"cluster{cl}_{'own_smem' if local else 'dsmem'}"
            out[key] = {"us": us.value, "ctas": ctas.value, "span_words": span} if rc == 0 else {"cuda_error": rc}
            del q
    print(json.dumps(out))
    return 0


def run_spmm_only(args):
    """A short SpMM-only run (few launches) for profiler captures: k right-hand sides U[-1, 1] (seed 6),
    the launch-shape autotuning call, 5 warm-up launches, then `steps` timed launches."""
    import numpy as np
    import torch

    from diploma_research_gb300 import build as B

    B.build()
    from diploma_research_gb300.csr5 import csr5, spmm, spmm_shape

    m, _, _ = _workload()
    n, nnz, k = m.dimensions.rows, m.nnz, int(args.spmm_only)
    A = csr5.from_csr(m)
    dt = torch.float32 if args.f32 else torch.float64
    X = torch.tensor(np.random.default_rng(6).uniform(-1, 1, (n, k)), device="cuda", dtype=dt)
    Y = torch.empty((n, k), device="cuda", dtype=dt)
    for _ in range(5):
        spmm(A, X, Y)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        spmm(A, X, Y)
    ev1.record(stream)
    torch.cuda.synchronize()
    s = ev0.elapsed_time(ev1) * 1e-3 / args.steps
    w = 4 if args.f32 else 8
    nbytes = (w + 4) * nnz + 2 * w * n * k
    print(json.dumps({"spmm_seconds": s, "gbps": nbytes / s / 1e9, "k": k, "nnz": nnz, "n": n, "f32": bool(args.f32),
                      "shape": spmm_shape(A, k, bool(args.f32))}))
    return 0


def run_batch(args):
    """Multi-RHS workload: 3-D 7-point Laplacian 192^3 (n = 7,077,888), k right-hand sides b_j = A x*_j
    (x* ~ U[-1,1], seed 3), block CG to 1e-10 per column in FP64 and mixed precision, against k separate
    FP64 solves (each column solved and timed).  Prints one JSON line per k."""
    import numpy as np
    import torch

    from diploma_research_gb300 import build as B

    B.build()
    from diploma_research_gb300.cg import BlockCGSolver, CGSolver
    from diploma_research_gb300.csr5 import csr5
    from diploma_research_gb300.generators import WORKLOADS, rhs

    m = WORKLOADS["lap3d7_192"]["build"]()
    n = m.dimensions.rows
    A = csr5.from_csr(m)
    stream = torch.cuda.current_stream()
    single = CGSolver(A, tol=TOL, precision="fp64", stream=stream)
    for k in [int(v) for v in args.batch.split(",")]:
        xs, Bh = rhs(m, 3, k=k)
        Bd = torch.tensor(Bh, device="cuda", dtype=torch.float64)
        out = {"workload": f"lap3d7_192: 3-D 7-point Laplacian 192^3, n={n}, nnz={m.nnz}, k={k}, CG to {TOL:g}"}
        for prec in ("fp64", "mixed"):
            s = BlockCGSolver(A, k, tol=TOL, precision=prec, stream=stream, use_graph=not args.no_graph)
            Xd = torch.zeros((n, k), device="cuda", dtype=torch.float64)
            s.solve(Bd, Xd, stream=stream)  # warm-up
            Xd.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            _, res = s.solve(Bd, Xd, stream=stream)
            torch.cuda.synchronize()
            sec = time.perf_counter() - t
            err = float(np.linalg.norm(Xd.cpu().numpy() - xs) / np.linalg.norm(xs))
            out[prec] = {"seconds": sec, "rhs_solves_per_s": k / sec, "iterations": res.iterations,
                         "converged_columns": res.converged_columns, "max_rel_residual": res.max_rel_residual,
                         "reliable_updates": res.reliable_updates, "rel_error_vs_xstar": err}
            out[prec]["spmm_shape"] = res.spmm_shape
            del s
        sep = []
        for j in range(k):
            b = torch.tensor(np.ascontiguousarray(Bh[:, j]), device="cuda", dtype=torch.float64)
            x = torch.zeros(n, device="cuda", dtype=torch.float64)
            single.solve(b, x, stream=stream)
            x.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            _, r1 = single.solve(b, x, stream=stream)
            torch.cuda.synchronize()
            sep.append((time.perf_counter() - t, r1.iterations))
        sep_s = sum(v[0] for v in sep)
        out["separate_fp64"] = {"seconds": sep_s, "rhs_solves_per_s": k / sep_s,
                                "iterations": [v[1] for v in sep], "note": "all k columns solved one after another"}
        out["speedup_block_fp64"] = sep_s / out["fp64"]["seconds"]
        out["speedup_block_mixed"] = sep_s / out["mixed"]["seconds"]
        print(json.dumps(out), flush=True)
    return 0


def run_adjoint(args):
    """Differentiable-solve workload: 2-D anisotropic diffusion 1024^2 (5-point, kappa = exp(g), g a
    Gaussian random field with length scale 16 cells, variance 1, seed 4, x:y anisotropy 10:1),
    b = A x* (seed 4), loss L = ||x - x_t||^2 with x_t ~ U[-1,1].  Forward CG and adjoint CG
    (lambda = A^{-T} dL/dx) to 1e-10 in FP64 and mixed precision, then dL/dA = -lambda x^T on the
    pattern.  Gradients are checked by the adjoint identity on 16 random directions: lambda.db against
    g.(A^{-1} db) and -lambda.(dA x) against g.(-A^{-1} dA x), the right-hand sides from FP64 forward
    solves to 1e-12.  Prints one JSON line."""
    import numpy as np
    import torch

    from diploma_research_gb300 import build as B

    B.build()
    from diploma_research_gb300.adjoint import cg_adjoint, spmv_transpose
    from diploma_research_gb300.cg import CGSolver
    from diploma_research_gb300.csr5 import csr5
    from diploma_research_gb300.generators import WORKLOADS, rhs

    w = WORKLOADS["aniso2d_1024"]
    m = w["build"]()
    n, nnz = m.dimensions.rows, m.nnz
    xs, bh = rhs(m, w["seed"])
    xt = np.random.default_rng(w["seed"] + 1).uniform(-1.0, 1.0, n)
    A = csr5.from_csr(m)
    stream = torch.cuda.current_stream()
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda", dtype=torch.float64)
    b, xtd = dev(bh), dev(xt)
    out = {"workload": f"aniso2d_1024: 2-D anisotropic diffusion 1024^2, n={n}, nnz={nnz}, CG to {TOL:g}"}
    torch.cuda.synchronize()
    t = time.perf_counter()
    spmv_transpose(A, b, torch.empty_like(b), stream=stream)  # builds A^T once
    torch.cuda.synchronize()
    out["transpose_build_seconds"] = time.perf_counter() - t
    tight = CGSolver(A, tol=1e-12, precision="fp64", stream=stream)
    results = {}
    for prec in ("fp64", "mixed"):
        fwd = CGSolver(A, tol=TOL, precision=prec, stream=stream)
        gv = torch.empty(nnz, device="cuda", dtype=torch.float64)
        for rep in range(2):  # the first pass warms the graphs
            x = torch.zeros(n, device="cuda", dtype=torch.float64)
            lam = torch.zeros(n, device="cuda", dtype=torch.float64)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, rf = fwd.solve(b, x, stream=stream, raise_on_failure=False)
            g = 2.0 * (x - xtd)
            ra = cg_adjoint(A, g, x, lam, gv, tol=TOL, precision=prec, stream=stream, raise_on_failure=False,
                            **({"reliable_delta": args.reliable_delta} if args.reliable_delta else {}))
            torch.cuda.synchronize()
            sec = time.perf_counter() - t0
        results[prec] = (x, lam, gv)
        out[prec] = {"seconds": sec, "forward_iterations": rf.iterations, "adjoint_iterations": ra.iterations,
                     "forward_converged": rf.converged, "adjoint_converged": ra.converged,
                     "forward_rel_residual": rf.rel_residual, "adjoint_rel_residual": ra.rel_residual,
                     "forward_seconds_device": rf.seconds, "adjoint_seconds_device": ra.seconds}
    # adjoint identity on random directions (FP64 forward solves to 1e-12 give the right-hand sides)
    rng = np.random.default_rng(11)
    Sd = m.to_scipy()
    for prec in ("fp64", "mixed"):
        x, lam, gv = results[prec]
        g = 2.0 * (x - xtd)
        xh = x.cpu().numpy()
        ad, fd = [], []
        for j in range(16):
            if j % 2 == 0:
                db = rng.standard_normal(n)
                ad.append(float(lam @ dev(db)))
                rhs_v = dev(db)
            else:
                dv = rng.standard_normal(nnz) * 0.1
                dA = Sd.copy()
                dA.data = dv
                ad.append(float(gv @ dev(dv)))
                rhs_v = dev(-(dA @ xh))
            z = torch.zeros(n, device="cuda", dtype=torch.float64)
            tight.solve(rhs_v, z, stream=stream)
            fd.append(float(g @ z))
        ad, fd = np.array(ad), np.array(fd)
        out[prec]["adjoint_identity_rel_error"] = float(np.linalg.norm(ad - fd) / np.linalg.norm(fd))
    lam64, lamx = results["fp64"][1], results["mixed"][1]
    out["mixed_vs_fp64_lambda_rel_error"] = float(torch.linalg.norm(lamx - lam64) / torch.linalg.norm(lam64))
    out["mixed_speedup"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
    # the FP64 CPU adjoint: one sparse LU factorisation of A gives x = A^-1 b and lambda = A^-T g
    import scipy.sparse.linalg as spla

    t = time.perf_counter()
    lu = spla.splu(Sd.tocsc(), permc_spec="MMD_AT_PLUS_A")
    x_ref = lu.solve(bh)
    lam_ref = lu.solve(2.0 * (x_ref - xt), trans="T")
    rows = np.repeat(np.arange(n), np.diff(m.row_start_offsets.astype(np.int64)))
    gv_ref = -lam_ref[rows] * x_ref[m.col_indices]
    out["cpu_adjoint_seconds"] = time.perf_counter() - t
    rel = lambda a, r: float(np.linalg.norm(a - r) / np.linalg.norm(r))
    for prec in ("fp64", "mixed"):
        x, lam, gv = results[prec]
        out[prec]["rel_error_x_vs_cpu"] = rel(x.cpu().numpy(), x_ref)
        out[prec]["rel_error_lambda_vs_cpu"] = rel(lam.cpu().numpy(), lam_ref)
        out[prec]["rel_error_grad_vals_vs_cpu"] = rel(gv.cpu().numpy(), gv_ref)
    out["tol"] = TOL
    out["reliable_delta"] = args.reliable_delta
    print(json.dumps(out), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="dimgpu", choices=["dimgpu", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--spmv-only", action="store_true", help="few SpMV launches only (for profiler captures)")
    ap.add_argument("--spmm-only", type=int, default=0, metavar="K",
                    help="few SpMM launches with K right-hand sides only (for profiler captures)")
    ap.add_argument("--f32", action="store_true", help="with --spmv-only / --spmm-only: the f32 product")
    ap.add_argument("--layout", default="as_generated", choices=["as_generated", "hub_first"],
                    help="with --spmv-only: the matrix as generated or renumbered by decreasing row length")
    ap.add_argument("--all-launches", action="store_true",
                    help="with --spmv-only: time the f64 and f32 SpMV in every launch configuration")
    ap.add_argument("--gather-ceiling", action="store_true",
                    help="with --spmv-only: the SpMV against gather-only kernels over its column indices")
    ap.add_argument("--no-graph", action="store_true",
                    help="host-driven CG loop instead of the CUDA graph (profilers list every kernel)")
    ap.add_argument("--batch", default=None, help="comma-separated k: the multi-RHS block-CG workload")
    ap.add_argument("--adjoint", action="store_true", help="the differentiable-solve workload (adjoint CG)")
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(DESCR),
                    help="the system of the CG comparison (default: the 27-point 128^3 stencil)")
    ap.add_argument("--tol", type=float, default=None,
                    help="relative residual to solve to (default: the workload's, 1e-8 for lap2d_512, else 1e-10)")
    ap.add_argument("--reliable-delta", type=float, default=None,
                    help="with --adjoint: the mixed adjoint solve's residual drop between f64 replacements")
    args = ap.parse_args()
    globals()["WORKLOAD"] = args.workload
    globals()["TOL"] = args.tol if args.tol is not None else __import__(
        "diploma_research_gb300.generators", fromlist=["WORKLOADS"]).WORKLOADS[args.workload]["tol"]
    if args.adjoint:
        return run_adjoint(args)
    if args.batch:
        return run_batch(args)
    if args.spmv_only:
        return run_spmv_only(args)
    if args.spmm_only:
        return run_spmm_only(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
