// cg.cu -- conjugate gradients on the device, FP64 and mixed precision.
//
// The algorithm is the reference's single-process CG loop (benchmarks/conjugate_gradient/dim_sp/
// main.cpp:89-127) with the residual threshold of docs/paper/thesis.tex:2127-2160, stopping when
// sqrt(r.r) <= tol * ||b||:
//     As = A s; alpha = rr / (s.As); x += alpha s; r -= alpha As; rr' = r.r; beta = rr'/rr; s = r + beta s
//
// One iteration is three kernels, all deterministic (fixed grids, fixed-order reductions):
//   A  SpMV As = A s fused with s.As and alpha = rr / s.As (spmv.cu's last-CTA epilogue)
//   B  r -= alpha As and r.r; its last block decides convergence, beta and the loop condition
//   C  x += alpha s and s = r + beta s in one pass (x is updated here, from the old s)
// and the whole solve is one CUDA graph: init kernels, then a conditional WHILE node whose body is
// A, B, C; B sets the loop condition from the device, so the solve runs without host round trips.
//
// The mixed-precision solver runs the same recurrence on f32 values and f32 vectors s, As, r with
// f64 dot products, f64 alpha/beta and an f64 iterate x, and replaces the recurrence residual by the
// true f64 residual b - A x ("reliable update") whenever r.r has dropped by reliable_delta^2 since
// the last replacement, and before convergence is accepted.  Convergence is only declared on a true
// f64 residual, so the mixed solver meets the same ||b - A x|| <= tol ||b|| as the f64 solver.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.hpp"

namespace dimgpu {
namespace {

constexpr int kVecThreads = 512;

struct cg_state {
    double rr;       // r.r of the current residual
    double rr_new;   // r.r after this iteration's update
    double alpha, beta;
    double dot;      // s.As
    double thresh2;  // (tol ||b||)^2
    double bb;       // b.b
    double maxrr;    // mixed: largest r.r since the last reliable update
    double delta2;   // mixed: reliable_delta^2
    double rr_true;  // last true residual r.r (f64)
    int64_t iter, max_it, ru_count;
    uint32_t stop;       // the solve has finished
    uint32_t x_pending;  // kernel C owes x += alpha s
    uint32_t no_ru;      // mixed: no reliable update this iteration (guards its kernels)
    uint32_t converged;
};

struct vec_ctx {
    cg_state* st;
    double* part;       // [grid * 2] block partials
    uint32_t* counter;  // completion ticket
    cudaGraphConditionalHandle cond;
    int has_cond;
};

// Reduces (a, b) over the grid.  Returns true in exactly one thread (thread 0 of the last block to
// finish) with the totals in *ta, *tb, summed in block order.
__device__ bool grid_reduce2(double a, double b, const vec_ctx& c, double* ta, double* tb) {
    __shared__ double sa[kVecThreads / 32], sb[kVecThreads / 32];
    __shared__ uint32_t s_last;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) {
        sa[warp] = a;
        sb[warp] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0, y = 0;
        for (int w = 0; w < kVecThreads / 32; ++w) {
            x += sa[w];
            y += sb[w];
        }
        c.part[2 * blockIdx.x] = x;
        c.part[2 * blockIdx.x + 1] = y;
        __threadfence();
        s_last = (atomicAdd(c.counter, 1u) == gridDim.x - 1) ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last)
        return false;
    __threadfence();
    double x = 0, y = 0;
    for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
        x += __ldcg(&c.part[2 * i]);
        y += __ldcg(&c.part[2 * i + 1]);
    }
    x = warp_sum(x);
    y = warp_sum(y);
    __syncthreads();
    if (lane == 0) {
        sa[warp] = x;
        sb[warp] = y;
    }
    __syncthreads();
    if (threadIdx.x != 0)
        return false;
    x = 0;
    y = 0;
    for (int w = 0; w < kVecThreads / 32; ++w) {
        x += sa[w];
        y += sb[w];
    }
    *ta = x;
    *tb = y;
    *c.counter = 0u;
    return true;
}

__device__ __forceinline__ void set_cond(const vec_ctx& c, bool go) {
    if (c.has_cond)
        cudaGraphSetConditional(c.cond, go ? 1u : 0u);
}

template <typename F>
__device__ __forceinline__ void grid_loop(uint64_t n, F f) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        f(i);
}

// ---------------------------------------------------------------------------------------------
// f64 solver
// ---------------------------------------------------------------------------------------------

// r = b - Ax; s = r; rr = r.r; bb = b.b
__global__ void __launch_bounds__(kVecThreads) k_init64(const double* b, const double* Ax, double* r, double* s,
                                                        uint64_t n, vec_ctx c) {
    double rr = 0, bb = 0;
    grid_loop(n, [&](uint64_t i) {
        const double bi = b[i];
        const double ri = bi - Ax[i];
        r[i] = ri;
        s[i] = ri;
        rr = fma(ri, ri, rr);
        bb = fma(bi, bi, bb);
    });
    double trr, tbb;
    if (grid_reduce2(rr, bb, c, &trr, &tbb)) {
        cg_state* st = c.st;
        st->rr = trr;
        st->bb = tbb;
        st->thresh2 = st->thresh2 * (tbb > 0 ? tbb : 1.0);  // holds tol^2 on entry
        st->iter = 0;
        st->x_pending = 0;
        st->converged = trr <= st->thresh2 ? 1u : 0u;
        st->stop = st->converged || st->max_it <= 0;
        set_cond(c, !st->stop);
    }
}

// r -= alpha As; rr' = r.r; decide
__global__ void __launch_bounds__(kVecThreads) k_update_r64(const double* As, double* r, uint64_t n, vec_ctx c) {
    cg_state* st = c.st;
    if (*reinterpret_cast<volatile uint32_t*>(&st->stop)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            st->x_pending = 0;
            set_cond(c, false);
        }
        return;
    }
    const double alpha = st->alpha;
    double rr = 0;
    grid_loop(n, [&](uint64_t i) {
        const double ri = r[i] + -alpha * As[i];
        r[i] = ri;
        rr = fma(ri, ri, rr);
    });
    double t, unused;
    if (grid_reduce2(rr, 0.0, c, &t, &unused)) {
        st->rr_new = t;
        st->iter += 1;
        st->x_pending = 1;
        if (t <= st->thresh2) {
            st->converged = 1;
            st->stop = 1;
        } else if (st->iter >= st->max_it || !isfinite(t)) {
            st->stop = 1;
        } else {
            st->beta = t / st->rr;
        }
        st->rr = t;
        set_cond(c, !st->stop);
    }
}

// x += alpha s; s = r + beta s (the latter only while the solve continues)
__global__ void __launch_bounds__(kVecThreads) k_update_xs64(double* x, double* s, const double* r, uint64_t n,
                                                             const cg_state* st) {
    if (!*reinterpret_cast<const volatile uint32_t*>(&st->x_pending))
        return;
    const double alpha = st->alpha, beta = st->beta;
    const bool more = !*reinterpret_cast<const volatile uint32_t*>(&st->stop);
    if (more)
        grid_loop(n, [&](uint64_t i) {
            const double si = s[i];
            x[i] = x[i] + alpha * si;
            s[i] = r[i] + beta * si;
        });
    else
        grid_loop(n, [&](uint64_t i) { x[i] = x[i] + alpha * s[i]; });
}

// ---------------------------------------------------------------------------------------------
// mixed solver: f32 inner recurrence, f64 x and reliable f64 residual updates
// ---------------------------------------------------------------------------------------------

// r64 = b - Ax; r32 = s32 = r64; rr = r64.r64; bb = b.b
__global__ void __launch_bounds__(kVecThreads) k_init_mixed(const double* b, const double* Ax, float* r32, float* s32,
                                                            uint64_t n, vec_ctx c) {
    double rr = 0, bb = 0;
    grid_loop(n, [&](uint64_t i) {
        const double bi = b[i];
        const double ri = bi - Ax[i];
        const float rf = (float)ri;
        r32[i] = rf;
        s32[i] = rf;
        rr = fma(ri, ri, rr);
        bb = fma(bi, bi, bb);
    });
    double trr, tbb;
    if (grid_reduce2(rr, bb, c, &trr, &tbb)) {
        cg_state* st = c.st;
        st->rr = trr;
        st->rr_true = trr;
        st->maxrr = trr;
        st->bb = tbb;
        st->thresh2 = st->thresh2 * (tbb > 0 ? tbb : 1.0);
        st->iter = 0;
        st->ru_count = 0;
        st->x_pending = 0;
        st->no_ru = 1;
        st->converged = trr <= st->thresh2 ? 1u : 0u;
        st->stop = st->converged || st->max_it <= 0;
        set_cond(c, !st->stop);
    }
}

// r32 -= alpha As32; rr' = r32.r32 (f64 sum); decide whether a reliable update is due
__global__ void __launch_bounds__(kVecThreads) k_update_r_mixed(const float* As, float* r, uint64_t n, vec_ctx c) {
    cg_state* st = c.st;
    if (*reinterpret_cast<volatile uint32_t*>(&st->stop)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            st->x_pending = 0;
            st->no_ru = 1;
            set_cond(c, false);
        }
        return;
    }
    const double alpha = st->alpha;
    double rr = 0;
    grid_loop(n, [&](uint64_t i) {
        const float ri = (float)((double)r[i] - alpha * (double)As[i]);
        r[i] = ri;
        rr = fma((double)ri, (double)ri, rr);
    });
    double t, unused;
    if (grid_reduce2(rr, 0.0, c, &t, &unused)) {
        st->rr_new = t;
        st->iter += 1;
        st->x_pending = 1;
        const bool ru = t <= st->thresh2 || t < st->delta2 * st->maxrr || st->iter >= st->max_it || !isfinite(t);
        st->no_ru = ru ? 0u : 1u;
        if (!ru) {
            st->beta = t / st->rr;
            st->rr = t;
            st->maxrr = fmax(st->maxrr, t);
        }
        set_cond(c, true);
    }
}

// reliable update, part 1: x += alpha s (the step of this iteration, before b - A x is formed)
__global__ void __launch_bounds__(kVecThreads) k_ru_x_mixed(double* x, const float* s, uint64_t n,
                                                            const cg_state* st) {
    if (*reinterpret_cast<const volatile uint32_t*>(&st->no_ru))
        return;
    const double alpha = st->alpha;
    grid_loop(n, [&](uint64_t i) { x[i] = x[i] + alpha * (double)s[i]; });
}

// reliable update, part 2 (after Ax = A x in f64): r64 = b - Ax; r32 = r64; decide convergence
__global__ void __launch_bounds__(kVecThreads) k_ru_r_mixed(const double* b, const double* Ax, float* r32, uint64_t n,
                                                            vec_ctx c) {
    cg_state* st = c.st;
    if (*reinterpret_cast<volatile uint32_t*>(&st->no_ru))
        return;
    double rr = 0;
    grid_loop(n, [&](uint64_t i) {
        const double ri = b[i] - Ax[i];
        r32[i] = (float)ri;
        rr = fma(ri, ri, rr);
    });
    double t, unused;
    if (grid_reduce2(rr, 0.0, c, &t, &unused)) {
        st->ru_count += 1;
        st->rr_true = t;
        st->x_pending = 0;  // x already holds this iteration's step
        if (t <= st->thresh2) {
            st->converged = 1;
            st->stop = 1;
        } else if (st->iter >= st->max_it || !isfinite(t)) {
            st->stop = 1;
        } else {
            st->beta = t / st->rr;
            st->rr = t;
            st->maxrr = t;
        }
        set_cond(c, !st->stop);
    }
}

// x += alpha s (unless the reliable update did it); s32 = r32 + beta s32 while the solve continues
__global__ void __launch_bounds__(kVecThreads) k_update_xs_mixed(double* x, float* s, const float* r, uint64_t n,
                                                                 const cg_state* st) {
    const bool xp = *reinterpret_cast<const volatile uint32_t*>(&st->x_pending) != 0;
    const bool more = !*reinterpret_cast<const volatile uint32_t*>(&st->stop);
    if (!xp && !more)
        return;
    const double alpha = st->alpha;
    const float beta = (float)st->beta;
    grid_loop(n, [&](uint64_t i) {
        const float si = s[i];
        if (xp)
            x[i] = x[i] + alpha * (double)si;
        if (more)
            s[i] = fmaf(beta, si, r[i]);
    });
}

__global__ void k_residual_norms(const double* b, const double* Ax, uint64_t n, double* out2) {
    // out2[0] += (b-Ax).(b-Ax) partial, out2[1] += b.b partial (atomics: diagnostics only)
    double rr = 0, bb = 0;
    grid_loop(n, [&](uint64_t i) {
        const double ri = b[i] - Ax[i];
        rr = fma(ri, ri, rr);
        bb = fma(b[i], b[i], bb);
    });
    rr = warp_sum(rr);
    bb = warp_sum(bb);
    if ((threadIdx.x & 31u) == 0) {
        atomicAdd(&out2[0], rr);
        atomicAdd(&out2[1], bb);
    }
}

}  // namespace
}  // namespace dimgpu

using namespace dimgpu;

struct dimgpu_cg_solver {
    const dimgpu_csr5* m = nullptr;
    dimgpu_cg_params params{};
    int grid = 1;
    uint64_t n = 0;
    // f64 vectors
    double *b = nullptr, *x = nullptr, *r = nullptr, *s = nullptr, *As = nullptr, *Ax = nullptr;
    // f32 vectors (mixed)
    float *r32 = nullptr, *s32 = nullptr, *As32 = nullptr;
    cg_state* st = nullptr;
    double* part = nullptr;
    uint32_t* counter = nullptr;
    double* norms = nullptr;
    dimgpu_calibrator cal{};   // SpMV scratch of this solver (f32 and f64 products take turns)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

void solver_free(dimgpu_cg_solver* s) {
    if (!s)
        return;
    if (s->exec)
        cudaGraphExecDestroy(s->exec);
    if (s->graph)
        cudaGraphDestroy(s->graph);
    if (s->ev0)
        cudaEventDestroy(s->ev0);
    if (s->ev1)
        cudaEventDestroy(s->ev1);
    calibrator_release(&s->cal);
    for (void* p : {(void*)s->b, (void*)s->x, (void*)s->r, (void*)s->s, (void*)s->As, (void*)s->Ax, (void*)s->r32,
                    (void*)s->s32, (void*)s->As32, (void*)s->st, (void*)s->part, (void*)s->counter, (void*)s->norms})
        dev_free(p);
    delete s;
}

vec_ctx make_ctx(dimgpu_cg_solver* s, cudaGraphConditionalHandle h, int has) {
    vec_ctx c;
    c.st = s->st;
    c.part = s->part;
    c.counter = s->counter;
    c.cond = h;
    c.has_cond = has;
    return c;
}

// Enqueues the init kernels (needs s->x and s->b filled).
int enqueue_init(dimgpu_cg_solver* s, cudaGraphConditionalHandle h, int has, cudaStream_t st) {
    vec_ctx c = make_ctx(s, h, has);
    DG_CHECK(launch_spmv_f64(s->m, s->x, s->Ax, &s->cal, spmv_epilogue{}, st));
    if (s->params.precision == DIMGPU_CG_MIXED)
        k_init_mixed<<<s->grid, kVecThreads, 0, st>>>(s->b, s->Ax, s->r32, s->s32, s->n, c);
    else
        k_init64<<<s->grid, kVecThreads, 0, st>>>(s->b, s->Ax, s->r, s->s, s->n, c);
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

// Enqueues one iteration.
int enqueue_iteration(dimgpu_cg_solver* s, cudaGraphConditionalHandle h, int has, cudaStream_t st) {
    vec_ctx c = make_ctx(s, h, has);
    spmv_epilogue ep;
    ep.dot_out = &s->st->dot;
    ep.rr = &s->st->rr;
    ep.alpha_out = &s->st->alpha;
    ep.halt = &s->st->stop;
    if (s->params.precision == DIMGPU_CG_MIXED) {
        DG_CHECK(launch_spmv_f32(s->m, s->s32, s->As32, &s->cal, ep, st));
        k_update_r_mixed<<<s->grid, kVecThreads, 0, st>>>(s->As32, s->r32, s->n, c);
        k_ru_x_mixed<<<s->grid, kVecThreads, 0, st>>>(s->x, s->s32, s->n, s->st);
        spmv_epilogue ru;
        ru.halt = &s->st->no_ru;
        DG_CHECK(launch_spmv_f64(s->m, s->x, s->Ax, &s->cal, ru, st));
        k_ru_r_mixed<<<s->grid, kVecThreads, 0, st>>>(s->b, s->Ax, s->r32, s->n, c);
        k_update_xs_mixed<<<s->grid, kVecThreads, 0, st>>>(s->x, s->s32, s->r32, s->n, s->st);
    } else {
        DG_CHECK(launch_spmv_f64(s->m, s->s, s->As, &s->cal, ep, st));
        k_update_r64<<<s->grid, kVecThreads, 0, st>>>(s->As, s->r, s->n, c);
        k_update_xs64<<<s->grid, kVecThreads, 0, st>>>(s->x, s->s, s->r, s->n, s->st);
    }
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

int build_graph(dimgpu_cg_solver* s, cudaStream_t stream) {
    cudaGraph_t g = nullptr;
    DG_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(e, "cudaGraphConditionalHandleCreate");
    }
    int rc = DIMGPU_OK;
    cudaStream_t cap = nullptr;
    e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(e, "cudaStreamCreate");
    }
    do {
        // init part
        e = cudaStreamBeginCaptureToGraph(cap, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "begin capture (init)");
            break;
        }
        rc = enqueue_init(s, h, 1, cap);
        // the WHILE node follows the captured init nodes
        const cudaGraphNode_t* deps = nullptr;
        const cudaGraphEdgeData* edges = nullptr;
        size_t ndeps = 0;
        cudaStreamCaptureStatus cs;
        e = cudaStreamGetCaptureInfo(cap, &cs, nullptr, nullptr, &deps, &edges, &ndeps);
        if (rc != DIMGPU_OK || e != cudaSuccess) {
            cudaGraph_t dummy;
            cudaStreamEndCapture(cap, &dummy);
            if (rc == DIMGPU_OK)
                rc = cuda_fail(e, "capture info");
            break;
        }
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t wnode;
        cudaGraph_t dummy;
        // close the init capture, then add the WHILE node after its leaf nodes
        std::vector<cudaGraphNode_t> leaves(deps, deps + ndeps);
        e = cudaStreamEndCapture(cap, &dummy);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "end capture (init)");
            break;
        }
        e = cudaGraphAddNode(&wnode, g, leaves.data(), nullptr, leaves.size(), &cp);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "add WHILE node");
            break;
        }
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "begin capture (body)");
            break;
        }
        rc = enqueue_iteration(s, h, 1, cap);
        e = cudaStreamEndCapture(cap, &dummy);
        if (rc != DIMGPU_OK)
            break;
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "end capture (body)");
            break;
        }
        e = cudaGraphInstantiate(&s->exec, g, 0);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "cudaGraphInstantiate");
            break;
        }
    } while (false);
    cudaStreamDestroy(cap);
    if (rc != DIMGPU_OK) {
        cudaGraphDestroy(g);
        (void)cudaGetLastError();
        return rc;
    }
    s->graph = g;
    (void)stream;
    return DIMGPU_OK;
}

}  // namespace

extern "C" {

int dimgpu_cg_create(const dimgpu_csr5* m, const dimgpu_cg_params* params, void* stream, dimgpu_cg_solver** out) {
    if (!m || !params || !out)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (m->rows != m->cols)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "CG needs a square matrix (%u x %u)", m->rows, m->cols);
    if (!(params->tol >= 0) || params->max_it < 0)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "tol must be >= 0 and max_it >= 0");
    if (params->precision != DIMGPU_CG_FP64 && params->precision != DIMGPU_CG_MIXED)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "unknown precision %d", params->precision);
    if (m->layout != kLayoutDevice)
        return fail(DIMGPU_ERR_UNSUPPORTED, "CG needs a device-layout matrix");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    dimgpu_cg_solver* s = new dimgpu_cg_solver();
    s->m = m;
    s->params = *params;
    if (s->params.reliable_delta <= 0 || s->params.reliable_delta >= 1)
        s->params.reliable_delta = 0.1;
    s->n = m->rows;
    const int sms = device_sm_count(m->device);
    s->grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * 2, (s->n + kVecThreads - 1) / kVecThreads));
    const uint64_t n = std::max<uint64_t>(1, s->n);
    int rc = DIMGPU_OK;
    do {
        if ((rc = dev_alloc_n(&s->b, n)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->x, n)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->Ax, n)) != DIMGPU_OK) break;
        if (params->precision == DIMGPU_CG_MIXED) {
            if ((rc = dev_alloc_n(&s->r32, n)) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&s->s32, n)) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&s->As32, n)) != DIMGPU_OK) break;
            if ((rc = ensure_vals32(m, st)) != DIMGPU_OK) break;
        } else {
            if ((rc = dev_alloc_n(&s->r, n)) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&s->s, n)) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&s->As, n)) != DIMGPU_OK) break;
        }
        if ((rc = dev_alloc_n(&s->st, 1)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->part, 2 * (uint64_t)s->grid)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->counter, 4)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->norms, 2)) != DIMGPU_OK) break;
        if (cudaMemset(s->counter, 0, 16) != cudaSuccess) {
            rc = cuda_fail(cudaGetLastError(), "memset");
            break;
        }
        if ((rc = calibrator_init(&s->cal, m)) != DIMGPU_OK) break;
        if (cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess) {
            rc = cuda_fail(cudaGetLastError(), "cudaEventCreate");
            break;
        }
        if (params->use_graph && (rc = build_graph(s, st)) != DIMGPU_OK) break;
    } while (false);
    if (rc != DIMGPU_OK) {
        solver_free(s);
        return rc;
    }
    *out = s;
    return DIMGPU_OK;
}

int dimgpu_cg_destroy(dimgpu_cg_solver* s) {
    solver_free(s);
    return DIMGPU_OK;
}

int dimgpu_cg_solve(dimgpu_cg_solver* s, const double* b, double* x, dimgpu_cg_stats* stats, void* stream) {
    if (!s || (!b && s->n) || (!x && s->n))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint64_t n = s->n;
    DG_CUDA(cudaMemcpyAsync(s->b, b, sizeof(double) * n, cudaMemcpyDefault, st));
    DG_CUDA(cudaMemcpyAsync(s->x, x, sizeof(double) * n, cudaMemcpyDefault, st));
    cg_state init{};
    init.thresh2 = s->params.tol * s->params.tol;
    init.max_it = s->params.max_it;
    init.delta2 = s->params.reliable_delta * s->params.reliable_delta;
    init.alpha = init.beta = 0;
    DG_CUDA(cudaMemcpyAsync(s->st, &init, sizeof(init), cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemsetAsync(s->cal.status, 0, sizeof(uint32_t), st));
    DG_CUDA(cudaEventRecord(s->ev0, st));
    if (s->exec) {
        DG_CUDA(cudaGraphLaunch(s->exec, st));
    } else {
        DG_CHECK(enqueue_init(s, 0, 0, st));
        // host-driven loop: kernels turn into no-ops once the device state says stop; the host
        // looks at the state every `check` iterations
        const int64_t check = 16;
        int64_t it = 0;
        while (true) {
            for (int64_t k = 0; k < check; ++k)
                DG_CHECK(enqueue_iteration(s, 0, 0, st));
            it += check;
            uint32_t stop = 0;
            DG_CUDA(cudaMemcpyAsync(&stop, &s->st->stop, sizeof(stop), cudaMemcpyDeviceToHost, st));
            DG_CUDA(cudaStreamSynchronize(st));
            if (stop || it > s->params.max_it + check)
                break;
        }
    }
    DG_CUDA(cudaEventRecord(s->ev1, st));
    DG_CUDA(cudaMemcpyAsync(x, s->x, sizeof(double) * n, cudaMemcpyDefault, st));
    cg_state fin{};
    DG_CUDA(cudaMemcpyAsync(&fin, s->st, sizeof(fin), cudaMemcpyDeviceToHost, st));
    // true residual of the returned x
    DG_CHECK(launch_spmv_f64(s->m, s->x, s->Ax, &s->cal, spmv_epilogue{}, st));
    DG_CUDA(cudaMemsetAsync(s->norms, 0, 2 * sizeof(double), st));
    k_residual_norms<<<s->grid, kVecThreads, 0, st>>>(s->b, s->Ax, n, s->norms);
    double norms[2] = {0, 0};
    DG_CUDA(cudaMemcpyAsync(norms, s->norms, sizeof(norms), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    int rc = check_status(&s->cal, st);
    int status = DIMGPU_OK;
    if (rc == DIMGPU_ERR_BREAKDOWN)
        status = DIMGPU_ERR_BREAKDOWN;
    else if (rc != DIMGPU_OK)
        return rc;
    else if (!fin.converged)
        status = DIMGPU_ERR_NOT_CONVERGED;
    if (stats) {
        const double bn = norms[1] > 0 ? std::sqrt(norms[1]) : 1.0;
        stats->iterations = fin.iter;
        stats->reliable_updates = fin.ru_count;
        stats->rel_residual = std::sqrt(norms[0]) / bn;
        const double rrc = s->params.precision == DIMGPU_CG_MIXED ? fin.rr_true : fin.rr;
        stats->recurrence_rel_residual = std::sqrt(std::max(0.0, rrc)) / bn;
        stats->seconds = ms * 1e-3;
        stats->status = status;
    }
    if (status == DIMGPU_ERR_NOT_CONVERGED)
        set_error("CG reached max_it = %lld before tol", (long long)s->params.max_it);
    return status;
}

int dimgpu_cg_solve_host(dimgpu_cg_solver* s, const double* b_host, double* x_host, dimgpu_cg_stats* stats) {
    return dimgpu_cg_solve(s, b_host, x_host, stats, nullptr);
}

}  // extern "C"
