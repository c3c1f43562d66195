// cg.cu -- conjugate gradients on the device, FP64 and mixed precision.
//
// The algorithm is the reference's single-process CG loop (benchmarks/conjugate_gradient/dim_sp/
// main.cpp:89-127) with the residual threshold of docs/paper/thesis.tex:2127-2160, stopping when
// sqrt(r.r) <= tol * ||b||:
//     As = A s; alpha = rr / (s.As); x += alpha s; r -= alpha As; rr' = r.r; beta = rr'/rr; s = r + beta s
//
// FP64 iteration = three kernels, all deterministic (fixed grids, fixed-order reductions):
//   A  SpMV As = A s fused with s.As and alpha = rr / s.As (spmv.cu's last-CTA epilogue)
//   B  r -= alpha As and r.r; its last block decides convergence, beta and the loop condition
//   C  x += alpha s and s = r + beta s in one pass (x is updated here, from the old s)
// The whole solve is one CUDA graph: init kernels, then a conditional WHILE node whose body is four
// iterations; kernel B sets the loop condition from the device, so the solve makes no host round trip.
//
// Mixed precision runs the same recurrence on f32 values and f32 vectors s, As, r.  Products and short
// partial sums are f32, every dot product is accumulated in f64, alpha and beta are f64, and the
// iterate is kept as x (f64) + y (f32 correction since the last flush).  Whenever r.r has dropped by
// reliable_delta^2 since the last replacement, before convergence is accepted and at max_it, a
// reliable update flushes y into x and replaces r by the true f64 residual b - A x computed with the
// f64 matrix.  Convergence is declared on a true f64 residual only.  Iteration kernels:
//   A32 SpMV (f32) + s.As + alpha;  B32 r -= alpha As, y += alpha s, r.r, decides a reliable update;
//   IF(reliable update) { x += y, y = 0;  Ax = A x (f64 SpMV);  r = b - Ax, r.r (f64);  S32 };
//   beside the IF: S32 s = r + beta s (it returns at once when a reliable update is due).
// The IF is a conditional graph node, so iterations without a reliable update launch three kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "cg_common.cuh"
#include "internal.hpp"

namespace dimgpu {
namespace {

constexpr int kVecThreads = 512;
constexpr int kUnroll = 4;

struct vec_ctx {
    cg_state* st;
    double* part;       // [grid * 2] block partials
    uint32_t* counter;  // completion ticket
    cudaGraphConditionalHandle loop;
    cudaGraphConditionalHandle ru;
    int has_loop, has_ru;
};

// Sums the kWarps values v[0..kWarps) in warp 0 by a shuffle tree (a fixed order); lane 0 gets the total.
constexpr int kWarps = kVecThreads / 32;
static_assert(kWarps <= 32 && (kWarps & (kWarps - 1)) == 0, "the shuffle tree takes a power of two");
__device__ __forceinline__ double warp0_tree(const double* v, unsigned lane) {
    double x = lane < (unsigned)kWarps ? v[lane] : 0.0;
#pragma unroll
    for (int d = kWarps / 2; d > 0; d >>= 1)
        x += __shfl_xor_sync(kFull, x, d);
    return x;
}

// Reduces (a, b) over the grid.  Returns true in exactly one thread (thread 0 of the last block to
// finish) with the totals in *ta, *tb, summed in a fixed order (warps by shuffles, the warps of a block
// and the blocks' partials by shuffle trees), so the result does not depend on which block is last.
__device__ bool grid_reduce2(double a, double b, const vec_ctx& c, double* ta, double* tb) {
    __shared__ double sa[kWarps], sb[kWarps];
    __shared__ uint32_t s_last;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) {
        sa[warp] = a;
        sb[warp] = b;
    }
    __syncthreads();
    if (warp == 0) {
        const double x = warp0_tree(sa, lane), y = warp0_tree(sb, lane);
        if (lane == 0) {
            c.part[2 * blockIdx.x] = x;
            c.part[2 * blockIdx.x + 1] = y;
            s_last = (ticket_acq_rel(c.counter) == gridDim.x - 1) ? 1u : 0u;
        }
    }
    __syncthreads();
    if (!s_last)
        return false;
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
    if (warp != 0)
        return false;
    x = warp0_tree(sa, lane);
    y = warp0_tree(sb, lane);
    if (lane != 0)
        return false;
    *ta = x;
    *tb = y;
    *c.counter = 0u;
    return true;
}

__device__ __forceinline__ void set_loop(const vec_ctx& c, bool go) {
    if (c.has_loop)
        cudaGraphSetConditional(c.loop, go ? 1u : 0u);
}
__device__ __forceinline__ void set_ru(const vec_ctx& c, bool go) {
    if (c.has_ru)
        cudaGraphSetConditional(c.ru, go ? 1u : 0u);
}

// Visits every vector index i in [0, nv): each thread takes U indices one grid stride apart per round
// and calls load(i, u) for all U of them before op(i, u) for any, so that the round's independent
// 16-byte loads are in flight together (op's stores may alias the next loads as far as the compiler
// knows, so interleaving the two would cost one memory round trip per element).  Indices left after the
// last full round go one at a time, in the same order.  The grid is two resident blocks per SM (every
// kernel here is register-bounded to allow that), so one wave covers it.
template <int U = kUnroll, typename Ld, typename Op>
__device__ __forceinline__ void vloop(uint64_t nv, Ld load, Op op) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    for (; i + (U - 1) * stride < nv; i += U * stride) {
#pragma unroll
        for (int u = 0; u < U; ++u)
            load(i + u * stride, u);
#pragma unroll
        for (int u = 0; u < U; ++u)
            op(i + u * stride, u);
    }
    for (; i < nv; i += stride) {
        load(i, 0);
        op(i, 0);
    }
}

// Visits every vector index i in [0, nv) in the same per-thread order as vloop, software-pipelined:
// rounds of U indices one grid stride apart, with round k+1's loads issued before round k's ops, so that
// the next round's loads are in flight while the FP64 pipe works through the current one (with a
// vector kernel's 2 DFMA per element the pipe is busy for about as long as the loads take).  load(i, slot)
// and op(i, slot) use slots [0, U) and [U, 2U) in turn; indices at or past nv are skipped, so a last
// partial round costs one memory round trip, not one per index.
//
// gate() is evaluated after the first round's loads are issued and before any op; when it returns false
// the loop does nothing more and vloop_pipe returns false.  A kernel whose work depends on solver state
// written by the previous kernel reads that state inside gate(), so the state's load latency overlaps
// the first round's loads (only loads of the vector data happen before the gate: nothing is written).
template <int U, typename Ld, typename Op, typename Gate>
__device__ __forceinline__ bool vloop_pipe(uint64_t nv, Ld load, Op op, Gate gate) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t span = U * stride;
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    auto ld_round = [&](uint64_t i0, int base) {
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (i0 + u * stride < nv)
                load(i0 + u * stride, base + u);
    };
    auto op_round = [&](uint64_t i0, int base) {
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (i0 + u * stride < nv)
                op(i0 + u * stride, base + u);
    };
    ld_round(i, 0);
    if (!gate())
        return false;
    while (i < nv) {
        ld_round(i + span, U);
        op_round(i, 0);
        i += span;
        if (i >= nv)
            break;
        ld_round(i + span, 0);
        op_round(i, U);
        i += span;
    }
    return true;
}

template <int U, typename Ld, typename Op>
__device__ __forceinline__ void vloop_pipe(uint64_t nv, Ld load, Op op) {
    vloop_pipe<U>(nv, load, op, [] { return true; });
}

// The scalar elements past the last full vector, visited by the first threads of block 0.
template <typename F>
__device__ __forceinline__ void vtail(uint64_t n, uint64_t width, F f) {
    const uint64_t first = (n / width) * width;
    if (blockIdx.x == 0 && first + threadIdx.x < n)
        f(first + threadIdx.x);
}

// ---------------------------------------------------------------------------------------------
// f64 solver
// ---------------------------------------------------------------------------------------------

// r = b - Ax; s = r; rr = r.r; bb = b.b
__global__ void __launch_bounds__(kVecThreads, 2) k_init64(const double* b, const double* Ax, double* r, double* s,
                                                        uint64_t n, vec_ctx c) {
    const uint64_t pol = policy_evict_last();
    double rr = 0, bb = 0;
    constexpr int U = 1;  // runs once per solve; one element per round keeps it free of spills
    double2 bv[U], av[U];
    vloop<U>(
        n / 2,
        [&](uint64_t i, int u) {
            bv[u] = ld2_keep(b + 2 * i, pol);
            av[u] = ld2_keep(Ax + 2 * i, pol);
        },
        [&](uint64_t i, int u) {
            const double2 bi = bv[u], ai = av[u];
            const double2 ri = make_double2(bi.x - ai.x, bi.y - ai.y);
            st2_stream(r + 2 * i, ri, pol);
            st2_stream(s + 2 * i, ri, pol);
            rr = fma(ri.x, ri.x, fma(ri.y, ri.y, rr));
            bb = fma(bi.x, bi.x, fma(bi.y, bi.y, bb));
        });
    vtail(n, 2, [&](uint64_t i) {
        const double ri = b[i] - Ax[i];
        r[i] = ri;
        s[i] = ri;
        rr = fma(ri, ri, rr);
        bb = fma(b[i], b[i], bb);
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
        set_loop(c, !st->stop);
    }
}

// r -= alpha As; rr' = r.r; decide
__global__ void __launch_bounds__(kVecThreads, 2) k_update_r64(const double* As, double* r, uint64_t n, vec_ctx c) {
    cg_state* st = c.st;
    // the state was written by earlier kernels: read it once, both words in flight together and with
    // the first round's vector loads
    const uint32_t stop = st->stop;
    const double alpha = st->alpha;
    const uint64_t pol = policy_evict_last();
    double rrx = 0, rry = 0;  // two independent chains of the r.r accumulation
    constexpr int U = 2;
    double2 av[2 * U], qv[2 * U];
    const bool go = vloop_pipe<U>(
        n / 2,
        [&](uint64_t i, int u) {
            av[u] = ld2_keep(As + 2 * i, pol);
            qv[u] = ld2_keep(r + 2 * i, pol);
        },
        [&](uint64_t i, int u) {
            const double2 a = av[u];
            double2 q = qv[u];
            q.x = fma(-alpha, a.x, q.x);
            q.y = fma(-alpha, a.y, q.y);
            st2_stream(r + 2 * i, q, pol);
            rrx = fma(q.x, q.x, rrx);
            rry = fma(q.y, q.y, rry);
        },
        [&] { return stop == 0u; });
    if (!go) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            st->x_pending = 0;
            set_loop(c, false);
        }
        return;
    }
    vtail(n, 2, [&](uint64_t i) {
        const double ri = fma(-alpha, As[i], r[i]);
        r[i] = ri;
        rrx = fma(ri, ri, rrx);
    });
    double t, unused;
    if (grid_reduce2(rrx + rry, 0.0, c, &t, &unused)) {
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
        set_loop(c, !st->stop);
    }
}

// x += alpha s; s = r + beta s (the latter only while the solve continues)
__global__ void __launch_bounds__(kVecThreads, 2) k_update_xs64(double* x, double* s, const double* r, uint64_t n,
                                                             const cg_state* st) {
    // the state read overlaps the first round's loads of the continuing solve's update (the usual case)
    const uint32_t pending = st->x_pending, stop = st->stop;
    const double alpha = st->alpha, beta = st->beta;
    const uint64_t pol = policy_evict_last();
    constexpr int U = 1;  // three 16-byte loads per element, two rounds in flight: 24 registers of data
    double2 sv[2 * U], xv[2 * U], rv[2 * U];
    const bool more = vloop_pipe<U>(
        n / 2,
        [&](uint64_t i, int u) {
            sv[u] = ld2_keep(s + 2 * i, pol);
            xv[u] = ld2_keep(x + 2 * i, pol);
            rv[u] = ld2_keep(r + 2 * i, pol);
        },
        [&](uint64_t i, int u) {
            const double2 si = sv[u], xi = xv[u], ri = rv[u];
            st2_stream(x + 2 * i, make_double2(fma(alpha, si.x, xi.x), fma(alpha, si.y, xi.y)), pol);
            st2_stream(s + 2 * i, make_double2(fma(beta, si.x, ri.x), fma(beta, si.y, ri.y)), pol);
        },
        [&] { return pending != 0u && stop == 0u; });
    if (!pending)
        return;
    if (more) {
        vtail(n, 2, [&](uint64_t i) {
            const double si = s[i];
            x[i] = fma(alpha, si, x[i]);
            s[i] = fma(beta, si, r[i]);
        });
    } else {
        vloop_pipe<U>(
            n / 2,
            [&](uint64_t i, int u) {
                sv[u] = ld2_keep(s + 2 * i, pol);
                xv[u] = ld2_keep(x + 2 * i, pol);
            },
            [&](uint64_t i, int u) {
                const double2 si = sv[u], xi = xv[u];
                st2_stream(x + 2 * i, make_double2(fma(alpha, si.x, xi.x), fma(alpha, si.y, xi.y)), pol);
            });
        vtail(n, 2, [&](uint64_t i) { x[i] = fma(alpha, s[i], x[i]); });
    }
}

// ---------------------------------------------------------------------------------------------
// mixed solver
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ float sq4(float4 v) { return fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, v.w * v.w))); }

// r64 = b - Ax; r32 = s32 = r64; y32 = 0; rr = r64.r64; bb = b.b
__global__ void __launch_bounds__(kVecThreads, 2) k_init_mixed(const double* b, const double* Ax, float* r32, float* s32,
                                                            float* y32, uint64_t n, vec_ctx c) {
    const uint64_t pol = policy_evict_last();
    double rr = 0, bb = 0;
    constexpr int U = 1;  // four 16-byte loads per element; runs once per solve
    double2 b0v[U], b1v[U], a0v[U], a1v[U];
    vloop<U>(
        n / 4,
        [&](uint64_t i, int u) {
            b0v[u] = ld2_keep(b + 4 * i, pol);
            b1v[u] = ld2_keep(b + 4 * i + 2, pol);
            a0v[u] = ld2_keep(Ax + 4 * i, pol);
            a1v[u] = ld2_keep(Ax + 4 * i + 2, pol);
        },
        [&](uint64_t i, int u) {
            const double2 b0 = b0v[u], b1 = b1v[u], a0 = a0v[u], a1 = a1v[u];
            const double r0 = b0.x - a0.x, r1 = b0.y - a0.y, r2 = b1.x - a1.x, r3 = b1.y - a1.y;
            const float4 rf = make_float4((float)r0, (float)r1, (float)r2, (float)r3);
            st4_stream(r32 + 4 * i, rf, pol);
            st4_stream(s32 + 4 * i, rf, pol);
            st4_stream(y32 + 4 * i, make_float4(0.f, 0.f, 0.f, 0.f), pol);
            rr = fma(r0, r0, fma(r1, r1, fma(r2, r2, fma(r3, r3, rr))));
            bb = fma(b0.x, b0.x, fma(b0.y, b0.y, fma(b1.x, b1.x, fma(b1.y, b1.y, bb))));
        });
    vtail(n, 4, [&](uint64_t i) {
        const double ri = b[i] - Ax[i];
        r32[i] = (float)ri;
        s32[i] = (float)ri;
        y32[i] = 0.f;
        rr = fma(ri, ri, rr);
        bb = fma(b[i], b[i], bb);
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
        set_loop(c, !st->stop);
    }
}

// r32 -= alpha As32; y32 += alpha s32; rr' = r32.r32 (f32 partials of 4, summed in f64); decide whether a
// reliable update is due
__global__ void __launch_bounds__(kVecThreads, 2) k_update_r_mixed(const float* As, float* r, const float* s, float* y,
                                                                uint64_t n, vec_ctx c) {
    cg_state* st = c.st;
    // the state read overlaps the first round's loads
    const uint32_t stop = st->stop;
    const float af = (float)st->alpha;
    const uint64_t pol = policy_evict_last();
    double rr = 0;
    constexpr int U = 1;  // four 16-byte loads per element, two rounds in flight
    float4 av[2 * U], sv[2 * U], qv[2 * U], yv[2 * U];
    const bool go = vloop_pipe<U>(
        n / 4,
        [&](uint64_t i, int u) {
            av[u] = ld4_keep(As + 4 * i, pol);
            sv[u] = ld4_keep(s + 4 * i, pol);
            qv[u] = ld4_keep(r + 4 * i, pol);
            yv[u] = ld4_keep(y + 4 * i, pol);
        },
        [&](uint64_t i, int u) {
            const float4 a = av[u], si = sv[u];
            float4 q = qv[u], yi = yv[u];
            q = make_float4(fmaf(-af, a.x, q.x), fmaf(-af, a.y, q.y), fmaf(-af, a.z, q.z), fmaf(-af, a.w, q.w));
            yi = make_float4(fmaf(af, si.x, yi.x), fmaf(af, si.y, yi.y), fmaf(af, si.z, yi.z),
                             fmaf(af, si.w, yi.w));
            st4_stream(r + 4 * i, q, pol);
            st4_stream(y + 4 * i, yi, pol);
            rr += (double)sq4(q);
        },
        [&] { return stop == 0u; });
    if (!go) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            st->no_ru = 1;
            set_ru(c, false);
            set_loop(c, false);
        }
        return;
    }
    vtail(n, 4, [&](uint64_t i) {
        const float q = fmaf(-af, As[i], r[i]);
        r[i] = q;
        y[i] = fmaf(af, s[i], y[i]);
        rr += (double)(q * q);
    });
    double t, unused;
    if (grid_reduce2(rr, 0.0, c, &t, &unused)) {
        st->rr_new = t;
        st->iter += 1;
        const bool ru = t <= st->thresh2 || t < st->delta2 * st->maxrr || st->iter >= st->max_it || !isfinite(t);
        st->no_ru = ru ? 0u : 1u;
        if (!ru) {
            st->beta = t / st->rr;
            st->rr = t;
            st->maxrr = fmax(st->maxrr, t);
        }
        set_ru(c, ru);
        set_loop(c, true);
    }
}

// x += y; y = 0 (at reliable updates and at the end of the solve)
__global__ void __launch_bounds__(kVecThreads, 2) k_flush_mixed(double* x, float* y, uint64_t n, const cg_state* st,
                                                             int guarded) {
    if (guarded && *reinterpret_cast<const volatile uint32_t*>(&st->no_ru))
        return;
    const uint64_t pol = policy_evict_last();
    constexpr int U = 2;  // three 16-byte loads per element
    float4 yv[U];
    double2 x0v[U], x1v[U];
    vloop<U>(
        n / 4,
        [&](uint64_t i, int u) {
            yv[u] = ld4_keep(y + 4 * i, pol);
            x0v[u] = ld2_keep(x + 4 * i, pol);
            x1v[u] = ld2_keep(x + 4 * i + 2, pol);
        },
        [&](uint64_t i, int u) {
            const float4 yi = yv[u];
            const double2 x0 = x0v[u], x1 = x1v[u];
            st2_stream(x + 4 * i, make_double2(x0.x + (double)yi.x, x0.y + (double)yi.y), pol);
            st2_stream(x + 4 * i + 2, make_double2(x1.x + (double)yi.z, x1.y + (double)yi.w), pol);
            st4_stream(y + 4 * i, make_float4(0.f, 0.f, 0.f, 0.f), pol);
        });
    vtail(n, 4, [&](uint64_t i) {
        x[i] += (double)y[i];
        y[i] = 0.f;
    });
}

// reliable update, after Ax = A x in f64: r32 = b - Ax; decide convergence on the true residual
__global__ void __launch_bounds__(kVecThreads, 2) k_ru_r_mixed(const double* b, const double* Ax, float* r32, uint64_t n,
                                                            vec_ctx c) {
    cg_state* st = c.st;
    if (*reinterpret_cast<volatile uint32_t*>(&st->no_ru))
        return;
    const uint64_t pol = policy_evict_last();
    double rr = 0;
    constexpr int U = 2;  // four 16-byte loads per element
    double2 b0v[U], b1v[U], a0v[U], a1v[U];
    vloop<U>(
        n / 4,
        [&](uint64_t i, int u) {
            b0v[u] = ld2_keep(b + 4 * i, pol);
            b1v[u] = ld2_keep(b + 4 * i + 2, pol);
            a0v[u] = ld2_keep(Ax + 4 * i, pol);
            a1v[u] = ld2_keep(Ax + 4 * i + 2, pol);
        },
        [&](uint64_t i, int u) {
            const double2 b0 = b0v[u], b1 = b1v[u], a0 = a0v[u], a1 = a1v[u];
            const double r0 = b0.x - a0.x, r1 = b0.y - a0.y, r2 = b1.x - a1.x, r3 = b1.y - a1.y;
            st4_stream(r32 + 4 * i, make_float4((float)r0, (float)r1, (float)r2, (float)r3), pol);
            rr = fma(r0, r0, fma(r1, r1, fma(r2, r2, fma(r3, r3, rr))));
        });
    vtail(n, 4, [&](uint64_t i) {
        const double ri = b[i] - Ax[i];
        r32[i] = (float)ri;
        rr = fma(ri, ri, rr);
    });
    double t, unused;
    if (grid_reduce2(rr, 0.0, c, &t, &unused)) {
        st->ru_count += 1;
        st->rr_true = t;
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
        set_loop(c, !st->stop);
    }
}

// s32 = r32 + beta s32 while the solve continues: after_ru = 0 runs it in iterations without a reliable
// update (beside the reliable-update IF node in the graph, so that the node's evaluation is off the
// iteration's critical path), after_ru = 1 after one (inside the IF body, from the replaced residual).
__global__ void __launch_bounds__(kVecThreads, 2) k_update_s_mixed(float* s, const float* r, uint64_t n,
                                                                const cg_state* st, int after_ru) {
    const uint32_t stop = st->stop, no_ru = st->no_ru;
    const float beta = (float)st->beta;
    if (stop || (after_ru ? no_ru != 0u : no_ru == 0u))
        return;
    const uint64_t pol = policy_evict_last();
    constexpr int U = 1;
    float4 sv[2 * U], rv[2 * U];
    vloop_pipe<U>(
        n / 4,
        [&](uint64_t i, int u) {
            sv[u] = ld4_keep(s + 4 * i, pol);
            rv[u] = ld4_keep(r + 4 * i, pol);
        },
        [&](uint64_t i, int u) {
            const float4 si = sv[u], ri = rv[u];
            st4_stream(s + 4 * i,
                       make_float4(fmaf(beta, si.x, ri.x), fmaf(beta, si.y, ri.y), fmaf(beta, si.z, ri.z),
                                   fmaf(beta, si.w, ri.w)),
                       pol);
        });
    vtail(n, 4, [&](uint64_t i) { s[i] = fmaf(beta, s[i], r[i]); });
}

__global__ void k_residual_norms(const double* b, const double* Ax, uint64_t n, double* out2) {
    // out2[0] += (b-Ax).(b-Ax) partial, out2[1] += b.b partial (atomics: diagnostics only)
    double rr = 0, bb = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const double ri = b[i] - Ax[i];
        rr = fma(ri, ri, rr);
        bb = fma(b[i], b[i], bb);
    }
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
    float *r32 = nullptr, *s32 = nullptr, *As32 = nullptr, *y32 = nullptr;
    cg_state* st = nullptr;
    double* part = nullptr;
    uint32_t* counter = nullptr;
    double* norms = nullptr;
    dimgpu_calibrator cal{};  // SpMV scratch of this solver (f32 and f64 products take turns)
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
                    (void*)s->s32, (void*)s->As32, (void*)s->y32, (void*)s->st, (void*)s->part, (void*)s->counter,
                    (void*)s->norms})
        dev_free(p);
    delete s;
}

vec_ctx make_ctx(dimgpu_cg_solver* s) {
    vec_ctx c{};
    c.st = s->st;
    c.part = s->part;
    c.counter = s->counter;
    return c;
}

bool mixed(const dimgpu_cg_solver* s) { return s->params.precision == DIMGPU_CG_MIXED; }

// Enqueues the init kernels (needs s->x and s->b filled).
int enqueue_init(dimgpu_cg_solver* s, const vec_ctx& c, cudaStream_t st) {
    DG_CHECK(launch_spmv_f64(s->m, s->x, s->Ax, &s->cal, spmv_epilogue{}, st));
    if (mixed(s))
        k_init_mixed<<<s->grid, kVecThreads, 0, st>>>(s->b, s->Ax, s->r32, s->s32, s->y32, s->n, c);
    else
        k_init64<<<s->grid, kVecThreads, 0, st>>>(s->b, s->Ax, s->r, s->s, s->n, c);
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

spmv_epilogue cg_epilogue(dimgpu_cg_solver* s) {
    spmv_epilogue ep;
    ep.dot_out = &s->st->dot;
    ep.rr = &s->st->rr;
    ep.alpha_out = &s->st->alpha;
    ep.halt = &s->st->stop;
    return ep;
}

// The reliable-update kernels of the mixed solver, ending with the s update from the replaced residual
// (each guarded by st->no_ru).
int enqueue_reliable_update(dimgpu_cg_solver* s, const vec_ctx& c, cudaStream_t st) {
    k_flush_mixed<<<s->grid, kVecThreads, 0, st>>>(s->x, s->y32, s->n, s->st, 1);
    spmv_epilogue ru;
    ru.halt = &s->st->no_ru;
    DG_CHECK(launch_spmv_f64(s->m, s->x, s->Ax, &s->cal, ru, st));
    k_ru_r_mixed<<<s->grid, kVecThreads, 0, st>>>(s->b, s->Ax, s->r32, s->n, c);
    k_update_s_mixed<<<s->grid, kVecThreads, 0, st>>>(s->s32, s->r32, s->n, s->st, 1);
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

// One whole iteration as a plain stream of kernels (host-driven loop).
int enqueue_iteration(dimgpu_cg_solver* s, const vec_ctx& c, cudaStream_t st) {
    if (mixed(s)) {
        DG_CHECK(launch_spmv_f32(s->m, s->s32, s->As32, &s->cal, cg_epilogue(s), st));
        k_update_r_mixed<<<s->grid, kVecThreads, 0, st>>>(s->As32, s->r32, s->s32, s->y32, s->n, c);
        k_update_s_mixed<<<s->grid, kVecThreads, 0, st>>>(s->s32, s->r32, s->n, s->st, 0);
        DG_CHECK(enqueue_reliable_update(s, c, st));
    } else {
        DG_CHECK(launch_spmv_f64(s->m, s->s, s->As, &s->cal, cg_epilogue(s), st));
        k_update_r64<<<s->grid, kVecThreads, 0, st>>>(s->As, s->r, s->n, c);
        k_update_xs64<<<s->grid, kVecThreads, 0, st>>>(s->x, s->s, s->r, s->n, s->st);
    }
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

// Captures `body` into `graph` after `deps`; returns the capture's leaf nodes in *leaves.
template <typename F>
int capture_into(cudaStream_t cap, cudaGraph_t graph, const std::vector<cudaGraphNode_t>& deps,
                 std::vector<cudaGraphNode_t>* leaves, F body) {
    cudaError_t e = cudaStreamBeginCaptureToGraph(cap, graph, deps.empty() ? nullptr : deps.data(), nullptr,
                                                  deps.size(), cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess)
        return cuda_fail(e, "begin capture");
    int rc = body();
    if (rc == DIMGPU_OK && leaves) {
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* d = nullptr;
        size_t nd = 0;
        e = cudaStreamGetCaptureInfo(cap, &cs, nullptr, nullptr, &d, nullptr, &nd);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "capture info");
        else
            leaves->assign(d, d + nd);
    }
    cudaGraph_t out;
    e = cudaStreamEndCapture(cap, &out);
    if (rc == DIMGPU_OK && e != cudaSuccess)
        rc = cuda_fail(e, "end capture");
    return rc;
}

int add_conditional(cudaGraph_t graph, const std::vector<cudaGraphNode_t>& deps, cudaGraphConditionalHandle h,
                    cudaGraphConditionalNodeType type, cudaGraphNode_t* node, cudaGraph_t* body) {
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = type;
    cp.conditional.size = 1;
    DG_CUDA(cudaGraphAddNode(node, graph, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &cp));
    *body = cp.conditional.phGraph_out[0];
    return DIMGPU_OK;
}

// Iterations per pass of the WHILE body.  Each pass of the loop costs about 4 us more than a plain kernel
// boundary (measured with per-kernel timestamps inside the graph, 27-point 128^3), so the body holds
// several iterations; the kernels of the iterations after the one that stops return at once (one pass
// of a few empty kernels, at the end of the solve).  Eight rather than four: FP64 solves 0.3 % (27-point
// 128^3) and 1 % (2-D 512^2) faster, mixed solves unchanged within the run-to-run spread.
constexpr int kGraphUnroll = 8;

// Graph: init kernels -> WHILE(loop) { kGraphUnroll iterations }.  A mixed iteration is
// A32 -> B32 -> { IF(ru) { flush, f64 SpMV, residual, S32 after it }  ||  S32 (no reliable update) },
// each IF with its own condition handle; the next iteration waits for both branches.
int build_graph(dimgpu_cg_solver* s) {
    cudaGraph_t g = nullptr;
    DG_CUDA(cudaGraphCreate(&g, 0));
    cudaStream_t cap = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(e, "cudaStreamCreate");
    }
    int rc = DIMGPU_OK;
    do {
        vec_ctx c = make_ctx(s);
        if ((e = cudaGraphConditionalHandleCreate(&c.loop, g, 0, 0)) != cudaSuccess) {
            rc = cuda_fail(e, "cudaGraphConditionalHandleCreate");
            break;
        }
        c.has_loop = 1;
        std::vector<cudaGraphNode_t> leaves;
        if ((rc = capture_into(cap, g, {}, &leaves, [&] { return enqueue_init(s, c, cap); })) != DIMGPU_OK)
            break;
        cudaGraphNode_t wnode;
        cudaGraph_t body;
        if ((rc = add_conditional(g, leaves, c.loop, cudaGraphCondTypeWhile, &wnode, &body)) != DIMGPU_OK)
            break;
        if (!mixed(s)) {
            rc = capture_into(cap, body, {}, nullptr, [&]() -> int {
                for (int u = 0; u < kGraphUnroll; ++u)
                    DG_CHECK(enqueue_iteration(s, c, cap));
                return DIMGPU_OK;
            });
            if (rc != DIMGPU_OK)
                break;
        } else {
            std::vector<cudaGraphNode_t> prev;  // leaves of the previous iteration in the body
            for (int u = 0; u < kGraphUnroll && rc == DIMGPU_OK; ++u) {
                vec_ctx cu = c;
                if ((e = cudaGraphConditionalHandleCreate(&cu.ru, body, 0, 0)) != cudaSuccess) {
                    rc = cuda_fail(e, "cudaGraphConditionalHandleCreate (reliable update)");
                    break;
                }
                cu.has_ru = 1;
                std::vector<cudaGraphNode_t> ab;
                rc = capture_into(cap, body, prev, &ab, [&]() -> int {
                    DG_CHECK(launch_spmv_f32(s->m, s->s32, s->As32, &s->cal, cg_epilogue(s), cap));
                    k_update_r_mixed<<<s->grid, kVecThreads, 0, cap>>>(s->As32, s->r32, s->s32, s->y32, s->n, cu);
                    DG_CUDA(cudaGetLastError());
                    return DIMGPU_OK;
                });
                if (rc != DIMGPU_OK)
                    break;
                cudaGraphNode_t inode;
                cudaGraph_t ibody;
                if ((rc = add_conditional(body, ab, cu.ru, cudaGraphCondTypeIf, &inode, &ibody)) != DIMGPU_OK)
                    break;
                if ((rc = capture_into(cap, ibody, {}, nullptr,
                                       [&] { return enqueue_reliable_update(s, cu, cap); })) != DIMGPU_OK)
                    break;
                // the s update of iterations without a reliable update, beside the IF node
                std::vector<cudaGraphNode_t> sb;
                rc = capture_into(cap, body, ab, &sb, [&]() -> int {
                    k_update_s_mixed<<<s->grid, kVecThreads, 0, cap>>>(s->s32, s->r32, s->n, s->st, 0);
                    DG_CUDA(cudaGetLastError());
                    return DIMGPU_OK;
                });
                prev = sb;
                prev.push_back(inode);
            }
            if (rc != DIMGPU_OK)
                break;
        }
        if ((e = cudaGraphInstantiate(&s->exec, g, 0)) != cudaSuccess) {
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
    if (params->engine != DIMGPU_CG_ENGINE_AUTO && params->engine != DIMGPU_CG_ENGINE_GRAPH)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "unknown engine %d", params->engine);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    dimgpu_cg_solver* s = new dimgpu_cg_solver();
    s->m = m;
    s->params = *params;
    if (s->params.reliable_delta <= 0 || s->params.reliable_delta >= 1)
        s->params.reliable_delta = 0.03;
    s->n = m->rows;
    const int sms = device_sm_count(m->device);
    // two resident blocks per SM (fewer for short vectors)
    s->grid = (int)std::max<uint64_t>(
        1, std::min<uint64_t>((uint64_t)sms * 2, (s->n / 2 + kVecThreads - 1) / kVecThreads));
    const uint64_t n = std::max<uint64_t>(4, s->n);
    int rc = DIMGPU_OK;
    do {
        if ((rc = dev_alloc_n(&s->b, n)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->x, n)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->Ax, n)) != DIMGPU_OK) break;
        if (params->precision == DIMGPU_CG_MIXED) {
            if ((rc = dev_alloc_n(&s->r32, n)) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&s->s32, n)) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&s->As32, n)) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&s->y32, n)) != DIMGPU_OK) break;
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
        if (params->use_graph && (rc = build_graph(s)) != DIMGPU_OK) break;
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
    DG_CUDA(cudaMemcpyAsync(s->st, &init, sizeof(init), cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemsetAsync(s->cal.status, 0, sizeof(uint32_t), st));
    DG_CUDA(cudaEventRecord(s->ev0, st));
    if (s->exec) {
        DG_CUDA(cudaGraphLaunch(s->exec, st));
    } else {
        const vec_ctx c = make_ctx(s);
        DG_CHECK(enqueue_init(s, c, st));
        // host-driven loop: kernels turn into no-ops once the device state says stop; the host
        // looks at the state every `check` iterations
        const int64_t check = 16;
        int64_t it = 0;
        while (true) {
            for (int64_t k = 0; k < check; ++k)
                DG_CHECK(enqueue_iteration(s, c, st));
            it += check;
            uint32_t stop = 0;
            DG_CUDA(cudaMemcpyAsync(&stop, &s->st->stop, sizeof(stop), cudaMemcpyDeviceToHost, st));
            DG_CUDA(cudaStreamSynchronize(st));
            if (stop || it > s->params.max_it + check)
                break;
        }
    }
    if (mixed(s))  // whatever y still holds (it is empty after a reliable update)
        k_flush_mixed<<<s->grid, kVecThreads, 0, st>>>(s->x, s->y32, n, s->st, 0);
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
        const double rrc = mixed(s) ? fin.rr_true : fin.rr;
        stats->recurrence_rel_residual = std::sqrt(std::max(0.0, rrc)) / bn;
        stats->seconds = ms * 1e-3;
        stats->status = status;
    }
    if (status == DIMGPU_ERR_NOT_CONVERGED)
        set_error("CG reached max_it = %lld before tol", (long long)s->params.max_it);
    else if (status == DIMGPU_ERR_BREAKDOWN)
        set_error("CG breakdown: s.As <= 0 or not finite (is the matrix SPD?)");
    return status;
}

int dimgpu_cg_solve_host(dimgpu_cg_solver* s, const double* b_host, double* x_host, dimgpu_cg_stats* stats) {
    return dimgpu_cg_solve(s, b_host, x_host, stats, nullptr);
}

}  // extern "C"
