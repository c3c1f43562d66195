// block_cg.cu -- k simultaneous CG solves sharing one CSR5 SpMM per iteration ("block CG" with
// per-column convergence masks), FP64 and mixed precision.
//
// Column j runs the reference's CG recurrence (benchmarks/conjugate_gradient/dim_sp/main.cpp:89-127,
// stop at sqrt(r.r) <= tol ||b||, docs/paper/thesis.tex:2127-2160) on its own right-hand side b_j with
// its own alpha_j, beta_j.  The k columns are stored row-major (n x kp, kp = k rounded up to a power
// of two <= 32; padding columns stay inactive), so one SpMM pass streams the matrix once for all of
// them.  A column leaves the iteration when it converges (or reaches max_it); its mask bit clears and
// its data stop changing, while the others go on.  Masks are double-buffered ([2][32], selected by the
// state's phase word) so that one kernel can read this iteration's mask while writing the next.
//
// FP64 iteration: A SpMM AS = A S with per-column s.As and alpha (spmm.cu epilogue)
//                 B R -= alpha AS, per-column r.r; last block decides masks, beta, loop condition
//                 C X += alpha S (columns active this iteration), S = R + beta S (still active)
// Mixed: the same on f32 S, AS, R with f64 dots, an f32 correction Y of X, and batched reliable
// updates (flush Y into X, AX = A X in f64, R = B - AX) for every active column whenever one of them
// needs it; convergence is declared on true f64 residuals only.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.hpp"

namespace dimgpu {
namespace {

constexpr int kThreads = 512;

struct bcg_state {
    int64_t iter, max_it, ru_count;
    uint32_t phase;  // masks[phase] = columns active in the current iteration
    uint32_t any;    // some column is still active
    uint32_t no_ru;  // mixed: no reliable update this iteration
    uint32_t k;      // real columns
    uint32_t kp;     // padded columns (power of two)
    uint32_t pad;
};

struct bcg_cols {  // per-column state, 32 entries each (device)
    double rr[32], rr_new[32], alpha[32], beta[32], dot[32], thresh2[32], bb[32], maxrr[32], rr_true[32];
    int64_t iters[32];
    uint32_t conv[32];
    uint32_t masks[2][32];
};

struct bctx {
    bcg_state* st;
    bcg_cols* cols;
    double* part;  // [grid][32]
    uint32_t* counter;
    cudaGraphConditionalHandle loop, ru;
    int has_loop, has_ru;
    double tol2, delta2;
};

__device__ __forceinline__ void bset(cudaGraphConditionalHandle h, int has, bool v) {
    if (has)
        cudaGraphSetConditional(h, v ? 1u : 0u);
}

// Per-column grid reduction of two values (thread's column = threadIdx.x % kp).  Returns true in every
// thread of the last block; then t1[j], t2[j] (j < kp) hold column j's totals, summed in a fixed order
// (the blocks' partials in kThreads / 32 interleaved slices, then the slices in order).
__device__ bool grid_reduce_cols(double v1, double v2, uint32_t kp, const bctx& c, double* t1, double* t2) {
    __shared__ double s_w[kThreads / 32][64];
    __shared__ uint32_t s_last;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (unsigned o = kp; o < 32; o <<= 1) {
        v1 += __shfl_xor_sync(kFull, v1, o);
        v2 += __shfl_xor_sync(kFull, v2, o);
    }
    if (lane < kp) {
        s_w[warp][lane] = v1;
        s_w[warp][32 + lane] = v2;
    }
    __syncthreads();
    if (threadIdx.x < kp) {
        double a = 0, b = 0;
        for (int w = 0; w < kThreads / 32; ++w) {
            a += s_w[w][threadIdx.x];
            b += s_w[w][32 + threadIdx.x];
        }
        c.part[(uint64_t)blockIdx.x * 64 + threadIdx.x] = a;
        c.part[(uint64_t)blockIdx.x * 64 + 32 + threadIdx.x] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        s_last = (ticket_acq_rel(c.counter) == gridDim.x - 1) ? 1u : 0u;
    __syncthreads();
    if (!s_last)
        return false;
    // the blocks' partials: warp w sums blocks w, w + W, w + 2W, ... of its lane's column, then one thread
    // per column sums the W slices in warp order (a fixed order whichever block is last)
    constexpr unsigned W = kThreads / 32;
    if (lane < kp) {
        double a = 0, b = 0;
        for (unsigned blk = warp; blk < gridDim.x; blk += W) {
            a += __ldcg(&c.part[(uint64_t)blk * 64 + lane]);
            b += __ldcg(&c.part[(uint64_t)blk * 64 + 32 + lane]);
        }
        s_w[warp][lane] = a;
        s_w[warp][32 + lane] = b;
    }
    __syncthreads();
    if (threadIdx.x < kp) {
        double a = 0, b = 0;
        for (unsigned w = 0; w < W; ++w) {
            a += s_w[w][threadIdx.x];
            b += s_w[w][32 + threadIdx.x];
        }
        t1[threadIdx.x] = a;
        t2[threadIdx.x] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        *c.counter = 0u;
    return true;
}

template <typename F>
__device__ __forceinline__ void flat_loop(uint64_t total, F f) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x)
        f(i);
}

// Grid-stride loop over [0, total) in batches of U elements per thread: load(i, u) for the whole batch
// first, then op(i, u), so that U independent loads are in flight per thread.  Every element a thread
// visits belongs to the same column (the stride is a multiple of the padded column count).
template <int U, typename L, typename O>
__device__ __forceinline__ void batched_loop(uint64_t total, L load, O op) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    for (; i + (U - 1) * stride < total; i += U * stride) {
#pragma unroll
        for (int u = 0; u < U; ++u)
            load(i + u * stride, u);
#pragma unroll
        for (int u = 0; u < U; ++u)
            op(i + u * stride, u);
    }
    for (; i < total; i += stride) {
        load(i, 0);
        op(i, 0);
    }
}

// ---- FP64 ---------------------------------------------------------------------------------------

__global__ void __launch_bounds__(kThreads, 2) k_bcg_init64(const double* B, const double* AX, double* R, double* S,
                                                         uint64_t total, bctx c) {
    const uint32_t kp = c.st->kp, k = c.st->k;
    const uint32_t j = threadIdx.x % kp;
    double rr = 0, bb = 0;
    flat_loop(total, [&](uint64_t f) {
        const double r = B[f] - AX[f];
        R[f] = r;
        S[f] = r;
        rr = fma(r, r, rr);
        bb = fma(B[f], B[f], bb);
    });
    __shared__ double s_rr[32], s_bb[32];
    if (grid_reduce_cols(rr, bb, kp, c, s_rr, s_bb) && threadIdx.x == 0) {
        bcg_cols* cs = c.cols;
        uint32_t any = 0;
        for (uint32_t jj = 0; jj < 32; ++jj) {
            const bool real = jj < k;
            const double bbj = real ? s_bb[jj] : 0.0;
            cs->rr[jj] = real ? s_rr[jj] : 0.0;
            cs->rr_true[jj] = cs->rr[jj];
            cs->maxrr[jj] = cs->rr[jj];
            cs->bb[jj] = bbj;
            cs->thresh2[jj] = c.tol2 * (bbj > 0 ? bbj : 1.0);
            cs->iters[jj] = 0;
            cs->conv[jj] = real && cs->rr[jj] <= cs->thresh2[jj];
            cs->alpha[jj] = cs->beta[jj] = 0.0;
            const uint32_t act = real && !cs->conv[jj] && c.st->max_it > 0;
            cs->masks[0][jj] = act;
            cs->masks[1][jj] = 0;
            any |= act;
        }
        c.st->phase = 0;
        c.st->iter = 0;
        c.st->ru_count = 0;
        c.st->no_ru = 1;
        c.st->any = any;
        bset(c.loop, c.has_loop, any != 0);
    }
    (void)j;
}

__global__ void __launch_bounds__(kThreads, 2) k_bcg_update_r64(const double* AS, double* R, uint64_t total, bctx c) {
    const uint32_t kp = c.st->kp, k = c.st->k, ph = c.st->phase;
    const uint32_t j = threadIdx.x % kp;
    const bool act = c.cols->masks[ph][j] != 0;
    const double alpha = c.cols->alpha[j];
    double rr = 0;
    if (act) {
        double a[8], q[8];
        batched_loop<8>(
            total, [&](uint64_t f, int u) { a[u] = AS[f]; q[u] = R[f]; },
            [&](uint64_t f, int u) {
                const double r = fma(-alpha, a[u], q[u]);
                R[f] = r;
                rr = fma(r, r, rr);
            });
    }
    __shared__ double s_rr[32], s_unused[32];
    if (grid_reduce_cols(rr, 0.0, kp, c, s_rr, s_unused) && threadIdx.x == 0) {
        bcg_cols* cs = c.cols;
        uint32_t any = 0;
        for (uint32_t jj = 0; jj < 32; ++jj) {
            uint32_t nxt = 0;
            if (jj < k && cs->masks[ph][jj]) {
                const double t = s_rr[jj];
                cs->iters[jj] += 1;
                cs->rr_new[jj] = t;
                if (cs->alpha[jj] == 0.0) {
                    // s.As <= 0: breakdown (recorded by the SpMM epilogue); the column stops
                } else if (t <= cs->thresh2[jj]) {
                    cs->conv[jj] = 1;
                } else if (cs->iters[jj] < c.st->max_it && isfinite(t)) {
                    cs->beta[jj] = t / cs->rr[jj];
                    nxt = 1;
                }
                cs->rr[jj] = t;
            }
            cs->masks[ph ^ 1u][jj] = nxt;
            any |= nxt;
        }
        c.st->iter += 1;
        c.st->phase = ph ^ 1u;
        c.st->any = any;
        bset(c.loop, c.has_loop, any != 0);
    }
}

__global__ void __launch_bounds__(kThreads, 2) k_bcg_update_xs64(double* X, double* S, const double* R, uint64_t total,
                                                              const bcg_state* st, const bcg_cols* cols) {
    const uint32_t kp = st->kp, q = st->phase;
    const uint32_t j = threadIdx.x % kp;
    const bool was = cols->masks[q ^ 1u][j] != 0, more = cols->masks[q][j] != 0;
    const double alpha = cols->alpha[j], beta = cols->beta[j];
    if (!was)
        return;
    double sv[4], xv[4], rv[4];
    batched_loop<4>(
        total,
        [&](uint64_t f, int u) {
            sv[u] = S[f];
            xv[u] = X[f];
            rv[u] = more ? R[f] : 0.0;
        },
        [&](uint64_t f, int u) {
            X[f] = fma(alpha, sv[u], xv[u]);
            if (more)
                S[f] = fma(beta, sv[u], rv[u]);
        });
}

// ---- mixed --------------------------------------------------------------------------------------

__global__ void __launch_bounds__(kThreads, 2) k_bcg_init_mixed(const double* B, const double* AX, float* R, float* S,
                                                             float* Y, uint64_t total, bctx c) {
    const uint32_t kp = c.st->kp, k = c.st->k;
    double rr = 0, bb = 0;
    flat_loop(total, [&](uint64_t f) {
        const double r = B[f] - AX[f];
        R[f] = (float)r;
        S[f] = (float)r;
        Y[f] = 0.f;
        rr = fma(r, r, rr);
        bb = fma(B[f], B[f], bb);
    });
    __shared__ double s_rr[32], s_bb[32];
    if (grid_reduce_cols(rr, bb, kp, c, s_rr, s_bb) && threadIdx.x == 0) {
        bcg_cols* cs = c.cols;
        uint32_t any = 0;
        for (uint32_t jj = 0; jj < 32; ++jj) {
            const bool real = jj < k;
            const double bbj = real ? s_bb[jj] : 0.0;
            cs->rr[jj] = real ? s_rr[jj] : 0.0;
            cs->rr_true[jj] = cs->rr[jj];
            cs->maxrr[jj] = cs->rr[jj];
            cs->bb[jj] = bbj;
            cs->thresh2[jj] = c.tol2 * (bbj > 0 ? bbj : 1.0);
            cs->iters[jj] = 0;
            cs->conv[jj] = real && cs->rr[jj] <= cs->thresh2[jj];
            cs->alpha[jj] = cs->beta[jj] = 0.0;
            const uint32_t act = real && !cs->conv[jj] && c.st->max_it > 0;
            cs->masks[0][jj] = act;
            cs->masks[1][jj] = 0;
            any |= act;
        }
        c.st->phase = 0;
        c.st->iter = 0;
        c.st->ru_count = 0;
        c.st->no_ru = 1;
        c.st->any = any;
        bset(c.loop, c.has_loop, any != 0);
    }
}

__global__ void __launch_bounds__(kThreads, 2) k_bcg_update_r_mixed(const float* AS, float* R, const float* S, float* Y,
                                                                 uint64_t total, bctx c) {
    const uint32_t kp = c.st->kp, k = c.st->k, ph = c.st->phase;
    const uint32_t j = threadIdx.x % kp;
    const bool act = c.cols->masks[ph][j] != 0;
    const float af = (float)c.cols->alpha[j];
    double rr = 0;
    if (act) {
        float a[4], q[4], sv[4], yv[4];
        batched_loop<4>(
            total,
            [&](uint64_t f, int u) {
                a[u] = AS[f];
                q[u] = R[f];
                sv[u] = S[f];
                yv[u] = Y[f];
            },
            [&](uint64_t f, int u) {
                const float r = fmaf(-af, a[u], q[u]);
                R[f] = r;
                Y[f] = fmaf(af, sv[u], yv[u]);
                rr += (double)(r * r);
            });
    }
    __shared__ double s_rr[32], s_unused[32];
    if (grid_reduce_cols(rr, 0.0, kp, c, s_rr, s_unused) && threadIdx.x == 0) {
        bcg_cols* cs = c.cols;
        bool ru = false;
        for (uint32_t jj = 0; jj < k; ++jj) {
            if (!cs->masks[ph][jj])
                continue;
            const double t = s_rr[jj];
            cs->iters[jj] += 1;
            cs->rr_new[jj] = t;
            ru = ru || t <= cs->thresh2[jj] || t < c.delta2 * cs->maxrr[jj] || cs->iters[jj] >= c.st->max_it ||
                 !isfinite(t);
        }
        c.st->iter += 1;
        c.st->no_ru = ru ? 0u : 1u;
        if (!ru) {  // every active column goes on with its recurrence residual
            for (uint32_t jj = 0; jj < 32; ++jj) {
                const uint32_t a = jj < k && cs->masks[ph][jj];
                if (a) {
                    const double t = cs->rr_new[jj];
                    cs->beta[jj] = t / cs->rr[jj];
                    cs->rr[jj] = t;
                    cs->maxrr[jj] = fmax(cs->maxrr[jj], t);
                }
                cs->masks[ph ^ 1u][jj] = a;
            }
            c.st->phase = ph ^ 1u;
        }
        bset(c.ru, c.has_ru, ru);
        bset(c.loop, c.has_loop, true);
    }
}

// X += Y; Y = 0 (guarded: only during a reliable update)
__global__ void __launch_bounds__(kThreads, 2) k_bcg_flush(double* X, float* Y, uint64_t total, const bcg_state* st,
                                                        int guarded) {
    if (guarded && st->no_ru)
        return;
    flat_loop(total, [&](uint64_t f) {
        X[f] += (double)Y[f];
        Y[f] = 0.f;
    });
}

// reliable update: R = B - AX for the active columns, true residuals, convergence per column
__global__ void __launch_bounds__(kThreads, 2) k_bcg_ru(const double* B, const double* AX, float* R, uint64_t total,
                                                     bctx c) {
    if (c.st->no_ru)
        return;
    const uint32_t kp = c.st->kp, k = c.st->k, ph = c.st->phase;
    const uint32_t j = threadIdx.x % kp;
    const bool act = c.cols->masks[ph][j] != 0;
    double rr = 0;
    if (act)
        flat_loop(total, [&](uint64_t f) {
            const double r = B[f] - AX[f];
            R[f] = (float)r;
            rr = fma(r, r, rr);
        });
    __shared__ double s_rr[32], s_unused[32];
    if (grid_reduce_cols(rr, 0.0, kp, c, s_rr, s_unused) && threadIdx.x == 0) {
        bcg_cols* cs = c.cols;
        uint32_t any = 0;
        for (uint32_t jj = 0; jj < 32; ++jj) {
            uint32_t nxt = 0;
            if (jj < k && cs->masks[ph][jj]) {
                const double t = s_rr[jj];
                cs->rr_true[jj] = t;
                if (t <= cs->thresh2[jj]) {
                    cs->conv[jj] = 1;
                } else if (cs->iters[jj] < c.st->max_it && isfinite(t)) {
                    cs->beta[jj] = t / cs->rr[jj];
                    cs->rr[jj] = t;
                    cs->maxrr[jj] = t;
                    nxt = 1;
                }
            }
            cs->masks[ph ^ 1u][jj] = nxt;
            any |= nxt;
        }
        c.st->ru_count += 1;
        c.st->phase = ph ^ 1u;
        c.st->any = any;
        bset(c.loop, c.has_loop, any != 0);
    }
}

__global__ void __launch_bounds__(kThreads, 2) k_bcg_update_s_mixed(float* S, const float* R, uint64_t total,
                                                                 const bcg_state* st, const bcg_cols* cols) {
    const uint32_t kp = st->kp, q = st->phase;
    const uint32_t j = threadIdx.x % kp;
    if (!cols->masks[q][j])
        return;
    const float beta = (float)cols->beta[j];
    float sv[16], rv[16];
    batched_loop<16>(
        total, [&](uint64_t f, int u) { sv[u] = S[f]; rv[u] = R[f]; },
        [&](uint64_t f, int u) { S[f] = fmaf(beta, sv[u], rv[u]); });
}

// per-column ||B - AX||^2 and ||B||^2 (diagnostics, fixed order through grid_reduce_cols)
__global__ void __launch_bounds__(kThreads, 2) k_bcg_norms(const double* B, const double* AX, uint64_t total, bctx c,
                                                        double* out /* [2][32] */) {
    const uint32_t kp = c.st->kp;
    double rr = 0, bb = 0;
    flat_loop(total, [&](uint64_t f) {
        const double r = B[f] - AX[f];
        rr = fma(r, r, rr);
        bb = fma(B[f], B[f], bb);
    });
    __shared__ double s_rr[32], s_bb[32];
    if (grid_reduce_cols(rr, bb, kp, c, s_rr, s_bb) && threadIdx.x < kp) {
        out[threadIdx.x] = s_rr[threadIdx.x];
        out[32 + threadIdx.x] = s_bb[threadIdx.x];
    }
}

// copy between the caller's (ld) and the solver's (kp) row-major blocks
__global__ void k_pack(const double* src, uint64_t lds, double* dst, uint64_t ldd, uint64_t n, uint32_t k,
                       uint32_t kd) {
    const uint64_t total = n * kd;
    flat_loop(total, [&](uint64_t f) {
        const uint64_t i = f / kd, j = f % kd;
        dst[i * ldd + j] = j < k ? src[i * lds + j] : 0.0;
    });
}

}  // namespace
}  // namespace dimgpu

using namespace dimgpu;

struct dimgpu_block_cg {
    const dimgpu_csr5* m = nullptr;
    dimgpu_cg_params params{};
    uint32_t k = 0, kp = 0;
    uint64_t n = 0;
    int grid = 1;
    double *B = nullptr, *X = nullptr, *AX = nullptr, *R = nullptr, *S = nullptr, *AS = nullptr;
    float *R32 = nullptr, *S32 = nullptr, *AS32 = nullptr, *Y32 = nullptr;
    bcg_state* st = nullptr;
    bcg_cols* cols = nullptr;
    double* part = nullptr;
    uint32_t* counter = nullptr;
    double* norms = nullptr;
    spmm_scratch sc{};
    int shape64 = 1, shape32 = 1;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

bool bmixed(const dimgpu_block_cg* s) { return s->params.precision == DIMGPU_CG_MIXED; }

void bcg_free(dimgpu_block_cg* s) {
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
    spmm_scratch_release(&s->sc);
    for (void* p : {(void*)s->B, (void*)s->X, (void*)s->AX, (void*)s->R, (void*)s->S, (void*)s->AS, (void*)s->R32,
                    (void*)s->S32, (void*)s->AS32, (void*)s->Y32, (void*)s->st, (void*)s->cols, (void*)s->part,
                    (void*)s->counter, (void*)s->norms})
        dev_free(p);
    delete s;
}

bctx make_bctx(dimgpu_block_cg* s) {
    bctx c{};
    c.st = s->st;
    c.cols = s->cols;
    c.part = s->part;
    c.counter = s->counter;
    c.tol2 = s->params.tol * s->params.tol;
    c.delta2 = s->params.reliable_delta * s->params.reliable_delta;
    return c;
}

spmm_args mm_args(dimgpu_block_cg* s, const void* X, void* Y, bool dot) {
    spmm_args a;
    a.X = X;
    a.Y = Y;
    a.ldx = a.ldy = s->kp;
    a.k = s->kp;
    if (dot) {
        a.dot_out = s->cols->dot;
        a.rr = s->cols->rr;
        a.alpha_out = s->cols->alpha;
        a.mask = &s->cols->masks[0][0];
        a.mask_sel = &s->st->phase;
    }
    return a;
}

int enqueue_binit(dimgpu_block_cg* s, const bctx& c, cudaStream_t st) {
    const uint64_t total = s->n * s->kp;
    DG_CHECK(launch_spmm(s->m, false, mm_args(s, s->X, s->AX, false), s->sc, s->shape64, st));
    if (bmixed(s))
        k_bcg_init_mixed<<<s->grid, kThreads, 0, st>>>(s->B, s->AX, s->R32, s->S32, s->Y32, total, c);
    else
        k_bcg_init64<<<s->grid, kThreads, 0, st>>>(s->B, s->AX, s->R, s->S, total, c);
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

int enqueue_bru(dimgpu_block_cg* s, const bctx& c, cudaStream_t st) {
    const uint64_t total = s->n * s->kp;
    k_bcg_flush<<<s->grid, kThreads, 0, st>>>(s->X, s->Y32, total, s->st, 1);
    spmm_args a = mm_args(s, s->X, s->AX, false);
    a.halt = &s->st->no_ru;
    DG_CHECK(launch_spmm(s->m, false, a, s->sc, s->shape64, st));
    k_bcg_ru<<<s->grid, kThreads, 0, st>>>(s->B, s->AX, s->R32, total, c);
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

// A and B of one iteration (graph mode puts the reliable update behind an IF node after them)
int enqueue_bab(dimgpu_block_cg* s, const bctx& c, cudaStream_t st) {
    const uint64_t total = s->n * s->kp;
    if (bmixed(s)) {
        spmm_args a = mm_args(s, s->S32, s->AS32, true);
        DG_CHECK(launch_spmm(s->m, true, a, s->sc, s->shape32, st));
        k_bcg_update_r_mixed<<<s->grid, kThreads, 0, st>>>(s->AS32, s->R32, s->S32, s->Y32, total, c);
    } else {
        spmm_args a = mm_args(s, s->S, s->AS, true);
        DG_CHECK(launch_spmm(s->m, false, a, s->sc, s->shape64, st));
        k_bcg_update_r64<<<s->grid, kThreads, 0, st>>>(s->AS, s->R, total, c);
    }
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

int enqueue_bc(dimgpu_block_cg* s, cudaStream_t st) {
    const uint64_t total = s->n * s->kp;
    if (bmixed(s))
        k_bcg_update_s_mixed<<<s->grid, kThreads, 0, st>>>(s->S32, s->R32, total, s->st, s->cols);
    else
        k_bcg_update_xs64<<<s->grid, kThreads, 0, st>>>(s->X, s->S, s->R, total, s->st, s->cols);
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

int enqueue_biteration(dimgpu_block_cg* s, const bctx& c, cudaStream_t st) {
    DG_CHECK(enqueue_bab(s, c, st));
    if (bmixed(s))
        DG_CHECK(enqueue_bru(s, c, st));
    return enqueue_bc(s, st);
}

template <typename F>
int bcapture(cudaStream_t cap, cudaGraph_t graph, const std::vector<cudaGraphNode_t>& deps,
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

int bcond(cudaGraph_t graph, const std::vector<cudaGraphNode_t>& deps, cudaGraphConditionalHandle h,
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

int build_bgraph(dimgpu_block_cg* s) {
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
        bctx c = make_bctx(s);
        if ((e = cudaGraphConditionalHandleCreate(&c.loop, g, 0, 0)) != cudaSuccess) {
            rc = cuda_fail(e, "conditional handle");
            break;
        }
        c.has_loop = 1;
        std::vector<cudaGraphNode_t> leaves;
        if ((rc = bcapture(cap, g, {}, &leaves, [&] { return enqueue_binit(s, c, cap); })) != DIMGPU_OK)
            break;
        cudaGraphNode_t wnode;
        cudaGraph_t body;
        if ((rc = bcond(g, leaves, c.loop, cudaGraphCondTypeWhile, &wnode, &body)) != DIMGPU_OK)
            break;
        if (!bmixed(s)) {
            if ((rc = bcapture(cap, body, {}, nullptr, [&] { return enqueue_biteration(s, c, cap); })) != DIMGPU_OK)
                break;
        } else {
            if ((e = cudaGraphConditionalHandleCreate(&c.ru, body, 0, 0)) != cudaSuccess) {
                rc = cuda_fail(e, "conditional handle (reliable update)");
                break;
            }
            c.has_ru = 1;
            std::vector<cudaGraphNode_t> ab;
            if ((rc = bcapture(cap, body, {}, &ab, [&] { return enqueue_bab(s, c, cap); })) != DIMGPU_OK)
                break;
            cudaGraphNode_t inode;
            cudaGraph_t ibody;
            if ((rc = bcond(body, ab, c.ru, cudaGraphCondTypeIf, &inode, &ibody)) != DIMGPU_OK)
                break;
            if ((rc = bcapture(cap, ibody, {}, nullptr, [&] { return enqueue_bru(s, c, cap); })) != DIMGPU_OK)
                break;
            if ((rc = bcapture(cap, body, {inode}, nullptr, [&] { return enqueue_bc(s, cap); })) != DIMGPU_OK)
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

uint32_t pow2_at_least(uint32_t k) {
    uint32_t p = 1;
    while (p < k)
        p <<= 1;
    return p;
}

}  // namespace

extern "C" {

int dimgpu_block_cg_create(const dimgpu_csr5* m, uint32_t k, const dimgpu_cg_params* params, void* stream,
                           dimgpu_block_cg** out) {
    if (!m || !params || !out)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (k == 0 || k > 32)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "block CG takes 1..32 right-hand sides (got %u)", k);
    if (m->rows != m->cols)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "CG needs a square matrix (%u x %u)", m->rows, m->cols);
    if (!(params->tol >= 0) || params->max_it < 0)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "tol must be >= 0 and max_it >= 0");
    if (params->precision != DIMGPU_CG_FP64 && params->precision != DIMGPU_CG_MIXED)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "unknown precision %d", params->precision);
    if (m->layout != kLayoutDevice || m->sigma != 16)
        return fail(DIMGPU_ERR_UNSUPPORTED, "block CG needs the device layout with sigma 16");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    dimgpu_block_cg* s = new dimgpu_block_cg();
    s->m = m;
    s->params = *params;
    if (s->params.reliable_delta <= 0 || s->params.reliable_delta >= 1)
        s->params.reliable_delta = 0.1;
    s->k = k;
    s->kp = pow2_at_least(k);
    s->n = m->rows;
    const uint64_t total = std::max<uint64_t>(1, s->n * s->kp);
    const int sms = device_sm_count(m->device);
    s->grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * 2, (total + kThreads - 1) / kThreads));
    int rc = DIMGPU_OK;
    do {
        if ((rc = prepare_spmm_kernels()) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->B, total)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->X, total)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->AX, total)) != DIMGPU_OK) break;
        if (bmixed(s)) {
            if ((rc = dev_alloc_n(&s->R32, total)) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&s->S32, total)) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&s->AS32, total)) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&s->Y32, total)) != DIMGPU_OK) break;
            if ((rc = ensure_vals32(m, st)) != DIMGPU_OK) break;
        } else {
            if ((rc = dev_alloc_n(&s->R, total)) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&s->S, total)) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&s->AS, total)) != DIMGPU_OK) break;
        }
        if ((rc = dev_alloc_n(&s->st, 1)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->cols, 1)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->part, (uint64_t)s->grid * 64)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->counter, 4)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&s->norms, 64)) != DIMGPU_OK) break;
        if (cudaMemset(s->counter, 0, 16) != cudaSuccess || cudaMemset(s->X, 0, total * 8) != cudaSuccess ||
            cudaMemset(s->cols, 0, sizeof(bcg_cols)) != cudaSuccess) {
            rc = cuda_fail(cudaGetLastError(), "memset");
            break;
        }
        if ((rc = spmm_scratch_init(&s->sc, m)) != DIMGPU_OK) break;
        if (cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess) {
            rc = cuda_fail(cudaGetLastError(), "cudaEventCreate");
            break;
        }
        // autotune the SpMM launch shapes on the solver's own blocks (before any capture)
        if ((rc = autotune_spmm(m, false, mm_args(s, s->X, s->AX, false), s->sc, st, &s->shape64, nullptr)) !=
            DIMGPU_OK)
            break;
        if (bmixed(s) && (rc = autotune_spmm(m, true, mm_args(s, s->S32, s->AS32, false), s->sc, st, &s->shape32,
                                             nullptr)) != DIMGPU_OK)
            break;
        if (params->use_graph && (rc = build_bgraph(s)) != DIMGPU_OK) break;
    } while (false);
    if (rc != DIMGPU_OK) {
        bcg_free(s);
        return rc;
    }
    *out = s;
    return DIMGPU_OK;
}

int dimgpu_block_cg_destroy(dimgpu_block_cg* s) {
    bcg_free(s);
    return DIMGPU_OK;
}

int dimgpu_block_cg_solve(dimgpu_block_cg* s, const double* B, uint64_t ldb, double* X, uint64_t ldx,
                          dimgpu_block_cg_stats* stats, int64_t* col_iterations, double* col_rel_residual,
                          void* stream) {
    if (!s || !B || !X)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    if (ldb < s->k || ldx < s->k)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "leading dimensions must be >= k");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint64_t n = s->n, total = n * s->kp;
    k_pack<<<s->grid, kThreads, 0, st>>>(B, ldb, s->B, s->kp, n, s->k, s->kp);
    k_pack<<<s->grid, kThreads, 0, st>>>(X, ldx, s->X, s->kp, n, s->k, s->kp);
    bcg_state init{};
    init.max_it = s->params.max_it;
    init.k = s->k;
    init.kp = s->kp;
    init.no_ru = 1;
    DG_CUDA(cudaMemcpyAsync(s->st, &init, sizeof(init), cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemsetAsync(s->sc.status, 0, sizeof(uint32_t), st));
    DG_CUDA(cudaEventRecord(s->ev0, st));
    if (s->exec) {
        DG_CUDA(cudaGraphLaunch(s->exec, st));
    } else {
        const bctx c = make_bctx(s);
        DG_CHECK(enqueue_binit(s, c, st));
        const int64_t check = 16;
        int64_t it = 0;
        while (true) {
            for (int64_t q = 0; q < check; ++q) {
                DG_CHECK(enqueue_biteration(s, c, st));
            }
            it += check;
            uint32_t any = 0;
            DG_CUDA(cudaMemcpyAsync(&any, &s->st->any, sizeof(any), cudaMemcpyDeviceToHost, st));
            DG_CUDA(cudaStreamSynchronize(st));
            if (!any || it > s->params.max_it + check)
                break;
        }
    }
    if (bmixed(s))
        k_bcg_flush<<<s->grid, kThreads, 0, st>>>(s->X, s->Y32, total, s->st, 0);
    DG_CUDA(cudaEventRecord(s->ev1, st));
    k_pack<<<s->grid, kThreads, 0, st>>>(s->X, s->kp, X, ldx, n, s->k, s->k);
    // true residuals of the returned X
    DG_CHECK(launch_spmm(s->m, false, mm_args(s, s->X, s->AX, false), s->sc, s->shape64, st));
    k_bcg_norms<<<s->grid, kThreads, 0, st>>>(s->B, s->AX, total, make_bctx(s), s->norms);
    double norms[64];
    bcg_state fin{};
    std::vector<unsigned char> colbuf(sizeof(bcg_cols));
    DG_CUDA(cudaMemcpyAsync(norms, s->norms, sizeof(norms), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaMemcpyAsync(&fin, s->st, sizeof(fin), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaMemcpyAsync(colbuf.data(), s->cols, sizeof(bcg_cols), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    const bcg_cols* hc = reinterpret_cast<const bcg_cols*>(colbuf.data());
    uint32_t status_word = 0;
    DG_CUDA(cudaMemcpy(&status_word, s->sc.status, sizeof(status_word), cudaMemcpyDeviceToHost));
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    uint32_t nconv = 0;
    int64_t maxit = 0;
    double maxrel = 0;
    for (uint32_t j = 0; j < s->k; ++j) {
        const double bn = norms[32 + j] > 0 ? std::sqrt(norms[32 + j]) : 1.0;
        const double rel = std::sqrt(std::max(0.0, norms[j])) / bn;
        nconv += hc->conv[j] ? 1u : 0u;
        maxit = std::max<int64_t>(maxit, hc->iters[j]);
        maxrel = std::max(maxrel, rel);
        if (col_iterations)
            col_iterations[j] = hc->iters[j];
        if (col_rel_residual)
            col_rel_residual[j] = rel;
    }
    int status = DIMGPU_OK;
    if (status_word == kStatusBreakdown)
        status = DIMGPU_ERR_BREAKDOWN;
    else if (status_word != 0)
        return fail(DIMGPU_ERR_TIMEOUT, "device status %u", status_word);
    else if (nconv < s->k)
        status = DIMGPU_ERR_NOT_CONVERGED;
    if (status_word)
        cudaMemset(s->sc.status, 0, sizeof(uint32_t));
    if (stats) {
        stats->iterations = maxit;
        stats->reliable_updates = fin.ru_count;
        stats->max_rel_residual = maxrel;
        stats->seconds = ms * 1e-3;
        stats->converged_columns = (int32_t)nconv;
        stats->status = status;
        stats->spmm_shape = bmixed(s) ? s->shape32 : s->shape64;
        stats->reserved = 0;
    }
    if (status == DIMGPU_ERR_NOT_CONVERGED)
        set_error("block CG: %u of %u columns converged within max_it", nconv, s->k);
    else if (status == DIMGPU_ERR_BREAKDOWN)
        set_error("block CG breakdown: s.As <= 0 or not finite in some column");
    return status;
}

}  // extern "C"
