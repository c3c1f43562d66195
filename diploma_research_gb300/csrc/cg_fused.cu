// cg_fused.cu -- the whole CG solve as one persistent, cooperative kernel.
//
// Same algorithm and stop rule as cg.cu (the reference's dim_sp loop, benchmarks/conjugate_gradient/
// dim_sp/main.cpp:89-127, with the threshold of docs/paper/thesis.tex:2127-2160), FP64 or mixed
// precision, but with no kernel boundary inside the solve: one CTA per SM, every CTA resident (the
// launch is cooperative), and the phases of an iteration separated by grid barriers:
//
//   A  SpMV As = A s over the warps' tile runs, with s.As accumulated as rows close   | barrier
//   B  alpha = rr / s.As;  r -= alpha As;  x += alpha s;  r.r                         | barrier
//   C  beta = r.r' / r.r;  s = r + beta s                                             | barrier
//
// Mixed precision: A and C on f32 vectors, B keeps the f32 correction y (x += y at reliable updates),
// and a reliable update (flush, f64 SpMV A x, r = b - A x) runs when B's r.r calls for it.
//
// Calibrator without a serial pass.  A warp whose run ends inside a row (its carry) needs the head
// fragments of the following warps whose runs begin inside that row.  Every warp publishes its head
// fragment and a flag word as soon as its tiles are done; the owner of the open row then reads the
// fragments of its successors in order (a bounded look-back: the successors never wait on anyone
// before publishing) and writes the finished row.  The warp that owns the last tile also computes the
// CSR tail.  Every sum is in a fixed order, and every CTA reduces the per-CTA partials of a dot product
// in the same order, so all CTAs take the same decisions and the solve is bit-reproducible.
//
// Every wait is bounded (DIMGPU_WAIT_NS of %globaltimer): an expired wait records a status word and the
// kernel leaves at the next barrier; the host maps the word to DIMGPU_ERR_TIMEOUT.
#include <cuda_runtime.h>

#include <algorithm>

#include "cg_common.cuh"
#include "common.cuh"
#include "internal.hpp"
#include "layout.cuh"
#include "spmv_tile.cuh"

namespace dimgpu {
namespace {

constexpr int kFWPC = 16;                 // warps per CTA
constexpr int kFThreads = kFWPC * 32;
constexpr int kFStages = 2;               // TMA ring depth per warp
constexpr int kSigma = 16;
using G64 = tile_geom<double, kSigma>;
using G32 = tile_geom<float, kSigma>;
constexpr uint32_t kStageStride = G64::STAGE;  // f32 tiles use the same stage slots
constexpr uint32_t kRingOff = 128 * ((kFWPC * kFStages * 8 + 127) / 128);
constexpr size_t kFusedSmem = kRingOff + (size_t)kFWPC * kFStages * kStageStride;
constexpr int kUnroll = 4;

// ---- grid barrier (all CTAs resident: cooperative launch) -------------------------------------------

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Returns false in every thread of the CTA when the solve must stop because a device status word is
// set (an expired wait anywhere, a breakdown).  `gen` lives in thread 0.
__device__ __forceinline__ bool grid_sync(const cg_fused_args& p, uint32_t& gen) {
    __shared__ uint32_t s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t target = gen + 1;
        __threadfence();
        if (atomicAdd(&p.bar[0], 1u) == (uint32_t)gridDim.x - 1) {
            p.bar[0] = 0u;
            __threadfence();
            st_release_gpu(&p.bar[32], target);
        } else if (ld_acquire_gpu(&p.bar[32]) != target) {
            const uint64_t t0 = global_ns();
            while (ld_acquire_gpu(&p.bar[32]) != target) {
                if (global_ns() - t0 > DIMGPU_WAIT_NS) {
                    record_status(p.status, kStatusWaitTimeout);
                    break;
                }
            }
        }
        gen = target;
        __threadfence();
        s_ok = *reinterpret_cast<volatile const uint32_t*>(p.status) == kStatusOk ? 1u : 0u;
    }
    __syncthreads();
    return s_ok != 0;
}

// ---- reductions ---------------------------------------------------------------------------------------

// Block sums of (a, b) in warp order into part[2 * blockIdx.x + {0,1}] (made visible by the next barrier).
__device__ __forceinline__ void cta_partial2(double a, double b, double* part) {
    __shared__ double s_red[kFWPC][2];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) {
        s_red[warp][0] = a;
        s_red[warp][1] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int w = 0; w < kFWPC; ++w) {
            x += s_red[w][0];
            y += s_red[w][1];
        }
        part[2 * blockIdx.x] = x;
        part[2 * blockIdx.x + 1] = y;
    }
}

// Grid totals of the partials after a barrier; every CTA sums them in the same order.
__device__ __forceinline__ void grid_total2(const double* part, double& A, double& B) {
    __shared__ double s_tot[2];
    if (threadIdx.x < 32) {
        double x = 0.0, y = 0.0;
        for (unsigned i = threadIdx.x; i < gridDim.x; i += 32) {
            x += __ldcg(&part[2 * i]);
            y += __ldcg(&part[2 * i + 1]);
        }
        x = warp_sum(x);
        y = warp_sum(y);
        if (threadIdx.x == 0) {
            s_tot[0] = x;
            s_tot[1] = y;
        }
    }
    __syncthreads();
    A = s_tot[0];
    B = s_tot[1];
}

// ---- vector loops -------------------------------------------------------------------------------------
// The vectors are streamed once per phase: their loads bypass L1 (.cg), which also leaves L1 to the
// gathers of the SpMV phases.

__device__ __forceinline__ double2 ldv2(const double* p) {
    double2 v;
    asm volatile("ld.global.cg.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ float4 ldv4(const float* p) {
    float4 v;
    asm volatile("ld.global.cg.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
    return v;
}
__device__ __forceinline__ double ldv(const double* p) {
    double v;
    asm volatile("ld.global.cg.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ float ldv(const float* p) {
    float v;
    asm volatile("ld.global.cg.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}

// f(i) for every vector index i < nv: kUnroll elements one grid stride apart per round (guarded), their
// loads in flight together.
template <typename F>
__device__ __forceinline__ void vloop(uint64_t nv, F f) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; base < nv; base += kUnroll * stride) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const uint64_t i = base + u * stride;
            if (i < nv)
                f(i);
        }
    }
}

// The scalar elements past the last full vector, visited by the first threads of block 0.
template <typename F>
__device__ __forceinline__ void vtail(uint64_t n, uint64_t width, F f) {
    const uint64_t first = (n / width) * width;
    if (blockIdx.x == 0 && first + threadIdx.x < n)
        f(first + threadIdx.x);
}

__device__ __forceinline__ float sq4(float4 v) { return fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, v.w * v.w))); }

// ---- the SpMV phase -----------------------------------------------------------------------------------

struct ring_state {
    uint64_t* bars;       // this warp's kFStages mbarriers
    unsigned char* ring;  // this warp's stages
    uint64_t n;           // tiles this warp has consumed over all phases (stage = n % kFStages)
};

// Bounded wait for warp w2's flag of phase `phase`.
__device__ __forceinline__ uint32_t wait_flag(const cg_fused_args& p, uint32_t w2, uint32_t phase) {
    const uint32_t* f = p.flag + w2;
    uint32_t v = ld_acquire_gpu(f);
    if ((v >> 1) == phase)
        return v;
    const uint64_t t0 = global_ns();
    while (((v = ld_acquire_gpu(f)) >> 1) != phase) {
        if (global_ns() - t0 > DIMGPU_WAIT_NS) {
            record_status(p.status, kStatusWaitTimeout);
            return 0u;
        }
    }
    return v;
}

// y = A x over the device-layout tiles (vals: f64 or f32 copy), DOT: dot_lane += this lane's share of
// x.y.  Rows are complete when the call returns in every warp; the caller's barrier publishes them.
template <typename VT, bool DOT>
__device__ __noinline__ void spmv_phase(const cg_fused_args& p, const VT* vals, const VT* x, VT* y, uint32_t phase,
                                        ring_state& rs, double& dot_lane) {
    using G = tile_geom<VT, kSigma>;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t gw = blockIdx.x * kFWPC + warp;
    const uint64_t t_begin = min(p.T, (uint64_t)gw * p.tpw);
    const uint64_t t_end = min(p.T, t_begin + p.tpw);
    const uint64_t pol_keep = policy_evict_last();
    warp_chain<VT> ch;
    const tile_io<VT> io{x, y, p.tdo_ptr, p.tdo, p.rows};

    if (t_begin < t_end) {
        const uint64_t pol = p.keep_matrix ? policy_evict_normal() : policy_evict_first();
        auto stage_of = [&](uint64_t q) { return rs.ring + (size_t)(q % kFStages) * kStageStride; };
        auto issue = [&](uint64_t q, uint64_t t) {
            unsigned char* st = stage_of(q);
            uint64_t* bar = &rs.bars[q % kFStages];
            mbar_arrive_expect_tx(bar, G::STAGE);
            bulk_g2s(st, vals + t * G::TS, G::VBYTES, bar, pol);
            bulk_g2s(st + G::VBYTES, p.col + t * G::TS, G::CBYTES, bar, pol);
            bulk_g2s(st + G::VBYTES + G::CBYTES, p.desc + t * 32, G::DBYTES, bar, pol);
        };
        if (lane == 0) {
            fence_proxy_async_smem();  // the stages held the previous phase's staged rows
            for (int j = 0; j < kFStages && t_begin + j < t_end; ++j)
                issue(rs.n + j, t_begin + j);
        }
        uint32_t raw_cur = __ldg(&p.tile_ptr[t_begin]);
        uint32_t raw_next = __ldg(&p.tile_ptr[t_begin + 1]);
        uint64_t t = t_begin;
        for (; t < t_end; ++t) {
            const uint64_t q = rs.n + (t - t_begin);
            const uint32_t raw = raw_cur, raw_n = raw_next;
            raw_cur = raw_next;
            raw_next = (t + 2 <= p.T) ? __ldg(&p.tile_ptr[t + 2]) : 0u;
            if (!mbar_wait_bounded(&rs.bars[q % kFStages], (uint32_t)((q / kFStages) & 1), p.status))
                break;
            process_tile<VT, kSigma, DOT, kXCoherent>(io, stage_of(q), lane, t, raw, raw_n, pol_keep, ch);
            __syncwarp();
            if (lane == 0 && t + kFStages < t_end) {
                fence_proxy_async_smem();
                issue(q + kFStages, t + kFStages);
            }
        }
        if (t < t_end) {
            // a copy did not arrive in time: wait (bounded) for the copies still in flight, then give up
            for (uint64_t t2 = t; t2 < t_end && t2 < t + kFStages; ++t2) {
                const uint64_t q2 = rs.n + (t2 - t_begin);
                (void)mbar_wait_bounded(&rs.bars[q2 % kFStages], (uint32_t)((q2 / kFStages) & 1), p.status);
            }
        }
        rs.n += t_end - t_begin;
    }

    // the CSR tail (csr5.h:756-782), by the warp that owns the last tile
    if (gw == p.tail_warp) {
        const uint64_t first_tail = p.T * G::TS;
        const bool cont = p.tail_start < p.rows && (uint64_t)p.row_ptr[p.tail_start] != first_tail;
        VT tpart = VT(0);
        for (uint64_t r = (uint64_t)p.tail_start + lane; r < p.rows; r += 32) {
            const uint64_t s0 = (r == p.tail_start) ? first_tail : (uint64_t)p.row_ptr[r];
            const uint64_t e = p.row_ptr[r + 1];
            VT acc = VT(0);
            for (uint64_t k = s0; k < e; ++k)
                acc = fma(vals[k], load_x<kXCoherent>(x + p.col[k], pol_keep), acc);
            if (r == p.tail_start && cont) {
                tpart = acc;  // finishes the row the tiles left open
            } else {
                y[r] = acc;
                if constexpr (DOT)
                    ch.dot_acc += (double)acc * (double)load_x<kXCoherent>(x + r, pol_keep);
            }
        }
        tpart = __shfl_sync(kFull, tpart, 0);
        if (cont) {
            if (ch.open)
                ch.carry += tpart;
            else if (ch.cal_valid)
                ch.cal += tpart;
        }
    }

    // publish this warp's head fragment, then finish the row it leaves open
    if (lane == 0) {
        p.cal_val[gw] = (double)ch.cal;
        p.cal_row[gw] = ch.cal_valid ? (ch.cal_row | kDirty) : 0u;
        const uint32_t through = (ch.cal_valid && !ch.open) ? 1u : 0u;
        __threadfence();
        st_release_gpu(&p.flag[gw], (phase << 1) | through);
        if (ch.open) {
            VT acc = ch.carry;
            for (uint32_t w2 = gw + 1; w2 < p.nwarps; ++w2) {
                const uint32_t f = wait_flag(p, w2, phase);
                if ((f >> 1) != phase)
                    break;
                const uint32_t cr = __ldcg(&p.cal_row[w2]);
                if (cr != (ch.carry_row | kDirty))
                    break;
                acc += (VT)__ldcg(&p.cal_val[w2]);
                if (!(f & 1u))
                    break;
            }
            y[ch.carry_row] = acc;
            if constexpr (DOT)
                ch.dot_acc += (double)acc * (double)load_x<kXCoherent>(x + ch.carry_row, pol_keep);
        }
    }
    dot_lane += ch.dot_acc;
}

// ---- the solve ----------------------------------------------------------------------------------------

struct scalars {
    double rr, bb, thresh2, maxrr, rr_true;
    int64_t iter, ru;
    bool converged;
};

__device__ void finish(const cg_fused_args& p, const scalars& sc) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        cg_state* st = p.st;
        st->rr = sc.rr;
        st->bb = sc.bb;
        st->thresh2 = sc.thresh2;
        st->rr_true = sc.rr_true;
        st->iter = sc.iter;
        st->ru_count = sc.ru;
        st->converged = sc.converged ? 1u : 0u;
        st->stop = 1u;
    }
}

__global__ void __launch_bounds__(kFThreads, 1) k_cg_fused(const __grid_constant__ cg_fused_args p) {
    extern __shared__ __align__(128) unsigned char smem[];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t gw = blockIdx.x * kFWPC + warp;
    ring_state rs{reinterpret_cast<uint64_t*>(smem) + warp * kFStages,
                  smem + kRingOff + (size_t)warp * kFStages * kStageStride, 0};
    if (lane == 0) {
        for (int j = 0; j < kFStages; ++j)
            mbar_init(&rs.bars[j], 1);
        fence_mbar_init();
        p.flag[gw] = 0u;
    }
    __syncwarp();
    uint32_t gen = 0;
    if (threadIdx.x == 0)
        gen = ld_acquire_gpu(&p.bar[32]);
    const uint64_t n = p.rows;
    double* part0 = p.part;
    double* part1 = p.part + 2 * (size_t)p.grid;
    double* part2 = p.part + 4 * (size_t)p.grid;
    scalars sc{};
    uint32_t phase = 0;

    // As, Ax, As32 start at zero: rows the SpMV never writes (empty rows) stay zero
    vloop(n, [&](uint64_t i) {
        p.Ax[i] = 0.0;
        if (p.mixed)
            p.As32[i] = 0.f;
        else
            p.As[i] = 0.0;
    });
    if (!grid_sync(p, gen))
        return;

    // ---- r0 = b - A x0 ----
    {
        double unused = 0.0;
        spmv_phase<double, false>(p, p.vals, p.x, p.Ax, ++phase, rs, unused);
    }
    if (!grid_sync(p, gen))
        return;
    {
        double rr = 0.0, bb = 0.0;
        if (p.mixed) {
            vloop(n / 4, [&](uint64_t i) {
                const double2 b0 = ldv2(p.b + 4 * i), b1 = ldv2(p.b + 4 * i + 2);
                const double2 a0 = ldv2(p.Ax + 4 * i), a1 = ldv2(p.Ax + 4 * i + 2);
                const double r0 = b0.x - a0.x, r1 = b0.y - a0.y, r2 = b1.x - a1.x, r3 = b1.y - a1.y;
                const float4 rf = make_float4((float)r0, (float)r1, (float)r2, (float)r3);
                reinterpret_cast<float4*>(p.r32)[i] = rf;
                reinterpret_cast<float4*>(p.s32)[i] = rf;
                reinterpret_cast<float4*>(p.y32)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                rr = fma(r0, r0, fma(r1, r1, fma(r2, r2, fma(r3, r3, rr))));
                bb = fma(b0.x, b0.x, fma(b0.y, b0.y, fma(b1.x, b1.x, fma(b1.y, b1.y, bb))));
            });
            vtail(n, 4, [&](uint64_t i) {
                const double bi = ldv(p.b + i), ri = bi - ldv(p.Ax + i);
                p.r32[i] = (float)ri;
                p.s32[i] = (float)ri;
                p.y32[i] = 0.f;
                rr = fma(ri, ri, rr);
                bb = fma(bi, bi, bb);
            });
        } else {
            vloop(n / 2, [&](uint64_t i) {
                const double2 bi = ldv2(p.b + 2 * i), ai = ldv2(p.Ax + 2 * i);
                const double2 ri = make_double2(bi.x - ai.x, bi.y - ai.y);
                reinterpret_cast<double2*>(p.r)[i] = ri;
                reinterpret_cast<double2*>(p.s)[i] = ri;
                rr = fma(ri.x, ri.x, fma(ri.y, ri.y, rr));
                bb = fma(bi.x, bi.x, fma(bi.y, bi.y, bb));
            });
            vtail(n, 2, [&](uint64_t i) {
                const double bi = ldv(p.b + i), ri = bi - ldv(p.Ax + i);
                p.r[i] = ri;
                p.s[i] = ri;
                rr = fma(ri, ri, rr);
                bb = fma(bi, bi, bb);
            });
        }
        cta_partial2(rr, bb, part0);
    }
    if (!grid_sync(p, gen))
        return;
    grid_total2(part0, sc.rr, sc.bb);
    sc.thresh2 = p.tol2 * (sc.bb > 0 ? sc.bb : 1.0);
    sc.rr_true = sc.rr;
    sc.maxrr = sc.rr;
    sc.converged = sc.rr <= sc.thresh2;
    if (sc.converged || p.max_it <= 0) {
        finish(p, sc);
        return;
    }

    while (true) {
        // ---- A: As = A s, s.As ----
        double dl = 0.0;
        if (p.mixed)
            spmv_phase<float, true>(p, p.vals32, p.s32, p.As32, ++phase, rs, dl);
        else
            spmv_phase<double, true>(p, p.vals, p.s, p.As, ++phase, rs, dl);
        cta_partial2(dl, 0.0, part1);
        if (!grid_sync(p, gen))
            return;
        double dot, unused;
        grid_total2(part1, dot, unused);
        if (!(dot > 0.0) || !isfinite(dot)) {
            if (threadIdx.x == 0)
                record_status(p.status, kStatusBreakdown);
            finish(p, sc);
            return;
        }
        const double alpha = sc.rr / dot;

        // ---- B: r -= alpha As, x += alpha s (f64) or y += alpha s (mixed), r.r ----
        double rp = 0.0;
        if (p.mixed) {
            const float af = (float)alpha;
            vloop(n / 4, [&](uint64_t i) {
                const float4 a = ldv4(p.As32 + 4 * i), si = ldv4(p.s32 + 4 * i);
                float4 q = ldv4(p.r32 + 4 * i), yi = ldv4(p.y32 + 4 * i);
                q = make_float4(fmaf(-af, a.x, q.x), fmaf(-af, a.y, q.y), fmaf(-af, a.z, q.z), fmaf(-af, a.w, q.w));
                yi = make_float4(fmaf(af, si.x, yi.x), fmaf(af, si.y, yi.y), fmaf(af, si.z, yi.z),
                                 fmaf(af, si.w, yi.w));
                reinterpret_cast<float4*>(p.r32)[i] = q;
                reinterpret_cast<float4*>(p.y32)[i] = yi;
                rp += (double)sq4(q);
            });
            vtail(n, 4, [&](uint64_t i) {
                const float q = fmaf(-af, ldv(p.As32 + i), ldv(p.r32 + i));
                p.r32[i] = q;
                p.y32[i] = fmaf(af, ldv(p.s32 + i), ldv(p.y32 + i));
                rp += (double)(q * q);
            });
        } else {
            vloop(n / 2, [&](uint64_t i) {
                const double2 a = ldv2(p.As + 2 * i), si = ldv2(p.s + 2 * i);
                double2 q = ldv2(p.r + 2 * i), xi = ldv2(p.x + 2 * i);
                q.x = fma(-alpha, a.x, q.x);
                q.y = fma(-alpha, a.y, q.y);
                xi.x = fma(alpha, si.x, xi.x);
                xi.y = fma(alpha, si.y, xi.y);
                reinterpret_cast<double2*>(p.r)[i] = q;
                reinterpret_cast<double2*>(p.x)[i] = xi;
                rp = fma(q.x, q.x, fma(q.y, q.y, rp));
            });
            vtail(n, 2, [&](uint64_t i) {
                const double q = fma(-alpha, ldv(p.As + i), ldv(p.r + i));
                p.r[i] = q;
                p.x[i] = fma(alpha, ldv(p.s + i), ldv(p.x + i));
                rp = fma(q, q, rp);
            });
        }
        cta_partial2(rp, 0.0, part2);
        if (!grid_sync(p, gen))
            return;
        double t;
        grid_total2(part2, t, unused);
        sc.iter += 1;
        double beta = 0.0;
        if (!p.mixed) {
            if (t <= sc.thresh2) {
                sc.rr = t;
                sc.converged = true;
                break;
            }
            if (sc.iter >= p.max_it || !isfinite(t)) {
                sc.rr = t;
                break;
            }
            beta = t / sc.rr;
            sc.rr = t;
        } else {
            const bool ru = t <= sc.thresh2 || t < p.delta2 * sc.maxrr || sc.iter >= p.max_it || !isfinite(t);
            if (!ru) {
                beta = t / sc.rr;
                sc.rr = t;
                sc.maxrr = fmax(sc.maxrr, t);
            } else {
                // reliable update: x += y, y = 0; Ax = A x (f64); r = b - Ax; convergence on the true residual
                vloop(n / 4, [&](uint64_t i) {
                    const float4 yi = ldv4(p.y32 + 4 * i);
                    const double2 x0 = ldv2(p.x + 4 * i), x1 = ldv2(p.x + 4 * i + 2);
                    reinterpret_cast<double2*>(p.x)[2 * i] = make_double2(x0.x + (double)yi.x, x0.y + (double)yi.y);
                    reinterpret_cast<double2*>(p.x)[2 * i + 1] =
                        make_double2(x1.x + (double)yi.z, x1.y + (double)yi.w);
                    reinterpret_cast<float4*>(p.y32)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                });
                vtail(n, 4, [&](uint64_t i) {
                    p.x[i] = ldv(p.x + i) + (double)ldv(p.y32 + i);
                    p.y32[i] = 0.f;
                });
                if (!grid_sync(p, gen))
                    return;
                double unused2 = 0.0;
                spmv_phase<double, false>(p, p.vals, p.x, p.Ax, ++phase, rs, unused2);
                if (!grid_sync(p, gen))
                    return;
                double rt = 0.0;
                vloop(n / 4, [&](uint64_t i) {
                    const double2 b0 = ldv2(p.b + 4 * i), b1 = ldv2(p.b + 4 * i + 2);
                    const double2 a0 = ldv2(p.Ax + 4 * i), a1 = ldv2(p.Ax + 4 * i + 2);
                    const double r0 = b0.x - a0.x, r1 = b0.y - a0.y, r2 = b1.x - a1.x, r3 = b1.y - a1.y;
                    reinterpret_cast<float4*>(p.r32)[i] = make_float4((float)r0, (float)r1, (float)r2, (float)r3);
                    rt = fma(r0, r0, fma(r1, r1, fma(r2, r2, fma(r3, r3, rt))));
                });
                vtail(n, 4, [&](uint64_t i) {
                    const double ri = ldv(p.b + i) - ldv(p.Ax + i);
                    p.r32[i] = (float)ri;
                    rt = fma(ri, ri, rt);
                });
                cta_partial2(rt, 0.0, part0);
                if (!grid_sync(p, gen))
                    return;
                double t2;
                grid_total2(part0, t2, unused);
                sc.ru += 1;
                sc.rr_true = t2;
                if (t2 <= sc.thresh2) {
                    sc.rr = t2;
                    sc.converged = true;
                    break;
                }
                if (sc.iter >= p.max_it || !isfinite(t2)) {
                    sc.rr = t2;
                    break;
                }
                beta = t2 / sc.rr;
                sc.rr = t2;
                sc.maxrr = t2;
            }
        }

        // ---- C: s = r + beta s ----
        if (p.mixed) {
            const float bf = (float)beta;
            vloop(n / 4, [&](uint64_t i) {
                const float4 si = ldv4(p.s32 + 4 * i), ri = ldv4(p.r32 + 4 * i);
                reinterpret_cast<float4*>(p.s32)[i] = make_float4(fmaf(bf, si.x, ri.x), fmaf(bf, si.y, ri.y),
                                                                  fmaf(bf, si.z, ri.z), fmaf(bf, si.w, ri.w));
            });
            vtail(n, 4, [&](uint64_t i) { p.s32[i] = fmaf(bf, ldv(p.s32 + i), ldv(p.r32 + i)); });
        } else {
            vloop(n / 2, [&](uint64_t i) {
                const double2 si = ldv2(p.s + 2 * i), ri = ldv2(p.r + 2 * i);
                reinterpret_cast<double2*>(p.s)[i] = make_double2(fma(beta, si.x, ri.x), fma(beta, si.y, ri.y));
            });
            vtail(n, 2, [&](uint64_t i) { p.s[i] = fma(beta, ldv(p.s + i), ldv(p.r + i)); });
        }
        if (!grid_sync(p, gen))
            return;
    }
    finish(p, sc);
}

}  // namespace

// Whether the persistent kernel can run on this matrix: cooperative launches, one resident CTA per SM.
int cg_fused_grid(const dimgpu_csr5* m, int* grid) {
    static int attr_done = 0;
    if (!attr_done) {
        DG_CUDA(cudaFuncSetAttribute(k_cg_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFusedSmem));
        attr_done = 1;
    }
    int coop = 0;
    DG_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, m->device));
    if (!coop)
        return fail(DIMGPU_ERR_UNSUPPORTED, "the device has no cooperative launches");
    int per_sm = 0;
    DG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_fused, kFThreads, kFusedSmem));
    if (per_sm < 1)
        return fail(DIMGPU_ERR_UNSUPPORTED, "the persistent CG kernel does not fit on an SM");
    *grid = device_sm_count(m->device);
    return DIMGPU_OK;
}

uint32_t cg_fused_warps(int grid) { return (uint32_t)grid * kFWPC; }

int launch_cg_fused(const cg_fused_args& a, cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)a.grid);
    cfg.blockDim = dim3(kFThreads);
    cfg.dynamicSmemBytes = kFusedSmem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    DG_CUDA(cudaLaunchKernelEx(&cfg, k_cg_fused, a));
    return DIMGPU_OK;
}

}  // namespace dimgpu
