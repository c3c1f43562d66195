// spmm.cu -- CSR5 SpMM on GB300: Y = A X for k right-hand sides (X, Y row-major, k <= 32 per pass).
//
// The matrix side is the SpMV's (spmv.cu): the same device layout, tiles streamed into shared memory
// by cp.async.bulk on an mbarrier ring, each warp owning a contiguous run of tiles, a per-warp
// calibrator slot for the row that began before the run, and the last CTA resolving the slots and
// the CSR tail.  What changes is the role of the lanes: lane j is right-hand side j.  The warp walks
// a tile's 512 elements in CSR order (tile column by tile column, csr5.h's element order before the
// transpose); every element broadcasts its value and column index from shared memory and every lane
// gathers X[col, j] -- one coalesced k-wide row per element -- and accumulates.  A set bit_flag bit
// (uniform across the warp) closes the running row, written as one coalesced Y row.  Rows crossing
// tiles go through the same in-order carry chain as the SpMV, with k-vectors.
//
// The optional epilogue of the block CG computes, per right-hand side, dot_j = sum_i X[i,j] Y[i,j]
// and alpha_j = rr_j / dot_j (columns whose mask is clear are skipped).
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "internal.hpp"
#include "layout.cuh"

namespace dimgpu {
namespace {

template <typename VT>
struct spmm_params {
    const VT* vals;
    const uint32_t* col;
    const uint32_t* desc;
    const uint32_t* tile_ptr;
    const uint32_t* tdo_ptr;
    const uint32_t* tdo;
    const uint32_t* row_ptr;
    const VT* X;
    VT* Y;
    uint64_t ldx, ldy;
    uint32_t k;
    uint64_t T;
    uint32_t rows;
    uint32_t tail_start;
    uint64_t tpw;
    uint32_t nwarps;
    const uint32_t* empty_rows;
    uint32_t n_empty;
    double* cal_val;     // [nwarps * 32]
    uint32_t* cal_row;   // [nwarps]
    double* dot_part;    // [nwarps * 32]
    uint32_t* counter;
    uint32_t* status;
    // block-CG epilogue (DOT): dot_out[j], alpha_out[j] = rr[j] / dot_out[j] where mask[j] != 0
    double* dot_out;
    const double* rr;
    double* alpha_out;
    const uint32_t* mask;
    const uint32_t* mask_sel;
    uint32_t* halt;
};

constexpr int kSigma = 16;
constexpr uint32_t kTS = kSigma * 32;

template <typename VT>
struct mm_geom {
    static constexpr uint32_t VBYTES = kTS * sizeof(VT);
    static constexpr uint32_t CBYTES = kTS * 4;
    static constexpr uint32_t DBYTES = 32 * 4;
    static constexpr uint32_t STAGE = VBYTES + CBYTES + DBYTES;
    static constexpr desc_fields F = fields_for(kSigma, 32);
};

template <typename VT>
__device__ __forceinline__ VT stage_val(const unsigned char* st, uint32_t c, uint32_t r) {
    const VT* sv = reinterpret_cast<const VT*>(st);
    return sizeof(VT) == 8 ? sv[pos_device_f64(c, r, 32)] : sv[pos_device_q32(c, r, 32)];
}

template <typename VT, int WPC, int STAGES, bool DOT>
__global__ void __launch_bounds__(WPC * 32) k_spmm(const spmm_params<VT> p) {
    using G = mm_geom<VT>;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint32_t s_last;
    __shared__ double s_dot[WPC][32];

    if (p.halt && *reinterpret_cast<volatile const uint32_t*>(p.halt))
        return;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t gw = blockIdx.x * WPC + warp;
    const bool active = lane < p.k;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem) + warp * STAGES;
    unsigned char* ring = smem + 128 * ((WPC * STAGES * 8 + 127) / 128) + (size_t)warp * STAGES * G::STAGE;

    // empty rows below the tail: zero rows of Y
    for (uint64_t i = blockIdx.x * (uint64_t)WPC + warp; i < p.n_empty; i += (uint64_t)gridDim.x * WPC)
        if (active)
            p.Y[(uint64_t)p.empty_rows[i] * p.ldy + lane] = VT(0);

    const uint64_t t_begin = min(p.T, (uint64_t)gw * p.tpw);
    const uint64_t t_end = min(p.T, t_begin + p.tpw);
    const uint64_t pol_keep = policy_evict_last();

    double dot_acc = 0.0;
    bool open = false, cal_valid = false;
    VT carry = VT(0), cal = VT(0);
    uint32_t carry_row = 0, cal_row = 0;

    auto write_row = [&](uint32_t row, VT val) {
        if (active) {
            st_keep(p.Y + (uint64_t)row * p.ldy + lane, val, pol_keep);
            if constexpr (DOT)
                dot_acc = fma((double)val, (double)ldg_x(p.X + (uint64_t)row * p.ldx + lane, pol_keep), dot_acc);
        }
    };

    if (t_begin < t_end) {
        const uint64_t pol = policy_evict_first();
        if (lane == 0) {
            for (int s = 0; s < STAGES; ++s)
                mbar_init(&bars[s], 1);
            fence_mbar_init();
        }
        __syncwarp();
        auto issue = [&](int s, uint64_t t) {
            unsigned char* st = ring + (size_t)s * G::STAGE;
            mbar_arrive_expect_tx(&bars[s], G::STAGE);
            bulk_g2s(st, p.vals + t * kTS, G::VBYTES, &bars[s], pol);
            bulk_g2s(st + G::VBYTES, p.col + t * kTS, G::CBYTES, &bars[s], pol);
            bulk_g2s(st + G::VBYTES + G::CBYTES, p.desc + t * 32, G::DBYTES, &bars[s], pol);
        };
        if (lane == 0)
            for (int s = 0; s < STAGES && t_begin + s < t_end; ++s)
                issue(s, t_begin + s);

        uint32_t raw_cur = __ldg(&p.tile_ptr[t_begin]);
        uint32_t raw_next = __ldg(&p.tile_ptr[t_begin + 1]);
        uint64_t i = 0;
        bool failed = false;
        for (uint64_t t = t_begin; t < t_end; ++t, ++i) {
            const int s = (int)(i % STAGES);
            const uint32_t par = (uint32_t)((i / STAGES) & 1);
            const uint32_t raw = raw_cur;
            const uint32_t row_start = raw & ~kDirty;
            raw_cur = raw_next;
            raw_next = (t + 2 <= p.T) ? __ldg(&p.tile_ptr[t + 2]) : 0u;
            if (!mbar_wait_bounded(&bars[s], par, p.status)) {
                failed = true;
                break;
            }
            const unsigned char* st = ring + (size_t)s * G::STAGE;
            const uint32_t* sc = reinterpret_cast<const uint32_t*>(st + G::VBYTES);
            const uint32_t* sd = reinterpret_cast<const uint32_t*>(st + G::VBYTES + G::CBYTES);
            const bool dirty = (raw & kDirty) != 0;
            const uint32_t optr = dirty ? __ldg(&p.tdo_ptr[t]) : 0u;
            auto row_of = [&](uint32_t idx) -> uint32_t {
                return row_start + (dirty ? __ldg(&p.tdo[optr + idx]) : idx);
            };
            const bool capped = ((sd[0] >> (G::F.yb + G::F.sb)) & 1u) != 0;

            VT acc = VT(0), head = VT(0);
            uint32_t seg = 0;
            // Column c's gathered X rows are fetched one column ahead (xa/xb), so the gathers of the next
            // column are in flight while this one accumulates; values come from shared memory.
            VT xa[kSigma], xb[kSigma];
            auto fetch = [&](uint32_t c, VT (&x)[kSigma]) {
#pragma unroll
                for (uint32_t r = 0; r < kSigma; ++r) {
                    const uint32_t cc = sc[pos_device_q32(c, r, 32)];
                    x[r] = active ? ldg_x(p.X + (uint64_t)cc * p.ldx + lane, pol_keep) : VT(0);
                }
            };
            auto walk = [&](uint32_t c, const VT (&x)[kSigma]) {
                const uint32_t fl = (sd[c] >> (G::F.yb + G::F.sb)) & 0xFFFFu;
#pragma unroll
                for (uint32_t r = 0; r < kSigma; ++r) {
                    if (((fl >> r) & 1u) && (c | r)) {  // a row starts here: the running row closes
                        if (seg == 0)
                            head = acc;
                        else
                            write_row(row_of(seg), acc);
                        ++seg;
                        acc = VT(0);
                    }
                    acc = fma(stage_val<VT>(st, c, r), x[r], acc);
                }
            };
            fetch(0, xa);
            for (uint32_t c = 0; c < 32; c += 2) {
                fetch(c + 1, xb);
                walk(c, xa);
                if (c + 2 < 32)
                    fetch(c + 2, xa);
                walk(c + 1, xb);
            }
            const uint32_t K = seg + 1;
            const VT Lt = acc;
            const VT H = (K == 1) ? Lt : head;
            const uint32_t row_last = (K == 1) ? row_start : row_of(seg);

            if (K == 1) {
                if (capped) {
                    if (open)
                        write_row(carry_row, carry);
                    open = true;
                    carry = H;
                    carry_row = row_start;
                } else if (open) {
                    carry += H;
                } else {
                    cal += H;
                    cal_row = row_start;
                    cal_valid = true;
                }
            } else {
                if (capped) {
                    if (open)
                        write_row(carry_row, carry);
                    write_row(row_start, H);
                } else if (open) {
                    write_row(row_start, carry + H);
                } else {
                    cal += H;
                    cal_row = row_start;
                    cal_valid = true;
                }
                open = true;
                carry = Lt;
                carry_row = row_last;
            }
            __syncwarp();
            if (lane == 0 && t + STAGES < t_end) {
                fence_proxy_async_smem();
                issue(s, t + STAGES);
            }
        }
        if (failed) {
            for (uint64_t t2 = t_begin + i; t2 < t_end && t2 < t_begin + i + STAGES; ++t2) {
                const uint64_t i2 = t2 - t_begin;
                (void)mbar_wait_bounded(&bars[i2 % STAGES], (uint32_t)((i2 / STAGES) & 1), p.status);
            }
        } else if (open) {
            write_row(carry_row, carry);
        }
    }
    p.cal_val[(uint64_t)gw * 32 + lane] = (double)cal;
    if (lane == 0)
        p.cal_row[gw] = cal_valid ? (cal_row | kDirty) : 0u;
    if constexpr (DOT)
        p.dot_part[(uint64_t)gw * 32 + lane] = dot_acc;

    // ---- last CTA: calibrator slots, CSR tail, per-column dots ----
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0)
        s_last = (atomicAdd(p.counter, 1u) == gridDim.x - 1) ? 1u : 0u;
    __syncthreads();
    if (!s_last)
        return;
    __threadfence();

    double fix_dot = 0.0;
    for (uint32_t wi = warp; wi < p.nwarps; wi += WPC) {
        const uint32_t cr = __ldcg(&p.cal_row[wi]);
        if (!(cr & kDirty))
            continue;
        if (wi > 0 && __ldcg(&p.cal_row[wi - 1]) == cr)
            continue;
        const uint32_t R = cr & ~kDirty;
        VT accr = active ? __ldcg(&p.Y[(uint64_t)R * p.ldy + lane]) : VT(0);
        double added = 0.0;
        for (uint32_t w2 = wi; w2 < p.nwarps; ++w2) {
            if (__ldcg(&p.cal_row[w2]) != cr)
                break;
            const VT cv = (VT)__ldcg(&p.cal_val[(uint64_t)w2 * 32 + lane]);
            accr += cv;
            added += (double)cv;
        }
        if (active) {
            p.Y[(uint64_t)R * p.ldy + lane] = accr;
            if constexpr (DOT)
                fix_dot += added * (double)p.X[(uint64_t)R * p.ldx + lane];
        }
    }
    __syncthreads();
    const uint64_t first_tail = p.T * kTS;
    for (uint64_t r = (uint64_t)p.tail_start + warp; r < p.rows; r += WPC) {
        const uint64_t s0 = (r == p.tail_start) ? first_tail : (uint64_t)p.row_ptr[r];
        const uint64_t e = p.row_ptr[r + 1];
        VT a = VT(0);
        for (uint64_t kk = s0; kk < e; ++kk)
            if (active)
                a = fma(p.vals[kk], p.X[(uint64_t)p.col[kk] * p.ldx + lane], a);
        if (active) {
            if (r == p.tail_start && (uint64_t)p.row_ptr[r] != first_tail)
                p.Y[r * p.ldy + lane] = __ldcg(&p.Y[r * p.ldy + lane]) + a;
            else
                p.Y[r * p.ldy + lane] = a;
            if constexpr (DOT)
                fix_dot += (double)a * (double)p.X[r * p.ldx + lane];
        }
    }
    if constexpr (DOT) {
        double part = fix_dot;
        for (uint32_t wi = warp; wi < p.nwarps; wi += WPC)
            part += __ldcg(&p.dot_part[(uint64_t)wi * 32 + lane]);
        s_dot[warp][lane] = part;
        __syncthreads();
        if (warp == 0 && active) {
            double d = 0.0;
            for (int w = 0; w < WPC; ++w)
                d += s_dot[w][lane];
            if (p.dot_out)
                p.dot_out[lane] = d;
            if (p.alpha_out) {
                const uint32_t* mk = p.mask ? p.mask + (p.mask_sel ? 32u * (*p.mask_sel) : 0u) : nullptr;
                const bool on = !mk || mk[lane];
                if (on && (!(d > 0.0) || !isfinite(d)))
                    record_status(p.status, kStatusBreakdown);
                p.alpha_out[lane] = (on && d > 0.0 && isfinite(d)) ? p.rr[lane] / d : 0.0;
            }
        }
    }
    if (threadIdx.x == 0)
        *p.counter = 0u;
}

template <typename VT, int WPC, int STAGES>
constexpr size_t mm_smem() {
    return 128 * ((WPC * STAGES * 8 + 127) / 128) + (size_t)WPC * STAGES * mm_geom<VT>::STAGE;
}

template <typename VT, int WPC, int STAGES, bool DOT>
cudaError_t mm_attr() {
    return cudaFuncSetAttribute(k_spmm<VT, WPC, STAGES, DOT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)mm_smem<VT, WPC, STAGES>());
}

template <typename VT, int WPC, int STAGES, bool DOT>
int mm_launch(const dimgpu_csr5* m, const VT* vals, const spmm_args& a, const spmm_scratch& sc, cudaStream_t st) {
    const spmv_plan pl = make_spmv_plan(m->tile_count, device_sm_count(m->device), WPC);
    if (pl.nwarps > sc.nslots)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "SpMM scratch holds %u warp slots, launch needs %u", sc.nslots,
                    pl.nwarps);
    spmm_params<VT> p;
    p.vals = vals;
    p.col = m->col;
    p.desc = reinterpret_cast<const uint32_t*>(m->tile_desc);
    p.tile_ptr = m->tile_ptr;
    p.tdo_ptr = m->tdo_ptr;
    p.tdo = m->tdo;
    p.row_ptr = m->row_ptr;
    p.X = static_cast<const VT*>(a.X);
    p.Y = static_cast<VT*>(a.Y);
    p.ldx = a.ldx;
    p.ldy = a.ldy;
    p.k = a.k;
    p.T = m->tile_count;
    p.rows = m->rows;
    p.tail_start = m->tail_start;
    p.tpw = pl.tiles_per_warp;
    p.nwarps = pl.nwarps;
    p.empty_rows = m->empty_rows;
    p.n_empty = m->n_empty;
    p.cal_val = sc.cal_val;
    p.cal_row = sc.cal_row;
    p.dot_part = sc.dot_part;
    p.counter = sc.counter;
    p.status = sc.status;
    p.dot_out = a.dot_out;
    p.rr = a.rr;
    p.alpha_out = a.alpha_out;
    p.mask = a.mask;
    p.mask_sel = a.mask_sel;
    p.halt = a.halt;
    k_spmm<VT, WPC, STAGES, DOT><<<pl.grid, WPC * 32, mm_smem<VT, WPC, STAGES>(), st>>>(p);
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

template <typename VT, bool DOT>
int mm_dispatch(const dimgpu_csr5* m, const VT* vals, const spmm_args& a, const spmm_scratch& sc, int shape,
                cudaStream_t st) {
    switch (shape) {
    case 0:
        return mm_launch<VT, 8, 3, DOT>(m, vals, a, sc, st);
    case 1:
        return mm_launch<VT, 16, 2, DOT>(m, vals, a, sc, st);
    default:
        return mm_launch<VT, 12, 2, DOT>(m, vals, a, sc, st);
    }
}

}  // namespace

int prepare_spmm_kernels() {
    static int done = 0;
    if (done)
        return DIMGPU_OK;
    DG_CUDA((mm_attr<double, 8, 3, false>()));
    DG_CUDA((mm_attr<double, 8, 3, true>()));
    DG_CUDA((mm_attr<double, 16, 2, false>()));
    DG_CUDA((mm_attr<double, 16, 2, true>()));
    DG_CUDA((mm_attr<double, 12, 2, false>()));
    DG_CUDA((mm_attr<double, 12, 2, true>()));
    DG_CUDA((mm_attr<float, 8, 3, false>()));
    DG_CUDA((mm_attr<float, 8, 3, true>()));
    DG_CUDA((mm_attr<float, 16, 2, false>()));
    DG_CUDA((mm_attr<float, 16, 2, true>()));
    DG_CUDA((mm_attr<float, 12, 2, false>()));
    DG_CUDA((mm_attr<float, 12, 2, true>()));
    done = 1;
    return DIMGPU_OK;
}

uint32_t spmm_max_slots(const dimgpu_csr5* m) {
    const int sms = device_sm_count(m->device);
    uint32_t n = 1;
    for (int wpc : {8, 12, 16})
        n = std::max<uint32_t>(n, make_spmv_plan(m->tile_count, sms, wpc).nwarps);
    return n;
}

int spmm_scratch_init(spmm_scratch* s, const dimgpu_csr5* m) {
    s->nslots = spmm_max_slots(m);
    DG_CHECK(dev_alloc_n(&s->cal_val, (uint64_t)s->nslots * 32));
    DG_CHECK(dev_alloc_n(&s->dot_part, (uint64_t)s->nslots * 32));
    DG_CHECK(dev_alloc_n(&s->cal_row, s->nslots));
    DG_CHECK(dev_alloc_n(&s->counter, 4));
    DG_CHECK(dev_alloc_n(&s->status, 4));
    DG_CUDA(cudaMemset(s->counter, 0, 16));
    DG_CUDA(cudaMemset(s->status, 0, 16));
    return DIMGPU_OK;
}

void spmm_scratch_release(spmm_scratch* s) {
    dev_free(s->cal_val);
    dev_free(s->dot_part);
    dev_free(s->cal_row);
    dev_free(s->counter);
    dev_free(s->status);
    *s = spmm_scratch{};
}

int launch_spmm(const dimgpu_csr5* m, bool f32, const spmm_args& a, const spmm_scratch& sc, int shape,
                cudaStream_t st) {
    if (m->layout != kLayoutDevice || m->omega != 32 || m->sigma != 16)
        return fail(DIMGPU_ERR_UNSUPPORTED, "SpMM needs the 32-lane device layout with sigma 16");
    if (a.k == 0 || a.k > 32)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "one SpMM pass takes 1..32 right-hand sides (got %u)", a.k);
    if (a.ldx < a.k || a.ldy < a.k)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "leading dimensions must be >= k");
    const bool dot = a.dot_out || a.alpha_out;
    if (f32) {
        DG_CHECK(ensure_vals32(m, st));
        return dot ? mm_dispatch<float, true>(m, m->vals32, a, sc, shape, st)
                   : mm_dispatch<float, false>(m, m->vals32, a, sc, shape, st);
    }
    return dot ? mm_dispatch<double, true>(m, m->vals, a, sc, shape, st)
               : mm_dispatch<double, false>(m, m->vals, a, sc, shape, st);
}

// Picks the launch shape (warps per CTA x pipeline stages) of one SpMM by timing each candidate on
// the caller's operands.  Deterministic choice: the fastest of two timed launches per shape.
int autotune_spmm(const dimgpu_csr5* m, bool f32, const spmm_args& a, const spmm_scratch& sc, cudaStream_t st,
                  int* best_shape, float* best_ms) {
    cudaEvent_t e0, e1;
    DG_CUDA(cudaEventCreate(&e0));
    DG_CUDA(cudaEventCreate(&e1));
    spmm_args plain = a;
    plain.dot_out = nullptr;
    plain.alpha_out = nullptr;
    plain.rr = nullptr;
    plain.mask = nullptr;
    plain.mask_sel = nullptr;
    plain.halt = nullptr;
    int best = 1;
    float bms = 1e30f;
    int rc = DIMGPU_OK;
    for (int shape = 0; shape < kSpmmShapes && rc == DIMGPU_OK; ++shape) {
        if ((rc = launch_spmm(m, f32, plain, sc, shape, st)) != DIMGPU_OK)
            break;
        float ms_min = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {
            cudaEventRecord(e0, st);
            if ((rc = launch_spmm(m, f32, plain, sc, shape, st)) != DIMGPU_OK)
                break;
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            ms_min = std::min(ms_min, ms);
        }
        if (ms_min < bms) {
            bms = ms_min;
            best = shape;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != DIMGPU_OK)
        return rc;
    *best_shape = best;
    if (best_ms)
        *best_ms = bms;
    return DIMGPU_OK;
}

}  // namespace dimgpu

// ------------------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------------------
namespace {
int spmm_entry(const dimgpu_csr5* cm, uint32_t k, const void* X, uint64_t ldx, void* Y, uint64_t ldy, bool f32,
               void* stream) {
    using namespace dimgpu;
    dimgpu_csr5* m = const_cast<dimgpu_csr5*>(cm);
    if (!m || (k && (!X || !Y)))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    if (k == 0)
        return DIMGPU_OK;
    if (ldx < k || ldy < k)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "leading dimensions must be >= k");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DG_CHECK(prepare_spmm_kernels());
    if (!m->spmm_sc) {
        spmm_scratch* sc = new spmm_scratch();
        int rc = spmm_scratch_init(sc, m);
        if (rc != DIMGPU_OK) {
            spmm_scratch_release(sc);
            delete sc;
            return rc;
        }
        m->spmm_sc = sc;
    }
    const spmm_scratch& sc = *static_cast<spmm_scratch*>(m->spmm_sc);
    const size_t esz = f32 ? 4 : 8;
    for (uint32_t c0 = 0; c0 < k; c0 += 32) {
        spmm_args a;
        a.k = std::min<uint32_t>(32, k - c0);
        a.X = static_cast<const unsigned char*>(X) + c0 * esz;
        a.Y = static_cast<unsigned char*>(Y) + c0 * esz;
        a.ldx = ldx;
        a.ldy = ldy;
        int& shape = m->spmm_shape[f32 ? 1 : 0][a.k];
        if (shape < 0)
            DG_CHECK(autotune_spmm(m, f32, a, sc, st, &shape, nullptr));
        DG_CHECK(launch_spmm(m, f32, a, sc, shape, st));
    }
    return DIMGPU_OK;
}
}  // namespace

extern "C" int dimgpu_csr5_spmm(const dimgpu_csr5* m, uint32_t k, const double* X, uint64_t ldx, double* Y,
                                uint64_t ldy, void* stream) {
    return spmm_entry(m, k, X, ldx, Y, ldy, false, stream);
}

extern "C" int dimgpu_csr5_spmm_f32(const dimgpu_csr5* m, uint32_t k, const float* X, uint64_t ldx, float* Y,
                                    uint64_t ldy, void* stream) {
    return spmm_entry(m, k, X, ldx, Y, ldy, true, stream);
}

extern "C" int dimgpu_csr5_spmm_shape(const dimgpu_csr5* m, uint32_t k, int f32, int* shape) {
    if (!m || !shape || k == 0 || k > 32)
        return dimgpu::fail(DIMGPU_ERR_INVALID_ARGUMENT, "bad argument");
    *shape = m->spmm_shape[f32 ? 1 : 0][k];
    return DIMGPU_OK;
}
