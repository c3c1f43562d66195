// spmv.cu -- CSR5 SpMV on GB300 (device layout: omega = 32 lanes, sigma rows per tile column).
//
// Reference: csr5::spmv and its helpers (include/dim/mat/storage_formats/csr5.h:495-829).
//
// Work split.  Each warp owns a contiguous run of tiles, as each OpenMP thread owns a contiguous
// chunk in the reference (csr5.h:608-630); lane c of the warp is tile column c (the reference's SIMD
// lane, csr5.h:553-560, widened from 4 to 32).
//
// Data movement.  Lane 0 of each warp streams its tiles into a ring of shared-memory stages with
// cp.async.bulk (TMA engine) completing on one mbarrier per stage: values (sigma*32*8 B), column
// indices (sigma*32*4 B) and the 32 descriptor words, all with an L2 evict-first policy so that the
// gathered vector x stays resident in L2.  Lanes then read their column with 16-byte shared loads
// (two f64 rows or four u32 rows at a time, see layout.cuh) and gather x.
//
// Arithmetic per tile (the csr5.h:640-745 algorithm restated for warps):
//   * a tile inside one row (tile_ptr[t] == tile_ptr[t+1], csr5.h:640-643) is a dot product;
//   * otherwise each lane walks its sigma rows, closing a segment at every set bit_flag bit
//     (csr5.h:688-724; column 0 gets an implicit row start, csr5.h:668); closed segments are
//     written to y[row_start + y_offset] (or through tile_desc_offset for tiles with empty rows,
//     csr5.h:650-655);
//   * the open segment at the bottom of each column takes the "red" head sums of the following
//     columns through a segmented suffix scan over warp shuffles (the role of fast_segmented_sum /
//     compute_last_sum, csr5.h:200-235), with as many doubling steps as the longest run of
//     columns without a row start needs;
//   * the head segment of the tile and the segment running off its end feed an in-order carry
//     chain inside the warp, so rows crossing tile boundaries are summed left to right.
// Calibrator (csr5.h:526-538, 750-754).  A warp's first row, when it started before the warp's
// first tile, is not written: its partial sum goes to the warp's calibrator slot.  The last CTA to
// finish (completion ticket) adds the slots to y in warp order, then computes the CSR tail
// (csr5.h:756-782) and, optionally, the fused dot x.y and alpha = rr / (x.y) for CG.  y is fully
// overwritten: empty rows below the tail are zeroed from the list built at conversion.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "internal.hpp"
#include "layout.cuh"

namespace dimgpu {
namespace {

template <int SIGMA>
struct word_of {
    using type = uint32_t;
};
template <>
struct word_of<32> {
    using type = uint64_t;
};

template <typename VT>
struct spmv_params {
    const VT* vals;
    const uint32_t* col;
    const void* desc;
    const uint32_t* tile_ptr;
    const uint32_t* tdo_ptr;
    const uint32_t* tdo;
    const uint32_t* row_ptr;
    const VT* x;
    VT* y;
    uint64_t T;
    uint32_t rows;
    uint32_t tail_start;
    uint64_t tpw;
    uint32_t nwarps;
    const uint32_t* empty_rows;
    uint32_t n_empty;
    double* cal_val;
    uint32_t* cal_row;
    double* dot_part;
    uint32_t* counter;
    uint32_t* status;
    double* dot_out;
    const double* rr;
    double* alpha_out;
    uint32_t* halt;
};

template <typename VT, int SIGMA>
struct tile_geom {
    using Word = typename word_of<SIGMA>::type;
    static constexpr uint32_t TS = SIGMA * 32;
    static constexpr uint32_t VBYTES = TS * sizeof(VT);
    static constexpr uint32_t CBYTES = TS * 4;
    static constexpr uint32_t DBYTES = 32 * sizeof(Word);
    static constexpr uint32_t STAGE = VBYTES + CBYTES + DBYTES;
    static constexpr desc_fields F = fields_for(SIGMA, 32);
    static constexpr uint64_t YMASK = (1ull << F.yb) - 1;
    static constexpr uint64_t FMASK = (SIGMA == 64) ? ~0ull : ((1ull << SIGMA) - 1);
};

// Loads lane `lane`'s column (SIGMA values and column indices) from a shared stage.
template <typename VT, int SIGMA>
__device__ __forceinline__ void load_column(const unsigned char* stage, unsigned lane, VT (&v)[SIGMA],
                                            uint32_t (&ci)[SIGMA]) {
    using G = tile_geom<VT, SIGMA>;
    const uint4* sc = reinterpret_cast<const uint4*>(stage + G::VBYTES);
#pragma unroll
    for (int j = 0; j < SIGMA / 4; ++j) {
        const uint4 q = sc[j * 32 + lane];
        ci[4 * j + 0] = q.x;
        ci[4 * j + 1] = q.y;
        ci[4 * j + 2] = q.z;
        ci[4 * j + 3] = q.w;
    }
    if constexpr (sizeof(VT) == 8) {
        const double2* sv = reinterpret_cast<const double2*>(stage);
#pragma unroll
        for (int j = 0; j < SIGMA / 2; ++j) {
            const double2 d = sv[j * 32 + lane];
            v[2 * j + 0] = d.x;
            v[2 * j + 1] = d.y;
        }
    } else {
        const float4* sv = reinterpret_cast<const float4*>(stage);
#pragma unroll
        for (int j = 0; j < SIGMA / 4; ++j) {
            const float4 d = sv[j * 32 + lane];
            v[4 * j + 0] = d.x;
            v[4 * j + 1] = d.y;
            v[4 * j + 2] = d.z;
            v[4 * j + 3] = d.w;
        }
    }
}

template <typename VT, int SIGMA, int WPC, int STAGES, bool DOT>
__global__ void __launch_bounds__(WPC * 32, 1) k_spmv(const spmv_params<VT> p) {
    using G = tile_geom<VT, SIGMA>;
    using Word = typename G::Word;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint32_t s_last;
    __shared__ double s_red[WPC];

    if (p.halt && *reinterpret_cast<volatile const uint32_t*>(p.halt))
        return;  // a previous stage of a CG iteration has already stopped the solve

    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t gw = blockIdx.x * WPC + warp;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem) + warp * STAGES;
    unsigned char* ring = smem + 128 * ((WPC * STAGES * 8 + 127) / 128) + (size_t)warp * STAGES * G::STAGE;

    // Empty rows below the tail get 0 (the reference leaves them to a zero-filled y).
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < p.n_empty;
         i += (uint64_t)gridDim.x * blockDim.x)
        p.y[p.empty_rows[i]] = VT(0);

    const uint64_t t_begin = min(p.T, (uint64_t)gw * p.tpw);
    const uint64_t t_end = min(p.T, t_begin + p.tpw);

    double dot_acc = 0.0;
    bool open = false, cal_valid = false;
    VT carry = VT(0), cal = VT(0);
    uint32_t carry_row = 0, cal_row = 0;

    auto write_row_lane0 = [&](uint32_t row, VT val) {
        if (lane == 0) {
            p.y[row] = val;
            if constexpr (DOT)
                dot_acc += (double)val * (double)ldg_keep(p.x + row);
        }
    };

    if (t_begin < t_end) {
        const Word* gdesc = reinterpret_cast<const Word*>(p.desc);
        const uint64_t pol = policy_evict_first();
        const uint64_t pol_keep = policy_evict_last();
        if (lane == 0) {
            for (int s = 0; s < STAGES; ++s)
                mbar_init(&bars[s], 1);
            fence_mbar_init();
        }
        __syncwarp();
        auto issue = [&](int s, uint64_t t) {
            unsigned char* st = ring + (size_t)s * G::STAGE;
            mbar_arrive_expect_tx(&bars[s], G::STAGE);
            bulk_g2s(st, p.vals + t * G::TS, G::VBYTES, &bars[s], pol);
            bulk_g2s(st + G::VBYTES, p.col + t * G::TS, G::CBYTES, &bars[s], pol);
            bulk_g2s(st + G::VBYTES + G::CBYTES, gdesc + t * 32, G::DBYTES, &bars[s], pol);
        };
        if (lane == 0)
            for (int s = 0; s < STAGES && t_begin + s < t_end; ++s)
                issue(s, t_begin + s);

        // tile_ptr runs two tiles ahead so that no tile waits on its load
        uint32_t raw_cur = __ldg(&p.tile_ptr[t_begin]);
        uint32_t raw_next = __ldg(&p.tile_ptr[t_begin + 1]);
        uint64_t i = 0;
        bool failed = false;
        for (uint64_t t = t_begin; t < t_end; ++t, ++i) {
            const int s = (int)(i % STAGES);
            const uint32_t par = (uint32_t)((i / STAGES) & 1);
            const uint32_t raw = raw_cur;
            const uint32_t row_stop = raw_next & ~kDirty;
            const uint32_t row_start = raw & ~kDirty;
            raw_cur = raw_next;
            raw_next = (t + 2 <= p.T) ? __ldg(&p.tile_ptr[t + 2]) : 0u;
            if (!mbar_wait_bounded(&bars[s], par, p.status)) {
                failed = true;
                break;
            }
            unsigned char* st = ring + (size_t)s * G::STAGE;
            const Word* sd = reinterpret_cast<const Word*>(st + G::VBYTES + G::CBYTES);

            VT v[SIGMA];
            uint32_t ci[SIGMA];
            load_column<VT, SIGMA>(st, lane, v, ci);
            const Word w = sd[lane];
            VT xv[SIGMA];
#pragma unroll
            for (int r = 0; r < SIGMA; ++r)
                xv[r] = ldg_x(p.x + ci[r], pol_keep);
            // the fused dot needs x at this tile's rows: fetch them now, off the write-out's path
            VT xrow = VT(0);
            if constexpr (DOT) {
                if (row_start + lane < p.rows)
                    xrow = ldg_x(p.x + row_start + lane, pol_keep);
            }
            const uint32_t flag = (uint32_t)((uint64_t(w) >> (G::F.yb + G::F.sb)) & G::FMASK);
            const bool capped = (__shfl_sync(kFull, flag, 0) & 1u) != 0;
            // Every lane now holds its column: the value area of the stage becomes the staging
            // buffer of this tile's segment sums (slot = segment index, at most sigma*32 of them).
            __syncwarp();
            VT* ystage = reinterpret_cast<VT*>(st);
            const bool dirty = (raw & kDirty) != 0;
            const uint32_t optr = dirty ? __ldg(&p.tdo_ptr[t]) : 0u;
            auto row_of = [&](uint32_t idx) -> uint32_t {
                return row_start + (dirty ? __ldg(&p.tdo[optr + idx]) : idx);
            };

            VT H, Lt;
            uint32_t K, row_last;
            if (raw == row_stop) {
                // partition_fast_track (csr5.h:562-574): the whole tile is one row
                VT acc = VT(0);
#pragma unroll
                for (int r = 0; r < SIGMA; ++r)
                    acc = fma(v[r], xv[r], acc);
                H = warp_sum(acc);
                Lt = H;
                K = 1;
                row_last = row_start;
            } else {
                const uint32_t yoff = (uint32_t)(uint64_t(w) & G::YMASK);
                const uint32_t fl = flag | (lane == 0 ? 1u : 0u);
                const uint32_t present = __ballot_sync(kFull, fl != 0);

                // Segments of this column: segment yoff + k is staged at slot[k].  Branch-free: a
                // row start closes the open segment (predicated store) and restarts the sum.
                VT* slot = ystage + yoff;
                VT sum = VT(0), red = VT(0);
                uint32_t k = 0;
                bool seen = false;
#pragma unroll
                for (int r = 0; r < SIGMA; ++r) {
                    const bool bit = ((fl >> r) & 1u) != 0;
                    const bool close = bit && seen;
                    if (close)
                        slot[k] = sum;
                    k += close ? 1u : 0u;
                    red = (bit && !seen) ? sum : red;
                    seen = seen || bit;
                    sum = bit ? VT(0) : sum;
                    sum = fma(v[r], xv[r], sum);
                }
                const VT L = seen ? sum : VT(0);
                red = seen ? red : sum;

                // segmented suffix sums of the red parts, terminated by columns with a row start
                VT U = red;
                uint32_t stopped = (present >> lane) & 1u;
                const int steps = scan_steps_for(present);
                for (int q = 0, d = 1; q < steps; ++q, d <<= 1) {
                    const VT u2 = __shfl_down_sync(kFull, U, d);
                    const uint32_t s2 = __shfl_down_sync(kFull, stopped, d);
                    if (!stopped && lane + d < 32) {
                        U += u2;
                        stopped |= s2;
                    }
                }
                const VT nxt = __shfl_down_sync(kFull, U, 1);
                const VT seg_total = L + (lane == 31 ? VT(0) : nxt);
                const uint32_t last_lane = 31u - __clz(present);
                const bool is_present = ((present >> lane) & 1u) != 0;
                if (is_present && lane != last_lane)
                    slot[k] = seg_total;  // the column's open segment, closed by a later column
                uint32_t my_row_last = 0;
                if (lane == last_lane)
                    my_row_last = row_of(yoff + k);
                K = __shfl_sync(kFull, yoff + k + 1, last_lane);
                Lt = __shfl_sync(kFull, seg_total, last_lane);
                row_last = __shfl_sync(kFull, my_row_last, last_lane);
                __syncwarp();
                H = (K == 1) ? Lt : ystage[0];  // segment 0 sits in slot 0 whenever it closed in this tile
            }

            // in-order carry chain over the warp's tiles (uniform across lanes)
            bool head_staged = false;
            if (K == 1) {
                if (capped) {
                    if (open)
                        write_row_lane0(carry_row, carry);
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
                if (capped || open) {
                    if (capped && open)
                        write_row_lane0(carry_row, carry);
                    if (!capped && lane == 0)
                        ystage[0] = carry + H;  // the row that began before this tile closes here
                    head_staged = true;
                } else {
                    cal += H;
                    cal_row = row_start;
                    cal_valid = true;
                }
                open = true;
                carry = Lt;
                carry_row = row_last;
            }
            // write the tile's closed rows coalesced (slots 0 or 1 .. K-2; slot K-1 is the carry)
            __syncwarp();
            if (K > 1) {
                const uint32_t lo = head_staged ? 0u : 1u;
                VT xfirst = VT(0);
                if constexpr (DOT)
                    xfirst = __shfl_down_sync(kFull, xrow, lo);  // x[row_start + lo + lane]
                for (uint32_t j = lo + lane; j + 1 < K; j += 32) {
                    const VT val = ystage[j];
                    const uint32_t row = row_of(j);
                    st_keep(p.y + row, val, pol_keep);
                    if constexpr (DOT) {
                        const bool have = !dirty && j == lo + lane && lane + lo < 32;
                        const VT xr = have ? xfirst : ldg_x(p.x + row, pol_keep);
                        dot_acc = fma((double)val, (double)xr, dot_acc);
                    }
                }
            }

            __syncwarp();
            if (lane == 0 && t + STAGES < t_end) {
                fence_proxy_async_smem();
                issue(s, t + STAGES);
            }
        }
        if (failed) {
            // drain the copies this warp still has in flight, then leave the results invalid
            for (uint64_t t2 = t_begin + i; t2 < t_end && t2 < t_begin + i + STAGES; ++t2) {
                const uint64_t i2 = t2 - t_begin;
                (void)mbar_wait_bounded(&bars[i2 % STAGES], (uint32_t)((i2 / STAGES) & 1), p.status);
            }
        } else if (open) {
            write_row_lane0(carry_row, carry);
        }
    }
    if (lane == 0) {
        p.cal_val[gw] = (double)cal;
        p.cal_row[gw] = cal_valid ? (cal_row | kDirty) : 0u;
    }
    if constexpr (DOT) {
        const double d = warp_sum(dot_acc);
        if (lane == 0)
            p.dot_part[gw] = d;
    }

    // ---- completion ticket; the last CTA resolves calibrators, the tail and the epilogue ----
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t ticket = atomicAdd(p.counter, 1u);
        s_last = (ticket == gridDim.x - 1) ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last)
        return;
    __threadfence();

    double fix_dot = 0.0;
    for (uint32_t wi = threadIdx.x; wi < p.nwarps; wi += blockDim.x) {
        const uint32_t cr = __ldcg(&p.cal_row[wi]);
        if (!(cr & kDirty))
            continue;
        if (wi > 0 && __ldcg(&p.cal_row[wi - 1]) == cr)
            continue;  // not the first slot of this row
        const uint32_t R = cr & ~kDirty;
        VT acc = __ldcg(&p.y[R]);
        double added = 0.0;
        for (uint32_t w2 = wi; w2 < p.nwarps; ++w2) {
            if (__ldcg(&p.cal_row[w2]) != cr)
                break;
            const VT c = (VT)__ldcg(&p.cal_val[w2]);
            acc += c;
            added += (double)c;
        }
        p.y[R] = acc;
        if constexpr (DOT)
            fix_dot += added * (double)p.x[R];
    }
    __syncthreads();
    const uint64_t first_tail = p.T * G::TS;
    for (uint64_t r = (uint64_t)p.tail_start + threadIdx.x; r < p.rows; r += blockDim.x) {
        const uint64_t s = (r == p.tail_start) ? first_tail : (uint64_t)p.row_ptr[r];
        const uint64_t e = p.row_ptr[r + 1];
        VT acc = VT(0);
        for (uint64_t k = s; k < e; ++k)
            acc = fma(p.vals[k], p.x[p.col[k]], acc);
        if (r == p.tail_start && (uint64_t)p.row_ptr[r] != first_tail)
            p.y[r] = __ldcg(&p.y[r]) + acc;
        else
            p.y[r] = acc;
        if constexpr (DOT)
            fix_dot += (double)acc * (double)p.x[r];
    }
    if constexpr (DOT) {
        double part = fix_dot;
        for (uint32_t wi = threadIdx.x; wi < p.nwarps; wi += blockDim.x)
            part += __ldcg(&p.dot_part[wi]);
        // warp sums, then the WPC warp sums in order (any block size; fixed order)
        part = warp_sum(part);
        if (lane == 0)
            s_red[warp] = part;
        __syncthreads();
        if (threadIdx.x == 0) {
            double dot = 0.0;
            for (int wi = 0; wi < WPC; ++wi)
                dot += s_red[wi];
            if (p.dot_out)
                *p.dot_out = dot;
            if (p.rr) {
                if (!(dot > 0.0) || !isfinite(dot)) {
                    record_status(p.status, kStatusBreakdown);
                    if (p.halt)
                        *p.halt = 1u;
                    if (p.alpha_out)
                        *p.alpha_out = 0.0;
                } else if (p.alpha_out) {
                    *p.alpha_out = *p.rr / dot;
                }
            }
        }
    }
    if (threadIdx.x == 0)
        *p.counter = 0u;
}

template <typename VT, int SIGMA, int WPC, int STAGES>
constexpr size_t smem_bytes() {
    return 128 * ((WPC * STAGES * 8 + 127) / 128) + (size_t)WPC * STAGES * tile_geom<VT, SIGMA>::STAGE;
}

template <typename VT, int SIGMA, int WPC, int STAGES, bool DOT>
int launch_cfg(const dimgpu_csr5* m, const VT* vals, const VT* x, VT* y, dimgpu_calibrator* cal,
               const spmv_epilogue& ep, cudaStream_t stream) {
    constexpr size_t smem = smem_bytes<VT, SIGMA, WPC, STAGES>();
    const spmv_plan& pl = sizeof(VT) == 8 ? m->plan : m->plan32;
    if (pl.warps_per_cta != WPC)
        return fail(DIMGPU_ERR_UNSUPPORTED, "launch plan has %d warps per CTA, kernel %d", pl.warps_per_cta, WPC);
    if (pl.nwarps > cal->nslots)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "calibrator has %u slots, plan needs %u", cal->nslots, pl.nwarps);
    spmv_params<VT> p;
    p.vals = vals;
    p.col = m->col;
    p.desc = m->tile_desc;
    p.tile_ptr = m->tile_ptr;
    p.tdo_ptr = m->tdo_ptr;
    p.tdo = m->tdo;
    p.row_ptr = m->row_ptr;
    p.x = x;
    p.y = y;
    p.T = m->tile_count;
    p.rows = m->rows;
    p.tail_start = m->tail_start;
    p.tpw = pl.tiles_per_warp;
    p.nwarps = pl.nwarps;
    p.empty_rows = m->empty_rows;
    p.n_empty = m->n_empty;
    p.cal_val = cal->cal_val;
    p.cal_row = cal->cal_row;
    p.dot_part = cal->dot_part;
    p.counter = cal->counter;
    p.status = cal->status;
    p.dot_out = ep.dot_out;
    p.rr = ep.rr;
    p.alpha_out = ep.alpha_out;
    p.halt = ep.halt;
    k_spmv<VT, SIGMA, WPC, STAGES, DOT><<<pl.grid, WPC * 32, smem, stream>>>(p);
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

constexpr int kWPC = 16;    // f64: 16 warps x 2 stages x 6.3 KB per SM (register-limited)
constexpr int kWPC32 = 24;  // f32: 24 warps x 2 stages x 4.2 KB per SM
constexpr int kStages = 2;

template <typename VT, int SIGMA, int WPC, int STAGES, bool DOT>
cudaError_t set_smem_attr() {
    return cudaFuncSetAttribute(k_spmv<VT, SIGMA, WPC, STAGES, DOT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_bytes<VT, SIGMA, WPC, STAGES>());
}

}  // namespace

// Sets the dynamic shared-memory limit of every SpMV kernel once per process (before any graph
// capture touches them).
int prepare_spmv_kernels() {
    static int done = 0;
    if (done)
        return DIMGPU_OK;
    DG_CUDA((set_smem_attr<double, 16, kWPC, kStages, false>()));
    DG_CUDA((set_smem_attr<double, 16, kWPC, kStages, true>()));
    DG_CUDA((set_smem_attr<float, 16, kWPC32, kStages, false>()));
    DG_CUDA((set_smem_attr<float, 16, kWPC32, kStages, true>()));
    done = 1;
    return DIMGPU_OK;
}

int device_sm_count(int device) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
        sms = 148;
    return sms;
}

spmv_plan make_spmv_plan(uint64_t tiles, int sms, int wpc) {
    spmv_plan pl;
    pl.warps_per_cta = wpc;
    const uint64_t max_warps = (uint64_t)sms * wpc;
    uint64_t warps = std::min<uint64_t>(max_warps, std::max<uint64_t>(1, tiles));
    pl.grid = (int)((warps + wpc - 1) / wpc);
    pl.nwarps = (uint32_t)pl.grid * wpc;
    pl.tiles_per_warp = tiles ? (tiles + pl.nwarps - 1) / pl.nwarps : 0;
    // shrink the grid when the last CTAs would have no tiles
    if (pl.tiles_per_warp) {
        const uint64_t used_warps = (tiles + pl.tiles_per_warp - 1) / pl.tiles_per_warp;
        pl.grid = (int)((used_warps + wpc - 1) / wpc);
        pl.nwarps = (uint32_t)pl.grid * wpc;
    }
    return pl;
}

spmv_plan make_spmv_plan32(uint64_t tiles, int sms) { return make_spmv_plan(tiles, sms, kWPC32); }

int calibrator_init(dimgpu_calibrator* c, const dimgpu_csr5* m) {
    cudaGetDevice(&c->device);
    c->nslots = std::max<uint32_t>(std::max(m->plan.nwarps, m->plan32.nwarps), 1);
    DG_CHECK(dev_alloc_n(&c->cal_val, c->nslots));
    DG_CHECK(dev_alloc_n(&c->cal_row, c->nslots));
    DG_CHECK(dev_alloc_n(&c->dot_part, c->nslots + 1));
    DG_CHECK(dev_alloc_n(&c->counter, 4));
    DG_CHECK(dev_alloc_n(&c->status, 4));
    DG_CUDA(cudaMemset(c->counter, 0, 16));
    DG_CUDA(cudaMemset(c->status, 0, 16));
    return DIMGPU_OK;
}

void calibrator_release(dimgpu_calibrator* c) {
    dev_free(c->cal_val);
    dev_free(c->cal_row);
    dev_free(c->dot_part);
    dev_free(c->counter);
    dev_free(c->status);
    c->cal_val = nullptr;
}

int launch_spmv_f64(const dimgpu_csr5* m, const double* x, double* y, dimgpu_calibrator* cal,
                    const spmv_epilogue& ep, cudaStream_t stream) {
    if (m->layout != kLayoutDevice || m->omega != 32)
        return fail(DIMGPU_ERR_UNSUPPORTED, "SpMV needs the 32-lane device layout");
    const bool dot = ep.dot_out || ep.alpha_out;
    switch (m->sigma) {
    case 16:
        return dot ? launch_cfg<double, 16, kWPC, kStages, true>(m, m->vals, x, y, cal, ep, stream)
                   : launch_cfg<double, 16, kWPC, kStages, false>(m, m->vals, x, y, cal, ep, stream);
    default:
        return fail(DIMGPU_ERR_UNSUPPORTED, "sigma %u has no SpMV kernel", m->sigma);
    }
}

int launch_spmv_f32(const dimgpu_csr5* m, const float* x, float* y, dimgpu_calibrator* cal,
                    const spmv_epilogue& ep, cudaStream_t stream) {
    if (m->layout != kLayoutDevice || m->omega != 32)
        return fail(DIMGPU_ERR_UNSUPPORTED, "SpMV needs the 32-lane device layout");
    DG_CHECK(ensure_vals32(m, stream));
    const bool dot = ep.dot_out || ep.alpha_out;
    switch (m->sigma) {
    case 16:
        return dot ? launch_cfg<float, 16, kWPC32, kStages, true>(m, m->vals32, x, y, cal, ep, stream)
                   : launch_cfg<float, 16, kWPC32, kStages, false>(m, m->vals32, x, y, cal, ep, stream);
    default:
        return fail(DIMGPU_ERR_UNSUPPORTED, "sigma %u has no SpMV kernel", m->sigma);
    }
}

int check_status(dimgpu_calibrator* cal, cudaStream_t stream) {
    uint32_t st = 0;
    DG_CUDA(cudaMemcpyAsync(&st, cal->status, sizeof(st), cudaMemcpyDeviceToHost, stream));
    DG_CUDA(cudaStreamSynchronize(stream));
    if (st == kStatusOk)
        return DIMGPU_OK;
    cudaMemsetAsync(cal->status, 0, sizeof(uint32_t), stream);
    if (st == kStatusWaitTimeout)
        return fail(DIMGPU_ERR_TIMEOUT, "a bounded device wait expired");
    if (st == kStatusBreakdown)
        return fail(DIMGPU_ERR_BREAKDOWN, "CG breakdown: s.As <= 0 or not finite");
    return fail(DIMGPU_ERR_BAD_INDEX, "device status %u", st);
}

}  // namespace dimgpu

// ------------------------------------------------------------------------------------------------
// SpMV without any allocation by the caller or the library.
//
// dimgpu_csr5_spmv needs a calibrator (scratch for the per-warp row fragments, the fused-dot
// partials, the completion ticket and the status word), and dimgpu_calibrator_create obtains it
// with cudaMalloc.  Some callers cannot do that: a plugin running inside a host application that
// reserved all device memory up front, a real-time loop where cudaMalloc's implicit device
// synchronisation would break the latency budget, or code that must not grow its memory footprint
// after start-up.  For them the scratch of this entry point is a fixed array compiled into the
// library: every GPU that loads the library holds it until the process exits.
// ------------------------------------------------------------------------------------------------
namespace dimgpu {
namespace {

constexpr uint32_t kStaticSlots = 4096;  // warp slots: enough for 256 SMs x 16 warps
constexpr size_t kStaticValBytes = 8 * kStaticSlots;
constexpr size_t kStaticDotBytes = 8 * (kStaticSlots + 32);
constexpr size_t kStaticRowBytes = 4 * kStaticSlots;
constexpr size_t kStaticWordBytes = 256;  // completion ticket + status word, own 256-byte block
constexpr size_t kStaticScratchBytes = kStaticValBytes + kStaticDotBytes + kStaticRowBytes + kStaticWordBytes;

// 82,432 bytes of device memory, shared by every call of dimgpu_csr5_spmv_static_scratch on a device.
static __device__ __align__(256) unsigned char g_spmv_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
unsigned char* g_static_addr[kMaxDevices] = {};

// Device address of the static scratch on `device` (which must be current).  Host code cannot use
// the symbol itself: on the host, g_spmv_static_scratch is only a stand-in, not a device address.
int static_scratch_on(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices)
        return fail(DIMGPU_ERR_UNSUPPORTED, "device ordinal %d is beyond %d", device, kMaxDevices);
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_spmv_static_scratch);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaGetSymbolAddress(static SpMV scratch)");
        g_static_addr[device] = static_cast<unsigned char*>(p);
    }
    *out = g_static_addr[device];
    return DIMGPU_OK;
}

}  // namespace
}  // namespace dimgpu

extern "C" int dimgpu_csr5_spmv_static_scratch(const dimgpu_csr5* m, const double* x, double* y, void* stream) {
    using namespace dimgpu;
    if (!m || (!x && m->cols) || (!y && m->rows))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    int device = -1;
    DG_CUDA(cudaGetDevice(&device));
    if (device != m->device)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "the matrix lives on device %d, the current device is %d",
                    m->device, device);
    if (m->plan.nwarps > kStaticSlots)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT,
                    "this matrix's SpMV uses %u warp slots; the static scratch holds at most %u "
                    "(use dimgpu_csr5_spmv with a calibrator)",
                    m->plan.nwarps, kStaticSlots);
    unsigned char* base = nullptr;
    DG_CHECK(static_scratch_on(device, &base));
    dimgpu_calibrator cal;
    cal.device = device;
    cal.nslots = kStaticSlots;
    cal.cal_val = reinterpret_cast<double*>(base);
    cal.dot_part = reinterpret_cast<double*>(base + kStaticValBytes);
    cal.cal_row = reinterpret_cast<uint32_t*>(base + kStaticValBytes + kStaticDotBytes);
    cal.counter = reinterpret_cast<uint32_t*>(base + kStaticValBytes + kStaticDotBytes + kStaticRowBytes);
    cal.status = cal.counter + 1;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The array keeps whatever the previous call left; the completion ticket and the status word must
    // start at zero.  (The slots themselves are written by every warp before they are read.)
    DG_CUDA(cudaMemsetAsync(cal.counter, 0, 2 * sizeof(uint32_t), s));
    return launch_spmv_f64(m, x, y, &cal, spmv_epilogue{}, s);
}
