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
// Calibrator (csr5.h:526-538, 750-754) as a decoupled look-back.  CTAs take consecutive run numbers
// in the order they start (one atomic per CTA), each warp owning run number cta * WPC + warp.  A row
// that crosses runs is finished by the run holding its last element: when a run ends, it publishes
// the fragment a later run needs (its open row's partial sum, or -- when no row starts in the whole
// run -- the run's sum of the row passing through) under a flag word tagged with the launch epoch;
// the finishing run looks back over the flags of earlier runs (bounded waits; earlier runs have always
// started, so no wait depends on residency) and adds the fragments in run order, left to right as the
// reference's serial calibrator pass does.  The last CTA to finish (completion ticket) computes the
// CSR tail (csr5.h:756-782) and, optionally, the fused dot x.y (per-CTA partials, fixed order) and
// alpha = rr / (x.y) for CG.  y is fully overwritten: empty rows below the tail are zeroed from the
// list built at conversion.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "internal.hpp"
#include "layout.cuh"
#include "spmv_tile.cuh"

namespace dimgpu {
namespace {

#ifdef DIMGPU_TEST_HOOKS
// Test builds only (libdimgpu_test.so): the warp run whose look-back flag the next launches withhold, so
// that a later run's bounded look-back wait expires and the status query reports it.
uint32_t g_test_withhold_run = 0xffffffffu;
#endif

template <typename VT>
struct spmv_params {
    const VT* vals;
    const uint32_t* col;
    const uint16_t* col16;     // 16-bit column offsets of the full tiles (kernels with IDX16)
    const uint32_t* col_base;  // [T] their bases
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
    int keep_matrix;     // the matrix stays in L2 between products (no evict-first policy)
    double* frag_val;    // [nwarps] fragment a run publishes for a later run
    uint32_t* frag_row;  // [nwarps] its row
    uint32_t* flag;      // [nwarps] (epoch << 2) | fragment kind, release-stored after the fragment
    double* cta_part;    // [grid] per-CTA partials of the fused dot
    uint32_t* words;     // [0] completion ticket, [2] run counter, [3] launch epoch
    uint32_t* status;
    double* dot_out;
    const double* rr;
    double* alpha_out;
    uint32_t* halt;
#ifdef DIMGPU_TEST_HOOKS
    uint32_t withhold_run;  // test builds only: this run never publishes its flag word (0xffffffff = none)
#endif
};

// Final value of row R, whose last fragment `own` this caller holds: the runs before `run` that hold
// R's earlier fragments are found by looking back (through-fragments, then the run where R started,
// which published its carry); the fragments are then added in run order, as a serial left-to-right
// pass over the runs would.  Runs are numbered in launch order, so every run waited on has started.
template <typename VT>
__device__ VT close_row(const spmv_params<VT>& p, uint32_t run, uint32_t R, VT own, uint32_t epoch) {
    uint32_t i = run;
    while (i > 0) {
        --i;
        const uint32_t kind = wait_run(&p.flag[i], epoch, p.status);
        const uint32_t fr = __ldcg(&p.frag_row[i]);
        if (fr != R || kind == kFragNone) {
            record_status(p.status, kStatusBadIndex);  // no earlier fragment of R: the format is inconsistent
            return own;
        }
        if (kind == kFragCarry)
            break;
    }
    VT acc = (VT)__ldcg(&p.frag_val[i]);
    for (uint32_t k = i + 1; k < run; ++k)
        acc += (VT)__ldcg(&p.frag_val[k]);
    return acc + own;
}

// The sum of v[0..N) for N <= 32 in warp 0: a shuffle tree over 32 lanes (lanes >= N add 0), in a fixed
// order; every lane gets the total.
template <int N>
__device__ __forceinline__ double warps_total(const double* v, unsigned lane) {
    static_assert(N >= 1 && N <= 32, "one value per lane");
    double x = lane < (unsigned)N ? v[lane] : 0.0;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
        x += __shfl_xor_sync(kFull, x, d);
    return x;
}

template <typename VT, int SIGMA, int WPC, int STAGES, bool DOT, int XM, bool IDX16>
__global__ void __launch_bounds__(WPC * 32, 1) k_spmv(const spmv_params<VT> p) {
    using G = tile_geom<VT, SIGMA, IDX16>;
    using Word = typename G::Word;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint32_t s_last, s_cta, s_epoch;
    __shared__ double s_red[WPC];

    if (p.halt && *reinterpret_cast<volatile const uint32_t*>(p.halt))
        return;  // a previous stage of a CG iteration has already stopped the solve

    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    // CTAs take run numbers in the order they start, so a run only ever waits for runs already running
    if (threadIdx.x == 0) {
        s_cta = atomicAdd(&p.words[2], 1u);
        s_epoch = *reinterpret_cast<volatile const uint32_t*>(&p.words[3]) + 1u;
    }
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem) + warp * STAGES;
    unsigned char* ring = smem + 128 * ((WPC * STAGES * 8 + 127) / 128) + (size_t)warp * STAGES * G::STAGE;

    // Empty rows below the tail get 0 (the reference leaves them to a zero-filled y).
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < p.n_empty;
         i += (uint64_t)gridDim.x * blockDim.x)
        p.y[p.empty_rows[i]] = VT(0);
    __syncthreads();
    const uint32_t cta = s_cta;
    const uint32_t epoch = (s_epoch & 0x3fffffffu) ? (s_epoch & 0x3fffffffu) : 1u;  // flags start at epoch 0
    const uint32_t run = cta * WPC + warp;

    const uint64_t t_begin = min(p.T, (uint64_t)run * p.tpw);
    const uint64_t t_end = min(p.T, t_begin + p.tpw);

    warp_chain<VT> ch;
    const tile_io<VT> io{p.x, p.y, p.tdo_ptr, p.tdo, p.rows};
    const uint64_t pol_keep = policy_evict_last();

    if (t_begin < t_end) {
        const Word* gdesc = reinterpret_cast<const Word*>(p.desc);
        const uint64_t pol = p.keep_matrix ? policy_evict_normal() : policy_evict_first();
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
            if constexpr (IDX16)
                bulk_g2s(st + G::VBYTES, p.col16 + t * G::TS, G::CBYTES, &bars[s], pol);
            else
                bulk_g2s(st + G::VBYTES, p.col + t * G::TS, G::CBYTES, &bars[s], pol);
            bulk_g2s(st + G::VBYTES + G::CBYTES, gdesc + t * 32, G::DBYTES, &bars[s], pol);
        };
        if (lane == 0)
            for (int s = 0; s < STAGES && t_begin + s < t_end; ++s)
                issue(s, t_begin + s);

        // tile_ptr (and the column base) run two tiles ahead so that no tile waits on its load
        uint32_t raw_cur = __ldg(&p.tile_ptr[t_begin]);
        uint32_t raw_next = __ldg(&p.tile_ptr[t_begin + 1]);
        uint32_t base_cur = 0, base_next = 0;
        if constexpr (IDX16) {
            base_cur = __ldg(&p.col_base[t_begin]);
            base_next = (t_begin + 1 < t_end) ? __ldg(&p.col_base[t_begin + 1]) : 0u;
        }
        uint64_t i = 0;
        bool failed = false;
        for (uint64_t t = t_begin; t < t_end; ++t, ++i) {
            const int s = (int)(i % STAGES);
            const uint32_t par = (uint32_t)((i / STAGES) & 1);
            const uint32_t raw = raw_cur;
            const uint32_t raw_n = raw_next;
            raw_cur = raw_next;
            raw_next = (t + 2 <= p.T) ? __ldg(&p.tile_ptr[t + 2]) : 0u;
            const uint32_t base = base_cur;
            if constexpr (IDX16) {
                base_cur = base_next;
                base_next = (t + 2 < t_end) ? __ldg(&p.col_base[t + 2]) : 0u;
            }
            if (!mbar_wait_bounded(&bars[s], par, p.status)) {
                failed = true;
                break;
            }
            process_tile<VT, SIGMA, DOT, XM, IDX16>(io, ring + (size_t)s * G::STAGE, lane, t, raw, raw_n, pol_keep, ch,
                                                    base);

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
        }

        // Does the row open at the end of this run go on after it?  Yes unless the next tile begins
        // with a row start (or, after the last tile, unless the CSR tail begins with a fresh row).
        bool cont_after;
        if (t_end < p.T) {
            const uint64_t w0 = (uint64_t)__ldg(&gdesc[t_end * 32]);
            cont_after = ((w0 >> (G::F.yb + G::F.sb)) & 1u) == 0;
        } else {
            cont_after = p.tail_start < p.rows && (uint64_t)p.row_ptr[p.tail_start] != p.T * G::TS;
        }
        const bool through = ch.cal_valid && !ch.open;
        if (lane == 0) {
            // publish the fragment a later run needs (the flag word is written for every run)
            uint32_t kind = kFragNone;
            if (ch.open && cont_after) {
                p.frag_val[run] = (double)ch.carry;
                p.frag_row[run] = ch.carry_row;
                kind = kFragCarry;
            } else if (through && cont_after) {
                p.frag_val[run] = (double)ch.cal;
                p.frag_row[run] = ch.cal_row;
                kind = kFragThrough;
            }
#ifdef DIMGPU_TEST_HOOKS
            if (run != p.withhold_run)
#endif
                st_release_u32(&p.flag[run], (epoch << 2) | kind);
            // rows this run finishes: its open row when it ends here, and the row it began inside
            if (ch.open && !cont_after)
                chain_write_row<VT, DOT>(io, ch, 0, ch.carry_row, ch.carry);
            if (ch.cal_valid && (!through || !cont_after)) {
                const VT v = close_row<VT>(p, run, ch.cal_row, ch.cal, epoch);
                chain_write_row<VT, DOT>(io, ch, 0, ch.cal_row, v);
            }
        }
    }
    // per-CTA partial of the fused dot, in warp order
    if constexpr (DOT) {
        const double d = warp_sum(ch.dot_acc);
        if (lane == 0)
            s_red[warp] = d;
    }

    // ---- completion ticket; the last CTA computes the CSR tail and the epilogue ----
    __syncthreads();
    if (warp == 0) {
        if constexpr (DOT) {
            const double d = warps_total<WPC>(s_red, lane);  // the CTA's warp partials, a fixed shuffle tree
            if (lane == 0)
                p.cta_part[cta] = d;
        }
        if (lane == 0) {
            const uint32_t ticket = ticket_acq_rel(&p.words[0]);
            s_last = (ticket == gridDim.x - 1) ? 1u : 0u;
        }
    }
    __syncthreads();
    if (!s_last)
        return;

    // CSR tail (csr5.h:756-782): one row per thread; a first row that began inside the tiles is closed
    // by looking back over the runs like any other row.
    double fix_dot = 0.0;
    const uint64_t first_tail = p.T * G::TS;
    const uint32_t nruns = p.T ? (uint32_t)((p.T + p.tpw - 1) / p.tpw) : 0u;
    for (uint64_t r = (uint64_t)p.tail_start + threadIdx.x; r < p.rows; r += blockDim.x) {
        const uint64_t s0 = (r == p.tail_start) ? first_tail : (uint64_t)p.row_ptr[r];
        const uint64_t e = p.row_ptr[r + 1];
        VT acc = VT(0);
        for (uint64_t k = s0; k < e; ++k)
            acc = fma(p.vals[k], p.x[p.col[k]], acc);
        if (r == p.tail_start && (uint64_t)p.row_ptr[r] != first_tail && nruns > 0)
            acc = close_row<VT>(p, nruns, (uint32_t)r, acc, epoch);
        p.y[r] = acc;
        if constexpr (DOT)
            fix_dot += (double)acc * (double)p.x[r];
    }
    if constexpr (DOT) {
        double part = fix_dot;
        for (uint32_t c = threadIdx.x; c < gridDim.x; c += blockDim.x)
            part += __ldcg(&p.cta_part[c]);
        // warp sums, then the WPC warp sums in order (fixed order)
        part = warp_sum(part);
        __syncthreads();
        if (lane == 0)
            s_red[warp] = part;
        __syncthreads();
        const double dot = warp == 0 ? warps_total<WPC>(s_red, lane) : 0.0;
        if (threadIdx.x == 0) {
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
    if (threadIdx.x == 0) {
        p.words[0] = 0u;
        p.words[2] = 0u;
        p.words[3] = epoch;
    }
}

template <typename VT, int SIGMA, int WPC, int STAGES, bool IDX16>
constexpr size_t smem_bytes() {
    return 128 * ((WPC * STAGES * 8 + 127) / 128) + (size_t)WPC * STAGES * tile_geom<VT, SIGMA, IDX16>::STAGE;
}

template <typename VT, int SIGMA, int WPC, int STAGES, bool DOT, bool IDX16>
int launch_cfg(const dimgpu_csr5* m, const VT* vals, const VT* x, VT* y, dimgpu_calibrator* cal,
               const spmv_epilogue& ep, cudaStream_t stream) {
    constexpr size_t smem = smem_bytes<VT, SIGMA, WPC, STAGES, IDX16>();
    const spmv_plan& pl = sizeof(VT) == 8 ? m->plan : m->plan32;
    if (pl.warps_per_cta != WPC)
        return fail(DIMGPU_ERR_UNSUPPORTED, "launch plan has %d warps per CTA, kernel %d", pl.warps_per_cta, WPC);
    if (pl.nwarps > cal->nslots)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "calibrator has %u slots, plan needs %u", cal->nslots, pl.nwarps);
    spmv_params<VT> p;
    p.vals = vals;
    p.col = m->col;
    p.col16 = m->col16;
    p.col_base = m->col_base;
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
    p.keep_matrix = m->keep_in_l2;
    p.frag_val = cal->cal_val;
    p.frag_row = cal->cal_row;
    p.flag = cal->flag;
    p.cta_part = cal->dot_part;
    p.words = cal->counter;
    p.status = cal->status;
    p.dot_out = ep.dot_out;
    p.rr = ep.rr;
    p.alpha_out = ep.alpha_out;
    p.halt = ep.halt;
#ifdef DIMGPU_TEST_HOOKS
    p.withhold_run = g_test_withhold_run;
#endif
    if ((sizeof(VT) == 8 ? m->x_mode : m->x_mode32) == kXStream)
        k_spmv<VT, SIGMA, WPC, STAGES, DOT, kXStream, IDX16><<<pl.grid, WPC * 32, smem, stream>>>(p);
    else
        k_spmv<VT, SIGMA, WPC, STAGES, DOT, kXReadOnly, IDX16><<<pl.grid, WPC * 32, smem, stream>>>(p);
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

// Warps per CTA (one CTA per SM).  Fewer warps hold less shared memory, which leaves more of the SM's
// 256 KB to L1: gathers that revisit a small part of x (the hub columns of a power-law matrix) then hit
// L1, and that can outweigh the latency hiding of more warps.  Each matrix gets the faster of the two
// per precision, timed at conversion (f64) and when its f32 values are made (f32).
constexpr int kWPC = 16;      // f64: 16 warps x 2 stages x 6.3 KB per SM (register-limited)
constexpr int kWPCL1 = 12;    // f64, L1-leaning: 12 warps, 151 KB of stages
constexpr int kWPC32 = 24;    // f32: 24 warps x 2 stages x 4.2 KB per SM
constexpr int kWPC32L1 = 20;  // f32, L1-leaning: 20 warps, 168 KB of stages
constexpr int kStages = 2;

// Dynamic shared memory a CTA may use on sm_103a (227 KB), less room for the kernel's static arrays.
constexpr size_t kMaxDynSmem = 232448 - 1024;

template <typename VT, int SIGMA, int WPC, int STAGES, bool DOT>
cudaError_t set_smem_attr() {
    static_assert(smem_bytes<VT, SIGMA, WPC, STAGES, false>() <= kMaxDynSmem, "stages exceed shared memory");
    static_assert(smem_bytes<VT, SIGMA, WPC, STAGES, true>() <= kMaxDynSmem, "stages exceed shared memory");
    cudaError_t e;
    const int bytes = (int)smem_bytes<VT, SIGMA, WPC, STAGES, false>();
    if ((e = cudaFuncSetAttribute(k_spmv<VT, SIGMA, WPC, STAGES, DOT, kXReadOnly, false>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_spmv<VT, SIGMA, WPC, STAGES, DOT, kXStream, false>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) != cudaSuccess)
        return e;
    const int bytes16 = (int)smem_bytes<VT, SIGMA, WPC, STAGES, true>();
    if ((e = cudaFuncSetAttribute(k_spmv<VT, SIGMA, WPC, STAGES, DOT, kXReadOnly, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes16)) != cudaSuccess)
        return e;
    return cudaFuncSetAttribute(k_spmv<VT, SIGMA, WPC, STAGES, DOT, kXStream, true>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, bytes16);
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
    DG_CUDA((set_smem_attr<double, 16, kWPCL1, kStages, false>()));
    DG_CUDA((set_smem_attr<double, 16, kWPCL1, kStages, true>()));
    DG_CUDA((set_smem_attr<float, 16, kWPC32, kStages, false>()));
    DG_CUDA((set_smem_attr<float, 16, kWPC32, kStages, true>()));
    DG_CUDA((set_smem_attr<float, 16, kWPC32L1, kStages, false>()));
    DG_CUDA((set_smem_attr<float, 16, kWPC32L1, kStages, true>()));
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
    // slots for every launch configuration the matrix may use, so that pinning another keeps it valid
    const int sms = device_sm_count(m->device);
    uint32_t most = std::max(m->plan.nwarps, m->plan32.nwarps);
    for (int w : {kWPC, kWPCL1, kWPC32, kWPC32L1})
        most = std::max(most, make_spmv_plan(m->tile_count, sms, w).nwarps);
    c->nslots = std::max<uint32_t>(most, 1);
    DG_CHECK(dev_alloc_n(&c->cal_val, c->nslots));
    DG_CHECK(dev_alloc_n(&c->cal_row, c->nslots));
    DG_CHECK(dev_alloc_n(&c->dot_part, c->nslots + 1));
    DG_CHECK(dev_alloc_n(&c->flag, c->nslots));
    DG_CUDA(cudaMemset(c->flag, 0, sizeof(uint32_t) * c->nslots));
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
    dev_free(c->flag);
    dev_free(c->counter);
    dev_free(c->status);
    c->cal_val = nullptr;
}

// The launch with 16-bit column offsets when the matrix has them, 32-bit indices otherwise.
template <typename VT, int SIGMA, int WPC, int STAGES, bool DOT>
int launch_idx(const dimgpu_csr5* m, const VT* vals, const VT* x, VT* y, dimgpu_calibrator* cal,
               const spmv_epilogue& ep, cudaStream_t stream) {
    if (m->col16)
        return launch_cfg<VT, SIGMA, WPC, STAGES, DOT, true>(m, vals, x, y, cal, ep, stream);
    return launch_cfg<VT, SIGMA, WPC, STAGES, DOT, false>(m, vals, x, y, cal, ep, stream);
}

int launch_spmv_f64(const dimgpu_csr5* m, const double* x, double* y, dimgpu_calibrator* cal,
                    const spmv_epilogue& ep, cudaStream_t stream) {
    if (m->layout != kLayoutDevice || m->omega != 32)
        return fail(DIMGPU_ERR_UNSUPPORTED, "SpMV needs the 32-lane device layout");
    const bool dot = ep.dot_out || ep.alpha_out;
    switch (m->sigma) {
    case 16:
        if (m->plan.warps_per_cta == kWPCL1)
            return dot ? launch_idx<double, 16, kWPCL1, kStages, true>(m, m->vals, x, y, cal, ep, stream)
                       : launch_idx<double, 16, kWPCL1, kStages, false>(m, m->vals, x, y, cal, ep, stream);
        return dot ? launch_idx<double, 16, kWPC, kStages, true>(m, m->vals, x, y, cal, ep, stream)
                   : launch_idx<double, 16, kWPC, kStages, false>(m, m->vals, x, y, cal, ep, stream);
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
        if (m->plan32.warps_per_cta == kWPC32L1)
            return dot ? launch_idx<float, 16, kWPC32L1, kStages, true>(m, m->vals32, x, y, cal, ep, stream)
                       : launch_idx<float, 16, kWPC32L1, kStages, false>(m, m->vals32, x, y, cal, ep, stream);
        return dot ? launch_idx<float, 16, kWPC32, kStages, true>(m, m->vals32, x, y, cal, ep, stream)
                   : launch_idx<float, 16, kWPC32, kStages, false>(m, m->vals32, x, y, cal, ep, stream);
    default:
        return fail(DIMGPU_ERR_UNSUPPORTED, "sigma %u has no SpMV kernel", m->sigma);
    }
}

// Times the SpMV of this matrix (x = 1) in each launch configuration `set(i)` installs, the faster of two
// timed launches after one untimed; returns the index of the fastest, which must beat configuration 0
// (the default) by 3 % to be chosen.
template <typename VT, typename Set>
int time_configs(dimgpu_csr5* m, int nconf, Set set, cudaStream_t stream, int* chosen) {
    *chosen = 0;
    VT *x = nullptr, *y = nullptr;
    DG_CHECK(dev_alloc_n(&x, m->cols));
    int rc = dev_alloc_n(&y, m->rows);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float best[4] = {1e30f, 1e30f, 1e30f, 1e30f};
    if (rc == DIMGPU_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
        rc = cuda_fail(cudaGetLastError(), "cudaEventCreate");
    if (rc == DIMGPU_OK) {
        if constexpr (sizeof(VT) == 8) {
            rc = vec_fill(m->cols, 1.0, x, stream);
        } else {
            std::vector<float> ones(m->cols, 1.0f);
            if (cudaMemcpyAsync(x, ones.data(), sizeof(float) * m->cols, cudaMemcpyHostToDevice, stream) !=
                    cudaSuccess ||
                cudaStreamSynchronize(stream) != cudaSuccess)
                rc = cuda_fail(cudaGetLastError(), "x = 1");
        }
    }
    for (int i = 0; i < nconf && i < 4 && rc == DIMGPU_OK; ++i) {
        set(i);
        for (int rep = 0; rep < 3 && rc == DIMGPU_OK; ++rep) {
            cudaEventRecord(e0, stream);
            if constexpr (sizeof(VT) == 8)
                rc = launch_spmv_f64(m, x, y, m->own_cal, spmv_epilogue{}, stream);
            else
                rc = launch_spmv_f32(m, x, y, m->own_cal, spmv_epilogue{}, stream);
            cudaEventRecord(e1, stream);
            if (rc == DIMGPU_OK && cudaEventSynchronize(e1) == cudaSuccess && rep > 0) {
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                best[i] = std::min(best[i], ms);
            }
        }
    }
    if (rc == DIMGPU_OK)
        rc = check_status(m->own_cal, stream);
    int b = 0;
    for (int i = 1; i < nconf && i < 4; ++i)
        if (best[i] < best[b])
            b = i;
    *chosen = (b != 0 && best[b] < 0.97f * best[0]) ? b : 0;
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    dev_free(x);
    dev_free(y);
    return rc;
}

// Chooses the f64 SpMV's launch for this matrix by timing: warps per CTA (16, or 12 to leave more L1)
// times how the x gathers load (kept in L1, or streamed past it).  Small matrices keep the default.
int autotune_gathers(dimgpu_csr5* m, cudaStream_t stream) {
    m->x_mode = kXReadOnly;
    if (m->tile_count < 4096 || m->rows == 0 || m->cols == 0)
        return DIMGPU_OK;
    const int sms = device_sm_count(m->device);
    const int wpc[2] = {kWPC, kWPCL1};
    const int mode[2] = {kXReadOnly, kXStream};
    auto set = [&](int i) {
        m->plan = make_spmv_plan(m->tile_count, sms, wpc[i / 2]);
        m->x_mode = mode[i % 2];
    };
    int c = 0;
    const int rc = time_configs<double>(m, 4, set, stream, &c);
    set(rc == DIMGPU_OK ? c : 0);
    return rc;
}

// The same for the f32 SpMV (24 or 20 warps per CTA), run once, when the f32 values are made.
int autotune_f32(dimgpu_csr5* m, cudaStream_t stream) {
    m->x_mode32 = m->x_mode;
    if (m->layout != kLayoutDevice || m->sigma != 16 || m->tile_count < 4096 || m->rows == 0 || m->cols == 0)
        return DIMGPU_OK;
    const int sms = device_sm_count(m->device);
    const int wpc[2] = {kWPC32, kWPC32L1};
    const int mode[2] = {kXReadOnly, kXStream};
    auto set = [&](int i) {
        m->plan32 = make_spmv_plan(m->tile_count, sms, wpc[i / 2]);
        m->x_mode32 = mode[i % 2];
    };
    int c = 0;
    const int rc = time_configs<float>(m, 4, set, stream, &c);
    set(rc == DIMGPU_OK ? c : 0);
    return rc;
}

int take_status_word(uint32_t* word, cudaStream_t stream, uint32_t* out) {
    *out = kStatusOk;
    if (!word)
        return DIMGPU_OK;
    DG_CUDA(cudaMemcpyAsync(out, word, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
    DG_CUDA(cudaStreamSynchronize(stream));
    if (*out != kStatusOk)
        DG_CUDA(cudaMemsetAsync(word, 0, sizeof(uint32_t), stream));
    return DIMGPU_OK;
}

int status_error(uint32_t st, const char* where) {
    if (st == kStatusOk)
        return DIMGPU_OK;
    if (st == kStatusWaitTimeout)
        return fail(DIMGPU_ERR_TIMEOUT, "%s: a bounded device wait expired (the results of that launch are invalid)",
                    where);
    if (st == kStatusBreakdown)
        return fail(DIMGPU_ERR_BREAKDOWN, "%s: CG breakdown: s.As <= 0 or not finite", where);
    return fail(DIMGPU_ERR_BAD_INDEX, "%s: a device-side consistency check on the CSR5 arrays failed (status %u)",
                where, st);
}

int check_status(dimgpu_calibrator* cal, cudaStream_t stream) {
    uint32_t st = 0;
    DG_CHECK(take_status_word(cal->status, stream, &st));
    return status_error(st, "SpMV");
}

}  // namespace dimgpu

// ------------------------------------------------------------------------------------------------
// SpMV without any allocation by the caller or the library.
//
// dimgpu_csr5_spmv needs a calibrator (scratch for the per-warp row fragments, the fused-dot
// partials, the completion ticket and the status word), and dimgpu_calibrator_create obtains it
// with cudaMalloc.  Some callers cannot do that: a plugin running inside a host application that
// reserved all device memory up front, a real-time loop where cudaMalloc's implicit device
// synchronisation would break its latency bound, or code that must not grow its memory footprint
// after start-up.  For them the scratch of this entry point is a fixed array compiled into the
// library: every GPU that loads the library holds it until the process exits.
// ------------------------------------------------------------------------------------------------
namespace dimgpu {
namespace {

constexpr uint32_t kStaticSlots = 4096;  // warp slots: enough for 256 SMs x 16 warps
constexpr size_t kStaticValBytes = 8 * kStaticSlots;
constexpr size_t kStaticDotBytes = 8 * (kStaticSlots + 32);
constexpr size_t kStaticRowBytes = 4 * kStaticSlots;
constexpr size_t kStaticFlagBytes = 4 * kStaticSlots;
// ticket, -, run counter, epoch (the kernel's control words), then the status word: own 256-byte block
constexpr size_t kStaticWordBytes = 256;
constexpr size_t kStaticScratchBytes =
    kStaticValBytes + kStaticDotBytes + kStaticRowBytes + kStaticFlagBytes + kStaticWordBytes;
constexpr size_t kStaticWordsOffset = kStaticValBytes + kStaticDotBytes + kStaticRowBytes + kStaticFlagBytes;
constexpr int kStaticStatusWord = 4;  // index of the status word in the control block

// 98,816 bytes of device memory, shared by every call of dimgpu_csr5_spmv_static_scratch on a device.
static __device__ __align__(256) unsigned char g_spmv_static_scratch[kStaticScratchBytes];

// The array's device address is looked up once per device and context and cached.  A context is named by
// its driver-assigned id (cuCtxGetId, unique for the life of the process), so a cached address is never
// used in a context other than the one it was looked up in -- after cudaDeviceReset the primary context
// is a new one, the module is loaded again and the address looked up again.
constexpr int kMaxDevices = 64;
struct static_slot {
    bool valid = false;
    unsigned long long ctx_id = 0;
    unsigned char* addr = nullptr;
};
std::mutex g_static_mu;
static_slot g_static[kMaxDevices];

using pfn_ctx_get_current = CUresult (*)(CUcontext*);
using pfn_ctx_get_id = CUresult (*)(CUcontext, unsigned long long*);

// Id of the calling thread's current context; false when there is none or the driver cannot say.
bool current_context_id(unsigned long long* id) {
    static std::once_flag once;
    static pfn_ctx_get_current get_current = nullptr;
    static pfn_ctx_get_id get_id = nullptr;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void* f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<pfn_ctx_get_current>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<pfn_ctx_get_id>(f);
        (void)cudaGetLastError();
    });
    if (!get_current || !get_id)
        return false;
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx)
        return false;
    return get_id(ctx, id) == CUDA_SUCCESS;
}

// Device address of the static scratch on `device` (which must be current).  Host code cannot use
// the symbol itself: on the host, g_spmv_static_scratch is only a stand-in, not a device address.
int static_scratch_on(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices)
        return fail(DIMGPU_ERR_UNSUPPORTED, "device ordinal %d is beyond %d", device, kMaxDevices);
    unsigned long long id = 0;
    bool have_id = current_context_id(&id);
    std::lock_guard<std::mutex> lock(g_static_mu);
    static_slot& slot = g_static[device];
    if (have_id && slot.valid && slot.ctx_id == id) {
        *out = slot.addr;
        return DIMGPU_OK;
    }
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_spmv_static_scratch);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetSymbolAddress(static SpMV scratch)");
    if (!have_id)
        have_id = current_context_id(&id);  // the lookup made the primary context current
    slot.valid = have_id;
    slot.ctx_id = id;
    slot.addr = static_cast<unsigned char*>(p);
    *out = slot.addr;
    return DIMGPU_OK;
}

// The static scratch of the current device, laid out as a calibrator.
int static_calibrator(const dimgpu_csr5* m, dimgpu_calibrator* cal) {
    int device = -1;
    DG_CUDA(cudaGetDevice(&device));
    if (m && device != m->device)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "the matrix lives on device %d, the current device is %d",
                    m->device, device);
    unsigned char* base = nullptr;
    DG_CHECK(static_scratch_on(device, &base));
    cal->device = device;
    cal->nslots = kStaticSlots;
    cal->cal_val = reinterpret_cast<double*>(base);
    cal->dot_part = reinterpret_cast<double*>(base + kStaticValBytes);
    cal->cal_row = reinterpret_cast<uint32_t*>(base + kStaticValBytes + kStaticDotBytes);
    cal->flag = reinterpret_cast<uint32_t*>(base + kStaticValBytes + kStaticDotBytes + kStaticRowBytes);
    cal->counter = reinterpret_cast<uint32_t*>(base + kStaticWordsOffset);
    cal->status = cal->counter + kStaticStatusWord;
    return DIMGPU_OK;
}

}  // namespace
}  // namespace dimgpu

extern "C" int dimgpu_csr5_get_spmv_launch(const dimgpu_csr5* m, int f32, uint32_t* warps_per_cta, int* gather) {
    using namespace dimgpu;
    if (!m || !warps_per_cta || !gather)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    if (f32)
        DG_CHECK(ensure_vals32(m, nullptr));
    *warps_per_cta = (uint32_t)(f32 ? m->plan32 : m->plan).warps_per_cta;
    *gather = (f32 ? m->x_mode32 : m->x_mode) == kXStream ? DIMGPU_GATHER_STREAM : DIMGPU_GATHER_L1;
    return DIMGPU_OK;
}

extern "C" int dimgpu_csr5_set_spmv_launch(dimgpu_csr5* m, int f32, uint32_t warps_per_cta, int gather) {
    using namespace dimgpu;
    if (!m)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL matrix");
    if (m->layout != kLayoutDevice || m->sigma != 16)
        return fail(DIMGPU_ERR_UNSUPPORTED, "the SpMV launch is chosen only for the 32-lane device layout at sigma 16");
    if (gather != DIMGPU_GATHER_L1 && gather != DIMGPU_GATHER_STREAM)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "gather mode %d", gather);
    const int wa = f32 ? kWPC32 : kWPC;
    const int wb = f32 ? kWPC32L1 : kWPCL1;
    if (warps_per_cta != (uint32_t)wa && warps_per_cta != (uint32_t)wb)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "%u warps per CTA is not an %s SpMV launch (%d or %d)",
                    warps_per_cta, f32 ? "f32" : "f64", wa, wb);
    const spmv_plan pl = make_spmv_plan(m->tile_count, device_sm_count(m->device), (int)warps_per_cta);
    const int mode = gather == DIMGPU_GATHER_STREAM ? kXStream : kXReadOnly;
    if (f32) {
        DG_CHECK(ensure_vals32(m, nullptr));  // makes (and tunes) the f32 values first, then the pin holds
        m->plan32 = pl;
        m->x_mode32 = mode;
    } else {
        m->plan = pl;
        m->x_mode = mode;
    }
    return DIMGPU_OK;
}

extern "C" int dimgpu_csr5_spmv_static_scratch(const dimgpu_csr5* m, const double* x, double* y, void* stream) {
    using namespace dimgpu;
    if (!m || (!x && m->cols) || (!y && m->rows))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    if (m->plan.nwarps > kStaticSlots)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT,
                    "this matrix's SpMV uses %u warp slots; the static scratch holds at most %u "
                    "(use dimgpu_csr5_spmv with a calibrator)",
                    m->plan.nwarps, kStaticSlots);
    dimgpu_calibrator cal;
    DG_CHECK(static_calibrator(m, &cal));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The array keeps whatever the previous call left.  The completion ticket and the run counter
    // (control words 0-2) must start at zero; every launch leaves them so, but a launch that never ran to
    // its end would not.  The launch epoch (word 3) carries over: the flags of earlier calls hold older
    // epochs, and a zero-initialised array starts at epoch 0, which no launch uses.  The status word is
    // left alone: a failure a kernel recorded stays there until dimgpu_static_scratch_status reads it.
    DG_CUDA(cudaMemsetAsync(cal.counter, 0, 3 * sizeof(uint32_t), s));
    return launch_spmv_f64(m, x, y, &cal, spmv_epilogue{}, s);
}

extern "C" int dimgpu_static_scratch_status(void* stream) {
    using namespace dimgpu;
    dimgpu_calibrator cal;
    DG_CHECK(static_calibrator(nullptr, &cal));
    uint32_t st = 0;
    DG_CHECK(take_status_word(cal.status, static_cast<cudaStream_t>(stream), &st));
    return status_error(st, "static-scratch SpMV");
}

extern "C" int dimgpu_csr5_status(const dimgpu_csr5* m, dimgpu_calibrator* cal, void* stream) {
    using namespace dimgpu;
    if (!m && !cal)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL matrix and calibrator");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t st = 0;
    if (cal) {
        DG_CHECK(take_status_word(cal->status, s, &st));
        return status_error(st, "SpMV (caller's calibrator)");
    }
    // the scratch the matrix owns: its calibrator, its SpMM scratch, and those of its cached transpose
    uint32_t first = kStatusOk;
    const char* where = "";
    for (const dimgpu_csr5* h = m; h; h = h->transposed) {
        const char* names[2] = {h == m ? "SpMV (matrix calibrator)" : "transpose SpMV",
                                h == m ? "SpMM" : "transpose SpMM"};
        uint32_t* words[2] = {h->own_cal ? h->own_cal->status : nullptr,
                              h->spmm_sc ? static_cast<spmm_scratch*>(h->spmm_sc)->status : nullptr};
        for (int i = 0; i < 2; ++i) {
            DG_CHECK(take_status_word(words[i], s, &st));
            if (st != kStatusOk && first == kStatusOk) {
                first = st;
                where = names[i];
            }
        }
    }
    return status_error(first, where);
}

#ifdef DIMGPU_TEST_HOOKS
// Test builds only (libdimgpu_test.so, compiled with a short DIMGPU_WAIT_NS): the next SpMV launches
// leave the look-back flag of warp run `run` unwritten, so that a later run's bounded wait expires
// (0xffffffff restores normal launches).
extern "C" DIMGPU_API void dimgpu_test_withhold_run(uint32_t run) { dimgpu::g_test_withhold_run = run; }

// Test builds only: gives the matrix's f64 SpMV plan `grid` CTAs (no launch is made with it; the
// static-scratch entry point must refuse a plan larger than its slots).
extern "C" DIMGPU_API int dimgpu_test_set_spmv_grid(dimgpu_csr5* m, int grid) {
    if (!m || grid < 1)
        return DIMGPU_ERR_INVALID_ARGUMENT;
    m->plan.grid = grid;
    m->plan.nwarps = (uint32_t)grid * (uint32_t)m->plan.warps_per_cta;
    return DIMGPU_OK;
}
#endif
