// spmm.cu -- CSR5 SpMM on GB300: Y = A X for k right-hand sides (X, Y row-major, k <= 32 per pass).
//
// The matrix side is the SpMV's (spmv.cu): the same device layout, tiles streamed into shared memory
// by cp.async.bulk on an mbarrier ring, each warp owning a contiguous run of tiles, rows that cross runs
// finished by a decoupled look-back, the CSR tail by the last CTA.
//
// Lanes.  KP = k rounded up to 8, 16 or 32.  Each lane holds V consecutive right-hand sides (f32: V = 4,
// 2 or 1, chosen by timing among those k and the leading dimensions allow with 16- or 8-byte vector
// accesses; FP64: V = 1), so a lane group has LG = KP / V lanes and a warp G = 32 / LG groups; lane j of a
// group holds right-hand sides [j V, (j+1) V).  Group g walks the tile elements of tile columns
// [g LG, (g+1) LG) -- 16 LG consecutive elements in CSR order -- one element per step: the element's value
// and column index come from shared memory (16-byte loads of a whole tile column), every lane gathers
// X[col, jV .. jV+V) (one coalesced k-wide row per group) and accumulates.  So one warp step does G
// elements x KP right-hand sides of useful work: GB300's FP64 pipe (a warp-wide DFMA costs the same
// whatever the number of active lanes) is kept full when k < 32, and with V > 1 the per-element overhead
// (flags, shared loads, shuffles), which bounds the f32 product (it is issue-bound), is paid once for V
// right-hand sides: a tile takes 16 LG warp steps.  A set bit_flag bit closes the group's running row
// (written as one k-wide Y row); after the tile the groups' head and tail sums are joined with shuffles,
// which finishes the rows that span groups and yields the tile's head and open segments for the in-order
// carry chain: in group order when a warp has one or two groups (the SpMV's left-to-right sums), as a
// log-step prefix over the groups' affine maps when it has four or more (a row spanning groups is then
// summed in a tree order).
//
// The optional epilogue of the block CG computes, per right-hand side, dot_j = sum_i X[i,j] Y[i,j]
// (products and per-tile partial sums in the value type, accumulated in f64 across tiles and CTAs in a
// fixed order) and alpha_j = rr_j / dot_j (columns whose mask is clear are skipped).  With several lane
// groups per warp the rows a tile finishes are read back right after it, while they are still cached,
// the groups taking them in turn: every FP64 instruction then serves NG rows, where a product at each row
// write would issue one for the single group that writes it.  With one group (the whole warp) the product
// is taken at the row write.
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
    uint64_t chunk;      // tiles per chunk
    uint32_t nchunks;
    const uint32_t* empty_rows;
    uint32_t n_empty;
    double* frag_val;    // [nchunks * 32] the k-vector fragment a chunk publishes for a later chunk
    uint32_t* frag_row;  // [nchunks]
    uint32_t* flag;      // [nchunks] (epoch << 2) | fragment kind
    double* cta_part;    // [grid * 32] per-CTA partials of the per-column dots
    uint32_t* words;     // [0] completion ticket, [2] run counter, [3] launch epoch
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
constexpr int kSpmmRounds = 4;  // chunks per warp

template <typename VT>
struct mm_geom {
    static constexpr uint32_t VBYTES = kTS * sizeof(VT);
    static constexpr uint32_t CBYTES = kTS * 4;
    static constexpr uint32_t DBYTES = 32 * 4;
    static constexpr uint32_t STAGE = VBYTES + CBYTES + DBYTES;
    static constexpr desc_fields F = fields_for(kSigma, 32);
    static constexpr uint32_t YMASK = (1u << F.yb) - 1u;
};

// The 16 column indices of tile column c (device layout, layout.cuh) from the stage's index area.
__device__ __forceinline__ void stage_cols(const unsigned char* cols, uint32_t c, uint32_t (&ci)[kSigma]) {
    const uint4* sc = reinterpret_cast<const uint4*>(cols);
#pragma unroll
    for (int q = 0; q < kSigma / 4; ++q) {
        const uint4 w = sc[q * 32 + c];
        ci[4 * q + 0] = w.x;
        ci[4 * q + 1] = w.y;
        ci[4 * q + 2] = w.z;
        ci[4 * q + 3] = w.w;
    }
}

// The 16 values of tile column c from the stage's value area.
template <typename VT>
__device__ __forceinline__ void stage_vals(const unsigned char* st, uint32_t c, VT (&v)[kSigma]) {
    if constexpr (sizeof(VT) == 8) {
        const double2* sv = reinterpret_cast<const double2*>(st);
#pragma unroll
        for (int q = 0; q < kSigma / 2; ++q) {
            const double2 d = sv[q * 32 + c];
            v[2 * q + 0] = d.x;
            v[2 * q + 1] = d.y;
        }
    } else {
        const float4* sv = reinterpret_cast<const float4*>(st);
#pragma unroll
        for (int q = 0; q < kSigma / 4; ++q) {
            const float4 d = sv[q * 32 + c];
            v[4 * q + 0] = d.x;
            v[4 * q + 1] = d.y;
            v[4 * q + 2] = d.z;
            v[4 * q + 3] = d.w;
        }
    }
}

// V consecutive right-hand sides of one lane.
template <typename VT, int V>
struct vv {
    VT a[V];
};

template <typename VT, int V>
__device__ __forceinline__ vv<VT, V> vv_zero() {
    vv<VT, V> r;
#pragma unroll
    for (int i = 0; i < V; ++i)
        r.a[i] = VT(0);
    return r;
}
template <typename VT, int V>
__device__ __forceinline__ void vv_add(vv<VT, V>& d, const vv<VT, V>& b) {
#pragma unroll
    for (int i = 0; i < V; ++i)
        d.a[i] += b.a[i];
}
template <typename VT, int V>
__device__ __forceinline__ vv<VT, V> vv_sum(const vv<VT, V>& x, const vv<VT, V>& y) {
    vv<VT, V> r;
#pragma unroll
    for (int i = 0; i < V; ++i)
        r.a[i] = x.a[i] + y.a[i];
    return r;
}
template <typename VT, int V>
__device__ __forceinline__ vv<VT, V> vv_shfl_up(const vv<VT, V>& x, unsigned d) {
    vv<VT, V> r;
#pragma unroll
    for (int i = 0; i < V; ++i)
        r.a[i] = __shfl_up_sync(kFull, x.a[i], d);
    return r;
}

template <typename VT, int V>
__device__ __forceinline__ vv<VT, V> vv_shfl(const vv<VT, V>& x, int src) {
    vv<VT, V> r;
#pragma unroll
    for (int i = 0; i < V; ++i)
        r.a[i] = __shfl_sync(kFull, x.a[i], src);
    return r;
}

// Read-only gather of V consecutive values (16-byte vector loads where V * sizeof(VT) allows), kept in L1
// and L2 like the SpMV's x gathers.
template <typename VT, int V>
__device__ __forceinline__ vv<VT, V> ldg_vec(const VT* p, uint64_t pol) {
    vv<VT, V> r;
    if constexpr (V == 1) {
        r.a[0] = ldg_x(p, pol);
    } else if constexpr (sizeof(VT) == 4 && V == 2) {
        asm("ld.global.nc.L1::evict_last.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
            : "=f"(r.a[0]), "=f"(r.a[1])
            : "l"(p), "l"(pol));
    } else if constexpr (sizeof(VT) == 4 && V == 4) {
        asm("ld.global.nc.L1::evict_last.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
            : "=f"(r.a[0]), "=f"(r.a[1]), "=f"(r.a[2]), "=f"(r.a[3])
            : "l"(p), "l"(pol));
    } else {
#pragma unroll
        for (int h = 0; h < V; h += 2)
            asm("ld.global.nc.L1::evict_last.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
                : "=d"(r.a[h]), "=d"(r.a[h + 1])
                : "l"(p + h), "l"(pol));
    }
    return r;
}

template <typename VT, int V>
__device__ __forceinline__ void st_vec(VT* p, const vv<VT, V>& v) {
    if constexpr (V == 1) {
        p[0] = v.a[0];
    } else if constexpr (sizeof(VT) == 4 && V == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(v.a[0], v.a[1]);
    } else if constexpr (sizeof(VT) == 4 && V == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(v.a[0], v.a[1], v.a[2], v.a[3]);
    } else {
#pragma unroll
        for (int h = 0; h < V; h += 2)
            *reinterpret_cast<double2*>(p + h) = make_double2(v.a[h], v.a[h + 1]);
    }
}

// Coherent load of V consecutive values this kernel wrote (read back past L1).
template <typename VT, int V>
__device__ __forceinline__ vv<VT, V> ldcg_vec(const VT* p) {
    vv<VT, V> r;
    if constexpr (V == 1) {
        r.a[0] = __ldcg(p);
    } else if constexpr (sizeof(VT) == 4 && V == 2) {
        const float2 f = __ldcg(reinterpret_cast<const float2*>(p));
        r.a[0] = f.x;
        r.a[1] = f.y;
    } else if constexpr (sizeof(VT) == 4 && V == 4) {
        const float4 f = __ldcg(reinterpret_cast<const float4*>(p));
        r.a[0] = f.x;
        r.a[1] = f.y;
        r.a[2] = f.z;
        r.a[3] = f.w;
    } else {
#pragma unroll
        for (int h = 0; h < V; ++h)
            r.a[h] = __ldcg(p + h);
    }
    return r;
}

// Y = A X.  KP = k rounded up to 8, 16 or 32; each lane holds V consecutive right-hand sides, so a lane
// group has LG = KP / V lanes and a warp NG = 32 / LG groups; group g walks tile columns [g LG, (g+1) LG).
template <typename VT, int KP, int V, int WPC, int STAGES, bool DOT>
__global__ void __launch_bounds__(WPC * 32, 1) k_spmm(const spmm_params<VT> p) {
    using G = mm_geom<VT>;
    using W = vv<VT, V>;
    constexpr int LG = KP / V;   // lanes per group
    constexpr int NG = 32 / LG;  // lane groups per warp
    // The f32 product with vector lanes is issue-bound: its walk closes rows with selects and a predicated
    // store (one instruction stream for every group).  FP64 (bound by the FP64 pipe) and one value per lane
    // keep the branch, which costs fewer instructions per step there.
    constexpr bool kSelectWalk = sizeof(VT) == 4 && V > 1;
    // rows gathered together (registers: RB x V values of x in flight per lane)
    constexpr int RB = (V * sizeof(VT) <= 8) ? kSigma : kSigma * 8 / (int)(V * sizeof(VT));
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint32_t s_last, s_epoch;
    __shared__ double s_dot[WPC][32];

    if (p.halt && *reinterpret_cast<volatile const uint32_t*>(p.halt))
        return;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned g = lane / LG, j = lane % LG;
    const bool active = j * V < p.k;  // the host sends V > 1 only when k is a multiple of V
    // Lane bases of X and Y: inactive lanes gather from the last active lane's columns (valid addresses,
    // values never stored), so the gathers need no select; row offsets are widening 32 x 32-bit products.
    const uint32_t jj = min(j, (uint32_t)(p.k / V) - 1u);
    const VT* __restrict__ Xl = p.X + jj * V;
    VT* __restrict__ Yl = p.Y + jj * V;
    const uint32_t ldx = (uint32_t)p.ldx, ldy = (uint32_t)p.ldy;
    if (threadIdx.x == 0)
        s_epoch = *reinterpret_cast<volatile const uint32_t*>(&p.words[3]) + 1u;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem) + warp * STAGES;
    unsigned char* ring = smem + 128 * ((WPC * STAGES * 8 + 127) / 128) + (size_t)warp * STAGES * G::STAGE;

    // empty rows below the tail: zero rows of Y
    for (uint64_t i = blockIdx.x * (uint64_t)WPC + warp; i < p.n_empty; i += (uint64_t)gridDim.x * WPC)
        if (lane < p.k)
            p.Y[(uint64_t)p.empty_rows[i] * p.ldy + lane] = VT(0);
    __syncthreads();
    const uint32_t epoch = (s_epoch & 0x3fffffffu) ? (s_epoch & 0x3fffffffu) : 1u;
    // Chunks of p.chunk consecutive tiles are dealt to the warps round-robin (chunk c to warp c mod nw),
    // so at any moment the warps work on one band of neighbouring tiles and the rows of X that several
    // tiles gather are still in L2 for all of them.  The launch is cooperative (every CTA resident), so a
    // chunk may wait for the previous chunk's fragment whichever warp holds it.
    const uint32_t gw = blockIdx.x * WPC + warp, nw = gridDim.x * WPC;
    const uint64_t C = p.chunk;
    const uint64_t pol_keep = policy_evict_last();

    double dot_acc[V];
#pragma unroll
    for (int i = 0; i < V; ++i)
        dot_acc[i] = 0.0;
    // dot epilogue: READBACK -- the rows this warp wrote in the current tile, read back after it; else the
    // tile's products, taken at each row write
    constexpr bool READBACK = NG > 1;
    W tdot = vv_zero<VT, V>();
    const bool no_empty = p.n_empty == 0;
    bool open = false, cal_valid = false;
    W carry = vv_zero<VT, V>(), cal = vv_zero<VT, V>();
    uint32_t carry_row = 0, cal_row = 0;

    // k-wide row write by the lanes of one group (`mine`), with its share of the dot when it is taken at
    // the write
    auto put_row = [&](bool mine, uint32_t row, const W& val) {
        if (mine) {
            if (active) {
                st_vec<VT, V>(Yl + (uint64_t)row * ldy, val);
                if constexpr (DOT && !READBACK) {
                    const W xr = ldg_vec<VT, V>(Xl + (uint64_t)row * ldx, pol_keep);
#pragma unroll
                    for (int q = 0; q < V; ++q)
                        tdot.a[q] = fma(val.a[q], xr.a[q], tdot.a[q]);
                }
            }
        }
    };
    // the same for the (at most two) rows a chunk finishes after its last tile, with their share of the dot
    auto put_row_dot = [&](bool mine, uint32_t row, const W& val) {
        if (mine && active) {
            st_vec<VT, V>(Yl + (uint64_t)row * ldy, val);
            if constexpr (DOT) {
                const W xr = ldg_vec<VT, V>(Xl + (uint64_t)row * ldx, pol_keep);
#pragma unroll
                for (int q = 0; q < V; ++q)
                    dot_acc[q] += (double)(val.a[q] * xr.a[q]);
            }
        }
    };
    // x.y over the rows [lo, hi] one tile finished, four rows per group in flight, summed in the value type
    // and folded into dot_acc.  Every non-empty row of the range was written by this warp in this tile.
    auto dot_rows = [&](uint32_t lo, uint32_t hi) {
        W ts = vv_zero<VT, V>();
#pragma unroll 1
        for (uint32_t r0 = lo; r0 <= hi; r0 += 4 * NG) {
            W yv[4], xr[4];
            bool on[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t r = r0 + (uint32_t)u * NG + g;
                // empty rows were zeroed by whichever CTA reached them; they add nothing
                on[u] = active && r <= hi && (no_empty || __ldg(&p.row_ptr[r]) != __ldg(&p.row_ptr[r + 1]));
                const uint32_t rr = r <= hi ? r : hi;
                yv[u] = ldcg_vec<VT, V>(Yl + (uint64_t)rr * ldy);
                xr[u] = ldg_vec<VT, V>(Xl + (uint64_t)rr * ldx, pol_keep);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int q = 0; q < V; ++q)
                    ts.a[q] = fma(on[u] ? yv[u].a[q] : VT(0), xr[u].a[q], ts.a[q]);
        }
#pragma unroll
        for (int q = 0; q < V; ++q)
            dot_acc[q] += (double)ts.a[q];
    };

    {
        const uint64_t pol = policy_evict_first();
        if (lane == 0) {
            for (int s = 0; s < STAGES; ++s)
                mbar_init(&bars[s], 1);
            fence_mbar_init();
        }
        __syncwarp();
        // this warp's j-th tile: chunk gw + (j / C) nw, tile j mod C of it (or T: no such tile)
        auto seq_tile = [&](uint64_t jt) -> uint64_t {
            const uint64_t c = gw + (jt / C) * (uint64_t)nw;
            if (c >= p.nchunks)
                return p.T;
            const uint64_t t = c * C + jt % C;
            return t < p.T ? t : p.T;
        };
        auto issue = [&](uint64_t q, uint64_t t) {  // ring position q <- tile t (lane 0)
            const int s = (int)(q % STAGES);
            unsigned char* st = ring + (size_t)s * G::STAGE;
            mbar_arrive_expect_tx(&bars[s], G::STAGE);
            bulk_g2s(st, p.vals + t * kTS, G::VBYTES, &bars[s], pol);
            bulk_g2s(st + G::VBYTES, p.col + t * kTS, G::CBYTES, &bars[s], pol);
            bulk_g2s(st + G::VBYTES + G::CBYTES, p.desc + t * 32, G::DBYTES, &bars[s], pol);
        };
        uint64_t qi = 0;  // ring positions issued (uniform across the lanes; lane 0 issues)
        for (int j0 = 0; j0 < STAGES; ++j0) {
            const uint64_t t = seq_tile(j0);
            if (t >= p.T)
                break;
            if (lane == 0)
                issue(j0, t);
            ++qi;
        }
        uint64_t q = 0;  // ring position of the tile being consumed
        bool failed = false;
        for (uint64_t c = gw; c < p.nchunks && !failed; c += nw) {
            const uint64_t cb = c * C, ce = min(p.T, cb + C);
            open = false;
            cal_valid = false;
            carry = vv_zero<VT, V>();
            cal = vv_zero<VT, V>();
            uint32_t raw_cur = __ldg(&p.tile_ptr[cb]);
            uint32_t raw_next = __ldg(&p.tile_ptr[cb + 1]);
            for (uint64_t t = cb; t < ce; ++t, ++q) {
                const int s = (int)(q % STAGES);
                const uint32_t par = (uint32_t)((q / STAGES) & 1);
                const uint32_t raw = raw_cur;
                const uint32_t row_start = raw & ~kDirty;
                raw_cur = raw_next;
                raw_next = (t + 2 <= p.T) ? __ldg(&p.tile_ptr[t + 2]) : 0u;
                if (!mbar_wait_bounded(&bars[s], par, p.status)) {
                    failed = true;
                    break;
                }
                const unsigned char* st = ring + (size_t)s * G::STAGE;
                const uint32_t* sd = reinterpret_cast<const uint32_t*>(st + G::VBYTES + G::CBYTES);
                const bool dirty = (raw & kDirty) != 0;
                const uint32_t optr = dirty ? __ldg(&p.tdo_ptr[t]) : 0u;
                auto row_of = [&](uint32_t idx) -> uint32_t {
                    return row_start + (dirty ? __ldg(&p.tdo[optr + idx]) : idx);
                };
                const bool capped = ((sd[0] >> (G::F.yb + G::F.sb)) & 1u) != 0;

                // ---- this group's elements: tile columns [c0, c0 + LG) ----
                const uint32_t c0 = g * LG;
                // segments are numbered by the row starts after tile element 0 (y_offset counts element 0 once)
                uint32_t seg = (c0 == 0) ? 0u : ((sd[c0] & G::YMASK) - 1u);
                const uint32_t seg0 = seg;  // the segment open when the group begins
                W acc = vv_zero<VT, V>(), head = vv_zero<VT, V>();
                bool hs = false;
                // gathers of rows [r0, r0 + RB) of tile column c (X[col, jV .. jV+V) per element)
                auto gather = [&](uint32_t c, int r0, W (&x)[RB]) {
                    uint32_t ci[kSigma];
                    stage_cols(st + G::VBYTES, c, ci);
    #pragma unroll
                    for (int r = 0; r < RB; ++r)
                        x[r] = ldg_vec<VT, V>(Xl + (uint64_t)ci[r0 + r] * ldx, pol_keep);
                };
                // rows [r0, r0 + RB) of tile column c, in CSR order, with their gathered x
                auto walk = [&](uint32_t c, int r0, const W (&x)[RB]) {
                    uint32_t fl = (sd[c] >> (G::F.yb + G::F.sb)) & 0xFFFFu;
                    if (c == 0)
                        fl &= ~1u;  // element 0 opens segment 0 without closing anything
                    VT v[kSigma];
                    stage_vals<VT>(st, c, v);
    #pragma unroll
                    for (int r = 0; r < RB; ++r) {
                        // a row start: the running row closes (written when it began in this group's range,
                        // else kept as the group's head)
                        const bool bit = ((fl >> (r0 + r)) & 1u) != 0;
                        if constexpr (kSelectWalk) {
                            put_row(bit && hs, row_of(seg), acc);
    #pragma unroll
                            for (int q = 0; q < V; ++q) {
                                head.a[q] = (bit && !hs) ? acc.a[q] : head.a[q];
                                acc.a[q] = fma(v[r0 + r], x[r].a[q], bit ? VT(0) : acc.a[q]);
                            }
                            seg += bit ? 1u : 0u;
                            hs = hs || bit;
                        } else {
                            if (bit) {
                                if (hs)
                                    put_row(true, row_of(seg), acc);  // a row that began in this group's range
                                else
                                    head = acc;
                                hs = true;
                                ++seg;
                                acc = vv_zero<VT, V>();
                            }
    #pragma unroll
                            for (int q = 0; q < V; ++q)
                                acc.a[q] = fma(v[r0 + r], x[r].a[q], acc.a[q]);
                        }
                    }
                };
                if constexpr (sizeof(VT) == 4 && V == 1) {
                    // f32, one value per lane: the next column's gathers are in flight while this one accumulates
                    W xa[RB], xb[RB];
                    gather(c0, 0, xa);
    #pragma unroll 1
                    for (uint32_t cc = 0; cc < (uint32_t)LG; cc += 2) {
                        gather(c0 + cc + 1, 0, xb);
                        walk(c0 + cc, 0, xa);
                        if (cc + 2 < (uint32_t)LG)
                            gather(c0 + cc + 2, 0, xa);
                        walk(c0 + cc + 1, 0, xb);
                    }
                } else {
    #pragma unroll 1
                    for (uint32_t cc = 0; cc < (uint32_t)LG; ++cc) {
    #pragma unroll
                        for (int r0 = 0; r0 < kSigma; r0 += RB) {
                            W xv[RB];
                            gather(c0 + cc, r0, xv);
                            walk(c0 + cc, r0, xv);
                        }
                    }
                }
                if (!hs)
                    head = acc;

                // ---- join the groups: rows spanning groups, the tile's head and open segments ----
                W H, Lt;
                uint32_t open_seg = 0;
                if constexpr (NG >= 4) {
                    // The partial R of the row open when group g begins follows R_{g+1} = f_g(R_g), with
                    // f_g(R) = hs_g ? acc_g : R + head_g (a group with a row start hands on its tail, one
                    // without adds its sum).  The prefixes of the maps f_g o ... o f_0 over the groups take
                    // log2(NG) shuffle steps (Hillis-Steele) instead of NG in turn; every group with a row
                    // start then closes its row, R_g + head_g, at once.
                    bool keep = !hs;             // f_g keeps R
                    W c = hs ? acc : head;       // and adds c
    #pragma unroll
                    for (unsigned d = 1; d < (unsigned)NG; d <<= 1) {
                        const bool keep_p = __shfl_up_sync(kFull, keep ? 1u : 0u, d * LG) != 0u;
                        const W c_p = vv_shfl_up<VT, V>(c, d * LG);
                        if (g >= d) {
                            if (keep)
                                vv_add<VT, V>(c, c_p);
                            keep = keep && keep_p;
                        }
                    }
                    W R = vv_shfl_up<VT, V>(c, LG);  // the prefix of the groups before g, applied to 0
                    if (g == 0)
                        R = vv_zero<VT, V>();
                    const W closed = vv_sum<VT, V>(R, head);
                    const uint32_t starts = __ballot_sync(kFull, hs);  // LG bits per group with a row start
                    Lt = vv_shfl<VT, V>(c, (NG - 1) * LG + (int)j);
                    if (starts) {
                        const int first = (int)((__ffs(starts) - 1) / LG), last = (int)((31 - __clz(starts)) / LG);
                        // the first row start closes the tile's head segment (segment 0, for the carry chain)
                        put_row(hs && g != (unsigned)first, row_of(seg0), closed);
                        H = vv_shfl<VT, V>(closed, first * LG + (int)j);
                        open_seg = __shfl_sync(kFull, seg, last * LG + (int)j);
                    } else {
                        H = Lt;
                    }
                } else {
                    W open_v = vv_zero<VT, V>();
                    H = vv_zero<VT, V>();
                    bool closed0 = false;
    #pragma unroll
                    for (int gg = 0; gg < NG; ++gg) {
                        const int src = gg * LG + (int)j;
                        const uint32_t ghs = __shfl_sync(kFull, hs ? 1u : 0u, src);
                        const W ghd = vv_shfl<VT, V>(head, src);
                        const W gtl = vv_shfl<VT, V>(acc, src);
                        const uint32_t gseg = __shfl_sync(kFull, seg, src);
                        vv_add<VT, V>(open_v, ghd);
                        if (ghs) {
                            if (open_seg == 0) {
                                H = open_v;
                                closed0 = true;
                            } else {
                                put_row(g == (unsigned)gg, row_of(open_seg), open_v);
                            }
                            open_v = gtl;
                            open_seg = gseg;
                        }
                    }
                    if (!closed0)
                        H = open_v;
                    Lt = open_v;
                }
                const uint32_t K = open_seg + 1;
                const uint32_t row_last = (K == 1) ? row_start : row_of(open_seg);

                // ---- in-order carry chain over the warp's tiles (per right-hand side, same in every group) ----
                const bool open_prev = open;
                const uint32_t carry_prev = carry_row;
                if (K == 1) {
                    if (capped) {
                        if (open)
                            put_row(g == 0, carry_row, carry);
                        open = true;
                        carry = H;
                        carry_row = row_start;
                    } else if (open) {
                        vv_add<VT, V>(carry, H);
                    } else {
                        vv_add<VT, V>(cal, H);
                        cal_row = row_start;
                        cal_valid = true;
                    }
                } else {
                    if (capped) {
                        if (open)
                            put_row(g == 0, carry_row, carry);
                        put_row(g == 0, row_start, H);
                    } else if (open) {
                        put_row(g == 0, row_start, vv_sum<VT, V>(carry, H));
                    } else {
                        vv_add<VT, V>(cal, H);
                        cal_row = row_start;
                        cal_valid = true;
                    }
                    open = true;
                    carry = Lt;
                    carry_row = row_last;
                }
                if constexpr (DOT && READBACK) {
                    // The rows this tile wrote, a range known from the tile alone: the previous tile's open
                    // row when this tile closed it (a capped tile, or one with a row start, after an open
                    // row), the head row unless it went to the chunk's look-back, and every row between it
                    // and the row left open at the end (the rows in between are closed here or empty).
                    uint32_t lo = 0xFFFFFFFFu, hi = 0u;
                    if (K > 1) {
                        lo = (capped && open_prev) ? carry_prev : ((capped || open_prev) ? row_start : row_start + 1u);
                        hi = row_last - 1u;
                    } else if (capped && open_prev) {
                        lo = hi = carry_prev;
                    }
                    __syncwarp();  // the rows' stores by the other lanes are visible to the loads below
                    if (lo <= hi)
                        dot_rows(lo, hi);
                } else if constexpr (DOT) {
#pragma unroll
                    for (int q = 0; q < V; ++q) {
                        dot_acc[q] += (double)tdot.a[q];
                        tdot.a[q] = VT(0);
                    }
                }
                __syncwarp();
                // refill this slot with the warp's tile STAGES positions ahead (this chunk or its next one)
                const uint64_t tn = seq_tile(q + STAGES);
                if (tn < p.T) {
                    if (lane == 0) {
                        fence_proxy_async_smem();
                        issue(q + STAGES, tn);
                    }
                    ++qi;
                }
            }
            if (failed) {
                for (uint64_t q2 = q; q2 < qi; ++q2)
                    (void)mbar_wait_bounded(&bars[q2 % STAGES], (uint32_t)((q2 / STAGES) & 1), p.status);
                break;
            }

            // ---- rows that cross chunks: publish this chunk's fragment, finish the rows that end here ----
            bool cont_after;
            if (ce < p.T)
                cont_after = ((__ldg(&p.desc[ce * 32]) >> (G::F.yb + G::F.sb)) & 1u) == 0;
            else
                cont_after = p.tail_start < p.rows && (uint64_t)p.row_ptr[p.tail_start] != p.T * kTS;
            const bool through = cal_valid && !open;
            uint32_t kind = kFragNone;
            if (open && cont_after)
                kind = kFragCarry;
            else if (through && cont_after)
                kind = kFragThrough;
            if (kind != kFragNone && g == 0) {
                const W& fv = kind == kFragCarry ? carry : cal;
    #pragma unroll
                for (int q = 0; q < V; ++q)
                    p.frag_val[(uint64_t)c * 32 + j * V + q] = (double)fv.a[q];
                if (j == 0)
                    p.frag_row[c] = kind == kFragCarry ? carry_row : cal_row;
                __threadfence();
            }
            __syncwarp();
            if (lane == 0)
                st_release_u32(&p.flag[c], (epoch << 2) | kind);
            if (open && !cont_after)
                put_row_dot(g == 0, carry_row, carry);
            if (cal_valid && (!through || !cont_after)) {
                // look back for the chunk where cal_row began, then add the fragments in chunk order
                uint32_t first = (uint32_t)c;
                if (lane == 0) {
                    while (first > 0) {
                        --first;
                        const uint32_t kd = wait_run(&p.flag[first], epoch, p.status);
                        if (__ldcg(&p.frag_row[first]) != cal_row || kd == kFragNone) {
                            record_status(p.status, kStatusBadIndex);
                            first = (uint32_t)c;
                            break;
                        }
                        if (kd == kFragCarry)
                            break;
                    }
                }
                first = __shfl_sync(kFull, first, 0);
                W v = vv_zero<VT, V>();
                if (first < (uint32_t)c && g == 0) {
    #pragma unroll
                    for (int q = 0; q < V; ++q) {
                        VT a = (VT)__ldcg(&p.frag_val[(uint64_t)first * 32 + j * V + q]);
                        for (uint32_t k2 = first + 1; k2 < (uint32_t)c; ++k2)
                            a += (VT)__ldcg(&p.frag_val[(uint64_t)k2 * 32 + j * V + q]);
                        v.a[q] = a;
                    }
                }
                put_row_dot(g == 0, cal_row, vv_sum<VT, V>(v, cal));
            }
        }
    }
    if constexpr (DOT) {
#pragma unroll
        for (int q = 0; q < V; ++q) {
            // sum over the groups (same right-hand sides), then per CTA in warp order
#pragma unroll
            for (int o = LG; o < 32; o <<= 1)
                dot_acc[q] += __shfl_xor_sync(kFull, dot_acc[q], o);
        }
        s_dot[warp][lane] = 0.0;
        __syncwarp();
        if (g == 0) {
#pragma unroll
            for (int q = 0; q < V; ++q)
                s_dot[warp][j * V + q] = dot_acc[q];
        }
    }

    // ---- completion ticket; the last CTA computes the CSR tail and the per-column dots ----
    __syncthreads();
    if constexpr (DOT) {
        if (threadIdx.x < 32) {
            double d = 0.0;
            for (int w = 0; w < WPC; ++w)
                d += s_dot[w][threadIdx.x];
            p.cta_part[(uint64_t)blockIdx.x * 32 + threadIdx.x] = d;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0)
        s_last = (ticket_acq_rel(&p.words[0]) == gridDim.x - 1) ? 1u : 0u;
    __syncthreads();
    if (!s_last)
        return;

    double fix_dot = 0.0;
    const uint64_t first_tail = p.T * kTS;
    const uint32_t nruns = p.nchunks;
    const bool lane_on = lane < p.k;
    for (uint64_t r = (uint64_t)p.tail_start + warp; r < p.rows; r += WPC) {
        const uint64_t s0 = (r == p.tail_start) ? first_tail : (uint64_t)p.row_ptr[r];
        const uint64_t e = p.row_ptr[r + 1];
        VT a = VT(0);
        for (uint64_t kk = s0; kk < e; ++kk)
            if (lane_on)
                a = fma(p.vals[kk], p.X[(uint64_t)p.col[kk] * p.ldx + lane], a);
        if (r == p.tail_start && (uint64_t)p.row_ptr[r] != first_tail && nruns > 0) {
            uint32_t first = nruns;
            if (lane == 0) {
                while (first > 0) {
                    --first;
                    const uint32_t kd = wait_run(&p.flag[first], epoch, p.status);
                    if (__ldcg(&p.frag_row[first]) != (uint32_t)r || kd == kFragNone) {
                        record_status(p.status, kStatusBadIndex);
                        first = nruns;
                        break;
                    }
                    if (kd == kFragCarry)
                        break;
                }
            }
            first = __shfl_sync(kFull, first, 0);
            if (first < nruns && lane_on) {
                VT v = (VT)__ldcg(&p.frag_val[(uint64_t)first * 32 + lane]);
                for (uint32_t k2 = first + 1; k2 < nruns; ++k2)
                    v += (VT)__ldcg(&p.frag_val[(uint64_t)k2 * 32 + lane]);
                a = v + a;
            }
        }
        if (lane_on) {
            p.Y[r * p.ldy + lane] = a;
            if constexpr (DOT)
                fix_dot += (double)a * (double)p.X[r * p.ldx + lane];
        }
    }
    if constexpr (DOT) {
        // the CTAs' partials in WPC interleaved slices (warp w: CTAs w, w + WPC, ...) beside the warp's
        // tail rows, then the slices in warp order: a fixed order whichever CTA is last
        double dw = fix_dot;
        for (uint32_t c = warp; c < gridDim.x; c += WPC)
            dw += __ldcg(&p.cta_part[(uint64_t)c * 32 + lane]);
        __syncthreads();
        s_dot[warp][lane] = dw;
        __syncthreads();
        if (warp == 0) {
            double d = 0.0;
            for (int w = 0; w < WPC; ++w)
                d += s_dot[w][lane];
            if (lane_on) {
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
    }
    if (threadIdx.x == 0) {
        p.words[0] = 0u;
        p.words[2] = 0u;
        p.words[3] = epoch;
    }
}

template <typename VT, int WPC, int STAGES>
constexpr size_t mm_smem() {
    return 128 * ((WPC * STAGES * 8 + 127) / 128) + (size_t)WPC * STAGES * mm_geom<VT>::STAGE;
}

template <typename VT, int KP, int V, int WPC, int STAGES, bool DOT>
cudaError_t mm_attr() {
    return cudaFuncSetAttribute(k_spmm<VT, KP, V, WPC, STAGES, DOT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)mm_smem<VT, WPC, STAGES>());
}

template <typename VT, int KP, int V, int WPC, int STAGES, bool DOT>
int mm_launch(const dimgpu_csr5* m, const VT* vals, const spmm_args& a, const spmm_scratch& sc, cudaStream_t st) {
    const spmv_plan pl = make_spmv_plan(m->tile_count, device_sm_count(m->device), WPC);
    // about kSpmmRounds chunks per warp (as many as the scratch holds), at least STAGES tiles each
    const uint64_t T = m->tile_count;
    const uint64_t target =
        std::max<uint64_t>(1, std::min<uint64_t>(sc.nslots, (uint64_t)kSpmmRounds * pl.nwarps));
    const uint64_t chunk = std::max<uint64_t>(STAGES, (T + target - 1) / target);
    const uint64_t nchunks = T ? (T + chunk - 1) / chunk : 0;
    if (nchunks > sc.nslots)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "SpMM scratch holds %u chunk slots, launch needs %llu", sc.nslots,
                    (unsigned long long)nchunks);
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
    p.chunk = chunk;
    p.nchunks = (uint32_t)nchunks;
    p.empty_rows = m->empty_rows;
    p.n_empty = m->n_empty;
    p.frag_val = sc.cal_val;
    p.frag_row = sc.cal_row;
    p.flag = sc.flag;
    p.cta_part = sc.dot_part;
    p.words = sc.counter;
    p.status = sc.status;
    p.dot_out = a.dot_out;
    p.rr = a.rr;
    p.alpha_out = a.alpha_out;
    p.mask = a.mask;
    p.mask_sel = a.mask_sel;
    p.halt = a.halt;
    // cooperative: every CTA resident (one per SM), so chunks can wait on each other's fragments
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(pl.grid);
    cfg.blockDim = dim3(WPC * 32);
    cfg.dynamicSmemBytes = mm_smem<VT, WPC, STAGES>();
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    DG_CUDA(cudaLaunchKernelEx(&cfg, k_spmm<VT, KP, V, WPC, STAGES, DOT>, p));
    return DIMGPU_OK;
}

template <typename VT, int KP, int V, bool DOT>
int mm_dispatch_kp(const dimgpu_csr5* m, const VT* vals, const spmm_args& a, const spmm_scratch& sc, int shape,
                   cudaStream_t st) {
    switch (shape) {
    case 0:
        return mm_launch<VT, KP, V, 8, 3, DOT>(m, vals, a, sc, st);
    default:
        return mm_launch<VT, KP, V, 16, 2, DOT>(m, vals, a, sc, st);
    }
}

// The most values per lane the operands allow: 4 or 2 (16- or 8-byte vector accesses) when k and both
// leading dimensions are multiples of it and X and Y are aligned to it, at most KP / 2 (a lane group keeps
// two lanes); one value per lane otherwise.
template <typename VT>
int lanes_vec(const spmm_args& a, int kp) {
    for (int v = std::min(4, kp / 2); v > 1; v /= 2) {
        const uintptr_t align = (uintptr_t)v * sizeof(VT);
        if (a.k % v == 0 && a.ldx % v == 0 && a.ldy % v == 0 && reinterpret_cast<uintptr_t>(a.X) % align == 0 &&
            reinterpret_cast<uintptr_t>(a.Y) % align == 0)
            return v;
    }
    return 1;
}

// Lane-group width for k right-hand sides.
inline int kp_for(uint32_t k) { return k <= 8 ? 8 : (k <= 16 ? 16 : 32); }

// Right-hand sides per lane that a shape code's lane grouping g (bits 1-2) selects for these operands: the
// widest the operands allow (f32: 4, 2 or 1) shifted right by g -- g = 0 the widest, 1 half of it, 2 a
// quarter.  -1 when that is below one (the grouping does not apply; it would repeat another).  FP64 keeps
// one value per lane: it is bound by the FP64 pipe, which a warp DFMA occupies the same way whatever its
// layout.
template <typename VT>
int lanes_for_shape(const spmm_args& a, int shape) {
    const int grouping = shape >> 1;
    if (sizeof(VT) == 8)
        return grouping == 0 ? 1 : -1;
    const int v = lanes_vec<VT>(a, kp_for(a.k)) >> grouping;
    return v >= 1 ? v : -1;
}

template <typename VT, bool DOT>
int mm_dispatch(const dimgpu_csr5* m, const VT* vals, const spmm_args& a, const spmm_scratch& sc, int shape,
                cudaStream_t st) {
    const int kp = kp_for(a.k);
    const int launch = shape & 1;
    int v = lanes_for_shape<VT>(a, shape);
    if (v < 0)
        v = lanes_for_shape<VT>(a, launch);  // a grouping these operands cannot use: the default one
    if constexpr (sizeof(VT) == 4) {
        // f32 is issue-bound: with V values per lane a group has KP / V lanes, each warp step serves
        // 32 V / KP elements, and a tile takes KP / V * 16 steps instead of KP * 16
        if (kp == 8 && v == 4)
            return mm_dispatch_kp<VT, 8, 4, DOT>(m, vals, a, sc, launch, st);
        if (kp == 8 && v == 2)
            return mm_dispatch_kp<VT, 8, 2, DOT>(m, vals, a, sc, launch, st);
        if (kp == 16 && v == 4)
            return mm_dispatch_kp<VT, 16, 4, DOT>(m, vals, a, sc, launch, st);
        if (kp == 16 && v == 2)
            return mm_dispatch_kp<VT, 16, 2, DOT>(m, vals, a, sc, launch, st);
        if (kp == 32 && v == 4)
            return mm_dispatch_kp<VT, 32, 4, DOT>(m, vals, a, sc, launch, st);
        if (kp == 32 && v == 2)
            return mm_dispatch_kp<VT, 32, 2, DOT>(m, vals, a, sc, launch, st);
    }
    switch (kp) {
    case 8:
        return mm_dispatch_kp<VT, 8, 1, DOT>(m, vals, a, sc, launch, st);
    case 16:
        return mm_dispatch_kp<VT, 16, 1, DOT>(m, vals, a, sc, launch, st);
    default:
        return mm_dispatch_kp<VT, 32, 1, DOT>(m, vals, a, sc, launch, st);
    }
}

template <typename VT, bool DOT>
cudaError_t mm_attrs() {
    cudaError_t e;
    if ((e = mm_attr<VT, 8, 1, 8, 3, DOT>()) != cudaSuccess) return e;
    if ((e = mm_attr<VT, 8, 1, 16, 2, DOT>()) != cudaSuccess) return e;
    if ((e = mm_attr<VT, 16, 1, 8, 3, DOT>()) != cudaSuccess) return e;
    if ((e = mm_attr<VT, 16, 1, 16, 2, DOT>()) != cudaSuccess) return e;
    if ((e = mm_attr<VT, 32, 1, 8, 3, DOT>()) != cudaSuccess) return e;
    if ((e = mm_attr<VT, 32, 1, 16, 2, DOT>()) != cudaSuccess) return e;
    if constexpr (sizeof(VT) == 4) {
        if ((e = mm_attr<VT, 8, 4, 8, 3, DOT>()) != cudaSuccess) return e;
        if ((e = mm_attr<VT, 8, 4, 16, 2, DOT>()) != cudaSuccess) return e;
        if ((e = mm_attr<VT, 8, 2, 8, 3, DOT>()) != cudaSuccess) return e;
        if ((e = mm_attr<VT, 8, 2, 16, 2, DOT>()) != cudaSuccess) return e;
        if ((e = mm_attr<VT, 16, 4, 8, 3, DOT>()) != cudaSuccess) return e;
        if ((e = mm_attr<VT, 16, 4, 16, 2, DOT>()) != cudaSuccess) return e;
        if ((e = mm_attr<VT, 16, 2, 8, 3, DOT>()) != cudaSuccess) return e;
        if ((e = mm_attr<VT, 16, 2, 16, 2, DOT>()) != cudaSuccess) return e;
        if ((e = mm_attr<VT, 32, 4, 8, 3, DOT>()) != cudaSuccess) return e;
        if ((e = mm_attr<VT, 32, 4, 16, 2, DOT>()) != cudaSuccess) return e;
        if ((e = mm_attr<VT, 32, 2, 8, 3, DOT>()) != cudaSuccess) return e;
        if ((e = mm_attr<VT, 32, 2, 16, 2, DOT>()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace

int prepare_spmm_kernels() {
    static int done = 0;
    if (done)
        return DIMGPU_OK;
    DG_CUDA((mm_attrs<double, false>()));
    DG_CUDA((mm_attrs<double, true>()));
    DG_CUDA((mm_attrs<float, false>()));
    DG_CUDA((mm_attrs<float, true>()));
    done = 1;
    return DIMGPU_OK;
}

uint32_t spmm_max_slots(const dimgpu_csr5* m) {
    const int sms = device_sm_count(m->device);
    uint32_t n = 1;
    for (int wpc : {8, 16})
        n = std::max<uint32_t>(n, make_spmv_plan(m->tile_count, sms, wpc).nwarps);
    return n * kSpmmRounds;
}

int spmm_scratch_init(spmm_scratch* s, const dimgpu_csr5* m) {
    s->nslots = spmm_max_slots(m);
    DG_CHECK(dev_alloc_n(&s->cal_val, (uint64_t)s->nslots * 32));
    DG_CHECK(dev_alloc_n(&s->dot_part, (uint64_t)s->nslots * 32));
    DG_CHECK(dev_alloc_n(&s->cal_row, s->nslots));
    DG_CHECK(dev_alloc_n(&s->flag, s->nslots));
    DG_CUDA(cudaMemset(s->flag, 0, sizeof(uint32_t) * s->nslots));
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
    dev_free(s->flag);
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
    if (a.ldx > 0xffffffffull || a.ldy > 0xffffffffull)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "leading dimensions must be < 2^32");
    const bool dot = a.dot_out || a.alpha_out;
    if (f32) {
        DG_CHECK(ensure_vals32(m, st));
        return dot ? mm_dispatch<float, true>(m, m->vals32, a, sc, shape, st)
                   : mm_dispatch<float, false>(m, m->vals32, a, sc, shape, st);
    }
    return dot ? mm_dispatch<double, true>(m, m->vals, a, sc, shape, st)
               : mm_dispatch<double, false>(m, m->vals, a, sc, shape, st);
}

bool spmm_shape_applies(bool f32, const spmm_args& a, int shape) {
    if (shape < 0 || shape >= kSpmmShapes)
        return false;
    return f32 ? lanes_for_shape<float>(a, shape) > 0 : lanes_for_shape<double>(a, shape) > 0;
}

// Picks the shape of one SpMM -- launch shape (warps per CTA x pipeline stages) and lane grouping
// (right-hand sides per lane) -- by timing each candidate that applies to the caller's operands.
// Deterministic choice: the fastest of two timed launches per candidate.
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
        if (!spmm_shape_applies(f32, plain, shape))
            continue;
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

extern "C" int dimgpu_csr5_set_spmm_shape(dimgpu_csr5* m, uint32_t k, int f32, int shape) {
    if (!m || k == 0 || k > 32)
        return dimgpu::fail(DIMGPU_ERR_INVALID_ARGUMENT, "bad argument");
    if (shape < -1 || shape >= dimgpu::kSpmmShapes)
        return dimgpu::fail(DIMGPU_ERR_INVALID_ARGUMENT, "shape %d is not in [-1, %d)", shape, dimgpu::kSpmmShapes);
    m->spmm_shape[f32 ? 1 : 0][k] = shape;
    return DIMGPU_OK;
}
