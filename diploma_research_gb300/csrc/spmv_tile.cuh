// spmv_tile.cuh -- one CSR5 tile of the SpMV kernel (spmv.cu).
//
// Reference: the per-tile part of csr5::spmv (include/dim/mat/storage_formats/csr5.h:640-745).
// A warp processes one staged tile: lane c owns tile column c (sigma rows), gathers x, closes a
// segment at every set bit_flag bit, joins the "red" heads of following columns through a segmented
// suffix scan on shuffles, and feeds the tile's head segment and the segment running off its end into
// the warp's in-order carry chain (warp_chain), so rows crossing tile boundaries are summed left to
// right.  Closed rows are staged in the consumed value area of the stage and written out coalesced.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"
#include "layout.cuh"

namespace dimgpu {

template <int SIGMA>
struct word_of {
    using type = uint32_t;
};
template <>
struct word_of<32> {
    using type = uint64_t;
};

// One staged tile: its values, its column indices (u32, or u16 offsets from the tile's smallest column
// when IDX16) and its 32 descriptor words.
template <typename VT, int SIGMA, bool IDX16 = false>
struct tile_geom {
    using Word = typename word_of<SIGMA>::type;
    static constexpr uint32_t TS = SIGMA * 32;
    static constexpr uint32_t VBYTES = TS * sizeof(VT);
    static constexpr uint32_t CBYTES = TS * (IDX16 ? 2 : 4);
    static constexpr uint32_t DBYTES = 32 * sizeof(Word);
    static constexpr uint32_t STAGE = VBYTES + CBYTES + DBYTES;
    static constexpr desc_fields F = fields_for(SIGMA, 32);
    static constexpr uint64_t YMASK = (1ull << F.yb) - 1;
    static constexpr uint64_t FMASK = (SIGMA == 64) ? ~0ull : ((1ull << SIGMA) - 1);
};

// Loads lane `lane`'s column (SIGMA values and column indices) from a shared stage; 16-bit indices are
// offsets from `col_base`.
template <typename VT, int SIGMA, bool IDX16 = false>
__device__ __forceinline__ void load_column(const unsigned char* stage, unsigned lane, uint32_t col_base,
                                            VT (&v)[SIGMA], uint32_t (&ci)[SIGMA]) {
    using G = tile_geom<VT, SIGMA, IDX16>;
    if constexpr (IDX16) {
        const uint2* sc = reinterpret_cast<const uint2*>(stage + G::VBYTES);
#pragma unroll
        for (int j = 0; j < SIGMA / 4; ++j) {
            const uint2 q = sc[j * 32 + lane];  // four u16 in quad order
            ci[4 * j + 0] = col_base + (q.x & 0xFFFFu);
            ci[4 * j + 1] = col_base + (q.x >> 16);
            ci[4 * j + 2] = col_base + (q.y & 0xFFFFu);
            ci[4 * j + 3] = col_base + (q.y >> 16);
        }
    } else {
        const uint4* sc = reinterpret_cast<const uint4*>(stage + G::VBYTES);
#pragma unroll
        for (int j = 0; j < SIGMA / 4; ++j) {
            const uint4 q = sc[j * 32 + lane];
            ci[4 * j + 0] = q.x;
            ci[4 * j + 1] = q.y;
            ci[4 * j + 2] = q.z;
            ci[4 * j + 3] = q.w;
        }
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

// The carry chain of one warp over its run of tiles (values uniform across the lanes).
template <typename VT>
struct warp_chain {
    double dot_acc = 0.0;     // this lane's share of x.y over the rows the warp wrote
    bool open = false;        // a row is open at the end of the tiles seen so far
    bool cal_valid = false;   // the warp's first row began before its first tile
    VT carry = VT(0), cal = VT(0);
    uint32_t carry_row = 0, cal_row = 0;
};

template <typename VT>
struct tile_io {
    const VT* x;
    VT* y;
    const uint32_t* tdo_ptr;
    const uint32_t* tdo;
    uint32_t rows;
};

// How the x gathers load: the read-only path kept in L1 (matrices whose column indices have locality)
// or the read-only path without L1 allocation (no locality).  The values name the kernels' template
// argument.
enum : int { kXReadOnly = 0, kXStream = 2 };

template <int XM, typename VT>
__device__ __forceinline__ VT load_x(const VT* p, uint64_t policy) {
    if constexpr (XM == kXStream)
        return ldg_x_stream(p, policy);
    else
        return ldg_x(p, policy);
}

// Writes a row the chain closed (lane 0) and accumulates its share of x.y.
template <typename VT, bool DOT>
__device__ __forceinline__ void chain_write_row(const tile_io<VT>& io, warp_chain<VT>& ch, unsigned lane,
                                                uint32_t row, VT val) {
    if (lane == 0) {
        io.y[row] = val;
        if constexpr (DOT)
            ch.dot_acc += (double)val * (double)ldg_keep(io.x + row);
    }
}

// Processes tile t staged at `st` (its values, column indices and descriptor words).  raw / raw_next are
// tile_ptr[t] and tile_ptr[t + 1] with their dirty bits.  The stage's value area is reused as the
// staging buffer of the tile's closed rows; the caller must __syncwarp() before refilling the stage.
template <typename VT, int SIGMA, bool DOT, int XM = kXReadOnly, bool IDX16 = false>
__device__ __forceinline__ void process_tile(const tile_io<VT>& io, unsigned char* st, unsigned lane, uint64_t t,
                                             uint32_t raw, uint32_t raw_next, uint64_t pol_keep, warp_chain<VT>& ch,
                                             uint32_t col_base = 0) {
    using G = tile_geom<VT, SIGMA, IDX16>;
    using Word = typename G::Word;
    const uint32_t row_stop = raw_next & ~kDirty;
    const uint32_t row_start = raw & ~kDirty;
    const Word* sd = reinterpret_cast<const Word*>(st + G::VBYTES + G::CBYTES);

    VT v[SIGMA];
    uint32_t ci[SIGMA];
    load_column<VT, SIGMA, IDX16>(st, lane, col_base, v, ci);
    const Word w = sd[lane];
    VT xv[SIGMA];
#pragma unroll
    for (int r = 0; r < SIGMA; ++r)
        xv[r] = load_x<XM>(io.x + ci[r], pol_keep);
    // the fused dot needs x at this tile's rows: fetch them now, off the write-out's path
    VT xrow = VT(0);
    if constexpr (DOT) {
        if (row_start + lane < io.rows)
            xrow = load_x<kXReadOnly>(io.x + row_start + lane, pol_keep);
    }
    const uint32_t flag = (uint32_t)((uint64_t(w) >> (G::F.yb + G::F.sb)) & G::FMASK);
    const bool capped = (__shfl_sync(kFull, flag, 0) & 1u) != 0;
    // Every lane now holds its column: the value area of the stage becomes the staging buffer of this
    // tile's segment sums (slot = segment index, at most sigma*32 of them).
    __syncwarp();
    VT* ystage = reinterpret_cast<VT*>(st);
    const bool dirty = (raw & kDirty) != 0;
    const uint32_t optr = dirty ? __ldg(&io.tdo_ptr[t]) : 0u;
    auto row_of = [&](uint32_t idx) -> uint32_t { return row_start + (dirty ? __ldg(&io.tdo[optr + idx]) : idx); };

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

        // Segments of this column: segment yoff + k is staged at slot[k].  Branch-free: a row start
        // closes the open segment (predicated store) and restarts the sum.
        VT* slot = ystage + yoff;
        VT sum = VT(0), red = VT(0);
        uint32_t k = 0;
        bool seen = false;
        if (!__any_sync(kFull, (flag & (flag - 1u)) != 0u)) {
            // No column holds two row starts (rows longer than sigma): no segment closes inside a column,
            // so the loop keeps only the products and the restart at the row start.  Lane 0's head bit
            // is applied afterwards; every sum is the same chain of fma as in the general loop.
#pragma unroll
            for (int r = 0; r < SIGMA; ++r) {
                const bool bit = ((flag >> r) & 1u) != 0;
                red = bit ? sum : red;
                sum = bit ? VT(0) : sum;
                sum = fma(v[r], xv[r], sum);
            }
            seen = flag != 0u;
            if (lane == 0) {
                if ((flag >> 1) != 0u) {  // segment 0 closes at the column's row start
                    slot[0] = red;
                    k = 1;
                }
                red = VT(0);
                seen = true;
            }
        } else {
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
            if (ch.open)
                chain_write_row<VT, DOT>(io, ch, lane, ch.carry_row, ch.carry);
            ch.open = true;
            ch.carry = H;
            ch.carry_row = row_start;
        } else if (ch.open) {
            ch.carry += H;
        } else {
            ch.cal += H;
            ch.cal_row = row_start;
            ch.cal_valid = true;
        }
    } else {
        if (capped || ch.open) {
            if (capped && ch.open)
                chain_write_row<VT, DOT>(io, ch, lane, ch.carry_row, ch.carry);
            if (!capped && lane == 0)
                ystage[0] = ch.carry + H;  // the row that began before this tile closes here
            head_staged = true;
        } else {
            ch.cal += H;
            ch.cal_row = row_start;
            ch.cal_valid = true;
        }
        ch.open = true;
        ch.carry = Lt;
        ch.carry_row = row_last;
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
            st_keep(io.y + row, val, pol_keep);
            if constexpr (DOT) {
                const bool have = !dirty && j == lo + lane && lane + lo < 32;
                const VT xr = have ? xfirst : load_x<kXReadOnly>(io.x + row, pol_keep);
                ch.dot_acc = fma((double)val, (double)xr, ch.dot_acc);
            }
        }
    }
}

}  // namespace dimgpu
