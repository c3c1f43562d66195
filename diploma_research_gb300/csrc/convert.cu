// convert.cu -- CSR -> CSR5 conversion on the device.
//
// Restates csr5_info_t::from_csr + csr5::transpose (include/dim/mat/storage_formats/csr5.h:323-446,
// 463-493, 791-803) as data-parallel kernels, for any (sigma <= 32, omega in {4, 8, 16, 32}):
//
//   k_tile_ptr      tile_ptr[t] = upper_bound(row_ptr, min(t*sigma*omega, nnz)) - 1   (csr5.h:411-421)
//   k_empty_flags   empty[r] = row_ptr[r] == row_ptr[r+1]; scanned into E[] (empty rows below r)
//   k_mark_dirty    MSB of tile_ptr[t] when rows [start, stop) hold an empty row     (csr5.h:423-430)
//   k_desc          bit_flag of each tile column from the row starts inside it (csr5.h:323-340),
//                   y_offset = exclusive scan of popcount(bit_flag | first) and
//                   scansum_offset = ctz(present >> (c+1)) with a sentinel bit omega (csr5.h:74-97),
//                   segment count + 1 for dirty multi-row tiles (csr5.h:342-361)
//   k_tdo           tile_desc_offset[ptr + y] = row of each segment, relative to the tile's first
//                   row (csr5.h:363-397)
//   k_permute       re-orders full tiles (csr5.h:463-493) into the chosen layout
//
// All integer work: the results are bit-identical to the reference's arrays at (16, 4) and to the
// same construction at omega = 32.  The reference's benign race on tile_desc_offset_ptr.back()
// (csr5.h:358) does not exist here: the counts go through an exclusive scan.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "internal.hpp"
#include "layout.cuh"

namespace dimgpu {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const unsigned lane = threadIdx.x & 31u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t o = __shfl_up_sync(kFull, v, d);
        if (lane >= (unsigned)d)
            v += o;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive prefix, *total = sum.
__device__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t inc = warp_incl_scan(v);
    if (lane == 31)
        warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
        uint32_t si = warp_incl_scan(s);
        if (lane < kScanThreads / 32)
            warp_sums[lane] = si - s;
        if (lane == 31)
            *total = si;
    }
    __syncthreads();
    uint32_t r = warp_sums[warp] + inc - v;
    __syncthreads();
    return r;
}

__global__ void k_scan_reduce(const uint32_t* in, uint64_t n, uint32_t* partial) {
    __shared__ uint32_t total;
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        uint64_t idx = base + (uint64_t)threadIdx.x * kScanItems + i;
        if (idx < n)
            s += in[idx];
    }
    (void)block_excl_scan(s, &total);
    if (threadIdx.x == 0)
        partial[blockIdx.x] = total;
}

// One block: exclusive scan of the per-block partials, in place.
__global__ void k_scan_partials(uint32_t* partial, uint64_t nblocks) {
    __shared__ uint32_t total;
    uint32_t carry = 0;
    for (uint64_t base = 0; base < nblocks; base += kScanThreads) {
        uint64_t idx = base + threadIdx.x;
        uint32_t v = idx < nblocks ? partial[idx] : 0;
        uint32_t ex = block_excl_scan(v, &total);
        if (idx < nblocks)
            partial[idx] = carry + ex;
        carry += total;
        __syncthreads();
    }
}

__global__ void k_scan_apply(const uint32_t* in, uint32_t* out, uint64_t n, const uint32_t* partial) {
    __shared__ uint32_t total;
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = (base + i < n) ? in[base + i] : 0;
        s += v[i];
    }
    uint32_t run = block_excl_scan(s, &total) + partial[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n)
            out[base + i] = run;
        run += v[i];
    }
}

// out[i] = sum_{j<i} in[j] (in and out may alias); tmp holds ceil(n / kScanTile) words.
int exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* tmp, cudaStream_t s) {
    if (n == 0)
        return DIMGPU_OK;
    const uint64_t nb = (n + kScanTile - 1) / kScanTile;
    k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, tmp);
    k_scan_partials<<<1, kScanThreads, 0, s>>>(tmp, nb);
    k_scan_apply<<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, tmp);
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

// first index in a[0, n) with a[i] > v
__device__ __forceinline__ uint64_t upper_bound_u32(const uint32_t* a, uint64_t n, uint64_t v) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if ((uint64_t)a[mid] <= v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// first index in a[0, n) with a[i] >= v
__device__ __forceinline__ uint64_t lower_bound_u32(const uint32_t* a, uint64_t n, uint64_t v) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if ((uint64_t)a[mid] < v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__global__ void k_tile_ptr(const uint32_t* row_ptr, uint32_t rows, uint64_t nnz, uint64_t T, uint32_t ts,
                           uint32_t* tile_ptr) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t <= T; t += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t b = t * ts < nnz ? t * ts : nnz;
        tile_ptr[t] = (uint32_t)(upper_bound_u32(row_ptr, (uint64_t)rows + 1, b) - 1);
    }
}

__global__ void k_empty_flags(const uint32_t* row_ptr, uint32_t rows, uint32_t* flags) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r <= rows;
         r += (uint64_t)gridDim.x * blockDim.x)
        flags[r] = (r < rows && row_ptr[r] == row_ptr[r + 1]) ? 1u : 0u;
}

__global__ void k_mark_dirty(const uint32_t* E, uint64_t T, uint32_t* tile_ptr) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < T; t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t start = tile_ptr[t] & ~kDirty, stop = tile_ptr[t + 1] & ~kDirty;
        if (start != stop && E[stop] != E[start])
            atomicOr(&tile_ptr[t], kDirty);
    }
}

template <typename Word>
__global__ void k_desc(const uint32_t* row_ptr, uint32_t rows, const uint32_t* tile_ptr, uint64_t T, uint32_t sigma,
                       uint32_t omega, desc_fields f, Word* desc, uint32_t* tdo_cnt) {
    const uint32_t ts = sigma * omega;
    const uint64_t gthreads = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t total_threads = ((T * omega + 31) / 32) * 32;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned group_base = lane & ~(omega - 1);
    const uint64_t group_mask = (omega == 32) ? 0xffffffffull : ((1ull << omega) - 1);
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < total_threads; g += gthreads) {
        const uint64_t t = g / omega;
        const uint32_t c = (uint32_t)(g % omega);
        const bool live = t < T;
        uint64_t flag = 0;
        uint32_t start = 0, stop = 0;
        if (live) {
            start = tile_ptr[t] & ~kDirty;
            stop = tile_ptr[t + 1] & ~kDirty;
            // row starts inside [base, base + sigma): one search per distinct row_ptr value
            const uint64_t base = t * ts + (uint64_t)c * sigma;
            uint64_t r = lower_bound_u32(row_ptr, (uint64_t)rows + 1, base);
            while (r <= rows) {
                uint64_t v = row_ptr[r];
                if (v >= base + sigma)
                    break;
                flag |= 1ull << (v - base);
                r = upper_bound_u32(row_ptr, (uint64_t)rows + 1, v);
            }
        }
        const uint64_t fl = flag | (c == 0 ? 1ull : 0ull);
        const uint32_t segn = live ? (uint32_t)__popcll(fl) : 0u;
        const unsigned ballot = __ballot_sync(kFull, segn != 0);
        const uint64_t present = ((uint64_t)(ballot >> group_base) & group_mask) | (1ull << omega);
        uint32_t inc = segn;
        for (unsigned d = 1; d < omega; d <<= 1) {
            uint32_t o = __shfl_up_sync(kFull, inc, d, omega);
            if (c >= d)
                inc += o;
        }
        const uint32_t total = __shfl_sync(kFull, inc, group_base + omega - 1);
        if (live) {
            const uint64_t y = inc - segn;
            const uint64_t s = ((present >> c) & 1) ? (uint64_t)__ffsll((long long)(present >> (c + 1))) - 1 : 0;
            desc[t * omega + c] = (Word)(y | (s << f.yb) | (flag << (f.yb + f.sb)));
            if (c == 0)
                tdo_cnt[t] = (start != stop && (tile_ptr[t] & kDirty)) ? total + 1 : 0u;
        }
    }
}

template <typename Word>
__global__ void k_tdo(const uint32_t* row_ptr, const uint32_t* tile_ptr, uint64_t T, uint32_t sigma, uint32_t omega,
                      desc_fields f, const Word* desc, const uint32_t* tdo_ptr, uint32_t* tdo) {
    const uint32_t ts = sigma * omega;
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < T * omega;
         g += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t t = g / omega;
        const uint32_t c = (uint32_t)(g % omega);
        const uint32_t raw = tile_ptr[t];
        if (!(raw & kDirty))
            continue;
        const uint32_t start = raw & ~kDirty, stop = tile_ptr[t + 1] & ~kDirty;
        const uint64_t w = desc[t * omega + c];
        uint64_t fl = (w >> (f.yb + f.sb)) & ((sigma == 64) ? ~0ull : ((1ull << sigma) - 1));
        if (c == 0)
            fl |= 1;
        uint64_t y = w & ((1ull << f.yb) - 1);
        const uint64_t base = t * ts + (uint64_t)c * sigma;
        const uint32_t* sub = row_ptr + start;
        const uint64_t nsub = (uint64_t)stop - start + 1;
        const uint32_t optr = tdo_ptr[t];
        while (fl) {
            const int r = __ffsll((long long)fl) - 1;
            fl &= fl - 1;
            tdo[optr + y] = (uint32_t)(upper_bound_u32(sub, nsub, base + r) - 1);
            ++y;
        }
    }
}

template <typename T_, int kind>  // kind: 0 reference order, 1 device f64 pairs, 2 device quads
__global__ void k_permute(const T_* in, T_* out, const uint32_t* tile_ptr, uint64_t T, uint64_t nnz, uint32_t sigma,
                          uint32_t omega) {
    const uint32_t ts = sigma * omega;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nnz; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t t = e / ts;
        uint64_t dst = e;
        // the reference order leaves single-row tiles alone (csr5.h:466-468); the device orders
        // re-order every full tile so that pair and quad reads always address the same elements
        if (t < T && (kind != 0 || (tile_ptr[t] & ~kDirty) != (tile_ptr[t + 1] & ~kDirty))) {
            const uint32_t k = (uint32_t)(e - t * ts);
            const uint32_t c = k / sigma, r = k % sigma;
            const uint32_t p = kind == 0 ? pos_reference(c, r, omega)
                               : kind == 1 ? pos_device_f64(c, r, omega)
                                           : pos_device_q32(c, r, omega);
            dst = t * ts + p;
        }
        out[dst] = in[e];
    }
}

__global__ void k_conv_scalars(const uint32_t* tile_ptr, uint64_t T, const uint32_t* tdo_ptr, const uint32_t* E,
                               uint32_t* out) {
    const uint32_t tail = tile_ptr[T] & ~kDirty;
    out[0] = tail;
    out[1] = tdo_ptr[T];
    out[2] = E[tail];
}

__global__ void k_empty_list(const uint32_t* flags, const uint32_t* E, uint32_t tail, uint32_t* list) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < tail; r += (uint64_t)gridDim.x * blockDim.x)
        if (flags[r])
            list[E[r]] = (uint32_t)r;
}

__global__ void k_to_f32(const double* in, float* out, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

// f32 copy of device-layout values: within every full tile the f64 pair order becomes quad order.
__global__ void k_vals32_device(const double* vals, float* out, const uint32_t* tile_ptr, uint64_t T, uint64_t nnz,
                                uint32_t sigma, uint32_t omega) {
    const uint32_t ts = sigma * omega;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nnz; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t t = e / ts;
        uint64_t src = e;
        if (t < T) {
            // e is the quad position of element (c, r); read that element from its pair position
            const uint32_t k = (uint32_t)(e - t * ts);
            const uint32_t q = k / (4 * omega), rem = k % (4 * omega);
            const uint32_t c = rem / 4, r = q * 4 + rem % 4;
            src = t * ts + pos_device_f64(c, r, omega);
        }
        out[e] = (float)vals[src];
    }
}

// Per full tile (one warp each): the smallest column of the tile into base[t]; sets *wide when the tile's
// columns span 2^16 or more.
__global__ void k_col_base(const uint32_t* col, uint64_t T, uint32_t ts, uint32_t* base, uint32_t* wide) {
    const unsigned lane = threadIdx.x & 31u;
    for (uint64_t t = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; t < T;
         t += (uint64_t)gridDim.x * blockDim.x / 32) {
        uint32_t lo = 0xFFFFFFFFu, hi = 0u;
        for (uint32_t k = lane; k < ts; k += 32) {
            const uint32_t c = col[t * ts + k];
            lo = min(lo, c);
            hi = max(hi, c);
        }
        for (int o = 16; o > 0; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) {
            base[t] = lo;
            if (hi - lo > 0xFFFFu)
                atomicOr(wide, 1u);
        }
    }
}

// col16[e] = col[e] - base[tile of e] for the full tiles.
__global__ void k_col16(const uint32_t* col, const uint32_t* base, uint64_t n, uint32_t ts, uint16_t* col16) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x)
        col16[e] = (uint16_t)(col[e] - base[e / ts]);
}

inline unsigned grid_for(uint64_t n, int threads = 256) {
    uint64_t b = (n + threads - 1) / threads;
    if (b == 0)
        b = 1;
    return (unsigned)std::min<uint64_t>(b, 1u << 20);
}

}  // namespace

int convert_csr5(dimgpu_csr5* m, const uint32_t* d_row_ptr, const uint32_t* d_col, const double* d_vals,
                 cudaStream_t s) {
    const uint32_t sigma = m->sigma, omega = m->omega, rows = m->rows;
    const uint32_t ts = sigma * omega;
    const uint64_t nnz = m->nnz;
    const uint64_t T = nnz / ts;  // csr5.h:438-439
    const desc_fields f = fields_for(sigma, omega);
    m->tile_count = T;
    m->desc_word_bytes = f.total() <= 32 ? 4 : 8;

    if (!m->row_ptr)
        DG_CHECK(dev_alloc_n(&m->row_ptr, (uint64_t)rows + 1));
    DG_CHECK(dev_alloc_n(&m->tile_ptr, T + 1));
    DG_CHECK(dev_alloc(&m->tile_desc, std::max<uint64_t>(1, T * omega) * m->desc_word_bytes));
    DG_CHECK(dev_alloc_n(&m->tdo_ptr, T + 1));
    DG_CHECK(dev_alloc_n(&m->vals, std::max<uint64_t>(1, nnz)));
    DG_CHECK(dev_alloc_n(&m->col, std::max<uint64_t>(1, nnz)));

    uint32_t *flags = nullptr, *E = nullptr, *tmp = nullptr, *scalars = nullptr;
    const uint64_t scan_n = std::max<uint64_t>((uint64_t)rows + 1, T + 1);
    int rc = DIMGPU_OK;
    do {
        if ((rc = dev_alloc_n(&flags, (uint64_t)rows + 1)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&E, (uint64_t)rows + 1)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&tmp, scan_n / kScanTile + 2)) != DIMGPU_OK) break;
        if ((rc = dev_alloc_n(&scalars, 4)) != DIMGPU_OK) break;

        k_tile_ptr<<<grid_for(T + 1), 256, 0, s>>>(d_row_ptr, rows, nnz, T, ts, m->tile_ptr);
        k_empty_flags<<<grid_for((uint64_t)rows + 1), 256, 0, s>>>(d_row_ptr, rows, flags);
        if ((rc = exclusive_scan_u32(flags, E, (uint64_t)rows + 1, tmp, s)) != DIMGPU_OK) break;
        if (T > 0)
            k_mark_dirty<<<grid_for(T), 256, 0, s>>>(E, T, m->tile_ptr);

        if (cudaMemsetAsync(m->tdo_ptr, 0, sizeof(uint32_t) * (T + 1), s) != cudaSuccess) {
            rc = cuda_fail(cudaGetLastError(), "cudaMemsetAsync");
            break;
        }
        if (T > 0) {
            const uint64_t thr = ((T * omega + 31) / 32) * 32;
            if (m->desc_word_bytes == 4)
                k_desc<uint32_t><<<grid_for(thr), 256, 0, s>>>(d_row_ptr, rows, m->tile_ptr, T, sigma, omega, f,
                                                               (uint32_t*)m->tile_desc, m->tdo_ptr);
            else
                k_desc<uint64_t><<<grid_for(thr), 256, 0, s>>>(d_row_ptr, rows, m->tile_ptr, T, sigma, omega, f,
                                                               (uint64_t*)m->tile_desc, m->tdo_ptr);
        }
        if ((rc = exclusive_scan_u32(m->tdo_ptr, m->tdo_ptr, T + 1, tmp, s)) != DIMGPU_OK) break;
        k_conv_scalars<<<1, 1, 0, s>>>(m->tile_ptr, T, m->tdo_ptr, E, scalars);
        uint32_t host_sc[3] = {0, 0, 0};
        if (cudaMemcpyAsync(host_sc, scalars, sizeof(host_sc), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            rc = cuda_fail(cudaGetLastError(), "conversion scalars");
            break;
        }
        m->tail_start = host_sc[0];
        m->tdo_len = host_sc[1];
        m->n_empty = host_sc[2];

        if ((rc = dev_alloc_n(&m->tdo, std::max<uint64_t>(1, m->tdo_len))) != DIMGPU_OK) break;
        if (m->tdo_len) {
            cudaMemsetAsync(m->tdo, 0, sizeof(uint32_t) * m->tdo_len, s);
            if (m->desc_word_bytes == 4)
                k_tdo<uint32_t><<<grid_for(T * omega), 256, 0, s>>>(d_row_ptr, m->tile_ptr, T, sigma, omega, f,
                                                                   (const uint32_t*)m->tile_desc, m->tdo_ptr, m->tdo);
            else
                k_tdo<uint64_t><<<grid_for(T * omega), 256, 0, s>>>(d_row_ptr, m->tile_ptr, T, sigma, omega, f,
                                                                   (const uint64_t*)m->tile_desc, m->tdo_ptr, m->tdo);
        }
        if ((rc = dev_alloc_n(&m->empty_rows, std::max<uint32_t>(1, m->n_empty))) != DIMGPU_OK) break;
        if (m->n_empty)
            k_empty_list<<<grid_for(m->tail_start), 256, 0, s>>>(flags, E, m->tail_start, m->empty_rows);

        if (nnz) {
            if (m->layout == kLayoutReference) {
                k_permute<double, 0><<<grid_for(nnz), 256, 0, s>>>(d_vals, m->vals, m->tile_ptr, T, nnz, sigma, omega);
                k_permute<uint32_t, 0><<<grid_for(nnz), 256, 0, s>>>(d_col, m->col, m->tile_ptr, T, nnz, sigma, omega);
            } else {
                k_permute<double, 1><<<grid_for(nnz), 256, 0, s>>>(d_vals, m->vals, m->tile_ptr, T, nnz, sigma, omega);
                k_permute<uint32_t, 2><<<grid_for(nnz), 256, 0, s>>>(d_col, m->col, m->tile_ptr, T, nnz, sigma, omega);
            }
        }
        if (m->row_ptr != d_row_ptr &&
            cudaMemcpyAsync(m->row_ptr, d_row_ptr, sizeof(uint32_t) * ((uint64_t)rows + 1), cudaMemcpyDeviceToDevice,
                            s) != cudaSuccess) {
            rc = cuda_fail(cudaGetLastError(), "row_ptr copy");
            break;
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "conversion kernels");
            break;
        }
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "conversion");
            break;
        }
    } while (false);
    dev_free(flags);
    dev_free(E);
    dev_free(tmp);
    dev_free(scalars);
    if (rc == DIMGPU_OK) {
        m->device_bytes = sizeof(uint32_t) * (2 * (T + 1) + m->tdo_len + m->n_empty + (uint64_t)rows + 1) +
                          T * omega * m->desc_word_bytes + nnz * (sizeof(double) + sizeof(uint32_t));
    }
    return rc;
}

// The 16-bit column offsets of the device layout, when every full tile's columns fit (see internal.hpp).
int build_col16(dimgpu_csr5* m, cudaStream_t s) {
    const uint64_t T = m->tile_count, ts = (uint64_t)m->sigma * m->omega;
    if (m->layout != kLayoutDevice || T == 0)
        return DIMGPU_OK;
    uint32_t *base = nullptr, *wide = nullptr;
    DG_CHECK(dev_alloc_n(&base, T));
    int rc = dev_alloc_n(&wide, 1);
    uint32_t w = 1;
    if (rc == DIMGPU_OK && cudaMemsetAsync(wide, 0, sizeof(uint32_t), s) != cudaSuccess)
        rc = cuda_fail(cudaGetLastError(), "memset");
    if (rc == DIMGPU_OK) {
        k_col_base<<<grid_for(T * 32), 256, 0, s>>>(m->col, T, (uint32_t)ts, base, wide);
        if (cudaMemcpyAsync(&w, wide, sizeof(w), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            rc = cuda_fail(cudaGetLastError(), "column span of the tiles");
    }
    dev_free(wide);
    uint16_t* c16 = nullptr;
    if (rc == DIMGPU_OK && w == 0 && (rc = dev_alloc_n(&c16, T * ts)) == DIMGPU_OK) {
        k_col16<<<grid_for(T * ts), 256, 0, s>>>(m->col, base, T * ts, (uint32_t)ts, c16);
        if (cudaStreamSynchronize(s) != cudaSuccess)
            rc = cuda_fail(cudaGetLastError(), "16-bit column offsets");
    }
    if (rc != DIMGPU_OK || w != 0) {
        dev_free(base);
        dev_free(c16);
        return rc;
    }
    m->col16 = c16;
    m->col_base = base;
    m->device_bytes += T * ts * sizeof(uint16_t) + T * sizeof(uint32_t);
    return DIMGPU_OK;
}

int ensure_vals32(const dimgpu_csr5* cm, cudaStream_t s) {
    dimgpu_csr5* m = const_cast<dimgpu_csr5*>(cm);
    if (m->vals32)
        return DIMGPU_OK;
    float* v = nullptr;
    DG_CHECK(dev_alloc_n(&v, std::max<uint64_t>(1, m->nnz)));
    if (m->nnz) {
        if (m->layout == kLayoutDevice)
            k_vals32_device<<<grid_for(m->nnz), 256, 0, s>>>(m->vals, v, m->tile_ptr, m->tile_count, m->nnz, m->sigma,
                                                              m->omega);
        else
            k_to_f32<<<grid_for(m->nnz), 256, 0, s>>>(m->vals, v, m->nnz);
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        dev_free(v);
        return cuda_fail(e, "f32 value copy");
    }
    m->vals32 = v;
    m->device_bytes += m->nnz * sizeof(float);
    return autotune_f32(m, s);
}

}  // namespace dimgpu
