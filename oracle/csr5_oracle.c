/*
 * csr5_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C restatement of the reference's CPU algorithms for the CSR5 hot path of
 * rurabori/diploma_research ("dim"):
 *
 *   - CSR -> CSR5 conversion       include/dim/mat/storage_formats/csr5.h:323-446, 463-493, 791-803
 *   - CSR5 SpMV (tiles, calibrator,
 *     tail)                        include/dim/mat/storage_formats/csr5.h:495-583, 608-782, 818-829
 *   - SIMD helper semantics        include/dim/simd.h:34-61, 70-81 and csr5.h:200-235
 *   - single-process CG loop       benchmarks/conjugate_gradient/dim_sp/main.cpp:89-127 with the
 *                                  residual threshold of docs/paper/thesis.tex:2127-2160
 *
 * Only the test-suite, the smoke check and the CPU-baseline leg of the benchmark load this file.
 * The product path never links it.
 *
 * The "oracle rule": the reference SpMV only yields A*x on a zero-filled y with a fresh calibrator
 * (the calibrator is never reset, csr5/calibrator.h:14-31, csr5.h:530; and csr5.h:744-745 passes
 * "first tile of the chunk AND row starts here" as `direct`).  This restatement zero-fills y and uses
 * a fresh calibrator on every call, and uses the row-starts-here flag as `direct` for every tile,
 * which gives the same bits as the reference under the rule.
 *
 * Floating-point order follows the reference's AVX2 code lane by lane: every product/accumulate is
 * an explicit fma(), the 4-lane inclusive scan adds neighbours in the order of simd.h:34-45 and the
 * horizontal sum pairs lanes as in simd.h:53-61.  The file must be compiled with
 * -ffp-contract=off so that no other contraction happens.
 *
 * Generalised to any (sigma, omega) with omega <= 32 and sigma <= 32 so that the same code describes
 * the 32-lane device layout; at (16, 4) it is the reference's csr5<double,16,4,uint32_t>.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MSB32 0x80000000u

static inline uint32_t strip_dirty(uint32_t v) { return v & ~MSB32; }
static inline int is_dirty(uint32_t v) { return (v & MSB32) != 0; }

/* std::bit_width */
static unsigned bit_width(uint64_t v) {
    unsigned w = 0;
    while (v) {
        ++w;
        v >>= 1;
    }
    return w;
}

/* detail::upper_bound_idx (csr5.h:194-198): index of the last element <= val, i.e.
 * upper_bound(range, val) - begin - 1. */
static int64_t upper_bound_idx(const uint32_t* a, uint64_t n, uint64_t val) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo) / 2;
        if ((uint64_t)a[mid] <= val)
            lo = mid + 1;
        else
            hi = mid;
    }
    return (int64_t)lo - 1;
}

/* Descriptor field widths (csr5.h:53-63). */
typedef struct {
    unsigned yb, sb, fb;
} oracle_fields;

static oracle_fields fields_for(unsigned sigma, unsigned omega) {
    oracle_fields f;
    f.yb = bit_width((uint64_t)sigma * omega);
    f.sb = bit_width(omega);
    f.fb = sigma;
    return f;
}

static inline uint64_t pack_word(oracle_fields f, uint64_t y, uint64_t s, uint64_t flag) {
    return y | (s << f.yb) | (flag << (f.yb + f.sb));
}
static inline uint64_t word_y(oracle_fields f, uint64_t w) { return w & ((1ull << f.yb) - 1); }
static inline uint64_t word_s(oracle_fields f, uint64_t w) { return (w >> f.yb) & ((1ull << f.sb) - 1); }
static inline uint64_t word_flag(oracle_fields f, uint64_t w) {
    return (w >> (f.yb + f.sb)) & ((f.fb == 64) ? ~0ull : ((1ull << f.fb) - 1));
}

/* Returns the number of packed descriptor bits per column (26 at sigma=16, omega=4). */
int oracle_desc_bits(unsigned sigma, unsigned omega) {
    oracle_fields f = fields_for(sigma, omega);
    return (int)(f.yb + f.sb + f.fb);
}

/* ----------------------------------------------------------------------------------------------
 * Conversion.  Two calls: oracle_csr5_plan() gives the sizes, oracle_csr5_convert() fills the
 * caller's buffers.  Layout of the outputs is exactly the reference's csr5_info_t:
 *   tile_ptr[T+1]          u32, MSB = "tile has an empty row"        (csr5.h:239-252, 411-431)
 *   tile_desc[T*omega]     packed column words, u64 here             (csr5.h:33-152, 323-361)
 *   tdo_ptr[T+1]           tile_desc_offset_ptr                      (csr5.h:342-366)
 *   tdo[tdo_size]          tile_desc_offset                          (csr5.h:363-397)
 *   vals/col_idx[nnz]      per-tile column-major -> row-major copies (csr5.h:463-493)
 * ---------------------------------------------------------------------------------------------- */

static void gen_tile_ptr(uint64_t T, unsigned ts, uint32_t rows, uint64_t nnz, const uint32_t* row_ptr,
                         uint32_t* tile_ptr) {
    /* csr5.h:411-421 */
    for (uint64_t t = 0; t <= T; ++t) {
        uint64_t boundary = t * ts < nnz ? t * ts : nnz;
        tile_ptr[t] = (uint32_t)upper_bound_idx(row_ptr, (uint64_t)rows + 1, boundary);
    }
    /* csr5.h:423-430: a tile covering rows [start, stop] is dirty when row_ptr has equal neighbours
     * among row_ptr[start..stop] (an empty row among rows start..stop-1). */
    for (uint64_t t = 0; t < T; ++t) {
        uint32_t start = strip_dirty(tile_ptr[t]), stop = strip_dirty(tile_ptr[t + 1]);
        if (start == stop)
            continue;
        for (uint32_t i = start; i < stop; ++i) {
            if (row_ptr[i] == row_ptr[i + 1]) {
                tile_ptr[t] |= MSB32;
                break;
            }
        }
    }
}

/* Fills tile_ptr (T+1 entries) and reports T and the tile_desc_offset length. */
int oracle_csr5_plan(uint32_t rows, uint64_t nnz, const uint32_t* row_ptr, unsigned sigma, unsigned omega,
                     uint64_t* tile_count, uint64_t* tdo_size) {
    if (sigma == 0 || omega == 0 || omega > 32 || sigma > 32)
        return -1;
    if (oracle_desc_bits(sigma, omega) > 64)
        return -1;
    const unsigned ts = sigma * omega;
    const uint64_t T = nnz / ts; /* csr5.h:438-439, floor */
    uint32_t* tile_ptr = (uint32_t*)malloc(sizeof(uint32_t) * (T + 1));
    if (!tile_ptr)
        return -2;
    gen_tile_ptr(T, ts, rows, nnz, row_ptr, tile_ptr);
    uint64_t total = 0;
    for (uint64_t t = 0; t < T; ++t) {
        uint32_t start = strip_dirty(tile_ptr[t]), stop = strip_dirty(tile_ptr[t + 1]);
        if (start == stop || !is_dirty(tile_ptr[t]))
            continue;
        /* number of segments = popcount of all columns' bits (column 0 forced), + 1 spare slot */
        uint64_t flags[32];
        memset(flags, 0, sizeof(flags));
        for (uint32_t rid = start; rid <= stop; ++rid) {
            uint64_t idx = row_ptr[rid];
            if (idx / ts != t)
                continue;
            flags[(idx / sigma) % omega] |= 1ull << (idx % sigma);
        }
        flags[0] |= 1;
        uint64_t segs = 0;
        for (unsigned c = 0; c < omega; ++c)
            segs += (uint64_t)__builtin_popcountll(flags[c]);
        total += segs + 1;
    }
    free(tile_ptr);
    *tile_count = T;
    *tdo_size = total;
    return 0;
}

int oracle_csr5_convert(uint32_t rows, uint64_t nnz, const uint32_t* row_ptr, const uint32_t* col_idx,
                        const double* vals, unsigned sigma, unsigned omega, uint32_t* tile_ptr, uint64_t* tile_desc,
                        uint32_t* tdo_ptr, uint32_t* tdo, double* out_vals, uint32_t* out_col) {
    if (sigma == 0 || omega == 0 || omega > 32 || sigma > 32 || oracle_desc_bits(sigma, omega) > 64)
        return -1;
    const oracle_fields f = fields_for(sigma, omega);
    const unsigned ts = sigma * omega;
    const uint64_t T = nnz / ts;

    gen_tile_ptr(T, ts, rows, nnz, row_ptr, tile_ptr);

    /* set_bit_flag (csr5.h:323-340) */
    memset(tile_desc, 0, sizeof(uint64_t) * T * omega);
    memset(tdo_ptr, 0, sizeof(uint32_t) * (T + 1));
    uint64_t* flags = (uint64_t*)calloc(T * omega + 1, sizeof(uint64_t));
    if (!flags)
        return -2;
    for (uint64_t t = 0; t < T; ++t) {
        uint32_t start = strip_dirty(tile_ptr[t]), stop = strip_dirty(tile_ptr[t + 1]);
        for (uint32_t rid = start; rid <= stop; ++rid) {
            uint64_t idx = row_ptr[rid];
            if (idx / ts != t)
                continue;
            flags[t * omega + (idx / sigma) % omega] |= 1ull << (idx % sigma);
        }
    }

    /* set_scansum_and_y_offsets + offset-pointer sizing (csr5.h:74-97, 342-361) */
    uint64_t any_dirty_total = 0;
    for (uint64_t t = 0; t < T; ++t) {
        uint64_t segn[33];
        uint64_t present = 1ull << omega; /* sentinel bit at omega */
        for (unsigned c = 0; c < omega; ++c) {
            uint64_t fl = flags[t * omega + c] | (c == 0 ? 1ull : 0ull);
            segn[c] = (uint64_t)__builtin_popcountll(fl);
            if (segn[c])
                present |= 1ull << c;
        }
        uint64_t acc = 0;
        for (unsigned c = 0; c < omega; ++c) {
            uint64_t y = acc;
            acc += segn[c];
            uint64_t s = ((present >> c) & 1) ? (uint64_t)__builtin_ctzll(present >> (c + 1)) : 0;
            tile_desc[t * omega + c] = pack_word(f, y, s, flags[t * omega + c]);
        }
        uint32_t start = strip_dirty(tile_ptr[t]), stop = strip_dirty(tile_ptr[t + 1]);
        if (start == stop)
            continue;
        if (is_dirty(tile_ptr[t])) {
            tdo_ptr[t] = (uint32_t)(acc + 1);
            any_dirty_total += acc + 1;
        }
    }

    /* generate_tile_offset (csr5.h:363-397) */
    if (any_dirty_total) {
        uint64_t run = 0;
        for (uint64_t t = 0; t <= T; ++t) {
            uint64_t v = (t < T) ? tdo_ptr[t] : 0;
            tdo_ptr[t] = (uint32_t)run;
            run += v;
        }
        memset(tdo, 0, sizeof(uint32_t) * any_dirty_total);
        for (uint64_t t = 0; t < T; ++t) {
            if (!is_dirty(tile_ptr[t]))
                continue;
            uint32_t start = strip_dirty(tile_ptr[t]), stop = strip_dirty(tile_ptr[t + 1]);
            const uint32_t* sub = row_ptr + start;
            uint64_t nsub = (uint64_t)stop - start + 1;
            uint32_t optr = tdo_ptr[t];
            for (unsigned c = 0; c < omega; ++c) {
                uint64_t w = tile_desc[t * omega + c];
                uint64_t fl = word_flag(f, w) | (c == 0 ? 1ull : 0ull);
                uint64_t y = word_y(f, w);
                uint64_t base = t * ts + (uint64_t)c * sigma;
                for (unsigned r = 0; r < sigma; ++r) {
                    if (!((fl >> r) & 1))
                        continue;
                    tdo[optr + y] = (uint32_t)upper_bound_idx(sub, nsub, base + r);
                    ++y;
                }
            }
        }
    }
    free(flags);

    /* transpose (csr5.h:463-493): full tiles that span more than one row */
    if (out_vals != vals)
        memcpy(out_vals, vals, sizeof(double) * nnz);
    if (out_col != col_idx)
        memcpy(out_col, col_idx, sizeof(uint32_t) * nnz);
    for (uint64_t t = 0; t < T; ++t) {
        uint32_t start = strip_dirty(tile_ptr[t]), stop = strip_dirty(tile_ptr[t + 1]);
        if (start == stop)
            continue;
        uint64_t off = t * ts;
        for (unsigned c = 0; c < omega; ++c)
            for (unsigned r = 0; r < sigma; ++r) {
                out_vals[off + (uint64_t)r * omega + c] = vals[off + (uint64_t)c * sigma + r];
                out_col[off + (uint64_t)r * omega + c] = col_idx[off + (uint64_t)c * sigma + r];
            }
    }
    return 0;
}

/* ----------------------------------------------------------------------------------------------
 * SpMV.  y := A*x on the CSR5 arrays above (the reference's csr5::spmv under the oracle rule).
 * nthreads plays the role of omp_get_max_threads(): it fixes the tile chunking and therefore where
 * calibrator slots are used (csr5.h:608-617).
 * ---------------------------------------------------------------------------------------------- */

typedef struct {
    uint32_t rows;
    uint64_t nnz;
    unsigned sigma, omega;
    uint64_t T;
    const uint32_t* row_ptr;
    const uint32_t* tile_ptr;
    const uint64_t* tile_desc;
    const uint32_t* tdo_ptr;
    const uint32_t* tdo;
    const double* vals;
    const uint32_t* col;
} oracle_view;

/* simd::inclusive_scan (simd.h:34-45), widened: lane i = (((a_i + a_{i-1}) + a_{i-2}) + ...) */
static void lane_inclusive_scan(const double* a, double* out, unsigned w) {
    for (unsigned i = 0; i < w; ++i) {
        double s = a[i];
        for (unsigned j = 1; j < w; ++j)
            s = s + (j <= i ? a[i - j] : 0.0);
        out[i] = s;
    }
}

/* simd::sum (simd.h:53-61), widened as a halving tree: for 4 lanes (a0+a2)+(a1+a3). */
static double lane_hsum(const double* a, unsigned w) {
    double t[32];
    for (unsigned i = 0; i < w; ++i)
        t[i] = a[i];
    while (w > 1) {
        w /= 2;
        for (unsigned i = 0; i < w; ++i)
            t[i] = t[i] + t[i + w];
    }
    return t[0];
}

typedef struct {
    double* y;
    double* calib; /* this chunk's slot */
    uint32_t start_row_start;
} chunk_ctx;

/* spmv_thread_data::store_to_row_start (csr5.h:526-538) */
static inline void store_to_row_start(chunk_ctx* ctx, uint32_t row_start, double val, int direct) {
    if (row_start == ctx->start_row_start && !direct) {
        *ctx->calib += val;
        return;
    }
    if (direct)
        ctx->y[row_start] = val;
    else
        ctx->y[row_start] += val;
}

static void spmv_tile(const oracle_view* A, const oracle_fields f, uint64_t t, const double* x, chunk_ctx* ctx) {
    const unsigned S = A->sigma, W = A->omega, TS = S * W;
    const double* v = A->vals + t * TS;
    const uint32_t* ci = A->col + t * TS;
    const uint32_t raw = A->tile_ptr[t];
    const uint32_t row_stop = strip_dirty(A->tile_ptr[t + 1]);

    uint64_t flag[32], yoff[32], soff[32];
    for (unsigned c = 0; c < W; ++c) {
        uint64_t w = A->tile_desc[t * W + c];
        flag[c] = word_flag(f, w);
        yoff[c] = word_y(f, w);
        soff[c] = word_s(f, w);
    }
    const int fast_direct = (int)(flag[0] & 1);

    if (raw == row_stop) { /* partition_fast_track (csr5.h:562-574) */
        double lane[32];
        for (unsigned c = 0; c < W; ++c)
            lane[c] = 0.0;
        for (unsigned i = 0; i < S; ++i)
            for (unsigned c = 0; c < W; ++c)
                lane[c] = fma(v[i * W + c], x[ci[i * W + c]], lane[c]);
        store_to_row_start(ctx, raw, lane_hsum(lane, W), fast_direct);
        return;
    }

    const int empty_rows = is_dirty(raw);
    const uint32_t row_start = strip_dirty(raw);
    double* y_local = ctx->y + row_start;
    const uint32_t optr = empty_rows ? (A->tdo_ptr[t] - A->tdo_ptr[0]) : 0;
#define Y_IDX(off) (empty_rows ? A->tdo[optr + (off)] : (uint32_t)(off))

    int start[32], stop[32], any_started[32];
    double sum[32], first_sum[32];
    flag[0] |= 1; /* csr5.h:668 */
    for (unsigned c = 0; c < W; ++c) {
        int bit0 = (int)(flag[c] & 1);
        start[c] = 1 - bit0;
        stop[c] = 0;
        any_started[c] = c == 0 ? 0 : bit0; /* csr5.h:677 */
        sum[c] = v[c] * x[ci[c]];           /* csr5.h:680-681 (a product, no fma) */
        first_sum[c] = 0.0;
    }
    yoff[0] += 1; /* csr5.h:684 */

    for (unsigned i = 1; i < S; ++i) {
        int any = 0;
        for (unsigned c = 0; c < W; ++c)
            any |= (int)((flag[c] >> i) & 1);
        if (any) {
            for (unsigned c = 0; c < W; ++c) {
                int lb = (int)((flag[c] >> i) & 1);
                if (any_started[c] && lb) { /* green segment, csr5.h:697-701 */
                    y_local[Y_IDX(yoff[c])] = sum[c];
                    yoff[c] += 1;
                }
                if (!any_started[c] && lb) /* end of the red segment, csr5.h:703-711 */
                    first_sum[c] = sum[c];
                if (lb)
                    sum[c] = 0.0; /* csr5.h:714 */
                any_started[c] |= lb;
                stop[c] += lb;
            }
        }
        for (unsigned c = 0; c < W; ++c)
            sum[c] = fma(v[i * W + c], x[ci[i * W + c]], sum[c]);
    }

    /* csr5.h:730-735 and compute_last_sum / fast_segmented_sum (csr5.h:200-235) */
    double red[32], rot[32], scan[32], last[32];
    for (unsigned c = 0; c < W; ++c) {
        if (!any_started[c])
            first_sum[c] = sum[c];
        red[c] = start[c] == 1 ? first_sum[c] : 0.0;
    }
    for (unsigned c = 0; c < W; ++c)
        rot[c] = (c + 1 < W) ? red[c + 1] : 0.0;
    lane_inclusive_scan(rot, scan, W);
    for (unsigned c = 0; c < W; ++c) {
        double next_prefix = (scan[c + soff[c]] - scan[c]) + rot[c];
        int not_red_column = start[c] > stop[c];
        last[c] = sum[c] + (not_red_column ? 0.0 : next_prefix);
    }
    for (unsigned c = 0; c < W; ++c)
        if (any_started[c])
            y_local[Y_IDX(yoff[c])] = last[c];
#undef Y_IDX
    /* csr5.h:741-745; `direct` is "a row starts at this tile's first element" (see header) */
    store_to_row_start(ctx, row_start, any_started[0] ? first_sum[0] : last[0], fast_direct);
}

int oracle_csr5_spmv(uint32_t rows, uint64_t nnz, unsigned sigma, unsigned omega, const uint32_t* row_ptr,
                     const uint32_t* tile_ptr, const uint64_t* tile_desc, const uint32_t* tdo_ptr, const uint32_t* tdo,
                     const double* vals, const uint32_t* col, const double* x, double* y, int nthreads) {
    const oracle_fields f = fields_for(sigma, omega);
    const unsigned ts = sigma * omega;
    const uint64_t T = nnz / ts;
    oracle_view A = {rows, nnz, sigma, omega, T, row_ptr, tile_ptr, tile_desc, tdo_ptr, tdo, vals, col};
    if (nthreads < 1)
        nthreads = omp_get_max_threads();

    memset(y, 0, sizeof(double) * rows); /* oracle rule: zero-filled y */

    if (T > 0) {
        /* get_parallel_data (csr5.h:608-617) */
        const uint64_t chunk = (T + (uint64_t)nthreads - 1) / (uint64_t)nthreads;
        const uint64_t active = (T + chunk - 1) / chunk;
        double* calib = (double*)calloc(active, sizeof(double)); /* oracle rule: fresh calibrator */
        if (!calib)
            return -2;
#pragma omp parallel for schedule(static, 1) num_threads(nthreads)
        for (int64_t k = 0; k < (int64_t)active; ++k) {
            chunk_ctx ctx;
            ctx.y = y;
            ctx.calib = &calib[k];
            ctx.start_row_start = strip_dirty(tile_ptr[(uint64_t)k * chunk]);
            uint64_t end = ((uint64_t)k + 1) * chunk < T ? ((uint64_t)k + 1) * chunk : T;
            for (uint64_t t = (uint64_t)k * chunk; t < end; ++t)
                spmv_tile(&A, f, t, x, &ctx);
        }
        /* spmv_calibrator (csr5.h:750-754) */
        for (uint64_t k = 0; k < active; ++k)
            y[strip_dirty(tile_ptr[k * chunk])] += calib[k];
        free(calib);
    }

    /* spmv_tail_partition (csr5.h:756-782) */
    const uint32_t tail_start = strip_dirty(tile_ptr[T]);
    const uint64_t first_tail = T * ts;
#pragma omp parallel for num_threads(nthreads)
    for (int64_t r = (int64_t)tail_start; r < (int64_t)rows; ++r) {
        uint64_t s = ((uint32_t)r == tail_start) ? first_tail : row_ptr[r];
        uint64_t e = row_ptr[r + 1];
        double acc = 0.0;
        /* `sum += vals * x` (csr5.h:773-774): GCC keeps this reduction chain as a multiply and an
         * add (its x86 tuning avoids FMA chains), so no fma here. */
        for (uint64_t k = s; k < e; ++k)
            acc = acc + vals[k] * x[col[k]];
        if ((uint32_t)r == tail_start && row_ptr[r] != first_tail)
            y[r] += acc;
        else
            y[r] = acc;
    }
    return 0;
}

/* Plain CSR row-by-row SpMV (same fma order along each row); a second, format-free check. */
void oracle_csr_spmv(uint32_t rows, const uint32_t* row_ptr, const uint32_t* col, const double* vals, const double* x,
                     double* y, int nthreads) {
    if (nthreads < 1)
        nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t r = 0; r < (int64_t)rows; ++r) {
        double acc = 0.0;
        for (uint64_t k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
            acc = fma(vals[k], x[col[k]], acc);
        y[r] = acc;
    }
}

/* (|A| |x|)_i, the scale of the componentwise SpMV tolerance. */
void oracle_csr_absspmv(uint32_t rows, const uint32_t* row_ptr, const uint32_t* col, const double* vals,
                        const double* x, double* y, int nthreads) {
    if (nthreads < 1)
        nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t r = 0; r < (int64_t)rows; ++r) {
        double acc = 0.0;
        for (uint64_t k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
            acc += fabs(vals[k]) * fabs(x[col[k]]);
        y[r] = acc;
    }
}

/* ----------------------------------------------------------------------------------------------
 * Vector kernels of include/dim/vec.h:29-84 and the CG loop.
 * Dots are summed in fixed blocks of 4096 elements, then over blocks in order, so the result does
 * not depend on the thread count.
 * ---------------------------------------------------------------------------------------------- */

static double dot_fixed(const double* a, const double* b, uint64_t n, int nthreads) {
    const uint64_t B = 4096;
    const uint64_t nb = (n + B - 1) / B;
    double* part = (double*)malloc(sizeof(double) * (nb ? nb : 1));
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t k = 0; k < (int64_t)nb; ++k) {
        double s = 0.0;
        uint64_t e = ((uint64_t)k + 1) * B < n ? ((uint64_t)k + 1) * B : n;
        for (uint64_t i = (uint64_t)k * B; i < e; ++i)
            s = fma(a[i], b[i], s);
        part[k] = s;
    }
    double s = 0.0;
    for (uint64_t k = 0; k < nb; ++k)
        s += part[k];
    free(part);
    return s;
}

double oracle_dot(const double* a, const double* b, uint64_t n, int nthreads) {
    if (nthreads < 1)
        nthreads = omp_get_max_threads();
    return dot_fixed(a, b, n, nthreads);
}

/*
 * CG of benchmarks/conjugate_gradient/dim_sp/main.cpp:89-127 with the stopping rule of
 * docs/paper/thesis.tex:2146-2148 in relative form: stop once sqrt(r.r) <= tol * ||b||.
 * x is the initial guess on entry (the reference uses x0 = 0) and the solution on return.
 * Returns the iteration count (>= 0) or a negative error code; *relres receives sqrt(r.r)/||b||
 * of the recurrence residual.
 */
int64_t oracle_cg(uint32_t rows, uint64_t nnz, unsigned sigma, unsigned omega, const uint32_t* row_ptr,
                  const uint32_t* tile_ptr, const uint64_t* tile_desc, const uint32_t* tdo_ptr, const uint32_t* tdo,
                  const double* vals, const uint32_t* col, const double* b, double* x, double tol, int64_t max_it,
                  int nthreads, double* relres) {
    if (nthreads < 1)
        nthreads = omp_get_max_threads();
    const uint64_t n = rows;
    double* r = (double*)malloc(sizeof(double) * n);
    double* s = (double*)malloc(sizeof(double) * n);
    double* As = (double*)malloc(sizeof(double) * n);
    if (!r || !s || !As) {
        free(r);
        free(s);
        free(As);
        return -2;
    }
    /* r = b - A x */
    oracle_csr5_spmv(rows, nnz, sigma, omega, row_ptr, tile_ptr, tile_desc, tdo_ptr, tdo, vals, col, x, As, nthreads);
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        r[i] = b[i] - As[i];
        s[i] = r[i];
    }
    const double bnorm = sqrt(dot_fixed(b, b, n, nthreads));
    const double thresh = tol * (bnorm > 0 ? bnorm : 1.0);
    double rr = dot_fixed(r, r, n, nthreads);
    int64_t it = 0;
    if (sqrt(rr) <= thresh) {
        *relres = sqrt(rr) / (bnorm > 0 ? bnorm : 1.0);
        free(r);
        free(s);
        free(As);
        return 0;
    }
    while (it < max_it) {
        oracle_csr5_spmv(rows, nnz, sigma, omega, row_ptr, tile_ptr, tile_desc, tdo_ptr, tdo, vals, col, s, As,
                         nthreads);
        const double alpha = rr / dot_fixed(s, As, n, nthreads);
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (int64_t i = 0; i < (int64_t)n; ++i) {
            x[i] = x[i] + alpha * s[i];   /* vec::axpy (vec.h:49-52) */
            r[i] = r[i] + -alpha * As[i]; /* r.axpy(As, -alpha) */
        }
        const double rr_new = dot_fixed(r, r, n, nthreads);
        ++it;
        if (sqrt(rr_new) <= thresh) {
            rr = rr_new;
            break;
        }
        const double beta = rr_new / rr;
        rr = rr_new;
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (int64_t i = 0; i < (int64_t)n; ++i)
            s[i] = r[i] + beta * s[i]; /* vec::aypx (vec.h:57-60) */
    }
    *relres = sqrt(rr) / (bnorm > 0 ? bnorm : 1.0);
    free(r);
    free(s);
    free(As);
    return it;
}

int oracle_max_threads(void) { return omp_get_max_threads(); }
