// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A C-ABI shim around the reference's own header-only CSR5 implementation
// (include/dim/mat/storage_formats/csr5.h, csr.h, include/dim/vec.h of rurabori/diploma_research),
// compiled from the reference sources where they lie by oracle/Makefile into oracle/_ref/.  It is
// used to pin the C restatement (csr5_oracle.c) and to generate golden fixtures; it is never part
// of the product.  The reference needs AVX2/FMA, so this shim only builds on x86-64 hosts.
//
// Every SpMV here follows the oracle rule: y zero-filled and a fresh calibrator per call
// (csr5.h:530,744-745 and csr5/calibrator.h:14-31 make the reference drift otherwise).
#include <dim/mat/storage_formats/coo.h>
#include <dim/mat/storage_formats/csr.h>
#include <dim/mat/storage_formats/csr5.h>
#include <dim/vec.h>

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <span>

namespace {
using csr_t = dim::mat::csr<double>;
using csr5_t = dim::mat::csr5<double>;
using coo_t = dim::mat::coo<double>;

struct handle_t
{
    csr5_t m;
};

struct csr_handle_t
{
    csr_t m;
};
} // namespace

extern "C" {

int dimref_max_threads() { return omp_get_max_threads(); }

// csr<double>::from_coo (csr.h:42-77) of a coo (coo.h:17-47) holding the caller's triplets; with
// symmetric != 0 the coo stands for its mirror entries too (coo::iterate, coo.h:33-46).  *out_nnz gets
// the CSR's non-zero count; dimref_csr_export copies the arrays out.
void* dimref_csr_from_coo(uint32_t rows, uint32_t cols, uint64_t nnz, const double* val, const uint32_t* row,
                          const uint32_t* col, int symmetric, uint64_t* out_nnz) {
    coo_t coo{dim::mat::dimensions_t{.rows = rows, .cols = cols}, nnz, symmetric != 0};
    std::copy(val, val + nnz, coo.values.begin());
    std::copy(row, row + nnz, coo.row_indices.begin());
    std::copy(col, col + nnz, coo.col_indices.begin());
    auto* h = new csr_handle_t{csr_t::from_coo(coo)};
    *out_nnz = h->m.values.size();
    return h;
}

void dimref_csr_export(void* h, uint32_t* row_ptr, uint32_t* col, double* val) {
    const auto& m = static_cast<csr_handle_t*>(h)->m;
    std::copy(m.row_start_offsets.begin(), m.row_start_offsets.end(), row_ptr);
    std::copy(m.col_indices.begin(), m.col_indices.end(), col);
    std::copy(m.values.begin(), m.values.end(), val);
}

void dimref_csr_free(void* h) { delete static_cast<csr_handle_t*>(h); }

// csr5<double,16,4,uint32_t>::from_csr (csr5.h:791-803) on copies of the caller's CSR arrays.
void* dimref_csr5_from_csr(uint32_t rows, uint32_t cols, uint64_t nnz, const uint32_t* row_ptr, const uint32_t* col,
                           const double* val) {
    csr_t::values_t v(val, val + nnz);
    csr_t::indices_t rp(row_ptr, row_ptr + rows + 1);
    csr_t::indices_t ci(col, col + nnz);
    csr_t csr{dim::mat::dimensions_t{.rows = rows, .cols = cols}, std::move(v), std::move(rp), std::move(ci)};
    return new handle_t{csr5_t::from_csr(std::move(csr))};
}

void dimref_csr5_free(void* h) { delete static_cast<handle_t*>(h); }

void dimref_csr5_sizes(void* h, uint64_t* tile_count, uint64_t* tdo_size, uint32_t* tail_start) {
    const auto& m = static_cast<handle_t*>(h)->m;
    *tile_count = m.csr5_info.tile_count;
    *tdo_size = m.csr5_info.tile_desc_offset.size();
    *tail_start = m.tail_partition_start();
}

// Raw arrays: tile_ptr words, tile_desc as 4 raw u32 words per tile (GCC bit-field layout),
// tile_desc_offset_ptr, tile_desc_offset, transposed vals and col_idx.
void dimref_csr5_export(void* h, uint32_t* tile_ptr, uint32_t* tile_desc_words, uint32_t* tdo_ptr, uint32_t* tdo,
                        double* vals, uint32_t* col) {
    const auto& m = static_cast<handle_t*>(h)->m;
    const auto& info = m.csr5_info;
    for (size_t i = 0; i < info.tile_ptr.size(); ++i)
        tile_ptr[i] = info.tile_ptr[i].raw;
    static_assert(sizeof(csr5_t::tile_descriptor_type) == 16, "4 u32 words per tile");
    if (!info.tile_desc.empty())
        std::memcpy(tile_desc_words, info.tile_desc.data(), info.tile_desc.size() * 16);
    std::copy(info.tile_desc_offset_ptr.begin(), info.tile_desc_offset_ptr.end(), tdo_ptr);
    std::copy(info.tile_desc_offset.begin(), info.tile_desc_offset.end(), tdo);
    std::copy(m.vals.begin(), m.vals.end(), vals);
    std::copy(m.col_idx.begin(), m.col_idx.end(), col);
}

// y := A x through csr5::spmv (csr5.h:818-829) under the oracle rule.  Returns 0, or -1 when the
// reference cannot run (tile_count == 0 divides by zero in get_parallel_data, csr5.h:610-616).
int dimref_csr5_spmv(void* h, const double* x, double* y) {
    const auto& m = static_cast<handle_t*>(h)->m;
    if (m.csr5_info.tile_count == 0)
        return -1;
    std::fill(y, y + m.dimensions.rows, 0.0);
    auto cal = m.create_calibrator();
    m.spmv({.x = std::span<const double>{x, m.dimensions.cols}, .y = std::span<double>{y, m.dimensions.rows},
            .calibrator = cal});
    return 0;
}

// The dim_sp CG loop (benchmarks/conjugate_gradient/dim_sp/main.cpp:89-127) with b given, x0 = x on
// entry, and the relative threshold stop of docs/paper/thesis.tex:2146-2148.  Uses the reference's
// dim::vec axpy/aypx/dot.  Returns iterations, *relres = sqrt(r.r)/||b||.
int64_t dimref_cg(void* h, const double* b, double* x_io, double tol, int64_t max_it, double* relres) {
    const auto& m = static_cast<handle_t*>(h)->m;
    if (m.csr5_info.tile_count == 0)
        return -1;
    const size_t n = m.dimensions.rows;
    auto x = dim::vec<double>(n, 0.);
    std::copy(x_io, x_io + n, x.raw().begin());
    auto bv = dim::vec<double>(n, 0.);
    std::copy(b, b + n, bv.raw().begin());
    auto As = dim::vec<double>(n, 0.);
    auto spmv = [&](const dim::vec<double>& in, dim::vec<double>& out) {
        std::fill(out.raw().begin(), out.raw().end(), 0.0);
        auto cal = m.create_calibrator();
        m.spmv({.x = in.raw(), .y = out.raw(), .calibrator = cal});
    };
    spmv(x, As);
    auto r = dim::vec<double>(n, 0.);
    for (size_t i = 0; i < n; ++i)
        r.raw()[i] = b[i] - As.raw()[i];
    auto s = dim::vec<double>(n, 0.);
    std::copy(r.raw().begin(), r.raw().end(), s.raw().begin());
    const double bnorm = std::sqrt(dot(bv, bv));
    const double thresh = tol * (bnorm > 0 ? bnorm : 1.0);
    double r_r = dot(r, r);
    int64_t it = 0;
    if (std::sqrt(r_r) > thresh) {
        while (it < max_it) {
            spmv(s, As);
            const auto alpha = r_r / dot(s, As);
            x.axpy(s, alpha);
            r.axpy(As, -alpha);
            const auto tmp = dot(r, r);
            ++it;
            if (std::sqrt(tmp) <= thresh) {
                r_r = tmp;
                break;
            }
            const auto beta = tmp / std::exchange(r_r, tmp);
            s.aypx(r, beta);
        }
    }
    *relres = std::sqrt(r_r) / (bnorm > 0 ? bnorm : 1.0);
    std::copy(x.raw().begin(), x.raw().end(), x_io);
    return it;
}

} // extern "C"
