// dimgpu.hpp -- C++ binding of the C ABI in dimgpu.h, shaped like the reference's interface.
//
// The reference ("dim") is used from C++ through the header-only template
// dim::mat::csr5<double,16,4,uint32_t> (include/dim/mat/storage_formats/csr5.h:254-881) and the CG loop
// of benchmarks/conjugate_gradient/dim_sp/main.cpp:78-141.  This header gives a C++ caller of dim the
// same calls on the GPU library:
//
//   reference                                          here
//   csr5::from_csr(csr) (csr5.h:791-803)               dim::gpu::csr5::from_csr(csr)
//   csr5::spmv(spmv_data_t{x, y, calibrator})          csr5::spmv(x, y) on host spans,
//     (csr5.h:280-285, 818-829)                          csr5::spmv_device(x, y, cal, stream) on device memory
//   csr5::create_calibrator() (csr5.h:809)             csr5::create_calibrator()
//   csr5::tail_partition_start(), non_zero_count()     the same names
//   the dim_sp CG loop                                 dim::gpu::cg_solver
//   (no counterpart: batching, differentiation)        csr5::spmm_device, block_cg_solver,
//                                                        csr5::spmv_transpose_device, cg_adjoint
//   dim::io::h5::read_matlab_compatible,               dim::gpu::io::read_matlab_compatible,
//     write_matlab_compatible, load_csr5, store          write_matlab_compatible, load_csr5, store
//     (include/dim/io/h5.h:68-115)                       (HDF5 files without libhdf5; see dimgpu.h)
//   dim::io::matrix_market::load_as_csr                dim::gpu::io::load_matrix_market (no scnlib)
//
// from_csr takes any matrix type with the members of dim::mat::csr<double> (csr.h:19-40):
// `dimensions.rows`, `dimensions.cols`, and contiguous `values`, `row_start_offsets` (u32) and
// `col_indices` (u32) containers -- the reference's own csr<double> among them.
//
// Handles are move-only (a copy would free the device matrix twice).  Errors are exceptions, as in the
// reference: a size mismatch or other bad argument throws std::invalid_argument (csr5.h:820-821), any
// other failure dim::gpu::error carrying the library's status code.
#pragma once

#include <cstddef>
#include <cstdint>
#include <span>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "dimgpu.h"

namespace dim::gpu {

class error : public std::runtime_error {
public:
    error(int code, const char* what) : std::runtime_error(what), code_(code) {}
    int code() const noexcept { return code_; }

private:
    int code_;
};

[[noreturn]] inline void raise(int rc) {
    const char* msg = dimgpu_last_error_string();
    if (rc == DIMGPU_ERR_INVALID_ARGUMENT)
        throw std::invalid_argument(msg);
    throw error(rc, msg);
}

inline void check(int rc) {
    if (rc != DIMGPU_OK)
        raise(rc);
}

class csr5;

// Scratch of one SpMV at a time (the reference's calibrator_t, csr5/calibrator.h:14-31).
class calibrator {
public:
    calibrator() = default;
    calibrator(const calibrator&) = delete;
    calibrator& operator=(const calibrator&) = delete;
    calibrator(calibrator&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
    calibrator& operator=(calibrator&& o) noexcept {
        if (this != &o) {
            reset();
            h_ = std::exchange(o.h_, nullptr);
        }
        return *this;
    }
    ~calibrator() { reset(); }

    dimgpu_calibrator* handle() const noexcept { return h_; }

private:
    friend class csr5;
    explicit calibrator(dimgpu_calibrator* h) : h_(h) {}
    void reset() noexcept {
        if (h_)
            dimgpu_calibrator_destroy(h_);
        h_ = nullptr;
    }
    dimgpu_calibrator* h_{};
};

struct dimensions_t {
    uint32_t rows{}, cols{};
};

// A CSR5 matrix in GPU memory.
class csr5 {
public:
    csr5() = default;
    csr5(const csr5&) = delete;
    csr5& operator=(const csr5&) = delete;
    csr5(csr5&& o) noexcept : h_(std::exchange(o.h_, nullptr)), info_(o.info_) {}
    csr5& operator=(csr5&& o) noexcept {
        if (this != &o) {
            reset();
            h_ = std::exchange(o.h_, nullptr);
            info_ = o.info_;
        }
        return *this;
    }
    ~csr5() { reset(); }

    // csr5::from_csr (csr5.h:791-803): conversion on the GPU from a host CSR matrix.  The reference
    // takes the csr by value and moves it in; here the caller keeps it (the device holds copies).
    template <typename Csr>
    static csr5 from_csr(const Csr& m, const dimgpu_csr5_options* opt = nullptr, void* stream = nullptr) {
        csr5 r;
        const auto nnz = static_cast<uint64_t>(std::size(m.values));
        if (std::size(m.col_indices) != nnz || std::size(m.row_start_offsets) != size_t(m.dimensions.rows) + 1)
            throw std::invalid_argument("csr arrays do not match the matrix dimensions");
        check(dimgpu_csr5_from_csr(static_cast<uint32_t>(m.dimensions.rows), static_cast<uint32_t>(m.dimensions.cols),
                                   nnz, std::data(m.row_start_offsets), nnz ? std::data(m.col_indices) : nullptr,
                                   nnz ? std::data(m.values) : nullptr, DIMGPU_MEM_HOST, opt, stream, &r.h_));
        check(dimgpu_csr5_get_info(r.h_, &r.info_));
        return r;
    }

    // y := A x on host spans (the reference's benchmark call with its spmv_data_t, csr5.h:818-829).
    // Throws std::invalid_argument on a size mismatch, as the reference does (csr5.h:820-821).
    void spmv(std::span<const double> x, std::span<double> y) const {
        if (x.size() != info_.cols)
            throw std::invalid_argument("can't multiply, vector size doesn't match column count of the matrix");
        if (y.size() != info_.rows)
            throw std::invalid_argument("output vector size doesn't match the row count of the matrix");
        check(dimgpu_csr5_spmv_host(h_, x.data(), y.data()));
    }

    // y := A x on device memory, asynchronous on `stream`; cal == nullptr uses the matrix's own scratch.
    // Device-side failures are reported by status(cal, stream).
    void spmv_device(const double* x, double* y, const calibrator* cal = nullptr, void* stream = nullptr) const {
        check(dimgpu_csr5_spmv(h_, x, y, cal ? cal->handle() : nullptr, stream));
    }

    // Synchronizes `stream` and throws dim::gpu::error when a product on this scratch recorded a failure.
    void status(const calibrator* cal = nullptr, void* stream = nullptr) const {
        check(dimgpu_csr5_status(h_, cal ? cal->handle() : nullptr, stream));
    }

    // Takes ownership of a handle made by the C ABI (dimgpu_csr5_from_csr, dimgpu_h5_load_csr5, ...).
    static csr5 adopt(dimgpu_csr5* h) {
        csr5 r;
        r.h_ = h;
        if (h)
            check(dimgpu_csr5_get_info(h, &r.info_));
        return r;
    }

    // Y := A X for k right-hand sides (device memory, row-major, leading dimensions ldx, ldy >= k); the
    // first call for a (k, precision) times the candidate shapes (not inside a stream capture).
    void spmm_device(uint32_t k, const double* X, uint64_t ldx, double* Y, uint64_t ldy, void* stream = nullptr) const {
        check(dimgpu_csr5_spmm(h_, k, X, ldx, Y, ldy, stream));
    }
    void spmm_device(uint32_t k, const float* X, uint64_t ldx, float* Y, uint64_t ldy, void* stream = nullptr) const {
        check(dimgpu_csr5_spmm_f32(h_, k, X, ldx, Y, ldy, stream));
    }

    // y := A^T x on device memory (x: rows, y: cols).
    void spmv_transpose_device(const double* x, double* y, void* stream = nullptr) const {
        check(dimgpu_csr5_spmv_transpose(h_, x, y, stream));
    }

    calibrator create_calibrator() const {
        dimgpu_calibrator* c = nullptr;
        check(dimgpu_calibrator_create(h_, &c));
        return calibrator(c);
    }

    uint32_t tail_partition_start() const noexcept { return info_.tail_partition_start; }
    size_t non_zero_count() const noexcept { return static_cast<size_t>(info_.nnz); }
    dimensions_t dimensions() const noexcept { return {info_.rows, info_.cols}; }
    const dimgpu_csr5_info& info() const noexcept { return info_; }
    dimgpu_csr5* handle() const noexcept { return h_; }

private:
    void reset() noexcept {
        if (h_)
            dimgpu_csr5_destroy(h_);
        h_ = nullptr;
    }
    dimgpu_csr5* h_{};
    dimgpu_csr5_info info_{};
};

// The dim_sp CG loop (benchmarks/conjugate_gradient/dim_sp/main.cpp:89-127) on the GPU, stopping at
// ||b - A x|| <= tol ||b|| (docs/paper/thesis.tex:2146-2148).  The matrix must outlive the solver.
class cg_solver {
public:
    cg_solver(const csr5& a, const dimgpu_cg_params& params, void* stream = nullptr) : rows_(a.dimensions().rows) {
        check(dimgpu_cg_create(a.handle(), &params, stream, &h_));
    }
    cg_solver(const cg_solver&) = delete;
    cg_solver& operator=(const cg_solver&) = delete;
    cg_solver(cg_solver&& o) noexcept : h_(std::exchange(o.h_, nullptr)), rows_(o.rows_) {}
    cg_solver& operator=(cg_solver&& o) noexcept {
        if (this != &o) {
            reset();
            h_ = std::exchange(o.h_, nullptr);
            rows_ = o.rows_;
        }
        return *this;
    }
    ~cg_solver() { reset(); }

    // Solves from the initial guess in x (host memory), overwriting it.  Returns the statistics; a solve
    // that stops at max_it or breaks down throws dim::gpu::error (DIMGPU_ERR_NOT_CONVERGED / _BREAKDOWN)
    // unless `throw_on_failure` is false, in which case stats.status tells.
    dimgpu_cg_stats solve(std::span<const double> b, std::span<double> x, bool throw_on_failure = true) {
        if (b.size() != rows_ || x.size() != rows_)
            throw std::invalid_argument("b and x must have as many elements as the matrix has rows");
        dimgpu_cg_stats st{};
        const int rc = dimgpu_cg_solve_host(h_, b.data(), x.data(), &st);
        if (rc != DIMGPU_OK && (throw_on_failure || (rc != DIMGPU_ERR_NOT_CONVERGED && rc != DIMGPU_ERR_BREAKDOWN)))
            raise(rc);
        return st;
    }

    // The same on device memory, on `stream`.
    dimgpu_cg_stats solve_device(const double* b, double* x, void* stream = nullptr) {
        dimgpu_cg_stats st{};
        check(dimgpu_cg_solve(h_, b, x, &st, stream));
        return st;
    }

private:
    void reset() noexcept {
        if (h_)
            dimgpu_cg_destroy(h_);
        h_ = nullptr;
    }
    dimgpu_cg_solver* h_{};
    size_t rows_{};
};

// k simultaneous CG solves sharing one SpMM per iteration, each column with its own convergence (the
// dim_sp recurrence per column).  The matrix must outlive the solver.
class block_cg_solver {
public:
    block_cg_solver(const csr5& a, uint32_t k, const dimgpu_cg_params& params, void* stream = nullptr) : k_(k) {
        check(dimgpu_block_cg_create(a.handle(), k, &params, stream, &h_));
    }
    block_cg_solver(const block_cg_solver&) = delete;
    block_cg_solver& operator=(const block_cg_solver&) = delete;
    block_cg_solver(block_cg_solver&& o) noexcept : h_(std::exchange(o.h_, nullptr)), k_(o.k_) {}
    block_cg_solver& operator=(block_cg_solver&& o) noexcept {
        if (this != &o) {
            reset();
            h_ = std::exchange(o.h_, nullptr);
            k_ = o.k_;
        }
        return *this;
    }
    ~block_cg_solver() { reset(); }

    // B and X (initial guesses, overwritten by the solutions): n x k row-major device blocks.  Per-column
    // iteration counts and true relative residuals go to `col_iterations` / `col_rel_residual` when
    // given (k entries each).  A column that stops at max_it makes it throw dim::gpu::error
    // (DIMGPU_ERR_NOT_CONVERGED) unless `throw_on_failure` is false.
    dimgpu_block_cg_stats solve_device(const double* B, uint64_t ldb, double* X, uint64_t ldx,
                                       std::span<int64_t> col_iterations = {}, std::span<double> col_rel_residual = {},
                                       void* stream = nullptr, bool throw_on_failure = true) {
        if ((!col_iterations.empty() && col_iterations.size() != k_) ||
            (!col_rel_residual.empty() && col_rel_residual.size() != k_))
            throw std::invalid_argument("per-column outputs must have k entries");
        dimgpu_block_cg_stats st{};
        const int rc = dimgpu_block_cg_solve(h_, B, ldb, X, ldx, &st,
                                             col_iterations.empty() ? nullptr : col_iterations.data(),
                                             col_rel_residual.empty() ? nullptr : col_rel_residual.data(), stream);
        if (rc != DIMGPU_OK && (throw_on_failure || (rc != DIMGPU_ERR_NOT_CONVERGED && rc != DIMGPU_ERR_BREAKDOWN)))
            raise(rc);
        return st;
    }

private:
    void reset() noexcept {
        if (h_)
            dimgpu_block_cg_destroy(h_);
        h_ = nullptr;
    }
    dimgpu_block_cg* h_{};
    uint32_t k_{};
};

// The adjoint of x = A^{-1} b for a loss L(x): lambda := A^{-T} g (g = dL/dx, device memory; lambda holds
// the initial guess on entry and dL/db on return) and, when grad_vals is given, dL/dA = -lambda x^T on
// the pattern, in the CSR order of the matrix given to from_csr.
inline dimgpu_cg_stats cg_adjoint(const csr5& a, const double* g, const double* x, double* lambda, double* grad_vals,
                                  const dimgpu_cg_params& params, void* stream = nullptr) {
    dimgpu_cg_stats st{};
    check(dimgpu_cg_adjoint(a.handle(), g, x, lambda, grad_vals, &params, &st, stream));
    return st;
}

// The reference's HDF5 matrix IO (dim::io::h5, include/dim/io/h5.h:68-115; libs/dim/io/h5.cpp:45-74).
// File errors throw dim::gpu::error with DIMGPU_ERR_IO, a missing group std::invalid_argument.
namespace io {

// A CSR matrix with the members of dim::mat::csr<double> (csr.h:19-40).
struct csr_matrix {
    dimensions_t dimensions;
    std::vector<double> values;
    std::vector<uint32_t> row_start_offsets;
    std::vector<uint32_t> col_indices;
};

// read_matlab_compatible (h5.h:78-97): datasets data, ir, jc and the attribute MATLAB_sparse.
inline csr_matrix read_matlab_compatible(const std::string& path, const std::string& group = "A") {
    uint32_t rows = 0, cols = 0;
    uint64_t nnz = 0;
    check(dimgpu_h5_csr_dimensions(path.c_str(), group.c_str(), &rows, &cols, &nnz));
    csr_matrix m{{rows, cols}, std::vector<double>(nnz), std::vector<uint32_t>(size_t(rows) + 1),
                 std::vector<uint32_t>(nnz)};
    check(dimgpu_h5_read_matlab_compatible(path.c_str(), group.c_str(), m.row_start_offsets.data(),
                                           m.col_indices.data(), m.values.data()));
    return m;
}

// write_matlab_compatible (h5.h:68-76) of any matrix with the members of dim::mat::csr<double>.
template <typename Csr>
void write_matlab_compatible(const std::string& path, const std::string& group, const Csr& m, bool append = false) {
    const auto nnz = static_cast<uint64_t>(std::size(m.values));
    if (std::size(m.col_indices) != nnz || std::size(m.row_start_offsets) != size_t(m.dimensions.rows) + 1)
        throw std::invalid_argument("csr arrays do not match the matrix dimensions");
    check(dimgpu_h5_write_matlab_compatible(path.c_str(), group.c_str(), static_cast<uint32_t>(m.dimensions.rows),
                                            static_cast<uint32_t>(m.dimensions.cols), nnz, std::data(m.row_start_offsets),
                                            nnz ? std::data(m.col_indices) : nullptr, nnz ? std::data(m.values) : nullptr,
                                            append ? 1 : 0));
}

// load_csr5 (h5.cpp:57-74): a stored CSR5 group, converted to the device layout (or `opt`'s).
inline csr5 load_csr5(const std::string& path, const std::string& group = "A", const dimgpu_csr5_options* opt = nullptr,
                      void* stream = nullptr) {
    dimgpu_csr5* h = nullptr;
    check(dimgpu_h5_load_csr5(path.c_str(), group.c_str(), opt, stream, &h));
    return csr5::adopt(h);
}

// store (h5.cpp:45-55) of a matrix converted with the reference's layout (sigma 16, omega 4).
inline void store(const std::string& path, const std::string& group, const csr5& m, bool append = false) {
    check(dimgpu_h5_store_csr5(path.c_str(), group.c_str(), m.handle(), append ? 1 : 0));
}

// The result vectors of benchmarks/csr5/dim/main.cpp:35-43.
inline std::vector<double> read_vector(const std::string& path, const std::string& dataset) {
    uint64_t n = 0;
    check(dimgpu_h5_vector_length(path.c_str(), dataset.c_str(), &n));
    std::vector<double> y(n);
    check(dimgpu_h5_read_vector(path.c_str(), dataset.c_str(), y.data()));
    return y;
}

inline void write_vector(const std::string& path, const std::string& dataset, std::span<const double> y,
                         bool overwrite = false) {
    check(dimgpu_h5_write_vector(path.c_str(), dataset.c_str(), y.size(), y.data(), overwrite ? 1 : 0));
}

// dim::io::matrix_market::load_as_csr (matrix_market.h:25-83): a coordinate Matrix Market file as CSR.
inline csr_matrix load_matrix_market(const std::string& path) {
    uint32_t rows = 0, cols = 0;
    uint64_t nnz = 0;
    check(dimgpu_mm_csr_dimensions(path.c_str(), &rows, &cols, &nnz));
    csr_matrix m{{rows, cols}, std::vector<double>(nnz), std::vector<uint32_t>(size_t(rows) + 1),
                 std::vector<uint32_t>(nnz)};
    check(dimgpu_mm_read_csr(path.c_str(), m.row_start_offsets.data(), m.col_indices.data(), m.values.data()));
    return m;
}

}  // namespace io

}  // namespace dim::gpu
