// adjoint.cu -- differentiation through the CG solve: transpose SpMV, adjoint CG, gradients on the
// sparsity pattern.
//
// For x = A^{-1} b and a loss L(x) with g = dL/dx:
//     lambda  = A^{-T} g          (adjoint CG: CG on A^T, which is SPD when A is)
//     dL/db   = lambda
//     dL/dA   = -lambda x^T       restricted to the stored entries of A
// A^T is built once per matrix, deterministically: the device arrays are put back in CSR order on the
// device, the transpose is a stable counting sort on the host (rows of A^T keep increasing column
// order), and the result goes through the normal device CSR5 conversion, so A^T x runs on the same
// SpMV kernel as A x.  The reference has no adjoint; this is the differentiation variant of its solver.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.hpp"
#include "layout.cuh"

namespace dimgpu {
namespace {

// Position in the device-layout arrays of CSR element e (full tiles re-ordered, tail in CSR order).
__device__ __forceinline__ uint64_t device_pos_q32(uint64_t e, uint64_t T) {
    const uint64_t t = e / 512;
    if (t >= T)
        return e;
    const uint32_t k = (uint32_t)(e - t * 512), c = k / 16, r = k % 16;
    return t * 512 + pos_device_q32(c, r, 32);
}
__device__ __forceinline__ uint64_t device_pos_f64(uint64_t e, uint64_t T) {
    const uint64_t t = e / 512;
    if (t >= T)
        return e;
    const uint32_t k = (uint32_t)(e - t * 512), c = k / 16, r = k % 16;
    return t * 512 + pos_device_f64(c, r, 32);
}

__global__ void k_to_csr_order(const double* vals, const uint32_t* col, uint64_t nnz, uint64_t T, double* v_out,
                               uint32_t* c_out) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nnz; e += (uint64_t)gridDim.x * blockDim.x) {
        v_out[e] = vals[device_pos_f64(e, T)];
        c_out[e] = col[device_pos_q32(e, T)];
    }
}

// out[e] = scale * u[row(e)] * v[col(e)] for every stored element e, in CSR order (one thread per row)
__global__ void k_pattern_outer(const uint32_t* row_ptr, const uint32_t* col, uint32_t rows, uint64_t T,
                                const double* u, const double* v, double scale, double* out) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < rows; r += (uint64_t)gridDim.x * blockDim.x) {
        const double ur = scale * u[r];
        for (uint64_t e = row_ptr[r]; e < row_ptr[r + 1]; ++e)
            out[e] = ur * v[col[device_pos_q32(e, T)]];
    }
}

}  // namespace

// Builds a new CSR5 handle of A^T.
int build_transpose(const dimgpu_csr5* m, cudaStream_t st, dimgpu_csr5** out) {
    if (m->layout != kLayoutDevice || m->sigma != 16)
        return fail(DIMGPU_ERR_UNSUPPORTED, "transpose needs the device layout with sigma 16");
    const uint64_t nnz = m->nnz;
    const uint32_t rows = m->rows, cols = m->cols;
    std::vector<uint32_t> rp(rows + 1), ci(nnz), tp(cols + 1, 0), tc(nnz);
    std::vector<double> cv(nnz), tv(nnz);
    if (nnz) {
        double* dv = nullptr;
        uint32_t* dc = nullptr;
        DG_CHECK(dev_alloc_n(&dv, nnz));
        int rc = dev_alloc_n(&dc, nnz);
        if (rc == DIMGPU_OK) {
            const unsigned grid = (unsigned)std::min<uint64_t>(4096, (nnz + 255) / 256);
            k_to_csr_order<<<grid, 256, 0, st>>>(m->vals, m->col, nnz, m->tile_count, dv, dc);
            cudaError_t e = cudaMemcpyAsync(cv.data(), dv, nnz * 8, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(ci.data(), dc, nnz * 4, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(st);
            if (e != cudaSuccess)
                rc = cuda_fail(e, "copying A for the transpose");
        }
        dev_free(dv);
        dev_free(dc);
        DG_CHECK(rc);
    }
    DG_CUDA(cudaMemcpy(rp.data(), m->row_ptr, (rows + 1) * 4ull, cudaMemcpyDeviceToHost));
    // stable counting sort by column: row r's entries are visited in increasing r
    for (uint64_t e = 0; e < nnz; ++e)
        ++tp[ci[e] + 1];
    for (uint32_t c = 0; c < cols; ++c)
        tp[c + 1] += tp[c];
    std::vector<uint32_t> cursor(tp.begin(), tp.end() - 1);
    for (uint32_t r = 0; r < rows; ++r)
        for (uint64_t e = rp[r]; e < rp[r + 1]; ++e) {
            const uint32_t pos = cursor[ci[e]]++;
            tc[pos] = r;
            tv[pos] = cv[e];
        }
    dimgpu_csr5_options opt{16, 32, DIMGPU_LAYOUT_DEVICE, 0};
    return dimgpu_csr5_from_csr(cols, rows, nnz, tp.data(), nnz ? tc.data() : nullptr, nnz ? tv.data() : nullptr,
                                DIMGPU_MEM_HOST, &opt, st, out);
}

// Builds (once) the CSR5 handle of A^T kept inside m.
int ensure_transpose(const dimgpu_csr5* cm, cudaStream_t st) {
    dimgpu_csr5* m = const_cast<dimgpu_csr5*>(cm);
    if (m->transposed)
        return DIMGPU_OK;
    dimgpu_csr5* t = nullptr;
    DG_CHECK(build_transpose(m, st, &t));
    m->transposed = t;
    return DIMGPU_OK;
}

}  // namespace dimgpu

using namespace dimgpu;

extern "C" {

int dimgpu_csr5_transpose(const dimgpu_csr5* m, void* stream, dimgpu_csr5** out) {
    if (!m || !out)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    return build_transpose(m, static_cast<cudaStream_t>(stream), out);
}

int dimgpu_csr5_spmv_transpose(const dimgpu_csr5* m, const double* x, double* y, void* stream) {
    if (!m || (!x && m->rows) || (!y && m->cols))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DG_CHECK(ensure_transpose(m, st));
    return launch_spmv_f64(m->transposed, x, y, m->transposed->own_cal, spmv_epilogue{}, st);
}

int dimgpu_csr5_pattern_outer(const dimgpu_csr5* m, const double* u, const double* v, double scale, double* out,
                              void* stream) {
    if (!m || (m->nnz && (!u || !v || !out)))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    if (m->layout != kLayoutDevice || m->sigma != 16)
        return fail(DIMGPU_ERR_UNSUPPORTED, "needs the device layout with sigma 16");
    if (m->rows) {
        const unsigned grid = (unsigned)std::min<uint64_t>(4096, (m->rows + 255) / 256);
        k_pattern_outer<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(m->row_ptr, m->col, m->rows,
                                                                               m->tile_count, u, v, scale, out);
        DG_CUDA(cudaGetLastError());
    }
    return DIMGPU_OK;
}

int dimgpu_cg_adjoint(const dimgpu_csr5* m, const double* g, const double* x, double* lambda, double* grad_vals,
                      const dimgpu_cg_params* params, dimgpu_cg_stats* stats, void* stream) {
    if (!m || !g || !x || !lambda || !params)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    if (m->rows != m->cols)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "the adjoint solve needs a square matrix");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DG_CHECK(ensure_transpose(m, st));
    dimgpu_cg_solver* s = nullptr;
    DG_CHECK(dimgpu_cg_create(m->transposed, params, stream, &s));
    int rc = dimgpu_cg_solve(s, g, lambda, stats, stream);  // lambda holds the initial guess on entry
    dimgpu_cg_destroy(s);
    if (rc != DIMGPU_OK && rc != DIMGPU_ERR_NOT_CONVERGED)
        return rc;
    if (grad_vals) {
        const int rc2 = dimgpu_csr5_pattern_outer(m, lambda, x, -1.0, grad_vals, stream);
        if (rc2 != DIMGPU_OK)
            return rc2;
    }
    return rc;
}

}  // extern "C"
