// api.cu -- the C ABI of include/dimgpu.h: matrix handles, calibrators, SpMV and vector entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "common.cuh"
#include "internal.hpp"

namespace dimgpu {

namespace {
thread_local std::string g_last_error;

__global__ void k_validate(const uint32_t* row_ptr, uint32_t rows, const uint32_t* col, uint64_t nnz, uint32_t cols,
                           uint32_t* bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < rows; r += stride)
        if (row_ptr[r] > row_ptr[r + 1])
            atomicOr(bad, 1u);
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < nnz; k += stride)
        if (col[k] >= cols)
            atomicOr(bad, 2u);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (row_ptr[0] != 0)
            atomicOr(bad, 4u);
        if ((uint64_t)row_ptr[rows] != nnz)
            atomicOr(bad, 8u);
    }
}

template <typename F>
__global__ void k_map(uint64_t n, F f) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        f(i);
}

// Deterministic dot: fixed grid of 256 blocks x 256 threads, fixed-order partials.
constexpr int kDotBlocks = 256;
constexpr int kDotThreads = 256;
__global__ void k_dot_part(const double* a, const double* b, uint64_t n, double* part) {
    __shared__ double sh[kDotThreads];
    double s = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)kDotThreads + threadIdx.x; i < n; i += (uint64_t)kDotBlocks * kDotThreads)
        s = fma(a[i], b[i], s);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int h = kDotThreads / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            sh[threadIdx.x] += sh[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        part[blockIdx.x] = sh[0];
}
__global__ void k_dot_final(const double* part, double* out) {
    __shared__ double sh[kDotBlocks];
    sh[threadIdx.x] = part[threadIdx.x];
    __syncthreads();
    for (int h = kDotBlocks / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            sh[threadIdx.x] += sh[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        *out = sh[0];
}

inline unsigned grid_n(uint64_t n) {
    uint64_t b = (n + 255) / 256;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(b, 4096));
}

}  // namespace

void set_error(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? DIMGPU_ERR_OUT_OF_MEMORY : DIMGPU_ERR_CUDA;
}

int dev_alloc(void** p, size_t bytes) {
    *p = nullptr;
    cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) {
        *p = nullptr;
        (void)cudaGetLastError();
        return fail(DIMGPU_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    }
    return DIMGPU_OK;
}

void dev_free(void* p) {
    if (p)
        cudaFree(p);
}

int dot_device(uint64_t n, const double* a, const double* b, double* d_out, double* d_part, cudaStream_t s) {
    k_dot_part<<<kDotBlocks, kDotThreads, 0, s>>>(a, b, n, d_part);
    k_dot_final<<<1, kDotBlocks, 0, s>>>(d_part, d_out);
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

}  // namespace dimgpu

using namespace dimgpu;

static void destroy_matrix(dimgpu_csr5* m) {
    if (!m)
        return;
    if (m->spmm_sc) {
        spmm_scratch_release(static_cast<spmm_scratch*>(m->spmm_sc));
        delete static_cast<spmm_scratch*>(m->spmm_sc);
    }
    if (m->transposed)
        destroy_matrix(m->transposed);
    if (m->own_cal) {
        calibrator_release(m->own_cal);
        delete m->own_cal;
    }
    dev_free(m->row_ptr);
    dev_free(m->vals);
    dev_free(m->col);
    dev_free(m->col16);
    dev_free(m->col_base);
    dev_free(m->tile_ptr);
    dev_free(m->tile_desc);
    dev_free(m->tdo_ptr);
    dev_free(m->tdo);
    dev_free(m->empty_rows);
    dev_free(m->vals32);
    delete m;
}

extern "C" {

const char* dimgpu_last_error_string(void) { return g_last_error.c_str(); }

int dimgpu_version(void) { return 2; }

int dimgpu_csr5_from_csr(uint32_t rows, uint32_t cols, uint64_t nnz, const uint32_t* row_ptr, const uint32_t* col_idx,
                         const double* vals, int mem, const dimgpu_csr5_options* opt, void* stream,
                         dimgpu_csr5** out) {
    if (!out)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!row_ptr || (nnz && (!col_idx || !vals)))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL CSR array");
    if (rows >= 0x80000000u)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "rows must be below 2^31 (the tile_ptr MSB is the dirty flag)");
    if (nnz > 0xFFFFFFFFull)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "nnz must fit u32 row offsets");
    if (mem != DIMGPU_MEM_HOST && mem != DIMGPU_MEM_DEVICE)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "mem must be DIMGPU_MEM_HOST or DIMGPU_MEM_DEVICE");
    uint32_t sigma = opt && opt->sigma ? opt->sigma : 16;
    uint32_t omega = opt && opt->omega ? opt->omega : 32;
    int layout = omega == 32 ? kLayoutDevice : (opt ? opt->layout : kLayoutReference);
    if (omega != 4 && omega != 8 && omega != 16 && omega != 32)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "omega must be 4, 8, 16 or 32");
    if (sigma < 1 || sigma > 32)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "sigma must be in [1, 32]");
    if (layout == kLayoutDevice && (sigma % 4 != 0 || omega != 32))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "the device layout needs omega = 32 and sigma a multiple of 4");
    if (fields_for(sigma, omega).total() > 64)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "descriptor does not fit 64 bits");
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    dimgpu_csr5* m = new dimgpu_csr5();
    for (auto& row : m->spmm_shape)
        for (int& v : row)
            v = -1;
    cudaGetDevice(&m->device);
    m->rows = rows;
    m->cols = cols;
    m->nnz = nnz;
    m->sigma = sigma;
    m->omega = omega;
    m->layout = layout;

    uint32_t *d_rp = nullptr, *d_ci = nullptr, *d_bad = nullptr;
    double* d_v = nullptr;
    int rc = DIMGPU_OK;
    do {
        if ((rc = dev_alloc_n(&m->row_ptr, (uint64_t)rows + 1)) != DIMGPU_OK) break;
        d_rp = m->row_ptr;
        if (mem == DIMGPU_MEM_HOST) {
            if ((rc = dev_alloc_n(&d_ci, std::max<uint64_t>(1, nnz))) != DIMGPU_OK) break;
            if ((rc = dev_alloc_n(&d_v, std::max<uint64_t>(1, nnz))) != DIMGPU_OK) break;
            cudaError_t e = cudaMemcpyAsync(d_rp, row_ptr, sizeof(uint32_t) * ((uint64_t)rows + 1),
                                            cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess && nnz)
                e = cudaMemcpyAsync(d_ci, col_idx, sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess && nnz)
                e = cudaMemcpyAsync(d_v, vals, sizeof(double) * nnz, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "copying the CSR arrays to the device");
                break;
            }
        } else {
            cudaError_t e = cudaMemcpyAsync(d_rp, row_ptr, sizeof(uint32_t) * ((uint64_t)rows + 1),
                                            cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "copying row_ptr");
                break;
            }
            d_ci = const_cast<uint32_t*>(col_idx);
            d_v = const_cast<double*>(vals);
        }
        // reject malformed CSR before any kernel indexes with it
        if ((rc = dev_alloc_n(&d_bad, 4)) != DIMGPU_OK) break;
        cudaMemsetAsync(d_bad, 0, sizeof(uint32_t), s);
        k_validate<<<grid_n(std::max<uint64_t>(rows, nnz)), 256, 0, s>>>(d_rp, rows, nnz ? d_ci : d_rp, nnz, cols,
                                                                        d_bad);
        uint32_t bad = 0;
        cudaError_t e = cudaMemcpyAsync(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "validating the CSR arrays");
            break;
        }
        if (bad) {
            rc = fail(DIMGPU_ERR_INVALID_ARGUMENT, "malformed CSR (%s%s%s%s)", (bad & 1) ? "row_ptr decreases " : "",
                      (bad & 2) ? "column index >= cols " : "", (bad & 4) ? "row_ptr[0] != 0 " : "",
                      (bad & 8) ? "row_ptr[rows] != nnz" : "");
            break;
        }
        if ((rc = prepare_spmv_kernels()) != DIMGPU_OK) break;
        if ((rc = convert_csr5(m, d_rp, d_ci, d_v, s)) != DIMGPU_OK) break;
        const bool kernel_sigma = m->layout == kLayoutDevice && m->sigma == 16;
        if (kernel_sigma && (rc = build_col16(m, s)) != DIMGPU_OK) break;
        m->plan = make_spmv_plan(m->tile_count, device_sm_count(m->device), 16);
        {
            // A matrix that fits in L2 together with the CG vectors (six f64 n-vectors) is better left
            // there between products than streamed with an evict-first policy.
            int l2 = 0;
            cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, m->device);
            const uint64_t matrix_bytes = m->nnz * 12 + (uint64_t)m->tile_count * 32 * 4;
            m->keep_in_l2 = (l2 > 0 && matrix_bytes + 48ull * m->rows <= (uint64_t)l2) ? 1 : 0;
        }
        m->plan32 = make_spmv_plan32(m->tile_count, device_sm_count(m->device));
        m->own_cal = new dimgpu_calibrator();
        if ((rc = calibrator_init(m->own_cal, m)) != DIMGPU_OK) break;
        if (kernel_sigma && (rc = autotune_gathers(m, s)) != DIMGPU_OK) break;
    } while (false);
    if (mem == DIMGPU_MEM_HOST) {
        dev_free(d_ci);
        dev_free(d_v);
    }
    dev_free(d_bad);
    if (rc != DIMGPU_OK) {
        destroy_matrix(m);
        return rc;
    }
    *out = m;
    return DIMGPU_OK;
}

int dimgpu_csr5_destroy(dimgpu_csr5* m) {
    destroy_matrix(m);
    return DIMGPU_OK;
}

int dimgpu_csr5_get_info(const dimgpu_csr5* m, dimgpu_csr5_info* o) {
    if (!m || !o)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    o->rows = m->rows;
    o->cols = m->cols;
    o->nnz = m->nnz;
    o->sigma = m->sigma;
    o->omega = m->omega;
    o->layout = m->layout;
    o->desc_word_bytes = m->desc_word_bytes;
    o->tile_count = m->tile_count;
    o->tile_desc_offset_len = m->tdo_len;
    o->tail_partition_start = m->tail_start;
    o->empty_rows = m->n_empty;
    o->device_bytes = m->device_bytes;
    return DIMGPU_OK;
}

int dimgpu_csr5_export(const dimgpu_csr5* m, uint32_t* tile_ptr, void* tile_desc, uint32_t* tdo_ptr, uint32_t* tdo,
                       double* vals, uint32_t* col_idx, uint32_t* row_ptr) {
    if (!m)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL matrix");
    const uint64_t T = m->tile_count;
    if (tile_ptr)
        DG_CUDA(cudaMemcpy(tile_ptr, m->tile_ptr, sizeof(uint32_t) * (T + 1), cudaMemcpyDeviceToHost));
    if (tile_desc && T)
        DG_CUDA(cudaMemcpy(tile_desc, m->tile_desc, T * m->omega * m->desc_word_bytes, cudaMemcpyDeviceToHost));
    if (tdo_ptr)
        DG_CUDA(cudaMemcpy(tdo_ptr, m->tdo_ptr, sizeof(uint32_t) * (T + 1), cudaMemcpyDeviceToHost));
    if (tdo && m->tdo_len)
        DG_CUDA(cudaMemcpy(tdo, m->tdo, sizeof(uint32_t) * m->tdo_len, cudaMemcpyDeviceToHost));
    if (vals && m->nnz)
        DG_CUDA(cudaMemcpy(vals, m->vals, sizeof(double) * m->nnz, cudaMemcpyDeviceToHost));
    if (col_idx && m->nnz)
        DG_CUDA(cudaMemcpy(col_idx, m->col, sizeof(uint32_t) * m->nnz, cudaMemcpyDeviceToHost));
    if (row_ptr)
        DG_CUDA(cudaMemcpy(row_ptr, m->row_ptr, sizeof(uint32_t) * ((uint64_t)m->rows + 1), cudaMemcpyDeviceToHost));
    return DIMGPU_OK;
}

int dimgpu_calibrator_create(const dimgpu_csr5* m, dimgpu_calibrator** out) {
    if (!m || !out)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    dimgpu_calibrator* c = new dimgpu_calibrator();
    int rc = calibrator_init(c, m);
    if (rc != DIMGPU_OK) {
        calibrator_release(c);
        delete c;
        return rc;
    }
    *out = c;
    return DIMGPU_OK;
}

int dimgpu_calibrator_destroy(dimgpu_calibrator* c) {
    if (c) {
        calibrator_release(c);
        delete c;
    }
    return DIMGPU_OK;
}

int dimgpu_csr5_spmv(const dimgpu_csr5* m, const double* x, double* y, dimgpu_calibrator* cal, void* stream) {
    if (!m || (!x && m->cols) || (!y && m->rows))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    return launch_spmv_f64(m, x, y, cal ? cal : m->own_cal, spmv_epilogue{}, static_cast<cudaStream_t>(stream));
}

int dimgpu_csr5_spmv_dot(const dimgpu_csr5* m, const double* x, double* y, double* dot, dimgpu_calibrator* cal,
                         void* stream) {
    if (!m || (!x && m->cols) || (!y && m->rows) || !dot)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    if (m->rows != m->cols)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "x.(A x) needs a square matrix (%u x %u)", m->rows, m->cols);
    spmv_epilogue ep;
    ep.dot_out = dot;
    return launch_spmv_f64(m, x, y, cal ? cal : m->own_cal, ep, static_cast<cudaStream_t>(stream));
}

int dimgpu_csr5_spmv_f32(const dimgpu_csr5* m, const float* x, float* y, dimgpu_calibrator* cal, void* stream) {
    if (!m || (!x && m->cols) || (!y && m->rows))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    return launch_spmv_f32(m, x, y, cal ? cal : m->own_cal, spmv_epilogue{}, static_cast<cudaStream_t>(stream));
}

int dimgpu_csr5_spmv_host(const dimgpu_csr5* m, const double* x_host, double* y_host) {
    if (!m || (!x_host && m->cols) || (!y_host && m->rows))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    double *dx = nullptr, *dy = nullptr;
    DG_CHECK(dev_alloc_n(&dx, std::max<uint32_t>(1, m->cols)));
    int rc = dev_alloc_n(&dy, std::max<uint32_t>(1, m->rows));
    if (rc == DIMGPU_OK) {
        cudaError_t e = cudaMemcpy(dx, x_host, sizeof(double) * m->cols, cudaMemcpyHostToDevice);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "x to device");
    }
    if (rc == DIMGPU_OK)
        rc = launch_spmv_f64(m, dx, dy, m->own_cal, spmv_epilogue{}, 0);
    if (rc == DIMGPU_OK) {
        cudaError_t e = cudaMemcpy(y_host, dy, sizeof(double) * m->rows, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "y to host");
    }
    if (rc == DIMGPU_OK)
        rc = check_status(m->own_cal, 0);
    dev_free(dx);
    dev_free(dy);
    return rc;
}

int dimgpu_vec_axpy(uint64_t n, double alpha, const double* x, double* y, void* stream) {
    if (n && (!x || !y))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL vector");
    if (n)
        k_map<<<grid_n(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            n, [=] __device__(uint64_t i) { y[i] = y[i] + alpha * x[i]; });
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

int dimgpu_vec_aypx(uint64_t n, double alpha, const double* x, double* y, void* stream) {
    if (n && (!x || !y))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL vector");
    if (n)
        k_map<<<grid_n(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            n, [=] __device__(uint64_t i) { y[i] = x[i] + alpha * y[i]; });
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

int dimgpu_vec_set(uint64_t n, double value, double* y, void* stream) {
    if (n && !y)
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL vector");
    if (n)
        k_map<<<grid_n(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(n,
                                                                          [=] __device__(uint64_t i) { y[i] = value; });
    DG_CUDA(cudaGetLastError());
    return DIMGPU_OK;
}

int dimgpu_vec_dot(uint64_t n, const double* l, const double* r, double* out, void* stream) {
    if (!out || (n && (!l || !r)))
        return fail(DIMGPU_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* scratch = nullptr;
    DG_CHECK(dev_alloc_n(&scratch, kDotBlocks + 1));
    int rc = dot_device(n, l, r, scratch + kDotBlocks, scratch, s);
    if (rc == DIMGPU_OK) {
        cudaError_t e = cudaMemcpyAsync(out, scratch + kDotBlocks, sizeof(double), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "dot");
    }
    dev_free(scratch);
    return rc;
}

}  // extern "C"

namespace dimgpu {
int vec_fill(uint64_t n, double v, double* y, cudaStream_t stream) { return dimgpu_vec_set(n, v, y, stream); }
}  // namespace dimgpu
