// internal.hpp -- host-side structures behind the C ABI (include/dimgpu.h).
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/dimgpu.h"
#include "layout.cuh"

namespace dimgpu {

// Last error message of the calling thread.
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

#define DG_CUDA(call)                                 \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess)                        \
            return ::dimgpu::cuda_fail(e_, #call);    \
    } while (0)

#define DG_CHECK(code_expr)            \
    do {                               \
        int rc_ = (code_expr);         \
        if (rc_ != DIMGPU_OK)          \
            return rc_;                \
    } while (0)

// Device allocation helpers: return DIMGPU_OK or DIMGPU_ERR_OUT_OF_MEMORY.
int dev_alloc(void** p, size_t bytes);
template <typename T>
int dev_alloc_n(T** p, size_t n) {
    return dev_alloc(reinterpret_cast<void**>(p), n * sizeof(T) + (n == 0 ? 16 : 0));
}
void dev_free(void* p);

// How one SpMV launch covers the tiles: each warp owns a contiguous run of tiles.
struct spmv_plan {
    int grid = 1;                  // CTAs
    int warps_per_cta = 1;
    uint64_t tiles_per_warp = 0;
    uint32_t nwarps = 1;           // grid * warps_per_cta (calibrator slots)
};

}  // namespace dimgpu

struct dimgpu_calibrator {
    int device = 0;
    uint32_t nslots = 0;
    double* cal_val = nullptr;    // [nslots] row fragment each warp run publishes for a later run
    uint32_t* cal_row = nullptr;  // [nslots] that fragment's row
    uint32_t* flag = nullptr;     // [nslots] (launch epoch << 2) | fragment kind of each run
    double* dot_part = nullptr;   // [nslots + 1] per-CTA partials of the fused dot product
    uint32_t* counter = nullptr;  // [4] completion ticket, -, run counter, launch epoch
    uint32_t* status = nullptr;   // device status word (dimgpu::device_status)
};

struct dimgpu_csr5 {
    int device = 0;
    uint32_t rows = 0, cols = 0;
    uint64_t nnz = 0;
    uint32_t sigma = 16, omega = 32;
    int layout = dimgpu::kLayoutDevice;
    uint64_t tile_count = 0;
    uint32_t tail_start = 0;
    uint32_t desc_word_bytes = 4;
    uint64_t tdo_len = 0;
    uint32_t n_empty = 0;

    uint32_t* row_ptr = nullptr;   // [rows+1]
    double* vals = nullptr;        // [nnz] re-ordered
    uint32_t* col = nullptr;       // [nnz] re-ordered
    // Device layout only, when every full tile's columns span less than 2^16: each tile's column indices
    // as u16 offsets from the tile's smallest column (same order as col), which the SpMV streams instead
    // of col (2 bytes per non-zero fewer).  nullptr when some tile spans more.
    uint16_t* col16 = nullptr;     // [T * sigma * omega]
    uint32_t* col_base = nullptr;  // [T]
    uint32_t* tile_ptr = nullptr;  // [T+1]
    void* tile_desc = nullptr;     // [T*omega] words
    uint32_t* tdo_ptr = nullptr;   // [T+1]
    uint32_t* tdo = nullptr;       // [tdo_len]
    uint32_t* empty_rows = nullptr;  // [n_empty]
    float* vals32 = nullptr;       // f32 values in the device layout (built on first f32 use)
    uint64_t device_bytes = 0;

    int spmm_shape[2][33];       // autotuned SpMM launch shape per (f32?, k); -1 = not tuned yet
    void* spmm_sc = nullptr;     // the handle's own SpMM scratch (dimgpu::spmm_scratch), built on first use
    dimgpu_csr5* transposed = nullptr;  // A^T, built on first transpose use
    int keep_in_l2 = 0;        // matrix + CG vectors fit in L2: stream the matrix without evict-first
    int x_mode = 0;            // how the f64 SpMV gathers x (spmv_tile.cuh: kXReadOnly or kXStream), autotuned
    int x_mode32 = 0;          // the same for the f32 SpMV (tuned when the f32 values are made)
    dimgpu::spmv_plan plan;    // f64 SpMV launch (warps per CTA autotuned at conversion)
    dimgpu::spmv_plan plan32;  // f32 SpMV launch (more warps per CTA; tuned with the f32 values)
    dimgpu_calibrator* own_cal = nullptr;
};

namespace dimgpu {

// convert.cu
int convert_csr5(dimgpu_csr5* m, const uint32_t* d_row_ptr, const uint32_t* d_col, const double* d_vals,
                 cudaStream_t stream);
int ensure_vals32(const dimgpu_csr5* m, cudaStream_t stream);
int build_col16(dimgpu_csr5* m, cudaStream_t stream);

// spmv.cu
spmv_plan make_spmv_plan(uint64_t tiles, int sms, int warps_per_cta);
spmv_plan make_spmv_plan32(uint64_t tiles, int sms);
int prepare_spmv_kernels();
int calibrator_init(dimgpu_calibrator* c, const dimgpu_csr5* m);
void calibrator_release(dimgpu_calibrator* c);

struct spmv_epilogue {
    // Optional CG epilogue, computed by the last CTA: dot = x.y (written to *dot_out) and, when
    // rr is given, alpha = *rr / dot (written to *alpha_out); a non-positive or non-finite dot sets
    // kStatusBreakdown and *halt = 1.
    double* dot_out = nullptr;
    const double* rr = nullptr;
    double* alpha_out = nullptr;
    uint32_t* halt = nullptr;        // when non-null and *halt != 0 on entry, the launch does nothing
};

int launch_spmv_f64(const dimgpu_csr5* m, const double* x, double* y, dimgpu_calibrator* cal,
                    const spmv_epilogue& ep, cudaStream_t stream);
int launch_spmv_f32(const dimgpu_csr5* m, const float* x, float* y, dimgpu_calibrator* cal,
                    const spmv_epilogue& ep, cudaStream_t stream);
int check_status(dimgpu_calibrator* cal, cudaStream_t stream);
// Copies a device status word to *out (after synchronizing `stream`) and clears it when it is set.
int take_status_word(uint32_t* word, cudaStream_t stream, uint32_t* out);
// DIMGPU_OK for kStatusOk, else the matching DIMGPU_ERR_* with a message naming `where`.
int status_error(uint32_t st, const char* where);
int autotune_gathers(dimgpu_csr5* m, cudaStream_t stream);
int autotune_f32(dimgpu_csr5* m, cudaStream_t stream);
int vec_fill(uint64_t n, double v, double* y, cudaStream_t stream);

// spmm.cu: CSR5 SpMM (lanes = right-hand sides, one pass takes k <= 32 columns)
// SpMM shape codes the autotuner chooses from: bit 0 the launch shape (0: 8 warps x 3 stages, 1: 16 x 2),
// bits 1-2 the lane grouping g (right-hand sides per lane: the widest the operands allow, >> g)
constexpr int kSpmmShapes = 6;
struct spmm_args {
    const void* X = nullptr;
    void* Y = nullptr;
    uint64_t ldx = 0, ldy = 0;
    uint32_t k = 0;
    double* dot_out = nullptr;      // block-CG epilogue: per-column X.Y
    const double* rr = nullptr;     // and alpha_j = rr_j / dot_j for the columns in `mask`
    double* alpha_out = nullptr;
    const uint32_t* mask = nullptr;      // [2][32]; the half selected by *mask_sel (when given)
    const uint32_t* mask_sel = nullptr;
    uint32_t* halt = nullptr;
};
struct spmm_scratch {
    uint32_t nslots = 0;
    double* cal_val = nullptr;   // [nslots * 32] k-vector fragments of the warp runs
    uint32_t* cal_row = nullptr; // [nslots] their rows
    uint32_t* flag = nullptr;    // [nslots] (launch epoch << 2) | fragment kind
    double* dot_part = nullptr;  // [nslots * 32] per-CTA partials of the per-column dots
    uint32_t* counter = nullptr; // [4] ticket, -, run counter, launch epoch
    uint32_t* status = nullptr;
};
int prepare_spmm_kernels();
uint32_t spmm_max_slots(const dimgpu_csr5* m);
int spmm_scratch_init(spmm_scratch* s, const dimgpu_csr5* m);
void spmm_scratch_release(spmm_scratch* s);
int launch_spmm(const dimgpu_csr5* m, bool f32, const spmm_args& a, const spmm_scratch& sc, int shape,
                cudaStream_t st);
bool spmm_shape_applies(bool f32, const spmm_args& a, int shape);
int autotune_spmm(const dimgpu_csr5* m, bool f32, const spmm_args& a, const spmm_scratch& sc, cudaStream_t st,
                  int* best_shape, float* best_ms);

// api.cu: deterministic dot product into device memory (d_part holds 256 partials)
int dot_device(uint64_t n, const double* a, const double* b, double* d_out, double* d_part, cudaStream_t s);

int device_sm_count(int device);

}  // namespace dimgpu
