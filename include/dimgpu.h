/*
 * dimgpu.h -- C ABI of the GB300-native CSR5 library (hand-written sm_103a kernels).
 *
 * The reference ("dim", rurabori/diploma_research) exposes this hot path as the header-only C++
 * template dim::mat::csr5<double,16,4,uint32_t> (include/dim/mat/storage_formats/csr5.h:254-881),
 * the vector helpers of include/dim/vec.h and the CG loops of benchmarks/conjugate_gradient/.  Each
 * entry point below names the reference interface it replaces.
 *
 * Conventions
 *   - Every function returns an int status: DIMGPU_OK (0) or a negative DIMGPU_ERR_* code; the
 *     message of the last failure on the calling thread is dimgpu_last_error_string().  Nothing
 *     throws across this boundary (the reference throws std::invalid_argument, csr5.h:820-821).
 *   - Pointers are plain pointers.  Functions whose name ends in _host take host memory and copy
 *     inside the call; all others take device memory of the current device.
 *   - `stream` is a cudaStream_t passed as void* (NULL = the legacy default stream).
 *   - A matrix handle is immutable after creation.  Scratch for one SpMV lives in a calibrator
 *     (the reference's calibrator_t, csr5/calibrator.h); calls that share a calibrator must not
 *     overlap on the device, calls with different calibrators may.
 *   - Index type u32 (row offsets, column indices), values f64, as csr5<double,16,4,uint32_t>.
 */
#ifndef DIMGPU_H
#define DIMGPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define DIMGPU_API __attribute__((visibility("default")))
#else
#define DIMGPU_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define DIMGPU_OK 0
#define DIMGPU_ERR_INVALID_ARGUMENT (-1) /* bad shape/pointer/option (std::invalid_argument) */
#define DIMGPU_ERR_CUDA (-2)             /* a CUDA runtime call failed */
#define DIMGPU_ERR_OUT_OF_MEMORY (-3)
#define DIMGPU_ERR_TIMEOUT (-4)          /* a bounded device-side wait expired */
#define DIMGPU_ERR_BREAKDOWN (-5)        /* CG: s.As <= 0 or not finite (matrix not SPD) */
#define DIMGPU_ERR_NOT_CONVERGED (-6)    /* CG: max_it reached before the tolerance */
#define DIMGPU_ERR_UNSUPPORTED (-7)
#define DIMGPU_ERR_BAD_INDEX (-8)        /* a device-side bounds check failed */
#define DIMGPU_ERR_IO (-9)               /* a file could not be read or written, or is outside the HDF5 subset */

typedef struct dimgpu_csr5 dimgpu_csr5;             /* device CSR5 matrix */
typedef struct dimgpu_calibrator dimgpu_calibrator; /* scratch of one SpMV at a time */
typedef struct dimgpu_cg_solver dimgpu_cg_solver;   /* CG workspace + captured CUDA graph */

typedef enum { DIMGPU_MEM_HOST = 0, DIMGPU_MEM_DEVICE = 1 } dimgpu_mem_kind;

/* Element order inside re-ordered tiles (see layout.cuh). */
typedef enum { DIMGPU_LAYOUT_REFERENCE = 0, DIMGPU_LAYOUT_DEVICE = 1 } dimgpu_layout;

typedef struct {
    uint32_t sigma;  /* rows per tile column; 0 = 16 */
    uint32_t omega;  /* lanes per tile: 32 for the device layout, 4 for the reference layout; 0 = 32 */
    int32_t layout;  /* dimgpu_layout; ignored (device) when omega == 32 */
    uint32_t flags;  /* reserved, 0 */
} dimgpu_csr5_options;

typedef struct {
    uint32_t rows, cols;
    uint64_t nnz;
    uint32_t sigma, omega;
    int32_t layout;
    uint32_t desc_word_bytes;      /* 4 or 8 */
    uint64_t tile_count;           /* csr5_info_t::tile_count (csr5.h:289) */
    uint64_t tile_desc_offset_len; /* tile_desc_offset.size() */
    uint32_t tail_partition_start; /* csr5::tail_partition_start() (csr5.h:806) */
    uint32_t empty_rows;           /* empty rows below tail_partition_start */
    uint64_t device_bytes;         /* HBM held by the handle */
} dimgpu_csr5_info;

/* ---- matrices --------------------------------------------------------------------------------- */

/* csr5::from_csr (csr5.h:791-803): builds the CSR5 arrays on the device from a CSR matrix held in
 * host (mem = DIMGPU_MEM_HOST) or device memory.  The handle owns device copies.  opt may be NULL. */
DIMGPU_API int dimgpu_csr5_from_csr(uint32_t rows, uint32_t cols, uint64_t nnz, const uint32_t* row_ptr,
                         const uint32_t* col_idx, const double* vals, int mem, const dimgpu_csr5_options* opt,
                         void* stream, dimgpu_csr5** out);

DIMGPU_API int dimgpu_csr5_destroy(dimgpu_csr5* m);

/* tile_count, tail_partition_start, non_zero_count (csr5.h:289, 806, 880) and sizes. */
DIMGPU_API int dimgpu_csr5_get_info(const dimgpu_csr5* m, dimgpu_csr5_info* out);

/* Copies the CSR5 arrays (csr5_info_t members, csr5.h:287-294, and csr5::vals/col_idx/row_ptr,
 * csr5.h:450-453) to host buffers sized from dimgpu_csr5_get_info.  tile_desc receives
 * tile_count*omega words of desc_word_bytes each.  Any pointer may be NULL to skip that array. */
DIMGPU_API int dimgpu_csr5_export(const dimgpu_csr5* m, uint32_t* tile_ptr, void* tile_desc, uint32_t* tile_desc_offset_ptr,
                       uint32_t* tile_desc_offset, double* vals, uint32_t* col_idx, uint32_t* row_ptr);

/* ---- SpMV ------------------------------------------------------------------------------------- */

/* csr5::create_calibrator (csr5.h:809): scratch for one SpMV at a time on this matrix. */
DIMGPU_API int dimgpu_calibrator_create(const dimgpu_csr5* m, dimgpu_calibrator** out);
DIMGPU_API int dimgpu_calibrator_destroy(dimgpu_calibrator* c);

/* csr5::spmv(spmv_data_t{x, y, calibrator}) (csr5.h:280-285, 818-829): y := A x.  y is overwritten
 * (empty rows get 0), so neither a zero-filled y nor a fresh calibrator is needed.  cal may be
 * NULL (the matrix's own calibrator; then calls on this matrix must not overlap).  x has cols
 * elements, y rows elements, both device memory.  Requires a device-layout matrix (omega = 32). */
DIMGPU_API int dimgpu_csr5_spmv(const dimgpu_csr5* m, const double* x, double* y, dimgpu_calibrator* cal, void* stream);

/* y := A x and *dot := x.y = x'Ax (the energy product CG needs) in one pass, for a square matrix.
 * dot is device memory; the sum is taken in a fixed order (bit-reproducible). */
DIMGPU_API int dimgpu_csr5_spmv_dot(const dimgpu_csr5* m, const double* x, double* y, double* dot,
                                    dimgpu_calibrator* cal, void* stream);

/* The same product with host x and y: copies x in, multiplies, copies y out, synchronizes. */
DIMGPU_API int dimgpu_csr5_spmv_host(const dimgpu_csr5* m, const double* x_host, double* y_host);

/* y := A x with f32 values, vectors and row sums (the inner kernel of the mixed-precision CG).
 * The first f32 use of a matrix (this call, an f32 SpMM, a mixed-precision solver, or
 * dimgpu_csr5_get_spmv_launch with f32) builds an f32 copy of the values inside the handle and times
 * the f32 launch configurations; it synchronizes, so make it outside stream capture. */
DIMGPU_API int dimgpu_csr5_spmv_f32(const dimgpu_csr5* m, const float* x, float* y, dimgpu_calibrator* cal, void* stream);

/* The SpMV launch configuration of this matrix: warps per CTA and how the x gathers load
 * (DIMGPU_GATHER_L1: kept in L1; DIMGPU_GATHER_STREAM: past L1).  The library chooses them by timing,
 * at conversion for the f64 product and when the f32 values are made for the f32 product (f32 != 0;
 * get makes them if needed).  Fewer warps leave more of the SM to L1, which helps matrices whose
 * gathers revisit a small part of x.  No reference counterpart (the reference's OpenMP SpMV has no
 * launch configuration). */
#define DIMGPU_GATHER_L1 0
#define DIMGPU_GATHER_STREAM 1
DIMGPU_API int dimgpu_csr5_get_spmv_launch(const dimgpu_csr5* m, int f32, uint32_t* warps_per_cta, int* gather);
/* Pins it (f64: 16 or 12 warps per CTA; f32: 24 or 20), e.g. for reproducible timings.  Calibrators
 * made before stay valid.  Must not overlap with products on the matrix in flight. */
DIMGPU_API int dimgpu_csr5_set_spmv_launch(dimgpu_csr5* m, int f32, uint32_t warps_per_cta, int gather);

/* y := A x like dimgpu_csr5_spmv, but neither this call nor the library allocates anything: the
 * scratch (per-warp row fragments, completion ticket, status word) is a fixed array of 98,816 bytes
 * compiled into the library, present on every GPU that loads it until the process exits.  It has no
 * counterpart in the reference; it exists for callers that cannot allocate device memory when they
 * multiply (a plugin whose host reserved all device memory, a latency-bound loop that cannot afford
 * cudaMalloc's implicit synchronisation, code whose footprint must not grow after start-up).
 *   - Limit: matrices whose SpMV launch uses more than 4096 warp slots (more than 256 SMs x 16
 *     warps) are rejected with DIMGPU_ERR_INVALID_ARGUMENT.
 *   - The first call on a device looks up the array's device address (cudaGetSymbolAddress) with
 *     that device current, and so does the first call in a new context of that device (after
 *     cudaDeviceReset, for instance); make that first call before any stream capture.
 *   - Every call on a device shares the one array: calls that overlap on the GPU (different streams,
 *     or concurrent graph branches) race and give wrong results.  Calls in one stream are safe.
 *   - A device-side failure (an expired bounded wait, an inconsistent format) is kept in the array's
 *     status word, which calls do not clear; dimgpu_static_scratch_status reads and clears it.
 *   - x, y: device memory of the matrix's device (the current device).  The call is asynchronous. */
DIMGPU_API int dimgpu_csr5_spmv_static_scratch(const dimgpu_csr5* m, const double* x, double* y, void* stream);

/* ---- device-side failures of asynchronous calls ------------------------------------------------ */

/* The asynchronous entry points (dimgpu_csr5_spmv, _spmv_dot, _spmv_f32, _spmm, _spmm_f32,
 * _spmv_transpose) return before their kernels run.  A kernel that meets a failure -- a bounded device
 * wait that expired, or a consistency check on the CSR5 arrays that failed -- records it in the status
 * word of the scratch it ran on and leaves its outputs invalid.  These calls synchronize `stream`, then
 * read and clear that word: DIMGPU_OK (no failure since the last query), DIMGPU_ERR_TIMEOUT or
 * DIMGPU_ERR_BAD_INDEX.  The reference reports its failures synchronously by exception
 * (std::invalid_argument, csr5.h:820-821); the _host entry points and the CG solvers read the word
 * themselves and return the code directly.
 *
 * cal != NULL: the calibrator the products ran on.  cal == NULL: the scratch matrix m owns (its own
 * calibrator, used when a product is given cal = NULL; its SpMM scratch; those of its cached A^T). */
DIMGPU_API int dimgpu_csr5_status(const dimgpu_csr5* m, dimgpu_calibrator* cal, void* stream);
/* The same for the static scratch of dimgpu_csr5_spmv_static_scratch on the current device. */
DIMGPU_API int dimgpu_static_scratch_status(void* stream);

/* ---- several right-hand sides ------------------------------------------------------------------- */

/* Y := A X for k right-hand sides (the batched form of csr5::spmv): X is cols x k, Y rows x k,
 * both row-major with leading dimensions ldx, ldy >= k (device memory).  k > 32 runs in passes of 32
 * columns.  The first call for a given (k, precision) times the candidate launch shapes on these
 * operands and keeps the fastest (make it outside any stream capture).  Calls on one matrix must not
 * overlap on the device (they share the matrix's SpMM scratch). */
DIMGPU_API int dimgpu_csr5_spmm(const dimgpu_csr5* m, uint32_t k, const double* X, uint64_t ldx, double* Y,
                                uint64_t ldy, void* stream);
DIMGPU_API int dimgpu_csr5_spmm_f32(const dimgpu_csr5* m, uint32_t k, const float* X, uint64_t ldx, float* Y,
                                    uint64_t ldy, void* stream);
/* The shape the autotuner picked for (k, f32), -1 before the first call.  Bit 0 is the launch shape
 * (0: 8 warps x 3 stages, 1: 16 x 2); bits 1-2 the lane grouping g: each lane holds w >> g right-hand
 * sides, w being the widest the operands allow (f32: 4 or 2 when k and the leading dimensions are
 * multiples of it and X, Y are aligned to it, else 1; FP64: 1), so g = 0 the widest, 1 half of it, 2 a
 * quarter.  No reference counterpart (the reference has no SpMM). */
DIMGPU_API int dimgpu_csr5_spmm_shape(const dimgpu_csr5* m, uint32_t k, int f32, int* shape);
/* Pins the shape for (k, f32) (0..5; -1 re-tunes on the next call), e.g. for reproducible timings.  A
 * grouping the operands cannot use falls back to grouping 0 with the same launch shape. */
DIMGPU_API int dimgpu_csr5_set_spmm_shape(dimgpu_csr5* m, uint32_t k, int f32, int shape);

/* ---- vectors (include/dim/vec.h:29-84), device memory ----------------------------------------- */

DIMGPU_API int dimgpu_vec_axpy(uint64_t n, double alpha, const double* x, double* y, void* stream); /* y += a x */
DIMGPU_API int dimgpu_vec_aypx(uint64_t n, double alpha, const double* x, double* y, void* stream); /* y = x + a y */
DIMGPU_API int dimgpu_vec_set(uint64_t n, double value, double* y, void* stream);
/* dot(l, r) (vec.h:78-84); deterministic order; result written to host *out (synchronizes). */
DIMGPU_API int dimgpu_vec_dot(uint64_t n, const double* l, const double* r, double* out, void* stream);

/* ---- CG (benchmarks/conjugate_gradient/dim_sp/main.cpp:78-141; docs/paper/thesis.tex:2127-2160) */

#define DIMGPU_CG_FP64 0  /* f64 everywhere */
#define DIMGPU_CG_MIXED 1 /* f32 values/vectors inside, f64 dots, f64 x and reliable f64 residual updates */

typedef struct {
    double tol;        /* stop when ||r|| <= tol * ||b|| */
    int64_t max_it;    /* iteration cap */
    int32_t precision; /* DIMGPU_CG_FP64 or DIMGPU_CG_MIXED */
    int32_t use_graph; /* 0: host-driven loop of kernels; otherwise the engine below */
    double reliable_delta; /* mixed only: replace the residual when it dropped by this factor; 0 = 0.03 (CG), 0.1 (block CG) */
    int32_t engine;    /* DIMGPU_CG_ENGINE_AUTO or _GRAPH: how a solve runs when use_graph != 0 */
} dimgpu_cg_params;

#define DIMGPU_CG_ENGINE_AUTO 0   /* the library's choice: the graph */
#define DIMGPU_CG_ENGINE_GRAPH 1  /* one CUDA graph per solve, the reference's recurrence: 3 kernels per iteration
                                     (SpMV + s.As, r update + r.r, x and s updates) in a device-side loop */

typedef struct {
    int64_t iterations;      /* CG iterations (inner iterations for the mixed solver) */
    int64_t reliable_updates; /* f64 residual replacements (mixed) */
    double rel_residual;      /* ||b - A x|| / ||b|| recomputed in f64 at the end */
    double recurrence_rel_residual; /* sqrt(r.r)/||b|| of the recurrence at exit */
    double seconds;           /* device time of the solve (CUDA events) */
    int32_t status;           /* DIMGPU_OK, _NOT_CONVERGED or _BREAKDOWN */
} dimgpu_cg_stats;

/* Allocates the CG workspace for matrix m (and, with use_graph, captures the solve graph). */
DIMGPU_API int dimgpu_cg_create(const dimgpu_csr5* m, const dimgpu_cg_params* params, void* stream, dimgpu_cg_solver** out);
DIMGPU_API int dimgpu_cg_destroy(dimgpu_cg_solver* s);
/* Solves A x = b from the initial guess in x (device memory).  Returns the solve status. */
DIMGPU_API int dimgpu_cg_solve(dimgpu_cg_solver* s, const double* b, double* x, dimgpu_cg_stats* stats, void* stream);
/* The same with host b and x (copies in and out inside the call). */
DIMGPU_API int dimgpu_cg_solve_host(dimgpu_cg_solver* s, const double* b_host, double* x_host, dimgpu_cg_stats* stats);

/* ---- block CG: k <= 32 right-hand sides, one SpMM per iteration -------------------------------- */

typedef struct dimgpu_block_cg dimgpu_block_cg;

typedef struct {
    int64_t iterations;       /* iterations of the slowest column */
    int64_t reliable_updates; /* batched f64 residual replacements (mixed) */
    double max_rel_residual;  /* max over columns of ||b_j - A x_j|| / ||b_j|| (f64, recomputed) */
    double seconds;           /* device time of the solve */
    int32_t converged_columns;
    int32_t status;           /* DIMGPU_OK, _NOT_CONVERGED or _BREAKDOWN */
    int32_t spmm_shape;       /* the autotuned shape of the iteration's SpMM (f32 for MIXED), as dimgpu_csr5_spmm_shape */
    int32_t reserved;
} dimgpu_block_cg_stats;

/* k simultaneous CG solves (the dim_sp recurrence per column, its own alpha_j/beta_j) sharing one
 * CSR5 SpMM per iteration; a column stops when it converges (per-column mask).  params as for
 * dimgpu_cg_create (precision FP64 or MIXED; engine AUTO or GRAPH).  Autotunes the SpMM shape (launch
 * shape and lane grouping) on its own blocks on creation. */
DIMGPU_API int dimgpu_block_cg_create(const dimgpu_csr5* m, uint32_t k, const dimgpu_cg_params* params,
                                      void* stream, dimgpu_block_cg** out);
DIMGPU_API int dimgpu_block_cg_destroy(dimgpu_block_cg* s);
/* B: n x k (leading dimension ldb), X: n x k initial guesses -> solutions (ldx); device memory.
 * col_iterations / col_rel_residual: optional host arrays of k entries. */
DIMGPU_API int dimgpu_block_cg_solve(dimgpu_block_cg* s, const double* B, uint64_t ldb, double* X, uint64_t ldx,
                                     dimgpu_block_cg_stats* stats, int64_t* col_iterations,
                                     double* col_rel_residual, void* stream);

/* ---- differentiation (adjoint of x = A^{-1} b; no counterpart in the reference) ----------------- */

/* A new handle holding A^T (deterministic: rows of A^T keep increasing column order). */
DIMGPU_API int dimgpu_csr5_transpose(const dimgpu_csr5* m, void* stream, dimgpu_csr5** out);
/* y := A^T x (x: rows, y: cols; device memory).  Builds A^T inside m on first use. */
DIMGPU_API int dimgpu_csr5_spmv_transpose(const dimgpu_csr5* m, const double* x, double* y, void* stream);
/* out[e] := scale * u[row(e)] * v[col(e)] for every stored element e, in the CSR order of the matrix
 * given to dimgpu_csr5_from_csr (with scale = -1, u = lambda, v = x: dL/dA on the pattern). */
DIMGPU_API int dimgpu_csr5_pattern_outer(const dimgpu_csr5* m, const double* u, const double* v, double scale,
                                         double* out, void* stream);
/* Adjoint CG: lambda := A^{-T} g by CG on A^T (lambda holds the initial guess on entry; dL/db = lambda),
 * then grad_vals := -lambda x^T on the pattern (dL/dA, CSR order; grad_vals may be NULL).  Returns the
 * solve status (DIMGPU_OK or _NOT_CONVERGED). */
DIMGPU_API int dimgpu_cg_adjoint(const dimgpu_csr5* m, const double* g, const double* x, double* lambda,
                                 double* grad_vals, const dimgpu_cg_params* params, dimgpu_cg_stats* stats,
                                 void* stream);

/* ---- diagnostics ------------------------------------------------------------------------------ */

/* ---- HDF5 matrix files ------------------------------------------------------------------------
 * The reference's dim::io::h5 (include/dim/io/h5.h:68-115, libs/dim/io/h5.cpp:45-74) on files it
 * writes with libhdf5, without libhdf5: the library reads and writes the part of the HDF5 format those
 * files use (superblock 0/1, version-1 object headers, symbol-table groups, contiguous, compact and
 * chunked 1-D datasets, the deflate filter; files written with libver "latest" are refused) and writes
 * the layout libhdf5's default settings produce.  Host memory only; DIMGPU_ERR_IO on a file that cannot
 * be read or written or lies outside that subset.  A writer with append != 0 keeps the other members
 * of an existing file (it is read, then rewritten through a temporary file). */

/* read_matlab_compatible (h5.h:78-97), first call: the sizes of the MATLAB-compatible CSR group
 * `group` (datasets data, ir, jc; attribute MATLAB_sparse = column count). */
DIMGPU_API int dimgpu_h5_csr_dimensions(const char* path, const char* group, uint32_t* rows, uint32_t* cols,
                                        uint64_t* nnz);
/* read_matlab_compatible, second call: row_ptr (rows + 1), col_indices and values (nnz each) into
 * caller buffers; indices stored in wider integer types are narrowed to u32 (an error if one does not fit). */
DIMGPU_API int dimgpu_h5_read_matlab_compatible(const char* path, const char* group, uint32_t* row_ptr,
                                                uint32_t* col_indices, double* values);
/* write_matlab_compatible (h5.h:68-76): replaces `group` (the whole file unless append). */
DIMGPU_API int dimgpu_h5_write_matlab_compatible(const char* path, const char* group, uint32_t rows, uint32_t cols,
                                                 uint64_t nnz, const uint32_t* row_ptr, const uint32_t* col_indices,
                                                 const double* values, int append);
/* store (h5.cpp:45-55): the reference's CSR5 group of a matrix converted with the reference layout
 * (dimgpu_csr5_options sigma 16, omega 4): attribute column_count; vals, col_idx, row_ptr, tile_ptr,
 * tile_desc (an array type of 4 u32 per tile), tile_desc_offset_ptr, tile_desc_offset. */
DIMGPU_API int dimgpu_h5_store_csr5(const char* path, const char* group, const dimgpu_csr5* m, int append);
/* load_csr5 (h5.cpp:57-74): reads a stored CSR5 group (sigma 16, omega 4), puts its transposed tiles
 * back into CSR order (the inverse of csr5::transpose, csr5.h:463-493) and converts it on the device
 * like dimgpu_csr5_from_csr with `opt` (NULL: the device layout the products run on). */
DIMGPU_API int dimgpu_h5_load_csr5(const char* path, const char* group, const dimgpu_csr5_options* opt, void* stream,
                                   dimgpu_csr5** out);
/* The result vectors of benchmarks/csr5/dim/main.cpp:35-43 (f64 datasets): length, read (converted to
 * f64), write (refused, DIMGPU_ERR_INVALID_ARGUMENT, when the dataset exists unless overwrite). */
DIMGPU_API int dimgpu_h5_vector_length(const char* path, const char* dataset, uint64_t* n);
DIMGPU_API int dimgpu_h5_read_vector(const char* path, const char* dataset, double* y);
DIMGPU_API int dimgpu_h5_write_vector(const char* path, const char* dataset, uint64_t n, const double* y,
                                      int overwrite);

/* ---- Matrix Market files ----------------------------------------------------------------------
 * dim::io::matrix_market::load_as_csr (include/dim/io/matrix_market.h:25-83) without scnlib: a coordinate
 * file (real, integer or pattern -- pattern entries get 1.0; general, symmetric or Hermitian) to CSR the
 * way csr::from_coo builds it (csr.h:42-77): entries in file order, each off-diagonal entry of a symmetric
 * file followed by its mirror (coo.h:33-46), rows sorted by column (stable: equal columns keep file order).
 * First call: the sizes (nnz after the symmetric expansion); second call: the arrays into caller buffers
 * (row_ptr rows + 1, col_indices and values nnz each).  Each call reads the file.  DIMGPU_ERR_INVALID_ARGUMENT
 * for a file that is not a coordinate Matrix Market matrix or whose entries do not scan or lie outside
 * the matrix; DIMGPU_ERR_IO when it cannot be read. */
DIMGPU_API int dimgpu_mm_csr_dimensions(const char* path, uint32_t* rows, uint32_t* cols, uint64_t* nnz);
DIMGPU_API int dimgpu_mm_read_csr(const char* path, uint32_t* row_ptr, uint32_t* col_indices, double* values);

DIMGPU_API const char* dimgpu_last_error_string(void);
/* ABI version of this library (2: status queries, SpMM shapes with lane grouping, no persistent CG engine). */
DIMGPU_API int dimgpu_version(void);

#ifdef __cplusplus
}
#endif

#endif /* DIMGPU_H */
