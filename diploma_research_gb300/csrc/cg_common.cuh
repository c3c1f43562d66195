// cg_common.cuh -- state shared by the CG drivers: the graph-driven kernels (cg.cu) and the persistent
// cooperative kernel (cg_fused.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

struct dimgpu_csr5;

namespace dimgpu {

// Device-resident state of one solve (written by the kernels, read back by the host at the end).
struct cg_state {
    double rr;       // r.r of the current residual
    double rr_new;   // r.r after this iteration's update
    double alpha, beta;
    double dot;      // s.As
    double thresh2;  // (tol ||b||)^2
    double bb;       // b.b
    double maxrr;    // mixed: largest r.r since the last reliable update
    double delta2;   // mixed: reliable_delta^2
    double rr_true;  // last true residual r.r (f64)
    int64_t iter, max_it, ru_count;
    uint32_t stop;       // the solve has finished
    uint32_t x_pending;  // f64: kernel C owes x += alpha s
    uint32_t no_ru;      // mixed: no reliable update this iteration (guards its kernels)
    uint32_t converged;
};

// Everything the persistent CG kernel touches.  The matrix is in the device layout (omega = 32,
// sigma = 16); the f32 fields are used by the mixed solver only.
struct cg_fused_args {
    // matrix
    const double* vals;
    const float* vals32;
    const uint32_t* col;
    const uint32_t* desc;
    const uint32_t* tile_ptr;
    const uint32_t* tdo_ptr;
    const uint32_t* tdo;
    const uint32_t* row_ptr;
    uint64_t T;
    uint32_t rows;
    uint32_t tail_start;
    uint64_t tpw;        // tiles per warp
    uint32_t nwarps;     // grid * warps per CTA
    uint32_t tail_warp;  // the warp that owns the last tile and computes the CSR tail
    int keep_matrix;     // the matrix stays in L2 between products
    // vectors (n = rows)
    const double* b;
    double *x, *r, *s, *As, *Ax;
    float *r32, *s32, *As32, *y32;
    // scratch
    double* cal_val;    // [nwarps] each warp's head fragment
    uint32_t* cal_row;  // [nwarps] its row | kDirty when valid
    uint32_t* flag;     // [nwarps] (phase << 1) | through, published after the warp's tiles
    double* part;       // [3][grid][2] per-CTA partial sums
    uint32_t* bar;      // grid barrier: [0] arrivals, [32] generation
    uint32_t* status;
    cg_state* st;
    // parameters
    double tol2, delta2;
    int64_t max_it;
    int mixed;
    int grid;
};

// cg_fused.cu: the grid the persistent kernel runs with on this matrix's device (an error when the device
// cannot run it), the number of warps of that grid, and the launch.
int cg_fused_grid(const struct ::dimgpu_csr5* m, int* grid);
uint32_t cg_fused_warps(int grid);
int launch_cg_fused(const cg_fused_args& a, cudaStream_t stream);

}  // namespace dimgpu
