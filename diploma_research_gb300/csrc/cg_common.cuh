// cg_common.cuh -- the device-resident state of one CG solve (cg.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

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

}  // namespace dimgpu
