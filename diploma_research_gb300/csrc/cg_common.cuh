// cg_common.cuh -- the device-resident state of one CG solve, shared by the CG kernels (cg.cu) and the
// SpMV epilogue that computes the step lengths (spmv.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

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
    double rr_prev;  // merged engine: r.r of the previous residual
    int64_t iter, max_it, ru_count;
    uint32_t stop;       // the solve has finished
    uint32_t x_pending;  // f64: kernel C owes x += alpha s
    uint32_t no_ru;      // mixed: no reliable update this iteration (guards its kernels)
    uint32_t converged;
};

// Step lengths of the merged (Chronopoulos-Gear) recurrence, computed by the SpMV's last CTA once
// delta = r.w (w = A r) is known, with gamma = r.r from the vector kernel before it:
//   first iteration  beta = 0, alpha = gamma / delta
//   otherwise        beta = gamma / gamma_prev, alpha = gamma / (delta - beta gamma / alpha_prev)
// The denominator is p.Ap of the new direction; a non-positive or non-finite one is a breakdown (the
// matrix is not SPD), which stops the solve.
__device__ __forceinline__ void merged_step_lengths(cg_state* st, double delta, uint32_t* status) {
    const double gamma = st->rr;
    double beta = 0.0, denom = delta;
    if (st->iter > 0) {
        beta = gamma / st->rr_prev;
        denom = delta - beta * gamma / st->alpha;
    }
    if (!(denom > 0.0) || !isfinite(denom)) {
        record_status(status, kStatusBreakdown);
        st->stop = 1u;
        st->alpha = 0.0;
        st->beta = 0.0;
        return;
    }
    st->beta = beta;
    st->alpha = gamma / denom;
    st->dot = delta;
}

}  // namespace dimgpu
