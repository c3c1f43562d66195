// common.cuh -- shared device helpers for the dimgpu CSR5 library (sm_103a only).
//
// Bulk copies (TMA engine, cp.async.bulk), mbarriers with bounded waits, L2 cache policies,
// warp helpers and the device-side error word.  Every wait in this library is bounded: after
// DIMGPU_WAIT_NS of global time a wait records an error code in the device status word and
// returns false; the caller then drains what it issued and leaves.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ < 1000)
#error "dimgpu is written for Blackwell (sm_103a); build with -gencode arch=compute_103a,code=sm_103a"
#endif

namespace dimgpu {

// ------------------------------------------------------------------------------------------------
// Status word written by device code when a bounded wait runs out or an index check fails.
// ------------------------------------------------------------------------------------------------
enum device_status : uint32_t {
    kStatusOk = 0,
    kStatusWaitTimeout = 1,   // an mbarrier wait exceeded its limit
    kStatusBadIndex = 2,      // a bounds check on an index read from the matrix failed
    kStatusBreakdown = 3,     // CG: s.As <= 0 or not finite
};

#ifndef DIMGPU_WAIT_NS
#define DIMGPU_WAIT_NS 2000000000ull  // 2 s of global time per wait, far beyond any legitimate wait
#endif

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void record_status(uint32_t* status, uint32_t code) {
    if (status)
        atomicCAS(status, 0u, code);
}

// ------------------------------------------------------------------------------------------------
// Shared-memory addresses and mbarriers.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on phase `parity`.  Returns false (and records kStatusWaitTimeout) on expiry.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t* status) {
    if (mbar_try_wait(bar, parity))
        return true;
    const uint64_t t0 = global_ns();
    while (true) {
        for (int i = 0; i < 64; ++i)
            if (mbar_try_wait(bar, parity))
                return true;
        if (global_ns() - t0 > DIMGPU_WAIT_NS) {
            record_status(status, kStatusWaitTimeout);
            return false;
        }
    }
}

// ------------------------------------------------------------------------------------------------
// Decoupled look-back between warp runs (spmv.cu, spmm.cu): each run release-stores a flag word
// (launch epoch << 2 | fragment kind) after publishing the row fragment a later run needs.
// ------------------------------------------------------------------------------------------------
constexpr uint32_t kFragNone = 0, kFragCarry = 1, kFragThrough = 2;

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Completion ticket: adds 1 to *p with acquire-release semantics at GPU scope and returns the old value.
// Called by one thread after a __syncthreads(): the block's earlier writes are released with it, and
// the block that draws the last ticket has acquired every earlier block's writes once it passes its next
// __syncthreads() (no separate fences on either side).
__device__ __forceinline__ uint32_t ticket_acq_rel(uint32_t* p) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

// Bounded wait for run k's flag of this launch; returns its fragment kind, or kFragNone after recording
// kStatusWaitTimeout.  Polls without acquire (no cache invalidation per poll), then one acquire.
__device__ __forceinline__ uint32_t wait_run(const uint32_t* flag, uint32_t epoch, uint32_t* status) {
    if ((ld_relaxed_u32(flag) >> 2) != epoch) {
        const uint64_t t0 = global_ns();
        while ((ld_relaxed_u32(flag) >> 2) != epoch) {
            if (global_ns() - t0 > DIMGPU_WAIT_NS) {
                record_status(status, kStatusWaitTimeout);
                return kFragNone;
            }
        }
    }
    return ld_acquire_u32(flag) & 3u;
}

// ------------------------------------------------------------------------------------------------
// L2 cache policies and the 1-D bulk copy global -> shared (TMA engine).
// Addresses must be 16-byte aligned and the size a multiple of 16 bytes.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ uint64_t policy_evict_normal() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ uint64_t policy_evict_last() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ void bulk_g2s(void* smem_dst, const void* gmem_src, uint32_t bytes, uint64_t* bar,
                                         uint64_t policy) {
    asm volatile(
        "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            smem_u32(smem_dst)),
        "l"(gmem_src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

// ------------------------------------------------------------------------------------------------
// Loads with explicit cache behaviour.
// ------------------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T ldg_keep(const T* p);  // read-only, keep in L2 (the gathered vector)

template <>
__device__ __forceinline__ double ldg_keep<double>(const double* p) {
    double v;
    asm volatile("ld.global.nc.L1::evict_last.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}
template <>
__device__ __forceinline__ float ldg_keep<float>(const float* p) {
    float v;
    asm volatile("ld.global.nc.L1::evict_last.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}

// Gathered-vector loads: read-only path, kept in L1 and (by `policy`) in L2.
__device__ __forceinline__ double ldg_x(const double* p, uint64_t policy) {
    double v;
    asm("ld.global.nc.L1::evict_last.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(policy));
    return v;
}
__device__ __forceinline__ float ldg_x(const float* p, uint64_t policy) {
    float v;
    asm("ld.global.nc.L1::evict_last.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(policy));
    return v;
}

// Read-only gathers that skip L1 allocation: for matrices whose column indices have no locality (an
// L1 line would be evicted before its next use), keeping L1 free for the stage traffic.
__device__ __forceinline__ double ldg_x_stream(const double* p, uint64_t policy) {
    double v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(policy));
    return v;
}
__device__ __forceinline__ float ldg_x_stream(const float* p, uint64_t policy) {
    float v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(policy));
    return v;
}

// Stores that the next kernel will read: kept in L2 by `policy`.
__device__ __forceinline__ void st_keep(double* p, double v, uint64_t policy) {
    asm volatile("st.global.L2::cache_hint.f64 [%0], %1, %2;" ::"l"(p), "d"(v), "l"(policy) : "memory");
}
__device__ __forceinline__ void st_keep(float* p, float v, uint64_t policy) {
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(policy) : "memory");
}

// 16-byte vector loads of the CG vectors with an L2 policy.  The loads carry no memory
// clobber so that independent loads can be batched; callers never load an element after storing it
// in the same kernel.
__device__ __forceinline__ double2 ld2_keep(const double* p, uint64_t policy) {
    double2 v;
    asm("ld.global.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(p), "l"(policy));
    return v;
}
// Stores of streamed vector elements that order nothing else: volatile (never dropped) but without a
// memory clobber, so the compiler may issue the next elements' loads ahead of them.
__device__ __forceinline__ void st2_stream(double* p, double2 v, uint64_t policy) {
    asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(p), "d"(v.x), "d"(v.y), "l"(policy));
}
__device__ __forceinline__ void st4_stream(float* p, float4 v, uint64_t policy) {
    asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x), "f"(v.y),
                 "f"(v.z), "f"(v.w), "l"(policy));
}
__device__ __forceinline__ float4 ld4_keep(const float* p, uint64_t policy) {
    float4 v;
    asm("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p), "l"(policy));
    return v;
}

// ------------------------------------------------------------------------------------------------
// Warp helpers.
// ------------------------------------------------------------------------------------------------
constexpr unsigned kFull = 0xffffffffu;

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
        v += __shfl_xor_sync(kFull, v, d);
    return v;
}

// Number of doubling steps a 32-lane segmented suffix scan needs when the lanes whose bit is set
// in `present` terminate segments: the smallest s with 2^s > longest run of clear bits.
__device__ __forceinline__ int scan_steps_for(uint32_t present) {
    uint32_t z = ~present;
    if (!z)
        return 0;
    uint32_t r2 = z & (z >> 1);
    if (!r2)
        return 1;
    uint32_t r4 = r2 & (r2 >> 2);
    if (!r4)
        return 2;
    uint32_t r8 = r4 & (r4 >> 4);
    if (!r8)
        return 3;
    uint32_t r16 = r8 & (r8 >> 8);
    if (!r16)
        return 4;
    return 5;
}

}  // namespace dimgpu
