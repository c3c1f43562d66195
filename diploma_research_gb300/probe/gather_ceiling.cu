// gather_ceiling.cu -- the random-gather ceiling that bounds an SpMV whose columns have no locality.
//
// A measurement library for bench.py (libdimgpu_probe.so); the product library does not contain it.
// Two gather-only kernels stream an index array (coalesced, evict-first) and sum the entries it selects:
//
//   k_gather_global   x in global memory (L2-resident when it fits): one L2 sector request per index
//                     whose sector is not in L1 -- the access pattern of the SpMV's x gathers with the
//                     matrix values and the row bookkeeping taken away;
//   k_gather_cluster  x spread over the shared memory of the CTAs of a thread-block cluster (words
//                     [r W, (r + 1) W) in CTA r), each index read from its owner's shared memory through
//                     the cluster's distributed shared memory, or (local) from the reading CTA's own.
//
// Each call times `reps` launches with CUDA events on the caller's stream after three untimed ones and
// returns the mean launch time.  Indices are clamped to the gathered span, so any index array is safe.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace cg = cooperative_groups;

namespace {

constexpr int kThreads = 1024;
constexpr int kUnroll = 8;                   // independent gathers in flight per thread
constexpr uint32_t kWordsPerCta = 48 * 1024; // 192 KB of f32 per CTA in the cluster kernel

template <typename T, bool BYPASS_L1>
__global__ void __launch_bounds__(kThreads, 2)
    k_gather_global(const uint32_t* __restrict__ idx, uint64_t n, const T* __restrict__ x, uint32_t span,
                    T* __restrict__ out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    T acc = 0;
    uint64_t j = t0;
    for (; j + (kUnroll - 1) * stride < n; j += kUnroll * stride) {
        uint32_t q[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            q[u] = min(__ldcs(idx + j + u * stride), span - 1);
        T g[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            g[u] = BYPASS_L1 ? __ldcg(x + q[u]) : __ldg(x + q[u]);
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            acc += g[u];
    }
    for (; j < n; j += stride)
        acc += __ldg(x + min(__ldcs(idx + j), span - 1));
    out[t0] = acc;
}

template <bool LOCAL>
__global__ void __launch_bounds__(kThreads, 1)
    k_gather_cluster(const uint32_t* __restrict__ idx, uint64_t n, float* __restrict__ out) {
    extern __shared__ float sx[];
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t rank = cl.block_rank();
    for (uint32_t i = threadIdx.x; i < kWordsPerCta; i += blockDim.x)
        sx[i] = (float)(rank * kWordsPerCta + i) * 1e-7f;
    cl.sync();
    const uint32_t span = LOCAL ? kWordsPerCta : cl.num_blocks() * kWordsPerCta;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float acc = 0.f;
    auto at = [&](uint32_t q) -> float {
        if (LOCAL)
            return sx[q];
        return *cl.map_shared_rank(sx + q % kWordsPerCta, q / kWordsPerCta);
    };
    uint64_t j = t0;
    for (; j + (kUnroll - 1) * stride < n; j += kUnroll * stride) {
        uint32_t q[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            q[u] = min(__ldcs(idx + j + u * stride), span - 1);
        float g[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            g[u] = at(q[u]);
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            acc += g[u];
    }
    for (; j < n; j += stride)
        acc += at(min(__ldcs(idx + j), span - 1));
    out[t0] = acc;
    cl.sync();  // no CTA leaves while another may still read its shared memory
}

template <typename F>
int time_launches(F&& launch, int reps, cudaStream_t stream, float* us) {
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t e = cudaEventCreate(&a);
    if (e == cudaSuccess)
        e = cudaEventCreate(&b);
    for (int i = 0; i < 3 && e == cudaSuccess; ++i)
        e = launch();
    if (e == cudaSuccess)
        e = cudaEventRecord(a, stream);
    for (int i = 0; i < reps && e == cudaSuccess; ++i)
        e = launch();
    if (e == cudaSuccess)
        e = cudaEventRecord(b, stream);
    if (e == cudaSuccess)
        e = cudaEventSynchronize(b);
    float ms = 0.f;
    if (e == cudaSuccess)
        e = cudaEventElapsedTime(&ms, a, b);
    if (a)
        cudaEventDestroy(a);
    if (b)
        cudaEventDestroy(b);
    *us = ms * 1e3f / (float)(reps > 0 ? reps : 1);
    return (int)e;
}

}  // namespace

extern "C" {

__attribute__((visibility("default"))) uint32_t dimgpu_probe_words_per_cta(void) { return kWordsPerCta; }

// Gathers x[idx[i]] for i < n from global memory (elem_bytes 4: f32, 8: f64; bypass_l1: ld.global.cg).
// Returns 0 or a CUDA error code; *us = mean launch time.
__attribute__((visibility("default"))) int dimgpu_probe_gather(const uint32_t* idx, uint64_t n, const void* x,
                                                               uint32_t x_len, int elem_bytes, int bypass_l1,
                                                               int reps, cudaStream_t stream, float* us) {
    if (!idx || !x || !us || x_len == 0 || (elem_bytes != 4 && elem_bytes != 8))
        return (int)cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess)
        return (int)e;
    const int grid = 2 * sms;
    void* out = nullptr;
    if ((e = cudaMalloc(&out, (size_t)grid * kThreads * 8)) != cudaSuccess)
        return (int)e;
    auto launch = [&]() -> cudaError_t {
        if (elem_bytes == 8) {
            if (bypass_l1)
                k_gather_global<double, true><<<grid, kThreads, 0, stream>>>(idx, n, (const double*)x, x_len,
                                                                             (double*)out);
            else
                k_gather_global<double, false><<<grid, kThreads, 0, stream>>>(idx, n, (const double*)x, x_len,
                                                                              (double*)out);
        } else {
            if (bypass_l1)
                k_gather_global<float, true><<<grid, kThreads, 0, stream>>>(idx, n, (const float*)x, x_len,
                                                                            (float*)out);
            else
                k_gather_global<float, false><<<grid, kThreads, 0, stream>>>(idx, n, (const float*)x, x_len,
                                                                             (float*)out);
        }
        return cudaGetLastError();
    };
    const int rc = time_launches(launch, reps, stream, us);
    cudaFree(out);
    return rc;
}

// Gathers over the shared memory of clusters of `cluster` CTAs (kWordsPerCta f32 words each), as many
// clusters as fit the GPU at once; local != 0 reads the reading CTA's own shared memory only.
// *ctas = CTAs launched.  Returns 0 or a CUDA error code (cudaErrorInvalidConfiguration: no cluster fits).
__attribute__((visibility("default"))) int dimgpu_probe_cluster_gather(const uint32_t* idx, uint64_t n,
                                                                       int cluster, int local, int reps,
                                                                       cudaStream_t stream, float* us, int* ctas) {
    if (!idx || !us || !ctas || cluster < 1 || cluster > 16)
        return (int)cudaErrorInvalidValue;
    const size_t smem = (size_t)kWordsPerCta * sizeof(float);
    void* fn = local ? (void*)k_gather_cluster<true> : (void*)k_gather_cluster<false>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess)
        return (int)e;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)cluster);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if ((e = cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg)) != cudaSuccess)
        return (int)e;
    if (clusters < 1)
        return (int)cudaErrorInvalidConfiguration;
    cfg.gridDim = dim3((unsigned)(clusters * cluster));
    *ctas = clusters * cluster;
    float* out = nullptr;
    if ((e = cudaMalloc(&out, (size_t)clusters * cluster * kThreads * sizeof(float))) != cudaSuccess)
        return (int)e;
    auto launch = [&]() -> cudaError_t {
        return local ? cudaLaunchKernelEx(&cfg, k_gather_cluster<true>, idx, n, out)
                     : cudaLaunchKernelEx(&cfg, k_gather_cluster<false>, idx, n, out);
    };
    const int rc = time_launches(launch, reps, stream, us);
    cudaFree(out);
    return rc;
}

}  // extern "C"
