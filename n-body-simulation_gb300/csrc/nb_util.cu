// nb_util.cu -- FMA throughput probe: the measured FP64 / FP32 pipe peaks that the pair and
// traversal kernels are reported against (the HBM peak comes from a copy, measured elsewhere).
#include "nb_internal.cuh"

namespace {

constexpr int PROBE_THREADS = 256;
constexpr int PROBE_CHAINS = 8;

template <typename T>
__global__ void __launch_bounds__(PROBE_THREADS) fma_probe_kernel(T* out, T s, int iters) {
    T a[PROBE_CHAINS];
#pragma unroll
    for (int i = 0; i < PROBE_CHAINS; ++i) a[i] = (T)(threadIdx.x * 1e-3 + i);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < PROBE_CHAINS; ++i) a[i] = fma(a[i], s, (T)1e-9);
    }
    T r = 0;
#pragma unroll
    for (int i = 0; i < PROBE_CHAINS; ++i) r += a[i];
    out[blockIdx.x * PROBE_THREADS + threadIdx.x] = r;
}

template <typename T>
nb_status probe(nb_ctx* ctx, int iters, double* flops) {
    const int blocks = ctx->sm_count * 8;
    T* out = nullptr;
    NB_CUDA_TRY(cudaMalloc(&out, (size_t)blocks * PROBE_THREADS * sizeof(T)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_probe_kernel<T><<<blocks, PROBE_THREADS>>>(out, (T)0.999, iters);  // warm-up
    cudaEventRecord(e0);
    fma_probe_kernel<T><<<blocks, PROBE_THREADS>>>(out, (T)0.999, iters);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return nb::cuda_error(e, "fma probe");
    const double fma_count = (double)blocks * PROBE_THREADS * PROBE_CHAINS * iters;
    *flops = 2.0 * fma_count / (ms * 1e-3);
    return NB_OK;
}

}  // namespace

extern "C" {

nb_status nb_util_fma_peak(nb_ctx* ctx, int fp64, double* flops_per_s) {
    NB_CHECK_CTX(ctx);
    if (!flops_per_s) return nb::set_error(NB_ERR_INVALID_ARG, "nb_util_fma_peak: null output");
    NB_CUDA_TRY(cudaSetDevice(ctx->device));
    return fp64 ? probe<double>(ctx, 2048, flops_per_s) : probe<float>(ctx, 16384, flops_per_s);
}

}  // extern "C"
