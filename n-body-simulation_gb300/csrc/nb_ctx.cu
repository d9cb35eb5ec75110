// nb_ctx.cu -- context lifetime, error reporting and scratch memory of libnbody_cuda.so.
#include <cstdarg>
#include <cstring>

#include "nb_internal.cuh"

namespace {
thread_local char g_last_error[512] = "no error";
}

namespace nb {

nb_status set_error(nb_status st, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return st;
}

nb_status cuda_error(cudaError_t err, const char* what) {
    return set_error(err == cudaErrorMemoryAllocation ? NB_ERR_OOM : NB_ERR_CUDA, "%s: %s (%s)",
                     what, cudaGetErrorName(err), cudaGetErrorString(err));
}

nb_status check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, what);
    return NB_OK;
}

nb_status scratch(nb_ctx* ctx, int slot, size_t bytes, void** out) {
    nb_scratch_buf& b = ctx->scratch[slot];
    if (b.bytes < bytes) {
        if (b.ptr) {
            // the previous user of this slot may still be running on some stream
            NB_CUDA_TRY(cudaDeviceSynchronize());
            NB_CUDA_TRY(cudaFree(b.ptr));
            b.ptr = nullptr;
            b.bytes = 0;
        }
        size_t want = bytes < 256 ? 256 : bytes;
        NB_CUDA_TRY(cudaMalloc(&b.ptr, want));
        b.bytes = want;
    }
    *out = b.ptr;
    return NB_OK;
}

}  // namespace nb

extern "C" {

const char* nb_last_error_string(void) { return g_last_error; }

const char* nb_version(void) { return "nbody-gb300 0.1 (sm_103a)"; }

nb_status nb_ctx_create(int device, nb_ctx** out) {
    if (!out) return nb::set_error(NB_ERR_INVALID_ARG, "nb_ctx_create: null output pointer");
    *out = nullptr;
    int count = 0;
    NB_CUDA_TRY(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_ctx_create: device %d out of range (%d)",
                             device, count);
    NB_CUDA_TRY(cudaSetDevice(device));
    nb_ctx* ctx = new nb_ctx();
    ctx->device = device;
    cudaError_t e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->dev_error, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(ctx->dev_error, 0, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->dev_counter, 64 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(ctx->dev_counter, 0, 64 * sizeof(unsigned int));
    if (e != cudaSuccess) {
        nb_ctx_destroy(ctx);
        return nb::cuda_error(e, "nb_ctx_create");
    }
    *out = ctx;
    return NB_OK;
}

nb_status nb_ctx_destroy(nb_ctx* ctx) {
    if (!ctx) return NB_OK;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    for (auto& b : ctx->scratch) {
        if (b.ptr) cudaFree(b.ptr);
        b.ptr = nullptr;
    }
    if (ctx->dev_error) cudaFree(ctx->dev_error);
    if (ctx->dev_counter) cudaFree(ctx->dev_counter);
    delete ctx;
    return NB_OK;
}

nb_status nb_ctx_set_fault_hooks(nb_ctx* ctx, long long wait_limit, unsigned int flags,
                                 unsigned int learned_stack_cap) {
    NB_CHECK_CTX(ctx);
    if (flags & ~(unsigned int)NB_FAULT_DROP_LOOKBACK)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_ctx_set_fault_hooks: unknown flags 0x%x",
                             flags);
    if (learned_stack_cap > NB_LEARNED_STACK_CAP)
        return nb::set_error(NB_ERR_INVALID_ARG,
                             "nb_ctx_set_fault_hooks: stack capacity %u above the kernel's %u",
                             learned_stack_cap, (unsigned)NB_LEARNED_STACK_CAP);
    ctx->wait_limit = wait_limit < 0 ? NB_WAIT_LIMIT_DEFAULT : (unsigned long long)wait_limit;
    ctx->fault_flags = flags;
    ctx->learned_stack_cap = learned_stack_cap;
    return NB_OK;
}

nb_status nb_sync(nb_ctx* ctx, nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    NB_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    uint32_t word = 0;
    NB_CUDA_TRY(cudaMemcpy(&word, ctx->dev_error, sizeof(word), cudaMemcpyDeviceToHost));
    if (word) {
        NB_CUDA_TRY(cudaMemset(ctx->dev_error, 0, sizeof(word)));
        if (word & NB_DEVERR_DRAIN) {
            ctx->unusable = true;
            return nb::set_error(NB_ERR_TIMEOUT,
                                 "device: a bounded wait ran out and its CTA could not drain its "
                                 "bulk copies in flight; the context refuses further work");
        }
        if (word & NB_DEVERR_POOL)
            return nb::set_error(NB_ERR_POOL_OVERFLOW, "device: octree node pool overflow");
        if (word & NB_DEVERR_DEPTH)
            return nb::set_error(NB_ERR_DEPTH_OVERFLOW, "device: maximum tree depth exceeded");
        if (word & NB_DEVERR_STACK)
            return nb::set_error(NB_ERR_STACK_OVERFLOW, "device: traversal stack overflow");
        if (word & NB_DEVERR_TIMEOUT)
            return nb::set_error(NB_ERR_TIMEOUT, "device: bounded wait ran out");
    }
    return NB_OK;
}

}  // extern "C"
