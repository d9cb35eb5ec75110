// nb_internal.cuh -- shared internals of libnbody_cuda.so (context, errors, scratch, math).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "nbody.h"

// Bits of the device error word a kernel raises instead of trapping or spinning forever.
enum : uint32_t {
    NB_DEVERR_POOL = 1u << 0,
    NB_DEVERR_DEPTH = 1u << 1,
    NB_DEVERR_STACK = 1u << 2,
    NB_DEVERR_TIMEOUT = 1u << 3,
    // a CTA whose wait ran out could not drain its own bulk copies in flight either and left
    // with them outstanding: the launch's memory state is undefined, the context refuses work
    NB_DEVERR_DRAIN = 1u << 4,
};

// Iterations of a bounded device-side wait (mbarrier polls, look-back polls) before it gives
// up. A context can lower it for the failure-path tests (nb_ctx_set_fault_hooks); the waits
// that drain a CTA's own copies in flight before it leaves always use this default.
constexpr unsigned long long NB_WAIT_LIMIT_DEFAULT = 1ull << 22;

struct nb_scratch_buf {
    void* ptr = nullptr;
    size_t bytes = 0;
};

enum nb_scratch_slot : int {
    NB_SCRATCH_NAIVE_F32 = 0,   // float4 sources for the FP32 pair kernel
    NB_SCRATCH_ENERGY = 1,      // per-block partial energies
    NB_SCRATCH_AABB = 2,        // per-block partial min/max
    NB_SCRATCH_LABELS = 3,      // sampled (group, cell) pairs of the label generator
    NB_SCRATCH_NAIVE_DF = 4,    // triple-float sources of the double-float pair kernel
    NB_SCRATCH_PAIR_SYM = 5,    // sources and partials of the symmetric FP32 pair kernel
    NB_SCRATCH_COUNT = 8,
};

// An instantiated CUDA graph of captured steps (nb_batch_graph_create, nb_bh_graph_create).
struct nb_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int steps = 0;
};

// Ends a capture on stream s (begun by the caller), instantiates the graph and wraps it; on any
// earlier failure (st != NB_OK) it only cleans up. Destroys s.
nb_status nb_finish_capture(cudaStream_t s, nb_status st, int steps, nb_graph** out);

struct nb_ctx {
    int device = 0;
    int sm_count = 0;
    uint32_t* dev_error = nullptr;  // device error word (NB_DEVERR_* bits)
    unsigned int* dev_counter = nullptr;  // last-block-done counters for fused grid reductions
    nb_scratch_buf scratch[NB_SCRATCH_COUNT];
    // failure-path test hooks (nb_ctx_set_fault_hooks)
    unsigned long long wait_limit = NB_WAIT_LIMIT_DEFAULT;
    unsigned int fault_flags = 0;
    unsigned int learned_stack_cap = 0;  // 0 = the kernel's full capacity
    // set when a launch left bulk copies outstanding (NB_DEVERR_DRAIN): every later call fails
    bool unusable = false;
};

namespace nb {

nb_status set_error(nb_status st, const char* fmt, ...);
nb_status cuda_error(cudaError_t err, const char* what);
// Grows scratch slot `slot` of the context to at least `bytes` (cudaMalloc; synchronous).
nb_status scratch(nb_ctx* ctx, int slot, size_t bytes, void** out);
nb_status check_launch(const char* what);

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace nb

#define NB_CHECK_CTX(ctx)                                                                  \
    do {                                                                                   \
        if (!(ctx)) return nb::set_error(NB_ERR_INVALID_ARG, "%s: null context", __func__); \
        if ((ctx)->unusable)                                                               \
            return nb::set_error(NB_ERR_TIMEOUT,                                           \
                                 "%s: context unusable after a launch left copies in "    \
                                 "flight; destroy it",                                     \
                                 __func__);                                                \
    } while (0)

#define NB_TRY(expr)                     \
    do {                                 \
        nb_status _st = (expr);          \
        if (_st != NB_OK) return _st;    \
    } while (0)

#define NB_CUDA_TRY(call)                                         \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return nb::cuda_error(_e, #call);  \
    } while (0)

// ---------------------------------------------------------------------------------------------
// Device math.
// ---------------------------------------------------------------------------------------------

// FP64 reciprocal square root: hardware approximation of the high word refined by one
// third-order Householder step (the Taylor series of (1-e)^(-1/2) = 1 + e/2 + 3e^2/8 + ...
// with e = 1 - x*y0^2), which cubes the approximation's relative error (~2^-22 -> ~2^-66),
// leaving only the final rounding (about 1 ulp).
__device__ __forceinline__ double nb_rsqrt_f64(double x) {
    double y0;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y0) : "d"(x));
    const double t = x * y0;
    const double e = fma(-t, y0, 1.0);
    const double p = fma(0.375, e, 0.5);
    const double u = y0 * e;
    return fma(u, p, y0);
}

// m * den^(-3/2) in FP64: hardware estimate y0 of den^(-1/2) and one correction of its cube,
// (1 - e)^(-3/2) = 1 + 3e/2 + 15e^2/8 + O(e^3) with e = 1 - den y0^2 (|e| < 2^-21, dropped terms
// below 2^-62): 7 FP64 operations.
__device__ __forceinline__ double nb_m_rinv3_f64(double m, double den) {
    double y0;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y0) : "d"(den));
    const double y2 = y0 * y0;
    const double e = fma(-den, y2, 1.0);
    const double p = fma(1.875, e, 1.5);
    const double w0 = m * (y2 * y0);
    return fma(w0 * e, p, w0);
}

// FP32 reciprocal square root (MUFU.RSQ, ~2 ulp).
__device__ __forceinline__ float nb_rsqrt_f32(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Packed FP32x2 arithmetic (sm_100+ f32x2 instructions): one instruction, two lanes.
typedef unsigned long long nb_f2;
__device__ __forceinline__ nb_f2 f2_pack(float lo, float hi) {
    nb_f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(nb_f2 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ nb_f2 f2_add(nb_f2 a, nb_f2 b) {
    nb_f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ nb_f2 f2_sub(nb_f2 a, nb_f2 b) {
    nb_f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ nb_f2 f2_mul(nb_f2 a, nb_f2 b) {
    nb_f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ nb_f2 f2_fma(nb_f2 a, nb_f2 b, nb_f2 c) {
    nb_f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// ---------------------------------------------------------------------------------------------
// Double-float arithmetic: a value is hi + lo with two FP32 numbers, |lo| <= ulp(hi)/2, which
// carries 48 significant bits (relative rounding ~2^-48 = 3.6e-15 per operation) on the FP32
// pipe. Error-free transformations after Knuth (TwoSum), Dekker/FMA (TwoProduct); products and
// sums as in the double-double literature (e.g. Hida, Li, Bailey, "Library for double-double
// and quad-double arithmetic", 2000), restated for float pairs.
// ---------------------------------------------------------------------------------------------
struct nb_df {
    float h, l;
};
// s + e = a + b exactly
__device__ __forceinline__ nb_df df_two_sum(float a, float b) {
    const float s = a + b, bb = s - a;
    return nb_df{s, (a - (s - bb)) + (b - bb)};
}
// s + e = a + b exactly, given |a| >= |b| (or a == 0)
__device__ __forceinline__ nb_df df_fast_two_sum(float a, float b) {
    const float s = a + b;
    return nb_df{s, b - (s - a)};
}
// a - b
__device__ __forceinline__ nb_df df_sub(nb_df a, nb_df b) {
    const nb_df s = df_two_sum(a.h, -b.h);
    return df_fast_two_sum(s.h, s.l + (a.l - b.l));
}
// a * b
__device__ __forceinline__ nb_df df_mul(nb_df a, nb_df b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return df_fast_two_sum(p, e);
}
// a * a
__device__ __forceinline__ nb_df df_sqr(nb_df a) {
    const float p = a.h * a.h;
    float e = fmaf(a.h, a.h, -p);
    e = fmaf(a.h + a.h, a.l, e);
    return df_fast_two_sum(p, e);
}
// (ch + cm + cl) - (ph + pm + pl) as a double-float, for two triple-float numbers (x = h + m + l
// with h = fl(x), m = fl(x - h), l = fl(x - h - m): 72 bits, so FP64 values are exact). The two
// leading differences are error-free, so the result is accurate to ~2^-48 of the difference
// itself however close the two numbers are.
__device__ __forceinline__ nb_df tf_diff(float ch, float cm, float cl, float ph, float pm,
                                         float pl) {
    const nb_df s = df_two_sum(ch, -ph);
    const nb_df t = df_two_sum(cm, -pm);
    const nb_df u = df_two_sum(s.h, t.h);
    return df_fast_two_sum(u.h, u.l + (s.l + t.l + (cl - pl)));
}
// The exact value of a - b (two FP64 numbers) as a triple-float h + m + l: FP64 TwoSum, then the
// rounded difference and its error split into FP32 terms.
__host__ __device__ __forceinline__ void tf_split_diff(double a, double b, float& h, float& m,
                                                       float& l) {
    const double s = a - b, bb = s - a;
    const double err = (a - (s - bb)) + (-b - bb);
    h = (float)s;
    const double rem = (s - (double)h) + err;
    m = (float)rem;
    l = (float)(rem - (double)m);
}
