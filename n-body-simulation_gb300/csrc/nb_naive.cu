// nb_naive.cu -- naive all-pairs acceleration (NaiveAlgorithm.cpp:262-482 semantics).
//
// Three arithmetic modes:
//  * NB_F64_IEEE: one thread per target body walks all sources j = 0..N-1 in order, every
//    operation separately rounded in the reference's order (r^2 summed left to right, den^3 as
//    (den*den)*den, 1/sqrt for rsqrt, acc += m*(r*den), G last). Bit-identical to the host
//    FP64 evaluation of NaiveAlgorithm.cpp:331-351.
//  * NB_F64: same loop with FMAs and the refined hardware rsqrt (FP64-pipe bound on GB300).
//  * NB_F32C: FP32 pair math with packed f32x2 instructions, per-j-tile FP32 partial sums folded
//    into a (hi, lo) TwoSum accumulator per body and component. Persistent CTAs (SMs x
//    resident CTAs) split the (i-block, j-tile) unit space into equal contiguous ranges
//    (stream-K), so every SM does the same number of pair interactions for any N; each CTA
//    writes one partial per i-block it touches and a combine pass adds the partials in CTA
//    order (deterministic). j-tiles are staged into shared memory by cp.async.bulk copies
//    completing on mbarriers (double-buffered), every wait bounded.
#include "nb_internal.cuh"

namespace {

// ---------------------------------------------------------------------------------------------
// FP64
// ---------------------------------------------------------------------------------------------
constexpr int F64_THREADS = 64;

template <bool IEEE>
__global__ void __launch_bounds__(F64_THREADS)
naive_f64_kernel(const double* __restrict__ m, const double* __restrict__ x,
                 const double* __restrict__ y, const double* __restrict__ z,
                 double* __restrict__ ax, double* __restrict__ ay, double* __restrict__ az,
                 uint32_t n, uint32_t i_begin, uint32_t i_end, double G, double eps2) {
    __shared__ double sx[F64_THREADS], sy[F64_THREADS], sz[F64_THREADS], sm[F64_THREADS];
    const uint32_t i = i_begin + blockIdx.x * F64_THREADS + threadIdx.x;
    const bool active = i < i_end;
    double px = 0, py = 0, pz = 0;
    if (active) {
        px = x[i];
        py = y[i];
        pz = z[i];
    }
    double acc_x = 0, acc_y = 0, acc_z = 0;
    for (uint32_t k = 0; k < n; k += F64_THREADS) {
        const uint32_t j = k + threadIdx.x;
        if (j < n) {
            sx[threadIdx.x] = x[j];
            sy[threadIdx.x] = y[j];
            sz[threadIdx.x] = z[j];
            sm[threadIdx.x] = m[j];
        }
        __syncthreads();
        const uint32_t cnt = min((uint32_t)F64_THREADS, n - k);
        if (active) {
            if (IEEE) {
                for (uint32_t jj = 0; jj < cnt; ++jj) {
                    const double r_x = __dsub_rn(sx[jj], px);
                    const double r_y = __dsub_rn(sy[jj], py);
                    const double r_z = __dsub_rn(sz[jj], pz);
                    double den = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(r_x, r_x), __dmul_rn(r_y, r_y)),
                                                     __dmul_rn(r_z, r_z)),
                                           eps2);
                    den = __dmul_rn(__dmul_rn(den, den), den);
                    den = __ddiv_rn(1.0, __dsqrt_rn(den));
                    acc_x = __dadd_rn(acc_x, __dmul_rn(sm[jj], __dmul_rn(r_x, den)));
                    acc_y = __dadd_rn(acc_y, __dmul_rn(sm[jj], __dmul_rn(r_y, den)));
                    acc_z = __dadd_rn(acc_z, __dmul_rn(sm[jj], __dmul_rn(r_z, den)));
                }
            } else {
#pragma unroll 4
                for (uint32_t jj = 0; jj < cnt; ++jj) {
                    const double r_x = sx[jj] - px;
                    const double r_y = sy[jj] - py;
                    const double r_z = sz[jj] - pz;
                    double den = fma(r_x, r_x, fma(r_y, r_y, fma(r_z, r_z, eps2)));
                    den = den * den * den;
                    const double inv = nb_rsqrt_f64(den);
                    const double s = sm[jj] * inv;
                    acc_x = fma(s, r_x, acc_x);
                    acc_y = fma(s, r_y, acc_y);
                    acc_z = fma(s, r_z, acc_z);
                }
            }
        }
        __syncthreads();
    }
    if (active) {
        if (IEEE) {
            ax[i] = __dmul_rn(acc_x, G);
            ay[i] = __dmul_rn(acc_y, G);
            az[i] = __dmul_rn(acc_z, G);
        } else {
            ax[i] = acc_x * G;
            ay[i] = acc_y * G;
            az[i] = acc_z * G;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// FP32, compensated
// ---------------------------------------------------------------------------------------------
constexpr int F32_THREADS = 128;   // threads per CTA
constexpr int F32_IP = 8;          // target bodies per thread (4 packed f32x2 slots)
constexpr int F32_IB = F32_THREADS * F32_IP;  // target bodies per i-block
constexpr int F32_JT = 256;        // sources per j-tile
constexpr int F32_SLOTS = F32_IP / 2;
constexpr unsigned long long WAIT_LIMIT = 1ull << 26;  // mbarrier polls before giving up

// Source record in the duplicated layout the packed pair loop consumes with two broadcast
// 16-byte shared loads: {x, x, y, y} {z, z, Gm, Gm}, positions relative to an FP64 anchor.
struct __align__(16) SrcDup {
    float x0, x1, y0, y1, z0, z1, m0, m1;
};

__global__ void f32_prepare_kernel(const double* __restrict__ m, const double* __restrict__ x,
                                   const double* __restrict__ y, const double* __restrict__ z,
                                   uint32_t n, double G, SrcDup* __restrict__ out,
                                   float4* __restrict__ tgt) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double ox = x[0], oy = y[0], oz = z[0];
    const float fx = (float)(x[j] - ox), fy = (float)(y[j] - oy), fz = (float)(z[j] - oz);
    const float fm = (float)(G * m[j]);
    out[j] = SrcDup{fx, fx, fy, fy, fz, fz, fm, fm};
    tgt[j] = make_float4(fx, fy, fz, fm);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Bounded wait on phase `parity` of an mbarrier. Returns false if the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (unsigned long long it = 0; it < WAIT_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

struct F32Plan {
    uint32_t n;
    uint32_t n_ib;     // i-blocks
    uint32_t n_jt;     // j-tiles
    uint64_t units;    // n_ib * n_jt
    uint32_t ctas;     // persistent CTAs
    uint32_t i_begin;  // first target body of block 0
};

__device__ __forceinline__ uint64_t unit_begin(const F32Plan& p, uint32_t cta) {
    return (p.units * (uint64_t)cta) / p.ctas;
}

// Partial layout: part[slot][6][F32_IB] floats, slot = cta + i_block (unique along the
// monotone staircase of CTA ranges over i-blocks).
__global__ void __launch_bounds__(F32_THREADS)
naive_f32c_kernel(const SrcDup* __restrict__ src, const float4* __restrict__ tgt, F32Plan plan,
                  float eps2, float* __restrict__ part, uint32_t* __restrict__ err_word) {
    __shared__ __align__(128) SrcDup tile[2][F32_JT];
    __shared__ __align__(8) uint64_t full[2];

    const uint32_t cta = blockIdx.x;
    const uint64_t u0 = unit_begin(plan, cta), u1 = unit_begin(plan, cta + 1);
    if (u0 >= u1) return;

    if (threadIdx.x == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // Sequence of j-tiles this CTA consumes: units u0..u1-1 in order; unit u -> tile u % n_jt.
    auto issue = [&](uint64_t u, int buf) {
        const uint32_t jt = (uint32_t)(u % plan.n_jt);
        const uint32_t j0 = jt * F32_JT;
        const uint32_t cnt = min((uint32_t)F32_JT, plan.n - j0);
        const uint32_t bytes = cnt * (uint32_t)sizeof(SrcDup);
        mbar_expect_tx(&full[buf], bytes);
        bulk_g2s(&tile[buf][0], src + j0, bytes, &full[buf]);
    };
    if (threadIdx.x == 0) {
        issue(u0, 0);
        if (u0 + 1 < u1) issue(u0 + 1, 1);
    }

    const nb_f2 eps2x2 = f2_pack(eps2, eps2);
    const nb_f2 zero2 = f2_pack(0.f, 0.f);
    nb_f2 xi[F32_SLOTS], yi[F32_SLOTS], zi[F32_SLOTS];
    nb_f2 tx[F32_SLOTS], ty[F32_SLOTS], tz[F32_SLOTS];   // per-tile sums
    nb_f2 hx[F32_SLOTS], hy[F32_SLOTS], hz[F32_SLOTS];   // compensated sums: high parts
    nb_f2 lx[F32_SLOTS], ly[F32_SLOTS], lz[F32_SLOTS];   // low parts

    uint64_t u = u0;
    uint32_t iter = 0;
    bool failed = false;
    while (u < u1 && !failed) {
        const uint32_t ib = (uint32_t)(u / plan.n_jt);
        const uint64_t seg_end = min(u1, (uint64_t)(ib + 1) * plan.n_jt);
        // load this i-block's targets (bodies past n get a far-away dummy; never stored)
#pragma unroll
        for (int s = 0; s < F32_SLOTS; ++s) {
            float4 a, b;
            const uint32_t ia = plan.i_begin + ib * F32_IB + (2 * s) * F32_THREADS + threadIdx.x;
            const uint32_t ibb = ia + F32_THREADS;
            a = ia < plan.n ? tgt[ia] : make_float4(1e18f, 1e18f, 1e18f, 0.f);
            b = ibb < plan.n ? tgt[ibb] : make_float4(1e18f, 1e18f, 1e18f, 0.f);
            xi[s] = f2_pack(a.x, b.x);
            yi[s] = f2_pack(a.y, b.y);
            zi[s] = f2_pack(a.z, b.z);
            hx[s] = hy[s] = hz[s] = zero2;
            lx[s] = ly[s] = lz[s] = zero2;
        }
        for (; u < seg_end; ++u, ++iter) {
            const int buf = iter & 1;
            const uint32_t jt = (uint32_t)(u % plan.n_jt);
            const uint32_t cnt = min((uint32_t)F32_JT, plan.n - jt * F32_JT);
            const bool ok = mbar_wait(&full[buf], (iter >> 1) & 1);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
#pragma unroll
            for (int s = 0; s < F32_SLOTS; ++s) tx[s] = ty[s] = tz[s] = zero2;
            const ulonglong2* t2 = reinterpret_cast<const ulonglong2*>(&tile[buf][0]);
#pragma unroll 2
            for (uint32_t j = 0; j < cnt; ++j) {
                const ulonglong2 A = t2[2 * j];      // {x,x} {y,y}
                const ulonglong2 B = t2[2 * j + 1];  // {z,z} {m,m}
#pragma unroll
                for (int s = 0; s < F32_SLOTS; ++s) {
                    const nb_f2 dx = f2_sub(A.x, xi[s]);
                    const nb_f2 dy = f2_sub(A.y, yi[s]);
                    const nb_f2 dz = f2_sub(B.x, zi[s]);
                    nb_f2 r2 = f2_fma(dx, dx, eps2x2);
                    r2 = f2_fma(dy, dy, r2);
                    r2 = f2_fma(dz, dz, r2);
                    float r2a, r2b;
                    f2_unpack(r2, r2a, r2b);
                    const nb_f2 inv = f2_pack(nb_rsqrt_f32(r2a), nb_rsqrt_f32(r2b));
                    const nb_f2 inv2 = f2_mul(inv, inv);
                    const nb_f2 mi = f2_mul(B.y, inv);
                    const nb_f2 s3 = f2_mul(mi, inv2);
                    tx[s] = f2_fma(dx, s3, tx[s]);
                    ty[s] = f2_fma(dy, s3, ty[s]);
                    tz[s] = f2_fma(dz, s3, tz[s]);
                }
            }
            // fold the tile sums into the compensated accumulators (Knuth TwoSum)
#pragma unroll
            for (int s = 0; s < F32_SLOTS; ++s) {
#define NB_TWOSUM(H, L, T)                                   \
    {                                                        \
        const nb_f2 sum = f2_add(H, T);                      \
        const nb_f2 bp = f2_sub(sum, H);                     \
        const nb_f2 e1 = f2_sub(H, f2_sub(sum, bp));         \
        const nb_f2 e2 = f2_sub(T, bp);                      \
        L = f2_add(L, f2_add(e1, e2));                       \
        H = sum;                                             \
    }
                NB_TWOSUM(hx[s], lx[s], tx[s]);
                NB_TWOSUM(hy[s], ly[s], ty[s]);
                NB_TWOSUM(hz[s], lz[s], tz[s]);
#undef NB_TWOSUM
            }
            __syncthreads();  // every thread is done with tile[buf]
            if (threadIdx.x == 0 && u + 2 < u1) issue(u + 2, buf);
        }
        if (failed) break;
        // partial of this (cta, i-block)
        float* out = part + (size_t)(cta + ib) * 6 * F32_IB;
#pragma unroll
        for (int s = 0; s < F32_SLOTS; ++s) {
            const int la = (2 * s) * F32_THREADS + threadIdx.x, lb = la + F32_THREADS;
            float a0, b0;
            f2_unpack(hx[s], a0, b0); out[0 * F32_IB + la] = a0; out[0 * F32_IB + lb] = b0;
            f2_unpack(hy[s], a0, b0); out[1 * F32_IB + la] = a0; out[1 * F32_IB + lb] = b0;
            f2_unpack(hz[s], a0, b0); out[2 * F32_IB + la] = a0; out[2 * F32_IB + lb] = b0;
            f2_unpack(lx[s], a0, b0); out[3 * F32_IB + la] = a0; out[3 * F32_IB + lb] = b0;
            f2_unpack(ly[s], a0, b0); out[4 * F32_IB + la] = a0; out[4 * F32_IB + lb] = b0;
            f2_unpack(lz[s], a0, b0); out[5 * F32_IB + la] = a0; out[5 * F32_IB + lb] = b0;
        }
    }
    if (failed) {
        if (threadIdx.x == 0) atomicOr(err_word, NB_DEVERR_TIMEOUT);
        // drain copies still in flight into this CTA's shared memory (bounded)
        const uint32_t done = iter;
        for (uint32_t k = done; k < done + 2 && u0 + k < u1; ++k) {
            mbar_wait(&full[k & 1], (k >> 1) & 1);
        }
    }
}

__device__ __forceinline__ uint32_t cta_of_unit(const F32Plan& p, uint64_t u) {
    uint32_t c = (uint32_t)((u * p.ctas) / p.units);
    while (c + 1 < p.ctas && unit_begin(p, c + 1) <= u) ++c;
    while (c > 0 && unit_begin(p, c) > u) --c;
    return c;
}

__global__ void naive_f32c_combine(F32Plan plan, const float* __restrict__ part,
                                   double* __restrict__ ax, double* __restrict__ ay,
                                   double* __restrict__ az, uint32_t i_end) {
    const uint32_t local = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = plan.i_begin + local;
    if (i >= i_end) return;
    const uint32_t ib = local / F32_IB, li = local % F32_IB;
    const uint32_t c0 = cta_of_unit(plan, (uint64_t)ib * plan.n_jt);
    const uint32_t c1 = cta_of_unit(plan, (uint64_t)(ib + 1) * plan.n_jt - 1);
    double sx = 0, sy = 0, sz = 0;
    for (uint32_t c = c0; c <= c1; ++c) {
        const float* p = part + (size_t)(c + ib) * 6 * F32_IB;
        sx += (double)p[0 * F32_IB + li] + (double)p[3 * F32_IB + li];
        sy += (double)p[1 * F32_IB + li] + (double)p[4 * F32_IB + li];
        sz += (double)p[2 * F32_IB + li] + (double)p[5 * F32_IB + li];
    }
    ax[i] = sx;
    ay[i] = sy;
    az[i] = sz;
}

int g_f32_ctas_per_sm = 0;

nb_status naive_f32c(nb_ctx* ctx, const double* m, const double* x, const double* y,
                     const double* z, double* ax, double* ay, double* az, uint32_t n,
                     uint32_t i_begin, uint32_t i_end, double G, double eps2,
                     cudaStream_t stream) {
    if (g_f32_ctas_per_sm == 0) {
        NB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_f32_ctas_per_sm,
                                                                  naive_f32c_kernel, F32_THREADS, 0));
        if (g_f32_ctas_per_sm < 1) g_f32_ctas_per_sm = 1;
    }
    const uint32_t n_t = i_end - i_begin;
    F32Plan plan;
    plan.n = n;
    plan.i_begin = i_begin;
    plan.n_ib = (n_t + F32_IB - 1) / F32_IB;
    plan.n_jt = (n + F32_JT - 1) / F32_JT;
    plan.units = (uint64_t)plan.n_ib * plan.n_jt;
    uint64_t ctas = (uint64_t)ctx->sm_count * g_f32_ctas_per_sm;
    if (ctas > plan.units) ctas = plan.units;
    plan.ctas = (uint32_t)ctas;
    // scratch: duplicated sources, float4 targets, partials
    const size_t src_bytes = ((size_t)n * sizeof(SrcDup) + 255) & ~(size_t)255;
    const size_t tgt_bytes = ((size_t)n * sizeof(float4) + 255) & ~(size_t)255;
    const size_t part_bytes = (size_t)(plan.ctas + plan.n_ib) * 6 * F32_IB * sizeof(float);
    void* base = nullptr;
    NB_TRY(nb::scratch(ctx, NB_SCRATCH_NAIVE_F32, src_bytes + tgt_bytes + part_bytes, &base));
    SrcDup* src = (SrcDup*)base;
    float4* tgt = (float4*)((char*)base + src_bytes);
    float* part = (float*)((char*)base + src_bytes + tgt_bytes);
    f32_prepare_kernel<<<nb::ceil_div(n, 256), 256, 0, stream>>>(m, x, y, z, n, G, src, tgt);
    NB_TRY(nb::check_launch("f32_prepare_kernel"));
    naive_f32c_kernel<<<plan.ctas, F32_THREADS, 0, stream>>>(src, tgt, plan, (float)eps2, part,
                                                             ctx->dev_error);
    NB_TRY(nb::check_launch("naive_f32c_kernel"));
    naive_f32c_combine<<<nb::ceil_div(n_t, 256), 256, 0, stream>>>(plan, part, ax, ay, az, i_end);
    return nb::check_launch("naive_f32c_combine");
}

nb_status naive_dispatch(nb_ctx* ctx, const double* m, const double* x, const double* y,
                         const double* z, double* ax, double* ay, double* az, uint32_t n,
                         uint32_t i_begin, uint32_t i_end, double G, double eps2,
                         nb_precision prec, cudaStream_t stream) {
    NB_CHECK_CTX(ctx);
    if (n == 0 || i_begin >= i_end) return NB_OK;
    if (!m || !x || !y || !z || !ax || !ay || !az)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_accel: null array pointer");
    if (i_end > n) return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_accel: i_end > n");
    const uint32_t n_t = i_end - i_begin;
    switch (prec) {
        case NB_F64_IEEE:
            naive_f64_kernel<true><<<nb::ceil_div(n_t, F64_THREADS), F64_THREADS, 0, stream>>>(
                m, x, y, z, ax, ay, az, n, i_begin, i_end, G, eps2);
            return nb::check_launch("naive_f64_kernel<ieee>");
        case NB_F64:
            naive_f64_kernel<false><<<nb::ceil_div(n_t, F64_THREADS), F64_THREADS, 0, stream>>>(
                m, x, y, z, ax, ay, az, n, i_begin, i_end, G, eps2);
            return nb::check_launch("naive_f64_kernel");
        case NB_F32C:
            return naive_f32c(ctx, m, x, y, z, ax, ay, az, n, i_begin, i_end, G, eps2, stream);
        default:
            return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_accel: unknown precision %d",
                                 (int)prec);
    }
}

}  // namespace

extern "C" {

nb_status nb_naive_accel(nb_ctx* ctx, const double* m, const double* x, const double* y,
                         const double* z, double* ax, double* ay, double* az, uint32_t n,
                         double G, double eps2, nb_precision prec, int block_size,
                         nb_stream_t stream) {
    if (block_size < 0)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_accel: block_size must be >= 0");
    return naive_dispatch(ctx, m, x, y, z, ax, ay, az, n, 0, n, G, eps2, prec,
                          (cudaStream_t)stream);
}

nb_status nb_naive_accel_range(nb_ctx* ctx, const double* m, const double* x, const double* y,
                               const double* z, double* ax, double* ay, double* az, uint32_t n,
                               uint32_t i_begin, uint32_t i_end, double G, double eps2,
                               nb_precision prec, nb_stream_t stream) {
    return naive_dispatch(ctx, m, x, y, z, ax, ay, az, n, i_begin, i_end, G, eps2, prec,
                          (cudaStream_t)stream);
}

}  // extern "C"
