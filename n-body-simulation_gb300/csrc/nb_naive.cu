// nb_naive.cu -- naive all-pairs acceleration (NaiveAlgorithm.cpp:262-482 semantics).
//
// Three arithmetic modes:
//  * NB_F64_IEEE: one thread per target body walks all sources j = 0..N-1 in order, every
//    operation separately rounded in the reference's order (r^2 summed left to right, den^3 as
//    (den*den)*den, 1/sqrt for rsqrt, acc += m*(r*den), G last). Bit-identical to the host
//    FP64 evaluation of NaiveAlgorithm.cpp:331-351.
//  * NB_F64: same loop with FMAs and m (r^2 + eps^2)^(-3/2) from the hardware rsqrt estimate with
//    one correction (nb_m_rinv3_f64; FP64-pipe bound on GB300).
//  * NB_F32C: the FP32-compensated pair kernel of nb_pair.cuh (scalar FP32 pair math, TwoSum
//    accumulation, stream-K persistent CTAs, cp.async.bulk j-tiles behind bounded mbarrier
//    waits), run as a batch of one system.
#include "nb_internal.cuh"
#include "nb_pair.cuh"

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
                    const double den = fma(r_x, r_x, fma(r_y, r_y, fma(r_z, r_z, eps2)));
                    const double s = nb_m_rinv3_f64(sm[jj], den);
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

// FP64 accelerations of listed target bodies (ax[t] for targets[t]); FMAs + refined rsqrt.
__global__ void __launch_bounds__(F64_THREADS)
naive_f64_targets_kernel(const double* __restrict__ m, const double* __restrict__ x,
                         const double* __restrict__ y, const double* __restrict__ z, uint32_t n,
                         const uint32_t* __restrict__ targets, uint32_t n_t,
                         double* __restrict__ ax, double* __restrict__ ay,
                         double* __restrict__ az, double G, double eps2) {
    __shared__ double sx[F64_THREADS], sy[F64_THREADS], sz[F64_THREADS], sm[F64_THREADS];
    const uint32_t t = blockIdx.x * F64_THREADS + threadIdx.x;
    const bool active = t < n_t;
    const uint32_t i = active ? targets[t] : 0;
    const double px = active ? x[i] : 0, py = active ? y[i] : 0, pz = active ? z[i] : 0;
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
#pragma unroll 4
            for (uint32_t jj = 0; jj < cnt; ++jj) {
                const double r_x = sx[jj] - px, r_y = sy[jj] - py, r_z = sz[jj] - pz;
                const double den = fma(r_x, r_x, fma(r_y, r_y, fma(r_z, r_z, eps2)));
                const double s = nb_m_rinv3_f64(sm[jj], den);
                acc_x = fma(s, r_x, acc_x);
                acc_y = fma(s, r_y, acc_y);
                acc_z = fma(s, r_z, acc_z);
            }
        }
        __syncthreads();
    }
    if (active) {
        ax[t] = acc_x * G;
        ay[t] = acc_y * G;
        az[t] = acc_z * G;
    }
}

// ---------------------------------------------------------------------------------------------
// FP32, compensated: the batched pair kernel (nb_pair.cuh) with a batch of one system whose
// targets are [i_begin, i_end).
// ---------------------------------------------------------------------------------------------
int g_naive_pair_cfg = 0;  // tile configuration (nb_naive_set_pair_config)

nb_status naive_f32c(nb_ctx* ctx, const double* m, const double* x, const double* y,
                     const double* z, double* ax, double* ay, double* az, uint32_t n,
                     uint32_t i_begin, uint32_t i_end, double G, double eps2,
                     cudaStream_t stream) {
    const int cfg = g_naive_pair_cfg;
    const nb::PairConfig& C = nb::kPairConfigs[cfg];
    int per_sm = 0;
    NB_TRY(nb::pair_ctas_per_sm(cfg, &per_sm));
    const uint32_t n_t = i_end - i_begin;
    const uint32_t ib = (uint32_t)(C.threads * C.ip);
    const uint32_t n_ib = (n_t + ib - 1) / ib;
    const uint32_t n_jt = (n + C.jt - 1) / C.jt;
    const uint64_t units = (uint64_t)n_ib * n_jt;
    uint64_t ctas = (uint64_t)ctx->sm_count * per_sm;
    if (ctas > units) ctas = units;
    // scratch: plan arrays, duplicated sources, float4 targets, partials
    const size_t plan_bytes = 512;
    const size_t src_bytes = ((size_t)n * sizeof(nbpair::SrcDup) + 255) & ~(size_t)255;
    const size_t tgt_bytes = ((size_t)n * sizeof(float4) + 255) & ~(size_t)255;
    const size_t part_bytes = nb::pair_partial_floats(cfg, (uint32_t)ctas, n_ib) * sizeof(float);
    void* base = nullptr;
    NB_TRY(nb::scratch(ctx, NB_SCRATCH_NAIVE_F32, plan_bytes + src_bytes + tgt_bytes + part_bytes,
                       &base));
    char* b = (char*)base;
    uint64_t* unit_off = (uint64_t*)b;
    uint32_t* sys_off = (uint32_t*)(b + 64);
    uint32_t* tgt_begin = (uint32_t*)(b + 128);
    uint32_t* t_off = (uint32_t*)(b + 192);
    uint32_t* ib_off = (uint32_t*)(b + 256);
    nbpair::SrcDup* src = (nbpair::SrcDup*)(b + plan_bytes);
    float4* tgt = (float4*)(b + plan_bytes + src_bytes);
    float* part = (float*)(b + plan_bytes + src_bytes + tgt_bytes);
    NB_TRY(nb::pair_plan_single(sys_off, tgt_begin, t_off, unit_off, ib_off, n, i_begin, i_end,
                                units, n_ib, stream));
    nbpair::Plan P;
    P.n_systems = 1;
    P.ctas = (uint32_t)ctas;
    P.units = units;
    P.sys_off = sys_off;
    P.tgt_begin = tgt_begin;
    P.t_off = t_off;
    P.unit_off = unit_off;
    P.ib_off = ib_off;
    return nb::pair_launch(cfg, P, m, x, y, z, n, n_t, G, eps2, src, tgt, part, ax, ay, az,
                           ctx->dev_error, stream);
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
        case NB_DF64:
            return nb::set_error(NB_ERR_UNSUPPORTED, "nb_naive_accel: NB_DF64 is a Barnes-Hut mode");
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

nb_status nb_naive_accel_targets(nb_ctx* ctx, const double* m, const double* x, const double* y,
                                 const double* z, uint32_t n, const uint32_t* targets,
                                 uint32_t n_targets, double* ax, double* ay, double* az, double G,
                                 double eps2, nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (!m || !x || !y || !z || !targets || !ax || !ay || !az)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_accel_targets: null pointer");
    if (n == 0 || n_targets == 0) return NB_OK;
    naive_f64_targets_kernel<<<nb::ceil_div(n_targets, F64_THREADS), F64_THREADS, 0,
                               (cudaStream_t)stream>>>(m, x, y, z, n, targets, n_targets, ax, ay,
                                                       az, G, eps2);
    return nb::check_launch("naive_f64_targets_kernel");
}

nb_status nb_naive_set_pair_config(int config) {
    if (config < 0 || config >= nb::NB_PAIR_CONFIGS)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_set_pair_config: config %d", config);
    g_naive_pair_cfg = config;
    return NB_OK;
}

nb_status nb_naive_accel_range(nb_ctx* ctx, const double* m, const double* x, const double* y,
                               const double* z, double* ax, double* ay, double* az, uint32_t n,
                               uint32_t i_begin, uint32_t i_end, double G, double eps2,
                               nb_precision prec, nb_stream_t stream) {
    return naive_dispatch(ctx, m, x, y, z, ax, ay, az, n, i_begin, i_end, G, eps2, prec,
                          (cudaStream_t)stream);
}

}  // extern "C"
