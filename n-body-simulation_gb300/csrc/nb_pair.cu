// nb_pair.cu -- tile configurations and launcher of the FP32-compensated pair kernel.
#include "nb_pair.cuh"

namespace nbpair {

// Positions relative to each system's first body (FP64 subtraction, then rounded), G*m in FP32.
__global__ void pair_prepare_kernel(Plan P, const double* __restrict__ m,
                                    const double* __restrict__ x, const double* __restrict__ y,
                                    const double* __restrict__ z, uint32_t n_total, double G,
                                    SrcDup* __restrict__ out, float4* __restrict__ tgt) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_total) return;
    const uint32_t s = upper_index<uint32_t>(P.sys_off, P.n_systems, b);
    const uint32_t a = P.sys_off[s];
    const float fx = (float)(x[b] - x[a]), fy = (float)(y[b] - y[a]), fz = (float)(z[b] - z[a]);
    const float fm = (float)(G * m[b]);
    out[b] = SrcDup{fx, fx, fy, fy, fz, fz, fm, fm};
    tgt[b] = make_float4(fx, fy, fz, fm);
}

// Writes the plan of one system (sources [0, n), targets [t_begin, t_end)) into device arrays.
__global__ void plan_single_kernel(uint32_t* sys_off, uint32_t* tgt_begin, uint32_t* t_off,
                                   uint64_t* unit_off, uint32_t* ib_off, uint32_t n,
                                   uint32_t t_begin, uint32_t t_end, uint64_t units,
                                   uint32_t n_ib) {
    sys_off[0] = 0;
    sys_off[1] = n;
    tgt_begin[0] = t_begin;
    t_off[0] = 0;
    t_off[1] = t_end - t_begin;
    unit_off[0] = 0;
    unit_off[1] = units;
    ib_off[0] = 0;
    ib_off[1] = n_ib;
}

}  // namespace nbpair

namespace nb {

// (threads, targets per thread, j-tile); X-macro so that the table, the occupancy query and the
// launch switch list the same instantiations
#define NB_PAIR_CONFIG_LIST(X)                                                                  \
    X(0, 128, 12, 256) X(1, 256, 8, 256) X(2, 128, 8, 256) X(3, 64, 8, 256) X(4, 128, 12, 512)      \
        X(5, 128, 4, 256) X(6, 64, 12, 256) X(7, 128, 8, 128)

const PairConfig kPairConfigs[NB_PAIR_CONFIGS] = {
#define NB_PAIR_ROW(i, T, IP, JT) {T, IP, JT},
    NB_PAIR_CONFIG_LIST(NB_PAIR_ROW)
#undef NB_PAIR_ROW
};

namespace {

int g_ctas_per_sm[NB_PAIR_CONFIGS] = {};

// Opts the instantiation into its dynamic shared memory and returns its resident CTAs per SM.
template <int T, int IP, int JT>
nb_status prepare(int* out) {
    constexpr size_t smem = nbpair::pair_smem_bytes<T, IP, JT>();
    NB_CUDA_TRY(cudaFuncSetAttribute(nbpair::pair_f32c_kernel<T, IP, JT>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    NB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        out, nbpair::pair_f32c_kernel<T, IP, JT>, T, smem));
    if (*out < 1) *out = 1;
    return NB_OK;
}

template <int T, int IP, int JT>
nb_status launch_cfg(const nbpair::Plan& plan, const double* m, const double* x, const double* y,
                     const double* z, uint32_t n_total, uint32_t n_targets, double G, double eps2,
                     nbpair::SrcDup* src, float4* tgt, float* part, double* ax, double* ay,
                     double* az, uint32_t* err_word, cudaStream_t stream) {
    nbpair::pair_prepare_kernel<<<ceil_div(n_total, 256), 256, 0, stream>>>(plan, m, x, y, z, n_total,
                                                                            G, src, tgt);
    NB_TRY(check_launch("pair_prepare_kernel"));
    nbpair::pair_f32c_kernel<T, IP, JT><<<plan.ctas, T, nbpair::pair_smem_bytes<T, IP, JT>(),
                                          stream>>>(plan, src, tgt, (float)eps2, part, err_word);
    NB_TRY(check_launch("pair_f32c_kernel"));
    nbpair::pair_combine_kernel<T * IP, JT><<<ceil_div(n_targets, 256), 256, 0, stream>>>(
        plan, part, n_targets, ax, ay, az);
    return check_launch("pair_combine_kernel");
}

}  // namespace

// Also makes the configuration launchable (dynamic shared memory opt-in): callers query it
// before their first launch of a configuration.
nb_status pair_ctas_per_sm(int cfg, int* out) {
    if (cfg < 0 || cfg >= NB_PAIR_CONFIGS) return set_error(NB_ERR_INVALID_ARG, "bad pair config %d", cfg);
    if (g_ctas_per_sm[cfg] == 0) {
        int v = 0;
        switch (cfg) {
#define NB_PAIR_PREP(i, T, IP, JT) \
    case i: NB_TRY((prepare<T, IP, JT>(&v))); break;
            NB_PAIR_CONFIG_LIST(NB_PAIR_PREP)
#undef NB_PAIR_PREP
        }
        g_ctas_per_sm[cfg] = v;
    }
    *out = g_ctas_per_sm[cfg];
    return NB_OK;
}

nb_status pair_plan_single(uint32_t* sys_off, uint32_t* tgt_begin, uint32_t* t_off,
                           uint64_t* unit_off, uint32_t* ib_off, uint32_t n, uint32_t t_begin,
                           uint32_t t_end, uint64_t units, uint32_t n_ib, cudaStream_t stream) {
    nbpair::plan_single_kernel<<<1, 1, 0, stream>>>(sys_off, tgt_begin, t_off, unit_off, ib_off, n,
                                                   t_begin, t_end, units, n_ib);
    return check_launch("plan_single_kernel");
}

size_t pair_partial_floats(int cfg, uint32_t ctas, uint32_t total_ib) {
    const size_t ib = (size_t)kPairConfigs[cfg].threads * kPairConfigs[cfg].ip;
    return ((size_t)ctas + total_ib) * 6 * ib;
}

nb_status pair_launch(int cfg, const nbpair::Plan& plan, const double* m, const double* x,
                      const double* y, const double* z, uint32_t n_total, uint32_t n_targets,
                      double G, double eps2, nbpair::SrcDup* src, float4* tgt, float* part,
                      double* ax, double* ay, double* az, uint32_t* err_word,
                      cudaStream_t stream) {
    int per_sm = 0;
    NB_TRY(pair_ctas_per_sm(cfg, &per_sm));  // shared-memory opt-in before the first launch
    switch (cfg) {
#define NB_PAIR_LAUNCH(i, T, IP, JT)                                                          \
    case i:                                                                                   \
        return launch_cfg<T, IP, JT>(plan, m, x, y, z, n_total, n_targets, G, eps2, src, tgt, \
                                     part, ax, ay, az, err_word, stream);
        NB_PAIR_CONFIG_LIST(NB_PAIR_LAUNCH)
#undef NB_PAIR_LAUNCH
        default: return set_error(NB_ERR_INVALID_ARG, "bad pair config %d", cfg);
    }
}

}  // namespace nb
