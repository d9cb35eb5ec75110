// nb_pair_sym.cuh -- plan and launcher of the symmetric FP32 pair kernel (nb_pair_sym.cu).
#pragma once
#include "nb_internal.cuh"

namespace nbsym {

// One system of n bodies in nb I-blocks of IB bodies and n_jt = nb * tpb j-tiles of JT bodies;
// row a of the unit sequence holds the j-tiles a * tpb .. n_jt - 1.
struct SymPlan {
    uint32_t n, nb, n_jt, tpb, ctas;
    uint64_t units;
};

// First unit of I-block a (a <= nb; unit_off(nb) = units).
__host__ __device__ __forceinline__ uint64_t unit_off(const SymPlan& S, uint32_t a) {
    const uint64_t aa = a;
    return aa * S.n_jt - (uint64_t)S.tpb * (aa == 0 ? 0 : aa * (aa - 1) / 2);
}

}  // namespace nbsym

namespace nb {

struct SymConfig {
    int warps, p, jt;
};
constexpr int NB_SYM_CONFIGS = 8;
extern const SymConfig kSymConfigs[NB_SYM_CONFIGS];

// Resident CTAs per SM of configuration cfg (also opts it into its dynamic shared memory).
nb_status sym_ctas_per_sm(int cfg, int* out);
// Plan of one system of n bodies with at most ctas_max persistent CTAs.
nbsym::SymPlan sym_plan(int cfg, uint32_t n, uint32_t ctas_max);
// Scratch sizes of a plan: padded FP32 sources (bytes) and the two partial buffers (floats).
size_t sym_src_bytes(int cfg, const nbsym::SymPlan& S);
size_t sym_part_i_floats(int cfg, const nbsym::SymPlan& S);
size_t sym_part_j_floats(int cfg, const nbsym::SymPlan& S);
// Launches prepare + symmetric pair kernel + combine.
nb_status sym_launch(int cfg, const nbsym::SymPlan& S, const double* m, const double* x,
                     const double* y, const double* z, double G, double eps2, float4* src,
                     float* part_i, float* part_j, double* ax, double* ay, double* az,
                     uint32_t* err_word, cudaStream_t stream);

}  // namespace nb
