// nb_pair_sym.cuh -- plan and launcher of the symmetric pair kernel (nb_pair_sym.cu): FP32 with
// compensated accumulation, FP64, or double-float.
#pragma once
#include <vector>

#include "nb_internal.cuh"

namespace nbsym {

// One entry per system plus a closing entry with the totals (prefix sums): first unit, first
// body in the FP64 arrays, first padded source record and first I-block of system s. System s
// has off[s+1] - off[s] bodies in boff[s+1] - boff[s] I-blocks of IB bodies (records padded to
// whole I-blocks) and ceil(n / JT) j-tiles of JT bodies.
struct SymSys {
    uint64_t uoff;
    uint32_t off, poff, boff, pad;
};

struct SymPlan {
    const SymSys* sys;  // device, n_systems + 1 entries
    uint32_t n_systems, ctas, n_total, n_records;
    uint64_t units;
    unsigned long long wait_limit;  // polls of a tile wait before it gives up (context's limit)
};

// First unit of I-block a of a system with n_jt j-tiles (row a holds the j-tiles a * tpb ..
// n_jt - 1; a = nb gives the system's unit count).
__host__ __device__ __forceinline__ uint64_t row_off(uint32_t n_jt, uint32_t tpb, uint32_t a) {
    const uint64_t aa = a;
    return aa * n_jt - (uint64_t)tpb * (aa == 0 ? 0 : aa * (aa - 1) / 2);
}

}  // namespace nbsym

namespace nb {

// Arithmetic form of the symmetric kernel: FP32 with compensated sums, FP64, or double-float
// (FP64-accurate pair arithmetic on the FP32 pipe).
enum SymForm : int { SYM_F32 = 0, SYM_F64 = 1, SYM_DF = 2 };

// Tile shape: warps per CTA, bodies per lane, j-tile bodies.
struct SymConfig {
    int warps, p, jt;
};
constexpr int NB_SYM_CONFIGS = 8;    // FP32 shapes
constexpr int NB_SYM64_CONFIGS = 4;  // FP64 shapes
constexpr int NB_SYMDF_CONFIGS = 2;  // double-float shapes
extern const SymConfig kSymConfigs[NB_SYM_CONFIGS];
extern const SymConfig kSym64Configs[NB_SYM64_CONFIGS];
extern const SymConfig kSymDfConfigs[NB_SYMDF_CONFIGS];
int sym_config_count(int form);

// Bodies per I-block of a shape, and bytes per source record (16 FP32, 32 FP64, 48 double-float).
uint32_t sym_ib(int form, int cfg);
size_t sym_record_bytes(int form);

// Resident CTAs per SM of a shape (also opts it into its dynamic shared memory).
nb_status sym_ctas_per_sm(int form, int cfg, int* out);

// Host side of a plan: the per-system table and the totals.
struct SymHostPlan {
    std::vector<nbsym::SymSys> sys;
    uint64_t units = 0;
    uint32_t n_total = 0, n_records = 0, n_blocks = 0, ctas = 0;
};
nb_status sym_host_plan(int form, int cfg, const uint32_t* counts, uint32_t n_systems,
                        int sm_count, SymHostPlan* out);
// Scratch of a plan: i-side and j-side partials (bytes); records take
// n_records * sym_record_bytes(form).
size_t sym_part_i_bytes(int form, int cfg, uint32_t ctas, uint32_t n_blocks);
size_t sym_part_j_bytes(int form, int cfg, uint64_t units);
// Writes the device table of a single-system plan (two entries) with a kernel.
nb_status sym_single_table(nbsym::SymSys* sys, const SymHostPlan& hp, cudaStream_t stream);
// Launches prepare + symmetric pair kernel + combine for a plan whose device table is filled.
nb_status sym_launch(int form, int cfg, const nbsym::SymPlan& S, const double* m, const double* x,
                     const double* y, const double* z, double G, double eps2, void* src,
                     void* part_i, void* part_j, double* ax, double* ay, double* az,
                     uint32_t* err_word, cudaStream_t stream);

}  // namespace nb
