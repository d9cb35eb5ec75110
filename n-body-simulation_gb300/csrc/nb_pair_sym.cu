// nb_pair_sym.cu -- symmetric FP32 pair kernel with compensated accumulation: every unordered
// pair {i, j} of one system is evaluated once and its force is added to both bodies (Newton's
// third law, a_i += G m_j r_ij / r^3, a_j -= G m_i r_ij / r^3), for nb_naive_accel(NB_F32C) over
// all bodies of a system. Same per-pair arithmetic as the one-sided kernel of nb_pair.cuh
// (3 sub, 3 FMA for r^2 + eps^2, MUFU rsqrt), then 2 multiplies for r^-3, 2 for the two mass
// factors and 3 FMAs into each body's sums: 16 FP32 instructions and one rsqrt per unordered
// pair, against 24 and two for the two ordered pairs one at a time.
//
// Decomposition: bodies in I-blocks of IB = 32 W P (W warps, P bodies per lane) and j-tiles of
// JT. The units (I-block a, j-tile t) with t at or above the block's first tile form one sequence
// (row a holds n_jt - a IB/JT units); persistent CTAs take equal contiguous ranges of it
// (stream-K). A unit whose tile lies inside its own I-block ("diagonal") adds both orders of its
// pairs to the i side only; a unit above it adds each pair to both sides.
//
// Inside a unit each lane holds P i bodies in registers and walks the tile in groups of 32 j
// bodies: at step s lane l pairs its P bodies with j = (l + s) mod 32 of the group, and the j
// body's running sum moves one lane down after every step (three shuffles), so after 32 steps
// lane l holds the complete sum of body l of the group over the warp's 32 P i bodies, without a
// reduction tree. The W warps' j sums of a unit are added in warp order through shared memory and
// written, as FP32, to the unit's own slot of part_j. The i sums are folded into per-body
// (hi, lo) TwoSum accumulators once per tile and written per (CTA, I-block) as in the one-sided
// kernel. A combine pass adds, per body and in a fixed order, its i-side partials and the j-side
// partials of every unit above the diagonal in its column, in FP64: the result is deterministic.
//
// j-tiles arrive with cp.async.bulk on mbarriers (two buffers, bounded waits: on timeout the CTA
// sets the timeout bit, drains its copies in flight with bounded waits and returns).
#include "nb_internal.cuh"
#include "nb_pair.cuh"
#include "nb_pair_sym.cuh"

namespace nbsym {

using nbpair::bulk_g2s;
using nbpair::mbar_expect_tx;
using nbpair::mbar_init;
using nbpair::mbar_wait;

// Largest s in [0, count) with key(s) <= v (key non-decreasing in s, key(0) <= v).
template <typename F, typename T>
__device__ __forceinline__ uint32_t last_le(uint32_t count, T v, F key) {
    uint32_t lo = 0, hi = count;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (key(mid) <= v) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint64_t unit_begin(const SymPlan& P, uint32_t cta) {
    return (P.units * (uint64_t)cta) / P.ctas;
}

__device__ __forceinline__ uint32_t cta_of_unit(const SymPlan& P, uint64_t u) {
    uint32_t c = (uint32_t)((u * P.ctas) / P.units);
    while (c + 1 < P.ctas && unit_begin(P, c + 1) <= u) ++c;
    while (c > 0 && unit_begin(P, c) > u) --c;
    return c;
}

// Where a unit lies: system s (its bodies, I-blocks, j-tiles, records and first unit and
// I-block), I-block a and j-tile jt inside it.
struct Loc {
    uint32_t s, nb, n_jt, poff, bbase, a, jt;
    uint64_t ubase;
};

template <uint32_t TPB, int JT>
__device__ __forceinline__ Loc locate(const SymPlan& P, uint64_t u) {
    Loc L;
    L.s = last_le(P.n_systems, u, [&](uint32_t k) { return P.sys[k].uoff; });
    const SymSys A = P.sys[L.s], B = P.sys[L.s + 1];
    L.nb = B.boff - A.boff;
    L.n_jt = (B.off - A.off + JT - 1) / JT;
    L.poff = A.poff;
    L.bbase = A.boff;
    L.ubase = A.uoff;
    const uint64_t lu = u - A.uoff;
    L.a = last_le(L.nb, lu, [&](uint32_t k) { return row_off(L.n_jt, TPB, k); });
    L.jt = L.a * TPB + (uint32_t)(lu - row_off(L.n_jt, TPB, L.a));
    return L;
}

// FP32 records of all systems, each padded to whole I-blocks: positions relative to the
// system's first body (FP64 subtraction, then rounded) and G*m; pad records are massless and
// far away (they add exactly 0 to every real body).
__global__ void sym_prepare_kernel(SymPlan P, const double* __restrict__ m,
                                   const double* __restrict__ x, const double* __restrict__ y,
                                   const double* __restrict__ z, double G,
                                   float4* __restrict__ out) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= P.n_records) return;
    const uint32_t s = last_le(P.n_systems, r, [&](uint32_t k) { return P.sys[k].poff; });
    const SymSys A = P.sys[s], B = P.sys[s + 1];
    const uint32_t t = r - A.poff;
    if (t < B.off - A.off) {
        const uint32_t b = A.off + t, a0 = A.off;
        out[r] = make_float4((float)(x[b] - x[a0]), (float)(y[b] - y[a0]), (float)(z[b] - z[a0]),
                             (float)(G * m[b]));
    } else {
        out[r] = make_float4(1e18f, 1e18f, 1e18f, 0.f);
    }
}

// The table of a single system of n bodies (nb I-blocks, `records` padded records, `units`
// units), written by a kernel so that it can be part of a captured graph.
__global__ void sym_single_table_kernel(SymSys* sys, uint32_t n, uint32_t nb, uint32_t records,
                                        uint64_t units) {
    sys[0] = SymSys{0, 0, 0, 0, 0};
    sys[1] = SymSys{units, n, records, nb, 0};
}

template <int W, int P, int JT>
__global__ void __launch_bounds__(32 * W)
pair_sym_kernel(SymPlan S, const float4* __restrict__ src, float eps2, float* __restrict__ part_i,
                float* __restrict__ part_j, uint32_t* __restrict__ err_word) {
    constexpr int THREADS = 32 * W;
    constexpr int IB = THREADS * P;
    constexpr uint32_t TPB = IB / JT;
    static_assert(IB % JT == 0 && JT % 32 == 0, "tile shape");
    extern __shared__ __align__(128) unsigned char sym_smem[];
    float4 (*tile)[JT] = reinterpret_cast<float4 (*)[JT]>(sym_smem);
    // per-warp j sums of the current unit, two buffers (alternating units)
    float (*jacc)[W][3][JT] =
        reinterpret_cast<float (*)[W][3][JT]>(sym_smem + 2 * JT * sizeof(float4));
    // compensated i sums hl[c][k][thread], c = hx, hy, hz, lx, ly, lz
    float (*hl)[P][THREADS] = reinterpret_cast<float (*)[P][THREADS]>(
        sym_smem + 2 * JT * sizeof(float4) + (size_t)2 * W * 3 * JT * sizeof(float));
    __shared__ __align__(8) uint64_t full[2];

    const uint32_t cta = blockIdx.x;
    const uint64_t u0 = unit_begin(S, cta), u1 = unit_begin(S, cta + 1);
    if (u0 >= u1) return;
    if (threadIdx.x == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // Thread 0 copies the j-tile of unit c_u into buffer buf and moves on to the next unit.
    uint64_t c_u = u0;
    auto issue = [&](int buf) {
        const Loc L = locate<TPB, JT>(S, c_u);
        mbar_expect_tx(&full[buf], JT * (uint32_t)sizeof(float4));
        bulk_g2s(&tile[buf][0], src + L.poff + (size_t)L.jt * JT, JT * (uint32_t)sizeof(float4),
                 &full[buf]);
        ++c_u;
    };
    if (threadIdx.x == 0) {
        issue(0);
        if (u0 + 1 < u1) issue(1);
    }

    const int th = threadIdx.x, lane = th & 31, w = th >> 5;
    float xi[P], yi[P], zi[P], mi[P], fx[P], fy[P], fz[P];
    uint64_t u = u0;
    uint32_t iter = 0;
    bool failed = false;
    while (u < u1 && !failed) {
        const Loc L = locate<TPB, JT>(S, u);
        const uint32_t a = L.a;
        const uint64_t seg_end = min(u1, L.ubase + row_off(L.n_jt, TPB, a + 1));
        uint32_t jt = L.jt;
        const float4* isrc = src + L.poff + (size_t)a * IB + w * 32 * P + lane;
#pragma unroll
        for (int k = 0; k < P; ++k) {
            const float4 b = isrc[k * 32];
            xi[k] = b.x;
            yi[k] = b.y;
            zi[k] = b.z;
            mi[k] = b.w;
#pragma unroll
            for (int c = 0; c < 6; ++c) hl[c][k][th] = 0.f;
        }
        for (; u < seg_end; ++u, ++iter, ++jt) {
            const int buf = iter & 1;
            const bool ok = mbar_wait(&full[buf], (iter >> 1) & 1);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
#pragma unroll
            for (int k = 0; k < P; ++k) fx[k] = fy[k] = fz[k] = 0.f;
#pragma unroll 1
            for (int g = 0; g < JT / 32; ++g) {
                const float4* G4 = &tile[buf][g * 32];
                float jx = 0.f, jy = 0.f, jz = 0.f;  // sums of body (lane + s) mod 32 of the group
#pragma unroll 4
                for (int s = 0; s < 32; ++s) {
                    const float4 J = G4[(lane + s) & 31];
#pragma unroll
                    for (int k = 0; k < P; ++k) {
                        const float dx = J.x - xi[k], dy = J.y - yi[k], dz = J.z - zi[k];
                        const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
                        const float inv = nb_rsqrt_f32(r2);
                        const float inv3 = (inv * inv) * inv;
                        const float sj = J.w * inv3, si = mi[k] * inv3;
                        fx[k] = fmaf(dx, sj, fx[k]);
                        fy[k] = fmaf(dy, sj, fy[k]);
                        fz[k] = fmaf(dz, sj, fz[k]);
                        jx = fmaf(-dx, si, jx);
                        jy = fmaf(-dy, si, jy);
                        jz = fmaf(-dz, si, jz);
                    }
                    // the sum of body (l + s + 1) mod 32 comes from lane l + 1
                    jx = __shfl_sync(0xffffffffu, jx, (lane + 1) & 31);
                    jy = __shfl_sync(0xffffffffu, jy, (lane + 1) & 31);
                    jz = __shfl_sync(0xffffffffu, jz, (lane + 1) & 31);
                }
                // after 32 rotations lane l holds the sum of body l of the group
                jacc[buf][w][0][g * 32 + lane] = jx;
                jacc[buf][w][1][g * 32 + lane] = jy;
                jacc[buf][w][2][g * 32 + lane] = jz;
            }
#pragma unroll
            for (int k = 0; k < P; ++k) {
                float h0 = hl[0][k][th], h1 = hl[1][k][th], h2 = hl[2][k][th];
                float l0 = hl[3][k][th], l1 = hl[4][k][th], l2 = hl[5][k][th];
                NB_TWOSUM(h0, l0, fx[k]);
                NB_TWOSUM(h1, l1, fy[k]);
                NB_TWOSUM(h2, l2, fz[k]);
                hl[0][k][th] = h0;
                hl[1][k][th] = h1;
                hl[2][k][th] = h2;
                hl[3][k][th] = l0;
                hl[4][k][th] = l1;
                hl[5][k][th] = l2;
            }
            __syncthreads();
            if (jt >= (a + 1) * TPB) {  // above the diagonal: the j sums of this unit
                float* out = part_j + u * 3 * JT;
                for (int jl = th; jl < JT; jl += THREADS) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        float s = jacc[buf][0][c][jl];
#pragma unroll
                        for (int v = 1; v < W; ++v) s += jacc[buf][v][c][jl];
                        out[c * JT + jl] = s;
                    }
                }
            }
            if (threadIdx.x == 0 && u + 2 < u1) issue(buf);  // the cursor is at u + 2
        }
        if (failed) break;
        float* out = part_i + (size_t)(cta + L.bbase + a) * 6 * IB + w * 32 * P + lane;
#pragma unroll
        for (int k = 0; k < P; ++k)
#pragma unroll
            for (int c = 0; c < 6; ++c) out[c * IB + k * 32] = hl[c][k][th];
    }
    if (failed) {
        if (threadIdx.x == 0) atomicOr(err_word, NB_DEVERR_TIMEOUT);
        for (uint32_t k = iter; k < iter + 2 && u0 + k < u1; ++k)
            mbar_wait(&full[k & 1], (k >> 1) & 1);
    }
}

// Per body: its i-side partials (CTA order) and the j-side partials of the units above the
// diagonal in its column (I-block order), summed in FP64.
template <int IB, int JT>
__global__ void sym_combine_kernel(SymPlan S, const float* __restrict__ part_i,
                                   const float* __restrict__ part_j, double* __restrict__ ax,
                                   double* __restrict__ ay, double* __restrict__ az) {
    constexpr uint32_t TPB = IB / JT;
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= S.n_total) return;
    const uint32_t s = last_le(S.n_systems, b, [&](uint32_t k) { return S.sys[k].off; });
    const SymSys A = S.sys[s], B = S.sys[s + 1];
    const uint32_t n_jt = (B.off - A.off + JT - 1) / JT;
    const uint32_t t = b - A.off;
    const uint32_t a = t / IB, li = t % IB, jt = t / JT, jl = t % JT;
    const uint32_t c0 = cta_of_unit(S, A.uoff + row_off(n_jt, TPB, a));
    const uint32_t c1 = cta_of_unit(S, A.uoff + row_off(n_jt, TPB, a + 1) - 1);
    double sx = 0, sy = 0, sz = 0;
    for (uint32_t c = c0; c <= c1; ++c) {
        const float* p = part_i + (size_t)(c + A.boff + a) * 6 * IB;
        sx += (double)p[0 * IB + li] + (double)p[3 * IB + li];
        sy += (double)p[1 * IB + li] + (double)p[4 * IB + li];
        sz += (double)p[2 * IB + li] + (double)p[5 * IB + li];
    }
    for (uint32_t r = 0; r < a; ++r) {
        const float* p = part_j + (A.uoff + row_off(n_jt, TPB, r) + (jt - r * TPB)) * 3 * JT;
        sx += (double)p[jl];
        sy += (double)p[JT + jl];
        sz += (double)p[2 * JT + jl];
    }
    ax[b] = sx;
    ay[b] = sy;
    az[b] = sz;
}

}  // namespace nbsym

namespace nb {

// (warps, bodies per lane, j-tile); the table, the occupancy query and the launch switch list
// the same instantiations
#define NB_SYM_CONFIG_LIST(X)                                                            \
    X(0, 8, 12, 128) X(1, 4, 12, 256) X(2, 4, 12, 128) X(3, 4, 16, 128) X(4, 8, 8, 256)       \
        X(5, 4, 8, 256) X(6, 8, 6, 256) X(7, 2, 12, 128)

const SymConfig kSymConfigs[NB_SYM_CONFIGS] = {
#define NB_SYM_ROW(i, W, P, JT) {W, P, JT},
    NB_SYM_CONFIG_LIST(NB_SYM_ROW)
#undef NB_SYM_ROW
};

namespace {

int g_sym_ctas_per_sm[NB_SYM_CONFIGS] = {};

template <int W, int P, int JT>
constexpr size_t sym_smem_bytes() {
    return 2 * JT * sizeof(float4) + (size_t)2 * W * 3 * JT * sizeof(float) +
           (size_t)6 * P * 32 * W * sizeof(float);
}

template <int W, int P, int JT>
nb_status sym_prepare(int* out) {
    constexpr size_t smem = sym_smem_bytes<W, P, JT>();
    NB_CUDA_TRY(cudaFuncSetAttribute(nbsym::pair_sym_kernel<W, P, JT>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    NB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        out, nbsym::pair_sym_kernel<W, P, JT>, 32 * W, smem));
    if (*out < 1) *out = 1;
    return NB_OK;
}

template <int W, int P, int JT>
nb_status sym_launch_cfg(const nbsym::SymPlan& S, const float4* src, float eps2, float* part_i,
                         float* part_j, double* ax, double* ay, double* az, uint32_t* err_word,
                         cudaStream_t stream) {
    nbsym::pair_sym_kernel<W, P, JT><<<S.ctas, 32 * W, sym_smem_bytes<W, P, JT>(), stream>>>(
        S, src, eps2, part_i, part_j, err_word);
    NB_TRY(check_launch("pair_sym_kernel"));
    nbsym::sym_combine_kernel<32 * W * P, JT><<<ceil_div(S.n_total, 256), 256, 0, stream>>>(
        S, part_i, part_j, ax, ay, az);
    return check_launch("sym_combine_kernel");
}

}  // namespace

nb_status sym_ctas_per_sm(int cfg, int* out) {
    if (cfg < 0 || cfg >= NB_SYM_CONFIGS)
        return set_error(NB_ERR_INVALID_ARG, "bad symmetric pair config %d", cfg);
    if (g_sym_ctas_per_sm[cfg] == 0) {
        int v = 0;
        switch (cfg) {
#define NB_SYM_PREP(i, W, P, JT) \
    case i: NB_TRY((sym_prepare<W, P, JT>(&v))); break;
            NB_SYM_CONFIG_LIST(NB_SYM_PREP)
#undef NB_SYM_PREP
        }
        g_sym_ctas_per_sm[cfg] = v;
    }
    *out = g_sym_ctas_per_sm[cfg];
    return NB_OK;
}

nb_status sym_host_plan(int cfg, const uint32_t* counts, uint32_t n_systems, int sm_count,
                        SymHostPlan* out) {
    const SymConfig& C = kSymConfigs[cfg];
    const uint32_t ib = sym_ib(cfg), tpb = ib / (uint32_t)C.jt;
    out->sys.assign(n_systems + 1, nbsym::SymSys{0, 0, 0, 0, 0});
    for (uint32_t s = 0; s < n_systems; ++s) {
        const nbsym::SymSys& A = out->sys[s];
        const uint32_t n = counts[s];
        const uint32_t nb = (n + ib - 1) / ib, n_jt = (n + C.jt - 1) / C.jt;
        const uint64_t records = (uint64_t)A.poff + (uint64_t)nb * ib;
        if (records > 0xffffffffull)
            return set_error(NB_ERR_INVALID_ARG, "symmetric pair plan: more than 2^32 records");
        out->sys[s + 1] = nbsym::SymSys{A.uoff + nbsym::row_off(n_jt, tpb, nb), A.off + n,
                                        (uint32_t)records, A.boff + nb, 0};
    }
    int per_sm = 0;
    NB_TRY(sym_ctas_per_sm(cfg, &per_sm));
    const nbsym::SymSys& E = out->sys[n_systems];
    out->units = E.uoff;
    out->n_total = E.off;
    out->n_records = E.poff;
    out->n_blocks = E.boff;
    uint64_t ctas = (uint64_t)sm_count * per_sm;
    if (ctas > out->units) ctas = out->units;
    out->ctas = (uint32_t)(ctas ? ctas : 1);
    return NB_OK;
}

size_t sym_part_i_floats(int cfg, uint32_t ctas, uint32_t n_blocks) {
    return ((size_t)ctas + n_blocks) * 6 * sym_ib(cfg);
}
size_t sym_part_j_floats(int cfg, uint64_t units) {
    return (size_t)units * 3 * kSymConfigs[cfg].jt;
}

nb_status sym_single_table(nbsym::SymSys* sys, const SymHostPlan& hp, cudaStream_t stream) {
    const nbsym::SymSys& E = hp.sys[1];
    nbsym::sym_single_table_kernel<<<1, 1, 0, stream>>>(sys, E.off, E.boff, E.poff, E.uoff);
    return check_launch("sym_single_table_kernel");
}

nb_status sym_launch(int cfg, const nbsym::SymPlan& S, const double* m, const double* x,
                     const double* y, const double* z, double G, double eps2, float4* src,
                     float* part_i, float* part_j, double* ax, double* ay, double* az,
                     uint32_t* err_word, cudaStream_t stream) {
    int per_sm = 0;
    NB_TRY(sym_ctas_per_sm(cfg, &per_sm));  // shared-memory opt-in before the first launch
    if (S.units == 0) return NB_OK;
    nbsym::sym_prepare_kernel<<<ceil_div(S.n_records, 256), 256, 0, stream>>>(S, m, x, y, z, G,
                                                                              src);
    NB_TRY(check_launch("sym_prepare_kernel"));
    switch (cfg) {
#define NB_SYM_LAUNCH(i, W, P, JT)                                                               \
    case i:                                                                                      \
        return sym_launch_cfg<W, P, JT>(S, src, (float)eps2, part_i, part_j, ax, ay, az, err_word, \
                                        stream);
        NB_SYM_CONFIG_LIST(NB_SYM_LAUNCH)
#undef NB_SYM_LAUNCH
        default: return set_error(NB_ERR_INVALID_ARG, "bad symmetric pair config %d", cfg);
    }
}

}  // namespace nb
