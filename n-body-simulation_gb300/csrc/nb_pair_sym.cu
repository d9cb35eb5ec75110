// nb_pair_sym.cu -- symmetric pair kernel: every unordered pair {i, j} of a system is evaluated
// once and its force is added to both bodies (Newton's third law, a_i += G m_j r_ij / r^3,
// a_j -= G m_i r_ij / r^3). Three arithmetic forms share the decomposition:
//  * FP32 with compensated accumulation (nb_naive_accel NB_F32C over whole systems, and batches):
//    positions relative to the system's first body and G*m in FP32; per unordered pair 3 sub,
//    3 FMA for r^2 + eps^2, one MUFU rsqrt, 2 multiplies for r^-3, 2 for the two mass factors and
//    3 FMAs into each body's sums: 16 FP32 instructions and one rsqrt, against 24 and two for the
//    two ordered pairs one at a time (nb_pair.cuh).
//  * FP64 (nb_naive_accel NB_F64 over whole systems): the positions and masses as given; r^-3 from
//    the hardware rsqrt estimate with one correction of its cube (6 FP64 operations), 20 FP64
//    operations per unordered pair against 32 for the two ordered pairs; G applied once at the end
//    as in NaiveAlgorithm.cpp:348-351.
//  * Double-float (nb_naive_accel NB_DF64 over whole systems): positions relative to the system's
//    first body as exact triple-floats and G*m as a double-float; the separation, r^2 + eps^2,
//    1/r and r^-3 in double-float arithmetic are shared by the two bodies, only the mass products,
//    the force terms and the compensated sums are per body (pair_sym_df_kernel).
//
// Decomposition: per system, bodies in I-blocks of IB = 32 W P (W warps, P bodies per lane) and
// j-tiles of JT; I-block a owns the j-tiles from its own first tile to the system's last, and the
// units (system, I-block, j-tile) of all systems form one sequence that persistent CTAs split into
// equal contiguous ranges (stream-K). A unit whose tile lies inside its own I-block ("diagonal")
// adds both orders of its pairs to the i side only; a unit above it adds each pair to both sides.
//
// Inside a unit each lane holds P i bodies in registers and walks the tile in groups of 32 j
// bodies: at step s lane l pairs its P bodies with j = (l + s) mod 32 of the group, and the j
// body's running sum moves one lane down after every step (three shuffles; six for the (hi, lo)
// sums of the double-float form), so after 32 steps
// lane l holds the complete sum of body l of the group over the warp's 32 P i bodies, without a
// reduction tree. The W warps' j sums of a unit are added in warp order through shared memory and
// written to the unit's own slot of part_j. FP32 i sums are folded into per-body (hi, lo) TwoSum
// accumulators once per tile; FP64 i sums stay in registers for the whole row segment; both are
// written per (CTA, I-block) as in the one-sided kernel. A combine pass adds, per body and in a
// fixed order, its i-side partials and the j-side partials of every unit above the diagonal in its
// column, in FP64: the result is deterministic.
//
// j-tiles arrive with cp.async.bulk on mbarriers (two buffers, bounded waits: on timeout the CTA
// sets the timeout bit, drains its copies in flight with bounded waits and returns).
#include <type_traits>

#include "nb_internal.cuh"
#include "nb_pair.cuh"
#include "nb_pair_sym.cuh"

namespace nbsym {

using nbpair::bulk_g2s;
using nbpair::mbar_expect_tx;
using nbpair::mbar_init;
using nbpair::mbar_wait;

// FP64 source record {x, y, z, m}.
struct __align__(32) Rec64 {
    double x, y, z, m;
};

template <typename R>
struct RecOf {
    using type = float4;
};
template <>
struct RecOf<double> {
    using type = Rec64;
};

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

// Where a unit lies: system s (its I-blocks, j-tiles, first record, first I-block and first
// unit), I-block a and j-tile jt inside it.
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

// Source records of all systems, each padded to whole I-blocks. FP32: positions relative to the
// system's first body (FP64 subtraction, then rounded) and G*m; FP64: positions and m as given.
// Pad records are massless and far away (they add exactly 0 to every real body).
template <typename R>
__global__ void sym_prepare_kernel(SymPlan P, const double* __restrict__ m,
                                   const double* __restrict__ x, const double* __restrict__ y,
                                   const double* __restrict__ z, double G,
                                   typename RecOf<R>::type* __restrict__ out) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= P.n_records) return;
    const uint32_t s = last_le(P.n_systems, r, [&](uint32_t k) { return P.sys[k].poff; });
    const SymSys A = P.sys[s], B = P.sys[s + 1];
    const uint32_t t = r - A.poff;
    const bool real = t < B.off - A.off;
    const uint32_t b = A.off + t;
    if constexpr (std::is_same<R, double>::value) {
        out[r] = real ? Rec64{x[b], y[b], z[b], m[b]} : Rec64{1e150, 1e150, 1e150, 0.0};
    } else {
        const uint32_t a0 = A.off;
        out[r] = real ? make_float4((float)(x[b] - x[a0]), (float)(y[b] - y[a0]),
                                    (float)(z[b] - z[a0]), (float)(G * m[b]))
                      : make_float4(1e18f, 1e18f, 1e18f, 0.f);
    }
}

// The table of a single system of n bodies (nb I-blocks, `records` padded records, `units`
// units), written by a kernel so that it can be part of a captured graph.
__global__ void sym_single_table_kernel(SymSys* sys, uint32_t n, uint32_t nb, uint32_t records,
                                        uint64_t units) {
    sys[0] = SymSys{0, 0, 0, 0, 0};
    sys[1] = SymSys{units, n, records, nb, 0};
}

// Double-float source record: the position minus the system's first body as exact
// triple-floats, G*m as a double-float.
struct __align__(16) RecTF {
    float xh, xm, xl, yh, ym, yl, zh, zm, zl, gh, gl, pad;
};

__global__ void sym_prepare_tf_kernel(SymPlan P, const double* __restrict__ m,
                                      const double* __restrict__ x, const double* __restrict__ y,
                                      const double* __restrict__ z, double G,
                                      RecTF* __restrict__ out) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= P.n_records) return;
    const uint32_t s = last_le(P.n_systems, r, [&](uint32_t k) { return P.sys[k].poff; });
    const SymSys A = P.sys[s], B = P.sys[s + 1];
    const uint32_t t = r - A.poff;
    RecTF o{1e18f, 0.f, 0.f, 1e18f, 0.f, 0.f, 1e18f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (t < B.off - A.off) {
        const uint32_t b = A.off + t, a0 = A.off;
        tf_split_diff(x[b], x[a0], o.xh, o.xm, o.xl);
        tf_split_diff(y[b], y[a0], o.yh, o.ym, o.yl);
        tf_split_diff(z[b], z[a0], o.zh, o.zm, o.zl);
        const double gm = G * m[b];
        o.gh = (float)gm;
        o.gl = (float)(gm - (double)o.gh);
    }
    out[r] = o;
}

template <typename R>
__device__ __forceinline__ R fma_r(R a, R b, R c) {
    if constexpr (std::is_same<R, float>::value) return fmaf(a, b, c); else return fma(a, b, c);
}

// den^(-3/2) in FP64: hardware estimate y0 of den^(-1/2) and one correction of its cube,
// (1 - e)^(-3/2) = 1 + 3e/2 + 15e^2/8 + O(e^3) with e = 1 - den y0^2 (|e| < 2^-21, dropped terms
// below 2^-62): 6 FP64 operations.
__device__ __forceinline__ double nb_rinv3_f64(double den) {
    double y0;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y0) : "d"(den));
    const double y2 = y0 * y0;
    const double e = fma(-den, y2, 1.0);
    const double p = fma(1.875, e, 1.5);
    const double w0 = y2 * y0;
    return fma(w0 * e, p, w0);
}

// Shared memory of a shape: two j-tiles, two buffers of per-warp j sums and, for FP32, the
// compensated i sums.
template <typename R, int W, int P, int JT>
constexpr size_t sym_smem_bytes() {
    return 2 * JT * sizeof(typename RecOf<R>::type) + (size_t)2 * W * 3 * JT * sizeof(R) +
           (std::is_same<R, float>::value ? (size_t)6 * P * 32 * W * sizeof(float) : 0);
}

template <typename R, int W, int P, int JT>
__global__ void __launch_bounds__(32 * W)
pair_sym_kernel(SymPlan S, const typename RecOf<R>::type* __restrict__ src, R eps2,
                R* __restrict__ part_i, R* __restrict__ part_j, uint32_t* __restrict__ err_word) {
    using Rec = typename RecOf<R>::type;
    constexpr bool F64 = std::is_same<R, double>::value;
    constexpr int THREADS = 32 * W;
    constexpr int IB = THREADS * P;
    constexpr uint32_t TPB = IB / JT;
    static_assert(IB % JT == 0 && JT % 32 == 0, "tile shape");
    extern __shared__ __align__(128) unsigned char sym_smem[];
    Rec (*tile)[JT] = reinterpret_cast<Rec (*)[JT]>(sym_smem);
    // per-warp j sums of the current unit, two buffers (alternating units)
    R (*jacc)[W][3][JT] = reinterpret_cast<R (*)[W][3][JT]>(sym_smem + 2 * JT * sizeof(Rec));
    // FP32: compensated i sums hl[c][k][thread], c = hx, hy, hz, lx, ly, lz
    float (*hl)[P][THREADS] = reinterpret_cast<float (*)[P][THREADS]>(
        sym_smem + 2 * JT * sizeof(Rec) + (size_t)2 * W * 3 * JT * sizeof(R));
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
        mbar_expect_tx(&full[buf], JT * (uint32_t)sizeof(Rec));
        bulk_g2s(&tile[buf][0], src + L.poff + (size_t)L.jt * JT, JT * (uint32_t)sizeof(Rec),
                 &full[buf]);
        ++c_u;
    };
    if (threadIdx.x == 0) {
        issue(0);
        if (u0 + 1 < u1) issue(1);
    }

    const int th = threadIdx.x, lane = th & 31, w = th >> 5;
    R xi[P], yi[P], zi[P], mi[P], fx[P], fy[P], fz[P];
    uint64_t u = u0;
    uint32_t iter = 0;
    bool failed = false;
    while (u < u1 && !failed) {
        const Loc L = locate<TPB, JT>(S, u);
        const uint32_t a = L.a;
        const uint64_t seg_end = min(u1, L.ubase + row_off(L.n_jt, TPB, a + 1));
        uint32_t jt = L.jt;
        const Rec* isrc = src + L.poff + (size_t)a * IB + w * 32 * P + lane;
#pragma unroll
        for (int k = 0; k < P; ++k) {
            const Rec b = isrc[k * 32];
            xi[k] = b.x;
            yi[k] = b.y;
            zi[k] = b.z;
            if constexpr (F64) {
                mi[k] = b.m;
                fx[k] = fy[k] = fz[k] = 0.0;
            } else {
                mi[k] = b.w;
#pragma unroll
                for (int c = 0; c < 6; ++c) hl[c][k][th] = 0.f;
            }
        }
        for (; u < seg_end; ++u, ++iter, ++jt) {
            const int buf = iter & 1;
            const bool ok = mbar_wait(&full[buf], (iter >> 1) & 1, S.wait_limit);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            if constexpr (!F64) {
#pragma unroll
                for (int k = 0; k < P; ++k) fx[k] = fy[k] = fz[k] = 0.f;
            }
#pragma unroll 1
            for (int g = 0; g < JT / 32; ++g) {
                const Rec* G4 = &tile[buf][g * 32];
                R jx = 0, jy = 0, jz = 0;  // sums of body (lane + s) mod 32 of the group
#pragma unroll 8
                for (int s = 0; s < 32; ++s) {
                    const Rec J = G4[(lane + s) & 31];
                    R jm;
                    if constexpr (F64) jm = J.m; else jm = J.w;
#pragma unroll
                    for (int k = 0; k < P; ++k) {
                        const R dx = J.x - xi[k], dy = J.y - yi[k], dz = J.z - zi[k];
                        R inv3;
                        if constexpr (F64) {
                            inv3 = nb_rinv3_f64(fma(dz, dz, fma(dy, dy, fma(dx, dx, eps2))));
                        } else {
                            const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
                            const float inv = nb_rsqrt_f32(r2);
                            inv3 = (inv * inv) * inv;
                        }
                        const R sj = jm * inv3, si = mi[k] * inv3;
                        fx[k] = fma_r(dx, sj, fx[k]);
                        fy[k] = fma_r(dy, sj, fy[k]);
                        fz[k] = fma_r(dz, sj, fz[k]);
                        jx = fma_r(-dx, si, jx);
                        jy = fma_r(-dy, si, jy);
                        jz = fma_r(-dz, si, jz);
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
            if constexpr (!F64) {
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
            }
            __syncthreads();
            if (jt >= (a + 1) * TPB) {  // above the diagonal: the j sums of this unit
                R* out = part_j + u * 3 * JT;
                for (int jl = th; jl < JT; jl += THREADS) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        R s = jacc[buf][0][c][jl];
#pragma unroll
                        for (int v = 1; v < W; ++v) s += jacc[buf][v][c][jl];
                        out[c * JT + jl] = s;
                    }
                }
            }
            if (threadIdx.x == 0 && u + 2 < u1) issue(buf);  // the cursor is at u + 2
        }
        if (failed) break;
        if constexpr (F64) {
            R* out = part_i + (size_t)(cta + L.bbase + a) * 3 * IB + w * 32 * P + lane;
#pragma unroll
            for (int k = 0; k < P; ++k) {
                out[0 * IB + k * 32] = fx[k];
                out[1 * IB + k * 32] = fy[k];
                out[2 * IB + k * 32] = fz[k];
            }
        } else {
            R* out = part_i + (size_t)(cta + L.bbase + a) * 6 * IB + w * 32 * P + lane;
#pragma unroll
            for (int k = 0; k < P; ++k)
#pragma unroll
                for (int c = 0; c < 6; ++c) out[c * IB + k * 32] = hl[c][k][th];
        }
    }
    if (failed) {  // drain the copies of units iter, iter + 1 before leaving (default limit)
        bool drained = true;
        for (uint32_t k = iter; k < iter + 2 && u0 + k < u1; ++k)
            drained &= mbar_wait(&full[k & 1], (k >> 1) & 1, NB_WAIT_LIMIT_DEFAULT);
        if (threadIdx.x == 0)
            atomicOr(err_word, NB_DEVERR_TIMEOUT | (drained ? 0u : NB_DEVERR_DRAIN));
    }
}

// Double-float form: the decomposition, copies and partial layout of the FP64 form (FP64 i
// totals per row segment, FP64 j partials per unit); per pair the arithmetic of the one-sided
// double-float kernel (exact triple-float separation, r^2 + eps^2 with TwoSums, 1/r from the
// hardware estimate with an error-free correction, products in double-float), once for both
// bodies; per-tile Neumaier-compensated FP32 sums folded into the FP64 totals.
template <int W, int P, int JT>
constexpr size_t sym_df_smem_bytes() {
    return 2 * JT * sizeof(RecTF) + (size_t)2 * W * 3 * JT * sizeof(double);
}

template <int W, int P, int JT>
__global__ void __launch_bounds__(32 * W)
pair_sym_df_kernel(SymPlan S, const RecTF* __restrict__ src, float e2h, float e2l,
                   double* __restrict__ part_i, double* __restrict__ part_j,
                   uint32_t* __restrict__ err_word) {
    constexpr int THREADS = 32 * W;
    constexpr int IB = THREADS * P;
    constexpr uint32_t TPB = IB / JT;
    static_assert(IB % JT == 0 && JT % 32 == 0, "tile shape");
    extern __shared__ __align__(128) unsigned char sym_smem[];
    RecTF (*tile)[JT] = reinterpret_cast<RecTF (*)[JT]>(sym_smem);
    double (*jacc)[W][3][JT] =
        reinterpret_cast<double (*)[W][3][JT]>(sym_smem + 2 * JT * sizeof(RecTF));
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
    uint64_t c_u = u0;
    auto issue = [&](int buf) {
        const Loc L = locate<TPB, JT>(S, c_u);
        mbar_expect_tx(&full[buf], JT * (uint32_t)sizeof(RecTF));
        bulk_g2s(&tile[buf][0], src + L.poff + (size_t)L.jt * JT, JT * (uint32_t)sizeof(RecTF),
                 &full[buf]);
        ++c_u;
    };
    if (threadIdx.x == 0) {
        issue(0);
        if (u0 + 1 < u1) issue(1);
    }

    const int th = threadIdx.x, lane = th & 31, w = th >> 5;
    RecTF I[P];
    double tx[P], ty[P], tz[P];
    uint64_t u = u0;
    uint32_t iter = 0;
    bool failed = false;
    while (u < u1 && !failed) {
        const Loc L = locate<TPB, JT>(S, u);
        const uint32_t a = L.a;
        const uint64_t seg_end = min(u1, L.ubase + row_off(L.n_jt, TPB, a + 1));
        uint32_t jt = L.jt;
        const RecTF* isrc = src + L.poff + (size_t)a * IB + w * 32 * P + lane;
#pragma unroll
        for (int k = 0; k < P; ++k) {
            I[k] = isrc[k * 32];
            tx[k] = ty[k] = tz[k] = 0.0;
        }
        for (; u < seg_end; ++u, ++iter, ++jt) {
            const int buf = iter & 1;
            const bool ok = mbar_wait(&full[buf], (iter >> 1) & 1, S.wait_limit);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            float ahx[P], alx[P], ahy[P], aly[P], ahz[P], alz[P];
#pragma unroll
            for (int k = 0; k < P; ++k) ahx[k] = alx[k] = ahy[k] = aly[k] = ahz[k] = alz[k] = 0.f;
#pragma unroll 1
            for (int g = 0; g < JT / 32; ++g) {
                const RecTF* G4 = &tile[buf][g * 32];
                // compensated sums of body (lane + s) mod 32 of the group
                float jhx = 0.f, jlx = 0.f, jhy = 0.f, jly = 0.f, jhz = 0.f, jlz = 0.f;
#pragma unroll 1
                for (int s = 0; s < 32; ++s) {
                    const RecTF J = G4[(lane + s) & 31];
#pragma unroll
                    for (int k = 0; k < P; ++k) {
                        const nb_df dx = tf_diff(J.xh, J.xm, J.xl, I[k].xh, I[k].xm, I[k].xl);
                        const nb_df dy = tf_diff(J.yh, J.ym, J.yl, I[k].yh, I[k].ym, I[k].yl);
                        const nb_df dz = tf_diff(J.zh, J.zm, J.zl, I[k].zh, I[k].zm, I[k].zl);
                        const nb_df sx = df_sqr(dx), sy = df_sqr(dy), sz = df_sqr(dz);
                        nb_df c1 = df_two_sum(sx.h, sy.h);
                        c1.l += sx.l + sy.l;
                        nb_df c2 = df_two_sum(c1.h, sz.h);
                        c2.l += c1.l + sz.l;
                        nb_df c3 = df_two_sum(c2.h, e2h);
                        c3.l += c2.l + e2l;
                        const nb_df r2 = df_two_sum(c3.h, c3.l);
                        const float y0 = nb_rsqrt_f32(r2.h);
                        const float q = y0 * y0, qe = fmaf(y0, y0, -q);  // y0^2 = q + qe
                        const float th2 = r2.h * q;
                        float te = fmaf(r2.h, q, -th2);
                        te = fmaf(r2.h, qe, te);
                        te = fmaf(r2.l, q, te);
                        const float e = (1.0f - th2) - te;
                        const nb_df inv = df_fast_two_sum(y0, y0 * (e * fmaf(0.375f, e, 0.5f)));
                        const nb_df inv3 = df_mul(df_sqr(inv), inv);
                        const nb_df wj = df_mul(nb_df{J.gh, J.gl}, inv3);
                        const nb_df wi = df_mul(nb_df{I[k].gh, I[k].gl}, inv3);
                        // body i: + (x_j - x_i) G m_j / r^3
                        nb_df t = df_mul(dx, wj);
                        nb_df v = df_two_sum(ahx[k], t.h);
                        ahx[k] = v.h;
                        alx[k] += v.l + t.l;
                        t = df_mul(dy, wj);
                        v = df_two_sum(ahy[k], t.h);
                        ahy[k] = v.h;
                        aly[k] += v.l + t.l;
                        t = df_mul(dz, wj);
                        v = df_two_sum(ahz[k], t.h);
                        ahz[k] = v.h;
                        alz[k] += v.l + t.l;
                        // body j: - (x_j - x_i) G m_i / r^3
                        t = df_mul(dx, wi);
                        v = df_two_sum(jhx, -t.h);
                        jhx = v.h;
                        jlx += v.l - t.l;
                        t = df_mul(dy, wi);
                        v = df_two_sum(jhy, -t.h);
                        jhy = v.h;
                        jly += v.l - t.l;
                        t = df_mul(dz, wi);
                        v = df_two_sum(jhz, -t.h);
                        jhz = v.h;
                        jlz += v.l - t.l;
                    }
                    // the sums of body (l + s + 1) mod 32 come from lane l + 1
                    const int src_lane = (lane + 1) & 31;
                    jhx = __shfl_sync(0xffffffffu, jhx, src_lane);
                    jlx = __shfl_sync(0xffffffffu, jlx, src_lane);
                    jhy = __shfl_sync(0xffffffffu, jhy, src_lane);
                    jly = __shfl_sync(0xffffffffu, jly, src_lane);
                    jhz = __shfl_sync(0xffffffffu, jhz, src_lane);
                    jlz = __shfl_sync(0xffffffffu, jlz, src_lane);
                }
                // after 32 rotations lane l holds the sums of body l of the group
                jacc[buf][w][0][g * 32 + lane] = (double)jhx + (double)jlx;
                jacc[buf][w][1][g * 32 + lane] = (double)jhy + (double)jly;
                jacc[buf][w][2][g * 32 + lane] = (double)jhz + (double)jlz;
            }
#pragma unroll
            for (int k = 0; k < P; ++k) {
                tx[k] += (double)ahx[k] + (double)alx[k];
                ty[k] += (double)ahy[k] + (double)aly[k];
                tz[k] += (double)ahz[k] + (double)alz[k];
            }
            __syncthreads();
            if (jt >= (a + 1) * TPB) {  // above the diagonal: the j sums of this unit
                double* out = part_j + u * 3 * JT;
                for (int jl = th; jl < JT; jl += THREADS) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        double s = jacc[buf][0][c][jl];
#pragma unroll
                        for (int v = 1; v < W; ++v) s += jacc[buf][v][c][jl];
                        out[c * JT + jl] = s;
                    }
                }
            }
            if (threadIdx.x == 0 && u + 2 < u1) issue(buf);  // the cursor is at u + 2
        }
        if (failed) break;
        double* out = part_i + (size_t)(cta + L.bbase + a) * 3 * IB + w * 32 * P + lane;
#pragma unroll
        for (int k = 0; k < P; ++k) {
            out[0 * IB + k * 32] = tx[k];
            out[1 * IB + k * 32] = ty[k];
            out[2 * IB + k * 32] = tz[k];
        }
    }
    if (failed) {  // drain the copies of units iter, iter + 1 before leaving (default limit)
        bool drained = true;
        for (uint32_t k = iter; k < iter + 2 && u0 + k < u1; ++k)
            drained &= mbar_wait(&full[k & 1], (k >> 1) & 1, NB_WAIT_LIMIT_DEFAULT);
        if (threadIdx.x == 0)
            atomicOr(err_word, NB_DEVERR_TIMEOUT | (drained ? 0u : NB_DEVERR_DRAIN));
    }
}

// Per body: its i-side partials (CTA order) and the j-side partials of the units above the
// diagonal in its column (I-block order), summed in FP64 and, for the FP64 form (whose masses are
// not scaled), multiplied by G.
template <typename R, int IB, int JT>
__global__ void sym_combine_kernel(SymPlan S, const R* __restrict__ part_i,
                                   const R* __restrict__ part_j, double G,
                                   double* __restrict__ ax, double* __restrict__ ay,
                                   double* __restrict__ az) {
    constexpr bool F64 = std::is_same<R, double>::value;
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
        if constexpr (F64) {
            const R* p = part_i + (size_t)(c + A.boff + a) * 3 * IB;
            sx += p[0 * IB + li];
            sy += p[1 * IB + li];
            sz += p[2 * IB + li];
        } else {
            const R* p = part_i + (size_t)(c + A.boff + a) * 6 * IB;
            sx += (double)p[0 * IB + li] + (double)p[3 * IB + li];
            sy += (double)p[1 * IB + li] + (double)p[4 * IB + li];
            sz += (double)p[2 * IB + li] + (double)p[5 * IB + li];
        }
    }
    for (uint32_t r = 0; r < a; ++r) {
        const R* p = part_j + (A.uoff + row_off(n_jt, TPB, r) + (jt - r * TPB)) * 3 * JT;
        sx += (double)p[jl];
        sy += (double)p[JT + jl];
        sz += (double)p[2 * JT + jl];
    }
    if constexpr (F64) {
        ax[b] = sx * G;
        ay[b] = sy * G;
        az[b] = sz * G;
    } else {
        ax[b] = sx;
        ay[b] = sy;
        az[b] = sz;
    }
}

}  // namespace nbsym

namespace nb {

// (warps, bodies per lane, j-tile) of each form; the tables, the occupancy queries and the launch
// switches list the same instantiations
#define NB_SYM_CONFIG_LIST(X)                                                            \
    X(0, 8, 12, 128) X(1, 4, 12, 256) X(2, 4, 12, 128) X(3, 4, 16, 128) X(4, 8, 8, 256)       \
        X(5, 4, 8, 256) X(6, 8, 6, 256) X(7, 2, 12, 128)
#define NB_SYM64_CONFIG_LIST(X) X(0, 4, 2, 64) X(1, 4, 4, 64) X(2, 8, 2, 64) X(3, 4, 2, 128)
#define NB_SYMDF_CONFIG_LIST(X) X(0, 4, 2, 64) X(1, 4, 4, 64)

#define NB_SYM_ROW(i, W, P, JT) {W, P, JT},
const SymConfig kSymConfigs[NB_SYM_CONFIGS] = {NB_SYM_CONFIG_LIST(NB_SYM_ROW)};
const SymConfig kSym64Configs[NB_SYM64_CONFIGS] = {NB_SYM64_CONFIG_LIST(NB_SYM_ROW)};
const SymConfig kSymDfConfigs[NB_SYMDF_CONFIGS] = {NB_SYMDF_CONFIG_LIST(NB_SYM_ROW)};
#undef NB_SYM_ROW

namespace {

int g_sym_ctas_per_sm[3][NB_SYM_CONFIGS] = {};

template <typename K>
nb_status occupancy(K kernel, int threads, size_t smem, int* out) {
    NB_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    NB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, kernel, threads, smem));
    if (*out < 1) *out = 1;
    return NB_OK;
}

template <typename R, int W, int P, int JT>
nb_status sym_prepare(int* out) {
    return occupancy(nbsym::pair_sym_kernel<R, W, P, JT>, 32 * W,
                     nbsym::sym_smem_bytes<R, W, P, JT>(), out);
}

template <int W, int P, int JT>
nb_status sym_df_prepare(int* out) {
    return occupancy(nbsym::pair_sym_df_kernel<W, P, JT>, 32 * W,
                     nbsym::sym_df_smem_bytes<W, P, JT>(), out);
}

template <typename R, int W, int P, int JT>
nb_status sym_launch_cfg(const nbsym::SymPlan& S, const void* src, double eps2, void* part_i,
                         void* part_j, double G, double* ax, double* ay, double* az,
                         uint32_t* err_word, cudaStream_t stream) {
    using Rec = typename nbsym::RecOf<R>::type;
    nbsym::pair_sym_kernel<R, W, P, JT>
        <<<S.ctas, 32 * W, nbsym::sym_smem_bytes<R, W, P, JT>(), stream>>>(
            S, (const Rec*)src, (R)eps2, (R*)part_i, (R*)part_j, err_word);
    NB_TRY(check_launch("pair_sym_kernel"));
    nbsym::sym_combine_kernel<R, 32 * W * P, JT><<<ceil_div(S.n_total, 256), 256, 0, stream>>>(
        S, (const R*)part_i, (const R*)part_j, G, ax, ay, az);
    return check_launch("sym_combine_kernel");
}

template <int W, int P, int JT>
nb_status sym_df_launch_cfg(const nbsym::SymPlan& S, const void* src, double eps2, void* part_i,
                            void* part_j, double* ax, double* ay, double* az, uint32_t* err_word,
                            cudaStream_t stream) {
    const float e2h = (float)eps2, e2l = (float)(eps2 - (double)e2h);
    nbsym::pair_sym_df_kernel<W, P, JT>
        <<<S.ctas, 32 * W, nbsym::sym_df_smem_bytes<W, P, JT>(), stream>>>(
            S, (const nbsym::RecTF*)src, e2h, e2l, (double*)part_i, (double*)part_j, err_word);
    NB_TRY(check_launch("pair_sym_df_kernel"));
    // G is folded into the double-float masses: the combine scales by 1
    nbsym::sym_combine_kernel<double, 32 * W * P, JT>
        <<<ceil_div(S.n_total, 256), 256, 0, stream>>>(S, (const double*)part_i,
                                                       (const double*)part_j, 1.0, ax, ay, az);
    return check_launch("sym_combine_kernel");
}

const SymConfig& config_of(int form, int cfg) {
    return form == SYM_F64 ? kSym64Configs[cfg]
                           : (form == SYM_DF ? kSymDfConfigs[cfg] : kSymConfigs[cfg]);
}

}  // namespace

int sym_config_count(int form) {
    return form == SYM_F64 ? NB_SYM64_CONFIGS
                           : (form == SYM_DF ? NB_SYMDF_CONFIGS : NB_SYM_CONFIGS);
}

uint32_t sym_ib(int form, int cfg) {
    const SymConfig& C = config_of(form, cfg);
    return 32u * C.warps * C.p;
}

size_t sym_record_bytes(int form) {
    return form == SYM_F64 ? sizeof(nbsym::Rec64)
                           : (form == SYM_DF ? sizeof(nbsym::RecTF) : sizeof(float4));
}

nb_status sym_ctas_per_sm(int form, int cfg, int* out) {
    if (form < SYM_F32 || form > SYM_DF || cfg < 0 || cfg >= sym_config_count(form))
        return set_error(NB_ERR_INVALID_ARG, "bad symmetric pair config %d/%d", form, cfg);
    int& cached = g_sym_ctas_per_sm[form][cfg];
    if (cached == 0) {
        int v = 0;
        if (form == SYM_F64) {
            switch (cfg) {
#define NB_SYM_PREP(i, W, P, JT) \
    case i: NB_TRY((sym_prepare<double, W, P, JT>(&v))); break;
                NB_SYM64_CONFIG_LIST(NB_SYM_PREP)
#undef NB_SYM_PREP
            }
        } else if (form == SYM_DF) {
            switch (cfg) {
#define NB_SYM_PREP(i, W, P, JT) \
    case i: NB_TRY((sym_df_prepare<W, P, JT>(&v))); break;
                NB_SYMDF_CONFIG_LIST(NB_SYM_PREP)
#undef NB_SYM_PREP
            }
        } else {
            switch (cfg) {
#define NB_SYM_PREP(i, W, P, JT) \
    case i: NB_TRY((sym_prepare<float, W, P, JT>(&v))); break;
                NB_SYM_CONFIG_LIST(NB_SYM_PREP)
#undef NB_SYM_PREP
            }
        }
        cached = v;
    }
    *out = cached;
    return NB_OK;
}

nb_status sym_host_plan(int form, int cfg, const uint32_t* counts, uint32_t n_systems,
                        int sm_count, SymHostPlan* out) {
    int per_sm = 0;
    NB_TRY(sym_ctas_per_sm(form, cfg, &per_sm));
    const SymConfig& C = config_of(form, cfg);
    const uint32_t ib = sym_ib(form, cfg), tpb = ib / (uint32_t)C.jt;
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

size_t sym_part_i_bytes(int form, int cfg, uint32_t ctas, uint32_t n_blocks) {
    // FP32: (hi, lo) per axis; FP64 and double-float: one FP64 value per axis
    return ((size_t)ctas + n_blocks) * sym_ib(form, cfg) * (form == SYM_F32 ? 6 * 4 : 3 * 8);
}
size_t sym_part_j_bytes(int form, int cfg, uint64_t units) {
    return (size_t)units * 3 * config_of(form, cfg).jt * (form == SYM_F32 ? 4 : 8);
}

nb_status sym_single_table(nbsym::SymSys* sys, const SymHostPlan& hp, cudaStream_t stream) {
    const nbsym::SymSys& E = hp.sys[1];
    nbsym::sym_single_table_kernel<<<1, 1, 0, stream>>>(sys, E.off, E.boff, E.poff, E.uoff);
    return check_launch("sym_single_table_kernel");
}

nb_status sym_launch(int form, int cfg, const nbsym::SymPlan& S, const double* m, const double* x,
                     const double* y, const double* z, double G, double eps2, void* src,
                     void* part_i, void* part_j, double* ax, double* ay, double* az,
                     uint32_t* err_word, cudaStream_t stream) {
    int per_sm = 0;
    NB_TRY(sym_ctas_per_sm(form, cfg, &per_sm));  // shared-memory opt-in before the first launch
    if (S.units == 0) return NB_OK;
    const int blocks = ceil_div(S.n_records, 256);
    if (form == SYM_F64) {
        nbsym::sym_prepare_kernel<double><<<blocks, 256, 0, stream>>>(S, m, x, y, z, G,
                                                                      (nbsym::Rec64*)src);
    } else if (form == SYM_DF) {
        nbsym::sym_prepare_tf_kernel<<<blocks, 256, 0, stream>>>(S, m, x, y, z, G,
                                                                 (nbsym::RecTF*)src);
    } else {
        nbsym::sym_prepare_kernel<float><<<blocks, 256, 0, stream>>>(S, m, x, y, z, G,
                                                                     (float4*)src);
    }
    NB_TRY(check_launch("sym_prepare_kernel"));
    if (form == SYM_F64) {
        switch (cfg) {
#define NB_SYM_LAUNCH(i, W, P, JT)                                                          \
    case i:                                                                                 \
        return sym_launch_cfg<double, W, P, JT>(S, src, eps2, part_i, part_j, G, ax, ay, az, \
                                                err_word, stream);
            NB_SYM64_CONFIG_LIST(NB_SYM_LAUNCH)
#undef NB_SYM_LAUNCH
        }
    } else if (form == SYM_DF) {
        switch (cfg) {
#define NB_SYM_LAUNCH(i, W, P, JT)                                                         \
    case i:                                                                                \
        return sym_df_launch_cfg<W, P, JT>(S, src, eps2, part_i, part_j, ax, ay, az, err_word, \
                                           stream);
            NB_SYMDF_CONFIG_LIST(NB_SYM_LAUNCH)
#undef NB_SYM_LAUNCH
        }
    } else {
        switch (cfg) {
#define NB_SYM_LAUNCH(i, W, P, JT)                                                          \
    case i:                                                                                 \
        return sym_launch_cfg<float, W, P, JT>(S, src, eps2, part_i, part_j, G, ax, ay, az, \
                                               err_word, stream);
            NB_SYM_CONFIG_LIST(NB_SYM_LAUNCH)
#undef NB_SYM_LAUNCH
        }
    }
    return set_error(NB_ERR_INVALID_ARG, "bad symmetric pair config %d/%d", form, cfg);
}

}  // namespace nb
