// nb_pair.cuh -- FP32 pair-force kernel with compensated accumulation over a batch of independent
// systems (a single system is a batch of one).
//
// Work decomposition: system s has n_t(s) targets in i-blocks of IB = THREADS*IP and n(s) sources
// in j-tiles of JT; the units (s, i-block, j-tile) of all systems form one sequence and each of
// the persistent CTAs (SMs x resident CTAs) takes an equal contiguous range of it ("stream-K"),
// so every SM computes the same number of pairs whatever the mix of system sizes. A CTA writes
// one (hi, lo) partial per i-block it touches into slot cta + global i-block (unique: the CTA
// ranges form a monotone staircase over the i-blocks), and a combine pass adds the partials of
// each target in CTA order (deterministic).
//
// j-tiles move into shared memory with cp.async.bulk copies that complete on mbarriers (two
// buffers, every wait bounded: on timeout the CTA sets the timeout bit, drains its in-flight
// copies with bounded waits and returns). Source records are 32 bytes ({x,x,y,y},{z,z,Gm,Gm});
// the scalar inner loop reads them with two broadcast 16-byte shared loads per source (measured
// faster than a single load of a packed 16-byte {x,y,z,Gm} record).
#pragma once
#include "nb_internal.cuh"

namespace nbpair {

struct __align__(16) SrcDup {
    float x0, x1, y0, y1, z0, z1, m0, m1;
};

// Device-resident description of a batch (all arrays on the device).
struct Plan {
    uint32_t n_systems;
    uint32_t ctas;
    uint64_t units;
    unsigned long long wait_limit;  // polls of a tile wait before it gives up (context's limit)
    const uint32_t* sys_off;    // [n_systems+1] first source body of each system
    const uint32_t* tgt_begin;  // [n_systems]   first target (relative to the system)
    const uint32_t* t_off;      // [n_systems+1] prefix of target counts
    const uint64_t* unit_off;   // [n_systems+1] prefix of units
    const uint32_t* ib_off;     // [n_systems+1] prefix of i-blocks
};


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
// Polls the mbarrier phase at most `limit` times; false when it has not completed by then.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          unsigned long long limit) {
    for (unsigned long long it = 0; it < limit; ++it) {
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

// Largest s in [0, count) with off[s] <= v (off non-decreasing, off[0] <= v).
template <typename T>
__device__ __forceinline__ uint32_t upper_index(const T* __restrict__ off, uint32_t count, T v) {
    uint32_t lo = 0, hi = count;  // off[lo] <= v, answer in [lo, hi)
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= v) lo = mid; else hi = mid;
    }
    return lo;
}

struct Where {
    uint32_t s, ib, jt, n_jt, n_src, src0;
};

template <int JT>
__device__ __forceinline__ Where locate(const Plan& P, uint64_t u) {
    Where w;
    w.s = upper_index<uint64_t>(P.unit_off, P.n_systems, u);
    w.src0 = P.sys_off[w.s];
    w.n_src = P.sys_off[w.s + 1] - w.src0;
    w.n_jt = (w.n_src + JT - 1) / JT;
    const uint64_t lu = u - P.unit_off[w.s];
    w.ib = (uint32_t)(lu / w.n_jt);
    w.jt = (uint32_t)(lu % w.n_jt);
    return w;
}

__device__ __forceinline__ uint64_t unit_begin(const Plan& P, uint32_t cta) {
    return (P.units * (uint64_t)cta) / P.ctas;
}

__device__ __forceinline__ uint32_t cta_of_unit(const Plan& P, uint64_t u) {
    uint32_t c = (uint32_t)((u * P.ctas) / P.units);
    while (c + 1 < P.ctas && unit_begin(P, c + 1) <= u) ++c;
    while (c > 0 && unit_begin(P, c) > u) --c;
    return c;
}

// (H, L) += T with Knuth's TwoSum: H + L carries the running sum to about twice FP32 precision.
#define NB_TWOSUM(H, L, T)                        \
    {                                             \
        const float sum_ = (H) + (T);             \
        const float bp_ = sum_ - (H);             \
        const float e1_ = (H) - (sum_ - bp_);     \
        const float e2_ = (T) - bp_;              \
        (L) = (L) + (e1_ + e2_);                  \
        (H) = sum_;                               \
    }

// Dynamic shared memory of a configuration: two j-tiles and the per-target (hi, lo) sums.
template <int THREADS, int IP, int JT>
constexpr size_t pair_smem_bytes() {
    return 2 * JT * sizeof(SrcDup) + (size_t)6 * IP * THREADS * sizeof(float);
}

// Each thread owns IP targets (k-th: i-block * IB + k * THREADS + thread) and walks the j-tile in
// scalar FP32: per pair 3 subtractions, 3 FMAs for r^2 + eps^2, one MUFU rsqrt, 3 multiplies for
// G m / r^3 and 3 FMAs into the tile sums, which are added into the compensated (hi, lo) sums
// once per tile. (Scalar FP32 issues faster here than the packed f32x2 forms of the same
// arithmetic, which were measured at 83% of its rate.)
template <int THREADS, int IP, int JT>
__global__ void __launch_bounds__(THREADS)
pair_f32c_kernel(Plan P, const SrcDup* __restrict__ src, const float4* __restrict__ tgt,
                 float eps2, float* __restrict__ part, uint32_t* __restrict__ err_word) {
    constexpr int IB = THREADS * IP;
    extern __shared__ __align__(128) unsigned char pair_smem[];
    SrcDup (*tile)[JT] = reinterpret_cast<SrcDup (*)[JT]>(pair_smem);
    // compensated per-target sums hl[c][k][thread], c = hx, hy, hz, lx, ly, lz: in shared
    // memory, since they change once per j-tile and the registers go to more targets per thread
    float (*hl)[IP][THREADS] =
        reinterpret_cast<float (*)[IP][THREADS]>(pair_smem + 2 * JT * sizeof(SrcDup));
    __shared__ __align__(8) uint64_t full[2];

    const uint32_t cta = blockIdx.x;
    const uint64_t u0 = unit_begin(P, cta), u1 = unit_begin(P, cta + 1);
    if (u0 >= u1) return;
    if (threadIdx.x == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // Thread 0 issues the j-tile copies two units ahead. It keeps the next unit's tile in
    // registers and reads the plan again only when the unit sequence enters another system.
    Where nxt{};
    uint64_t nxt_u = u0, nxt_sys_end = 0;
    auto seek = [&](uint64_t uu) {
        nxt = locate<JT>(P, uu);
        nxt_u = uu;
        nxt_sys_end = P.unit_off[nxt.s + 1];
    };
    auto issue_next = [&](int buf) {
        const uint32_t j0 = nxt.jt * JT;
        const uint32_t cnt = min((uint32_t)JT, nxt.n_src - j0);
        const uint32_t bytes = cnt * (uint32_t)sizeof(SrcDup);
        mbar_expect_tx(&full[buf], bytes);
        bulk_g2s(&tile[buf][0], src + nxt.src0 + j0, bytes, &full[buf]);
        ++nxt_u;  // advance the cursor to the following unit
        if (nxt_u >= nxt_sys_end) {
            if (nxt_u < u1) seek(nxt_u);
        } else if (++nxt.jt == nxt.n_jt) {
            nxt.jt = 0;
        }
    };
    if (threadIdx.x == 0) {
        seek(u0);
        issue_next(0);
        if (u0 + 1 < u1) issue_next(1);
    }

    const int th = threadIdx.x;
    float xi[IP], yi[IP], zi[IP], tx[IP], ty[IP], tz[IP];
    uint64_t u = u0;
    uint32_t iter = 0;
    bool failed = false;
    while (u < u1 && !failed) {
        const Where w = locate<JT>(P, u);
        const uint64_t seg_end = min(u1, P.unit_off[w.s] + (uint64_t)(w.ib + 1) * w.n_jt);
        const uint32_t n_t = P.t_off[w.s + 1] - P.t_off[w.s];
        const uint32_t t0 = w.src0 + P.tgt_begin[w.s];
#pragma unroll
        for (int k = 0; k < IP; ++k) {
            const uint32_t li = w.ib * IB + k * THREADS + th;
            const float4 a = li < n_t ? tgt[t0 + li] : make_float4(1e18f, 1e18f, 1e18f, 0.f);
            xi[k] = a.x;
            yi[k] = a.y;
            zi[k] = a.z;
#pragma unroll
            for (int c = 0; c < 6; ++c) hl[c][k][th] = 0.f;
        }
        uint32_t jt = w.jt;
        for (; u < seg_end; ++u, ++iter, ++jt) {
            const int buf = iter & 1;
            const uint32_t cnt = min((uint32_t)JT, w.n_src - jt * JT);
            const bool ok = mbar_wait(&full[buf], (iter >> 1) & 1, P.wait_limit);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
#pragma unroll
            for (int k = 0; k < IP; ++k) tx[k] = ty[k] = tz[k] = 0.f;
            const float4* t4 = reinterpret_cast<const float4*>(&tile[buf][0]);
#pragma unroll 2
            for (uint32_t j = 0; j < cnt; ++j) {
                const float4 A = t4[2 * j], B = t4[2 * j + 1];  // {x,x,y,y}, {z,z,Gm,Gm}
                const float sx = A.x, sy = A.z, sz = B.x, sm = B.z;
#pragma unroll
                for (int k = 0; k < IP; ++k) {
                    const float dx = sx - xi[k], dy = sy - yi[k], dz = sz - zi[k];
                    const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
                    const float inv = nb_rsqrt_f32(r2);
                    const float s3 = (sm * inv) * (inv * inv);
                    tx[k] = fmaf(dx, s3, tx[k]);
                    ty[k] = fmaf(dy, s3, ty[k]);
                    tz[k] = fmaf(dz, s3, tz[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < IP; ++k) {
                float h0 = hl[0][k][th], h1 = hl[1][k][th], h2 = hl[2][k][th];
                float l0 = hl[3][k][th], l1 = hl[4][k][th], l2 = hl[5][k][th];
                NB_TWOSUM(h0, l0, tx[k]);
                NB_TWOSUM(h1, l1, ty[k]);
                NB_TWOSUM(h2, l2, tz[k]);
                hl[0][k][th] = h0;
                hl[1][k][th] = h1;
                hl[2][k][th] = h2;
                hl[3][k][th] = l0;
                hl[4][k][th] = l1;
                hl[5][k][th] = l2;
            }
            __syncthreads();
            if (threadIdx.x == 0 && u + 2 < u1) issue_next(buf);  // the cursor is at u + 2
        }
        if (failed) break;
        float* out = part + (size_t)(cta + P.ib_off[w.s] + w.ib) * 6 * IB;
#pragma unroll
        for (int k = 0; k < IP; ++k)
#pragma unroll
            for (int c = 0; c < 6; ++c) out[c * IB + k * THREADS + th] = hl[c][k][th];
    }
    if (failed) {
        // the copies of units iter and iter + 1 were issued: wait for them (default limit)
        // before the CTA leaves, so that none lands in shared memory after it
        bool drained = true;
        for (uint32_t k = iter; k < iter + 2 && u0 + k < u1; ++k)
            drained &= mbar_wait(&full[k & 1], (k >> 1) & 1, NB_WAIT_LIMIT_DEFAULT);
        if (threadIdx.x == 0) atomicOr(err_word, NB_DEVERR_TIMEOUT | (drained ? 0u : NB_DEVERR_DRAIN));
    }
}

// Sum of each target's partials in CTA order; FP64 output.
template <int IB, int JT>
__global__ void pair_combine_kernel(Plan P, const float* __restrict__ part, uint32_t n_targets,
                                    double* __restrict__ ax, double* __restrict__ ay,
                                    double* __restrict__ az) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_targets) return;
    const uint32_t s = upper_index<uint32_t>(P.t_off, P.n_systems, g);
    const uint32_t lt = g - P.t_off[s];
    const uint32_t n_src = P.sys_off[s + 1] - P.sys_off[s];
    const uint32_t n_jt = (n_src + JT - 1) / JT;
    const uint32_t ib = lt / IB, li = lt % IB;
    const uint64_t us = P.unit_off[s] + (uint64_t)ib * n_jt;
    const uint32_t c0 = cta_of_unit(P, us), c1 = cta_of_unit(P, us + n_jt - 1);
    const uint32_t gib = P.ib_off[s] + ib;
    double sx = 0, sy = 0, sz = 0;
    for (uint32_t c = c0; c <= c1; ++c) {
        const float* p = part + (size_t)(c + gib) * 6 * IB;
        sx += (double)p[0 * IB + li] + (double)p[3 * IB + li];
        sy += (double)p[1 * IB + li] + (double)p[4 * IB + li];
        sz += (double)p[2 * IB + li] + (double)p[5 * IB + li];
    }
    const uint32_t b = P.sys_off[s] + P.tgt_begin[s] + lt;
    ax[b] = sx;
    ay[b] = sy;
    az[b] = sz;
}

}  // namespace nbpair

namespace nb {

// Tile configurations of the pair kernel (chosen by the batch autotuner).
struct PairConfig {
    int threads, ip, jt;
};
constexpr int NB_PAIR_CONFIGS = 8;
extern const PairConfig kPairConfigs[NB_PAIR_CONFIGS];

// Host-side plan numbers for a configuration.
struct PairHostPlan {
    uint32_t ctas;
    uint64_t units;
    uint32_t total_ib;
};

// Resident CTAs per SM of configuration `cfg` (cached occupancy query).
nb_status pair_ctas_per_sm(int cfg, int* out);
// Launches prepare + pair + combine for a batch whose device plan arrays are filled.
nb_status pair_launch(int cfg, const nbpair::Plan& plan, const double* m, const double* x,
                      const double* y, const double* z, uint32_t n_total, uint32_t n_targets,
                      double G, double eps2, nbpair::SrcDup* src, float4* tgt, float* part,
                      double* ax, double* ay, double* az, uint32_t* err_word,
                      cudaStream_t stream);
// Partial-buffer floats needed by a plan of configuration cfg.
size_t pair_partial_floats(int cfg, uint32_t ctas, uint32_t total_ib);
// Enqueues the device plan of one system (sources [0, n), targets [t_begin, t_end)).
nb_status pair_plan_single(uint32_t* sys_off, uint32_t* tgt_begin, uint32_t* t_off,
                           uint64_t* unit_off, uint32_t* ib_off, uint32_t n, uint32_t t_begin,
                           uint32_t t_end, uint64_t units, uint32_t n_ib, cudaStream_t stream);

}  // namespace nb
