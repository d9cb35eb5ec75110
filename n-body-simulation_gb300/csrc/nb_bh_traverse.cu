// nb_bh_traverse.cu -- Barnes-Hut accelerations over the DFS-ordered octree
// (replaces BarnesHutAlgorithm::computeAccelerations, BarnesHutAlgorithm.cpp:280-401).
//
// Nodes are stored in the order the reference's stack pops them (DFS pre-order, children in
// visit order 2,0,3,1,6,4,7,5), each with a skip link to the first node after its subtree.
// "Accept" (or skip) continues at the skip link and "open" continues at the next node, so a
// traversal needs no stack at all and visits nodes in exactly the reference's order.
//
//  * per-body rule (NB_OPEN_THETA), default schedule (bh_theta_lane_kernel, FP64; and
//    bh_theta_df_kernel, double-float): each lane walks its own body's DFS sequence, deciding each
//    cell with an FP32 pre-test whose rounding margin is proven and the reference's FP64
//    expression only inside that margin; find-then-compute, so the FP64 monopoles of all lanes
//    that found one run together. Warps take groups of 32 bodies close together in the tree, after
//    the first traversal of a tree sorted within windows of 1,024 by the length of their last
//    walk, so that the lanes of a warp finish together.
//  * per-body rule, lockstep schedule (bh_theta_f64_kernel, nb_bh_set_schedule(1)): the 32 lanes
//    of a warp hold 32 bodies adjacent in tree order, each with its own position in the DFS
//    sequence. Every iteration the warp takes the smallest position (__reduce_min_sync) and the
//    lanes sitting on it evaluate that node -- one broadcast load -- and advance by their own
//    decision.
//    Either way each body sees the reference's sequence of accepted nodes in the reference's
//    order.
//  * group rule (NB_OPEN_THETA_GROUP): the warp walks one sequence; a cell is opened when any
//    lane's rule opens it, otherwise all lanes accept it -- no divergence.
#include <algorithm>

#include "nb_bh.cuh"

namespace {

constexpr int TR_THREADS = 128;

enum Mode { IEEE64 = 0, FAST64 = 1, F32 = 2 };

template <int MODE>
struct Arith;

template <>
struct Arith<IEEE64> {
    __device__ static double sub(double a, double b) { return __dsub_rn(a, b); }
    __device__ static double norm2(double a, double b, double c) {
        return __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
    }
    __device__ static double rsqrt(double v) { return __ddiv_rn(1.0, __dsqrt_rn(v)); }
    __device__ static double mul(double a, double b) { return __dmul_rn(a, b); }
    __device__ static double add(double a, double b) { return __dadd_rn(a, b); }
    // acc += m * (d * inv), rounded as the reference writes it
    __device__ static double accum(double acc, double m, double d, double inv) {
        return __dadd_rn(acc, __dmul_rn(m, __dmul_rn(d, inv)));
    }
    __device__ static void monopole_xyz(double m, double dx, double dy, double dz, double eps2,
                                        double& ax, double& ay, double& az) {
        monopole(m, dx, dy, dz, norm2(dx, dy, dz), eps2, ax, ay, az);
    }
    // the reference's monopole: den = d2 + eps2, inv = 1/sqrt(den^3), acc += m * (d * inv)
    __device__ static void monopole(double m, double dx, double dy, double dz, double d2,
                                    double eps2, double& ax, double& ay, double& az) {
        double den = __dadd_rn(d2, eps2);
        den = __dmul_rn(__dmul_rn(den, den), den);
        const double inv = rsqrt(den);
        ax = accum(ax, m, dx, inv);
        ay = accum(ay, m, dy, inv);
        az = accum(az, m, dz, inv);
    }
};

template <>
struct Arith<FAST64> {
    __device__ static double sub(double a, double b) { return a - b; }
    __device__ static double norm2(double a, double b, double c) { return fma(a, a, fma(b, b, c * c)); }
    __device__ static double rsqrt(double v) { return nb_rsqrt_f64(v); }
    __device__ static double mul(double a, double b) { return a * b; }
    __device__ static double add(double a, double b) { return a + b; }
    __device__ static double accum(double acc, double m, double d, double inv) {
        return fma(m * inv, d, acc);
    }
    // m (d2 + eps2)^(-3/2) by nb_m_rinv3_f64: 7 FP64 operations instead of cubing den and
    // refining its rsqrt (8).
    __device__ static void monopole(double m, double dx, double dy, double dz, double d2,
                                    double eps2, double& ax, double& ay, double& az) {
        monopole_den(m, dx, dy, dz, d2 + eps2, ax, ay, az);
    }
    __device__ static void monopole_xyz(double m, double dx, double dy, double dz, double eps2,
                                        double& ax, double& ay, double& az) {
        monopole_den(m, dx, dy, dz, fma(dx, dx, fma(dy, dy, fma(dz, dz, eps2))), ax, ay, az);
    }
    __device__ static void monopole_den(double m, double dx, double dy, double dz, double den,
                                        double& ax, double& ay, double& az) {
        const double w = nb_m_rinv3_f64(m, den);
        ax = fma(w, dx, ax);
        ay = fma(w, dy, ay);
        az = fma(w, dz, az);
    }
};

// Per-body reference rule, FP64 (IEEE64 bit-identical to the host evaluation; FAST64 with FMAs).
template <int MODE>
__global__ void __launch_bounds__(TR_THREADS)
bh_theta_f64_kernel(const NodeRec64* __restrict__ rec, const uint32_t* __restrict__ info,
                    const uint32_t* __restrict__ ids, const double* __restrict__ x,
                    const double* __restrict__ y, const double* __restrict__ z, uint32_t n,
                    double theta, double eps2, double G, double* __restrict__ ax,
                    double* __restrict__ ay, double* __restrict__ az) {
    using A = Arith<MODE>;
    const uint32_t p = blockIdx.x * TR_THREADS + threadIdx.x;
    const bool valid = p < n;
    const uint32_t nn = info[0];
    const uint32_t me = valid ? ids[p] : NB_NONE;
    double px = 0, py = 0, pz = 0;
    if (valid) {
        px = x[me];
        py = y[me];
        pz = z[me];
    }
    double acx = 0, acy = 0, acz = 0;
    uint32_t kl = valid ? 0u : nn;
    for (;;) {
        const uint32_t k = __reduce_min_sync(0xffffffffu, kl);
        if (k >= nn) break;
        if (kl != k) continue;
        const NodeRec64 r = rec[k];
        if (r.mass != 0 && r.body != me) {  // BarnesHutAlgorithm.cpp:349
            const double dx = A::sub(r.cx, px), dy = A::sub(r.cy, py), dz = A::sub(r.cz, pz);
            const double d2 = A::norm2(dx, dy, dz);
            const double cur = A::mul(r.edge, A::rsqrt(d2));  // :355-357
            if (cur < theta || r.body != NB_NONE) {           // :359
                A::monopole(r.mass, dx, dy, dz, d2, eps2, acx, acy, acz);
                kl = r.skip;
            } else {
                kl = k + 1;
            }
        } else {
            kl = r.skip;
        }
    }
    if (valid) {
        ax[me] = A::mul(acx, G);
        ay[me] = A::mul(acy, G);
        az[me] = A::mul(acz, G);
    }
}

// Per-body reference rule, FP64, each lane walking its own DFS sequence (no union walk).
// The opening test is decided in FP32 on the anchored FP32 records whenever the FP32 error
// bound proves the answer; only undecided cells evaluate the reference's FP64 expression.
// FP32 error bound of d^2 with positions rounded relative to the box centre (|c-a|, |p-a| <=
// E/2 per axis, u = 2^-24): |d2f - d2| <= u d^2 (2*sqrt(3) E/d + 5); the test below widens it
// by 4x and adds the roundings of edge^2 and theta^2*d2f. Accumulation order per body is the
// reference's DFS order, so MODE IEEE64 stays bit-identical. Warps take groups of 32 sorted
// positions; with `order` != nullptr the bodies of the positions come from it (the previous
// walk's lengths regrouped within windows, regroup_kernel) instead of from ids. Each body's
// accepted-cell count goes to walk_len[body].
template <int MODE>
__global__ void __launch_bounds__(TR_THREADS)
bh_theta_lane_kernel(const NodeRec32* __restrict__ rec32, const NodeRec64* __restrict__ rec64,
                     const uint32_t* __restrict__ info, const uint32_t* __restrict__ ids,
                     const double* __restrict__ x, const double* __restrict__ y,
                     const double* __restrict__ z, const double* __restrict__ box, uint32_t n,
                     double theta, double eps2, double G, double* __restrict__ ax,
                     double* __restrict__ ay, double* __restrict__ az,
                     uint32_t* __restrict__ next_group, const uint32_t* __restrict__ order,
                     uint32_t* __restrict__ walk_len) {
    using A = Arith<MODE>;
    const uint32_t n_groups = (n + 31) / 32;
    const int lane = threadIdx.x & 31;
    // persistent warps: each takes the next 32 bodies until none are left, so no warp waits for
    // its block's slowest warp and the last wave's tail is one group long
    for (;;) {
        uint32_t grp = 0;
        if (lane == 0) grp = atomicAdd(next_group, 1u);
        grp = __shfl_sync(0xffffffffu, grp, 0);
        if (grp >= n_groups) break;
        const uint32_t p = grp * 32 + lane;
        const bool valid = p < n;  // lanes past the end stay (they take part in the warp votes)
        const uint32_t nn = info[0];
        const uint32_t me = valid ? (order != nullptr ? order[p] : ids[p]) : NB_NONE;
        uint32_t accepted = 0;
        const double px = valid ? x[me] : 0.0, py = valid ? y[me] : 0.0, pz = valid ? z[me] : 0.0;
        const double E = box[6];
        const double ox = box[0] + E / 2, oy = box[1] + E / 2, oz = box[2] + E / 2;
        const float pxf = (float)(px - ox), pyf = (float)(py - oy), pzf = (float)(pz - oz);
        const float th2 = (float)(theta * theta);
        const float u4 = 4.0f * 5.9604645e-8f;  // 4 * 2^-24
        const float Ef = (float)E;
        double acx = 0, acy = 0, acz = 0;
        uint32_t k = valid ? 0u : nn;
        // Find, then compute: every lane walks (FP32 tests, divergent but off the FP64 pipe) to its
        // next accepted cell, then the lanes evaluate their FP64 monopoles together, so the FP64
        // work runs with all unfinished lanes instead of the few that accept in the same iteration.
        for (;;) {
            bool found = false;
            uint32_t next = 0;
            while (k < nn) {
                const NodeRec32 r = rec32[k];
                if (r.body == me) {
                    k = r.skip;
                    continue;
                }
                bool accept = r.body != NB_NONE;
                if (!accept) {
                    const float dxf = r.cx - pxf, dyf = r.cy - pyf, dzf = r.cz - pzf;
                    const float d2f = fmaf(dxf, dxf, fmaf(dyf, dyf, dzf * dzf));
                    const float t = th2 * d2f;
                    const float rel = u4 * (3.5f * Ef * nb_rsqrt_f32(d2f) + 8.0f);
                    const float margin = t * rel + u4 * r.edge2;
                    if (r.edge2 > t + margin) {
                        accept = false;  // certainly opened
                    } else if (r.edge2 < t - margin) {
                        accept = true;   // certainly accepted
                    } else {             // undecided: the reference's FP64 expression
                        const NodeRec64 q = rec64[k];
                        const double dx = A::sub(q.cx, px), dy = A::sub(q.cy, py),
                                     dz = A::sub(q.cz, pz);
                        accept = A::mul(q.edge, A::rsqrt(A::norm2(dx, dy, dz))) < theta;
                    }
                }
                if (accept) {
                    found = true;
                    next = r.skip;
                    break;
                }
                k = k + 1;
            }
            if (!__any_sync(0xffffffffu, found)) break;
            if (found) {
                ++accepted;
                const NodeRec64 q = rec64[k];
                if (q.mass != 0) {
                    const double dx = A::sub(q.cx, px), dy = A::sub(q.cy, py), dz = A::sub(q.cz, pz);
                    A::monopole_xyz(q.mass, dx, dy, dz, eps2, acx, acy, acz);
                }
                k = next;
            }
        }
        if (valid) {
            ax[me] = A::mul(acx, G);
            ay[me] = A::mul(acy, G);
            az[me] = A::mul(acz, G);
            walk_len[me] = accepted;
        }
    }
}

// Walk order of the next per-body traversal: within each window of RG_WINDOW sorted positions
// (bodies close together in the tree), the bodies by decreasing length of their last walk (ties
// by position), so that the 32 lanes of a warp walk sequences of similar length and fewer lanes
// sit idle while the FP64 monopoles of the others run (a warp instruction costs the FP64 pipe the
// same however few lanes are active). Bitonic sort of (length, position) keys in shared memory.
constexpr int RG_WINDOW = 1024;

__global__ void __launch_bounds__(RG_WINDOW)
regroup_kernel(const uint32_t* __restrict__ ids, const uint32_t* __restrict__ walk_len, uint32_t n,
               uint32_t* __restrict__ order) {
    __shared__ unsigned long long key[RG_WINDOW];
    const uint32_t i = threadIdx.x, p = blockIdx.x * RG_WINDOW + i;
    // ascending keys: longest walk first, then position; positions past n sort last
    key[i] = p < n ? ((unsigned long long)(~walk_len[ids[p]]) << 32) | i : ~0ull;
    __syncthreads();
    for (uint32_t k = 2; k <= RG_WINDOW; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            const uint32_t q = i ^ j;
            if (q > i) {
                const unsigned long long a = key[i], b = key[q];
                if (((i & k) == 0) == (a > b)) {
                    key[i] = b;
                    key[q] = a;
                }
            }
            __syncthreads();
        }
    }
    if (p < n) order[p] = ids[blockIdx.x * RG_WINDOW + (uint32_t)(key[i] & 0xffffffffu)];
}

// Per-body reference rule with FP64-accurate double-float monopoles (NB_DF64). The walk and the
// opening decisions are those of bh_theta_lane_kernel (FP32 pre-test with a proven margin, the
// reference's FP64 expression for undecided cells), so each body accepts exactly the reference's
// cells; the accepted monopoles are evaluated in double-float arithmetic on the FP32 pipe
// (~2^-48 relative per operation) instead of on the FP64 pipe, which this part runs at 1/64 of
// the FP32 rate. Centres and the body are exact triple-floats relative to the box centre (rec32,
// rec32lo, rec32lo2), so the separation is accurate to ~2^-48 of itself; G*mass is rec32.gm +
// rec32lo.w. rsqrt: hardware estimate y0 plus the third-order step
// y = y0 (1 + e/2 + 3e^2/8), e = 1 - r^2 y0^2 evaluated with error-free products. The sums are
// Neumaier-compensated (hi + running lo), converted to FP64 at the end and scaled by G / G_build.
__global__ void __launch_bounds__(TR_THREADS)
bh_theta_df_kernel(const NodeRec32* __restrict__ rec32, const float4* __restrict__ rec32lo,
                   const float4* __restrict__ rec32lo2, const NodeRec64* __restrict__ rec64,
                   const uint32_t* __restrict__ info,
                   const uint32_t* __restrict__ ids, const double* __restrict__ x,
                   const double* __restrict__ y, const double* __restrict__ z,
                   const double* __restrict__ box, uint32_t n, double theta, double eps2,
                   double gscale, double* __restrict__ ax, double* __restrict__ ay,
                   double* __restrict__ az, const uint32_t* __restrict__ order,
                   uint32_t* __restrict__ walk_len) {
    using A = Arith<FAST64>;
    const uint32_t p = blockIdx.x * TR_THREADS + threadIdx.x;
    if (p >= n) return;
    const uint32_t nn = info[0];
    const uint32_t me = order != nullptr ? order[p] : ids[p];  // as bh_theta_lane_kernel
    uint32_t accepted = 0;
    const double px = x[me], py = y[me], pz = z[me];
    const double E = box[6];
    const double ox = box[0] + E / 2, oy = box[1] + E / 2, oz = box[2] + E / 2;
    const float pxf = (float)(px - ox), pyf = (float)(py - oy), pzf = (float)(pz - oz);
    // the body minus the box centre, exactly, as triple-floats (pxf etc. are their leading terms)
    float hx, hy, hz, pxm, pym, pzm, pxl, pyl, pzl;
    tf_split_diff(px, ox, hx, pxm, pxl);
    tf_split_diff(py, oy, hy, pym, pyl);
    tf_split_diff(pz, oz, hz, pzm, pzl);
    const float e2h = (float)eps2, e2l = (float)(eps2 - (double)e2h);
    const float th2 = (float)(theta * theta);
    const float u4 = 4.0f * 5.9604645e-8f;  // 4 * 2^-24
    const float Ef = (float)E;
    float ahx = 0.f, ahy = 0.f, ahz = 0.f, alx = 0.f, aly = 0.f, alz = 0.f;
    uint32_t k = 0;
    while (k < nn) {
        const NodeRec32 r = rec32[k];
        if (r.body == me) {
            k = r.skip;
            continue;
        }
        bool accept = r.body != NB_NONE;
        if (!accept) {
            const float dxf = r.cx - pxf, dyf = r.cy - pyf, dzf = r.cz - pzf;
            const float d2f = fmaf(dxf, dxf, fmaf(dyf, dyf, dzf * dzf));
            const float t = th2 * d2f;
            const float rel = u4 * (3.5f * Ef * nb_rsqrt_f32(d2f) + 8.0f);
            const float margin = t * rel + u4 * r.edge2;
            if (r.edge2 > t + margin) {
                accept = false;
            } else if (r.edge2 < t - margin) {
                accept = true;
            } else {
                const NodeRec64 q = rec64[k];
                const double dx = A::sub(q.cx, px), dy = A::sub(q.cy, py), dz = A::sub(q.cz, pz);
                accept = A::mul(q.edge, A::rsqrt(A::norm2(dx, dy, dz))) < theta;
            }
        }
        if (accept) {
            ++accepted;
            const float4 lo = rec32lo[k];
            if (r.gm != 0.f || lo.w != 0.f) {
                const float4 lo2 = rec32lo2[k];
                const nb_df dx = tf_diff(r.cx, lo.x, lo2.x, pxf, pxm, pxl);
                const nb_df dy = tf_diff(r.cy, lo.y, lo2.y, pyf, pym, pyl);
                const nb_df dz = tf_diff(r.cz, lo.z, lo2.z, pzf, pzm, pzl);
                // r^2 + eps^2
                const nb_df sx = df_sqr(dx), sy = df_sqr(dy), sz = df_sqr(dz);
                nb_df a = df_two_sum(sx.h, sy.h);
                a.l += sx.l + sy.l;
                nb_df b = df_two_sum(a.h, sz.h);
                b.l += a.l + sz.l;
                nb_df c = df_two_sum(b.h, e2h);  // eps^2 may be as large as r^2
                c.l += b.l + e2l;
                const nb_df r2 = df_two_sum(c.h, c.l);
                // 1/r
                const float y0 = nb_rsqrt_f32(r2.h);
                const float q = y0 * y0, qe = fmaf(y0, y0, -q);  // y0^2 = q + qe exactly
                const float th = r2.h * q;
                float te = fmaf(r2.h, q, -th);
                te = fmaf(r2.h, qe, te);
                te = fmaf(r2.l, q, te);
                const float e = (1.0f - th) - te;  // 1 - th is exact (th is within 2^-21 of 1)
                const nb_df inv = df_fast_two_sum(y0, y0 * (e * fmaf(0.375f, e, 0.5f)));
                // G m / r^3
                const nb_df w = df_mul(nb_df{r.gm, lo.w}, df_mul(df_sqr(inv), inv));
                // compensated sums
                const nb_df tx = df_mul(dx, w), ty = df_mul(dy, w), tz = df_mul(dz, w);
                nb_df s = df_two_sum(ahx, tx.h);
                ahx = s.h;
                alx += s.l + tx.l;
                s = df_two_sum(ahy, ty.h);
                ahy = s.h;
                aly += s.l + ty.l;
                s = df_two_sum(ahz, tz.h);
                ahz = s.h;
                alz += s.l + tz.l;
            }
            k = r.skip;
        } else {
            k = k + 1;
        }
    }
    walk_len[me] = accepted;
    ax[me] = ((double)ahx + (double)alx) * gscale;
    ay[me] = ((double)ahy + (double)aly) * gscale;
    az[me] = ((double)ahz + (double)alz) * gscale;
}

// Per-body reference rule with FP32 pair math and compensated accumulation.
__global__ void __launch_bounds__(TR_THREADS)
bh_theta_f32_kernel(const NodeRec32* __restrict__ rec, const uint32_t* __restrict__ info,
                    const uint32_t* __restrict__ ids, const double* __restrict__ x,
                    const double* __restrict__ y, const double* __restrict__ z,
                    const double* __restrict__ box, uint32_t n, float theta, float eps2,
                    double* __restrict__ ax, double* __restrict__ ay, double* __restrict__ az) {
    const uint32_t p = blockIdx.x * TR_THREADS + threadIdx.x;
    const bool valid = p < n;
    const uint32_t nn = info[0];
    const uint32_t me = valid ? ids[p] : NB_NONE;
    const double ox = box[0] + box[6] / 2, oy = box[1] + box[6] / 2, oz = box[2] + box[6] / 2;
    float px = 0, py = 0, pz = 0;
    if (valid) {
        px = (float)(x[me] - ox);
        py = (float)(y[me] - oy);
        pz = (float)(z[me] - oz);
    }
    float hx = 0, hy = 0, hz = 0, lx = 0, ly = 0, lz = 0;
    uint32_t kl = valid ? 0u : nn;
    const float theta2 = theta * theta;
    for (;;) {
        const uint32_t k = __reduce_min_sync(0xffffffffu, kl);
        if (k >= nn) break;
        if (kl != k) continue;
        const NodeRec32 r = rec[k];
        if (r.gm != 0 && r.body != me) {
            const float dx = r.cx - px, dy = r.cy - py, dz = r.cz - pz;
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (r.body != NB_NONE || r.edge2 < theta2 * d2) {
                const float inv = nb_rsqrt_f32(d2 + eps2);
                const float s = r.gm * inv * inv * inv;
                // TwoSum of each term into (h, l)
                const float tx = dx * s, ty = dy * s, tz = dz * s;
                float sh = hx + tx, bp = sh - hx;
                lx += (hx - (sh - bp)) + (tx - bp);
                hx = sh;
                sh = hy + ty;
                bp = sh - hy;
                ly += (hy - (sh - bp)) + (ty - bp);
                hy = sh;
                sh = hz + tz;
                bp = sh - hz;
                lz += (hz - (sh - bp)) + (tz - bp);
                hz = sh;
                kl = r.skip;
            } else {
                kl = k + 1;
            }
        } else {
            kl = r.skip;
        }
    }
    if (valid) {
        ax[me] = (double)hx + (double)lx;
        ay[me] = (double)hy + (double)ly;
        az[me] = (double)hz + (double)lz;
    }
}

// Group rule, FP64.
__global__ void __launch_bounds__(TR_THREADS)
bh_group_f64_kernel(const NodeRec64* __restrict__ rec, const uint32_t* __restrict__ info,
                    const uint32_t* __restrict__ ids, const double* __restrict__ x,
                    const double* __restrict__ y, const double* __restrict__ z, uint32_t n,
                    double theta, double eps2, double G, double* __restrict__ ax,
                    double* __restrict__ ay, double* __restrict__ az) {
    const uint32_t p = blockIdx.x * TR_THREADS + threadIdx.x;
    const bool valid = p < n;
    const uint32_t nn = info[0];
    const uint32_t me = valid ? ids[p] : NB_NONE;
    double px = 0, py = 0, pz = 0;
    if (valid) {
        px = x[me];
        py = y[me];
        pz = z[me];
    }
    const double theta2 = theta * theta;
    double acx = 0, acy = 0, acz = 0;
    uint32_t k = 0;
    while (k < nn) {
        const NodeRec64 r = rec[k];
        const double dx = r.cx - px, dy = r.cy - py, dz = r.cz - pz;
        const double d2 = fma(dx, dx, fma(dy, dy, dz * dz));
        const bool open = valid && r.body == NB_NONE && r.mass != 0 && r.edge * r.edge >= theta2 * d2;
        if (__any_sync(0xffffffffu, open)) {
            k = k + 1;
            continue;
        }
        if (valid && r.body != me && r.mass != 0) {
            const double s = nb_m_rinv3_f64(r.mass, d2 + eps2);
            acx = fma(s, dx, acx);
            acy = fma(s, dy, acy);
            acz = fma(s, dz, acz);
        }
        k = r.skip;
    }
    if (valid) {
        ax[me] = acx * G;
        ay[me] = acy * G;
        az[me] = acz * G;
    }
}

// Group rule, FP32 pair math; tile sums of 32 accepted cells folded into (hi, lo) by TwoSum.
__global__ void __launch_bounds__(TR_THREADS)
bh_group_f32_kernel(const NodeRec32* __restrict__ rec, const uint32_t* __restrict__ info,
                    const uint32_t* __restrict__ ids, const double* __restrict__ x,
                    const double* __restrict__ y, const double* __restrict__ z,
                    const double* __restrict__ box, uint32_t n, float theta, float eps2,
                    double* __restrict__ ax, double* __restrict__ ay, double* __restrict__ az) {
    const uint32_t p = blockIdx.x * TR_THREADS + threadIdx.x;
    const bool valid = p < n;
    const uint32_t nn = info[0];
    const uint32_t me = valid ? ids[p] : NB_NONE;
    const double ox = box[0] + box[6] / 2, oy = box[1] + box[6] / 2, oz = box[2] + box[6] / 2;
    float px = 0, py = 0, pz = 0;
    if (valid) {
        px = (float)(x[me] - ox);
        py = (float)(y[me] - oy);
        pz = (float)(z[me] - oz);
    }
    const float theta2 = theta * theta;
    float tx = 0, ty = 0, tz = 0, hx = 0, hy = 0, hz = 0, lx = 0, ly = 0, lz = 0;
    int batch = 0;
    uint32_t k = 0;
    while (k < nn) {
        const NodeRec32 r = rec[k];
        const float dx = r.cx - px, dy = r.cy - py, dz = r.cz - pz;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const bool open = valid && r.body == NB_NONE && r.edge2 >= theta2 * d2;
        if (__any_sync(0xffffffffu, open)) {
            k = k + 1;
            continue;
        }
        if (valid && r.body != me) {
            const float inv = nb_rsqrt_f32(d2 + eps2);
            const float s = r.gm * inv * inv * inv;
            tx = fmaf(dx, s, tx);
            ty = fmaf(dy, s, ty);
            tz = fmaf(dz, s, tz);
        }
        if (++batch == 32) {
            batch = 0;
            float sh = hx + tx, bp = sh - hx;
            lx += (hx - (sh - bp)) + (tx - bp);
            hx = sh;
            sh = hy + ty;
            bp = sh - hy;
            ly += (hy - (sh - bp)) + (ty - bp);
            hy = sh;
            sh = hz + tz;
            bp = sh - hz;
            lz += (hz - (sh - bp)) + (tz - bp);
            hz = sh;
            tx = ty = tz = 0;
        }
        k = r.skip;
    }
    if (valid) {
        ax[me] = ((double)hx + (double)lx) + (double)tx;
        ay[me] = ((double)hy + (double)ly) + (double)ty;
        az[me] = ((double)hz + (double)lz) + (double)tz;
    }
}

// Work model: per body, the number of cells accepted (interactions) and opened under the
// per-body rule (FP64 decisions); totals accumulated into out[0] (accepted), out[1] (opened).
__global__ void __launch_bounds__(TR_THREADS)
bh_count_kernel(const NodeRec64* __restrict__ rec, const uint32_t* __restrict__ info,
                const uint32_t* __restrict__ ids, const double* __restrict__ x,
                const double* __restrict__ y, const double* __restrict__ z, uint32_t n,
                double theta, int group, unsigned long long* __restrict__ out) {
    const uint32_t p = blockIdx.x * TR_THREADS + threadIdx.x;
    const bool valid = p < n;
    const uint32_t nn = info[0];
    const uint32_t me = valid ? ids[p] : NB_NONE;
    double px = 0, py = 0, pz = 0;
    if (valid) {
        px = x[me];
        py = y[me];
        pz = z[me];
    }
    unsigned long long acc = 0, opened = 0;
    uint32_t kl = valid ? 0u : nn;
    const double theta2 = theta * theta;
    for (;;) {
        const uint32_t k = group ? (valid ? kl : nn) : kl;
        const uint32_t kk = group ? __reduce_min_sync(0xffffffffu, k) : __reduce_min_sync(0xffffffffu, kl);
        if (kk >= nn) break;
        const NodeRec64 r = rec[kk];
        const double dx = r.cx - px, dy = r.cy - py, dz = r.cz - pz;
        const double d2 = fma(dx, dx, fma(dy, dy, dz * dz));
        const bool wants_open = valid && r.mass != 0 && r.body == NB_NONE &&
                                r.edge * r.edge >= theta2 * d2;
        if (group) {
            if (__any_sync(0xffffffffu, wants_open)) {
                if (valid) opened += 1;
                kl = kk + 1;
            } else {
                if (valid && r.body != me && r.mass != 0) acc += 1;
                kl = r.skip;
            }
        } else if (kl == kk) {
            if (r.mass == 0 || r.body == me) {
                kl = r.skip;
            } else if (wants_open) {
                opened += 1;
                kl = kk + 1;
            } else {
                acc += 1;
                kl = r.skip;
            }
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        acc += __shfl_down_sync(0xffffffffu, acc, off);
        opened += __shfl_down_sync(0xffffffffu, opened, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], acc);
        atomicAdd(&out[1], opened);
    }
}

// Schedule of the per-body FP64 traversal: 0 = per-lane walks (default), 1 = the warp's union
// walk (bh_theta_f64_kernel). Both produce identical results; the switch exists for comparison.
int g_lockstep = 0;

// Resident blocks per SM of the two lane-kernel instantiations (queried once, before any
// stream capture uses them).
int g_lane_per_sm[2] = {0, 0};

template <int MODE>
nb_status lane_per_sm(int* out) {
    int& ps = g_lane_per_sm[MODE == IEEE64 ? 0 : 1];
    if (ps == 0) {
        NB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, bh_theta_lane_kernel<MODE>,
                                                                  TR_THREADS, 0));
        if (ps < 1) ps = 1;
    }
    *out = ps;
    return NB_OK;
}

// The walk lengths of the last per-body traversal of the same bodies order this one's groups
// (*order = the regrouped bodies), else tree order (*order = nullptr). The results do not depend
// on the order: each body sums its own sequence.
nb_status walk_order(const nb_bh_tree* t, cudaStream_t s, const uint32_t** order) {
    *order = nullptr;
    if (t->walk_n != t->n) return NB_OK;
    regroup_kernel<<<nb::ceil_div(t->n, RG_WINDOW), RG_WINDOW, 0, s>>>(t->ids, t->walk_len, t->n,
                                                                       t->walk_ids);
    NB_TRY(nb::check_launch("regroup_kernel"));
    *order = t->walk_ids;
    return NB_OK;
}

// Persistent launch of bh_theta_lane_kernel: resident blocks only, groups from work[1], at most
// LANE_BLOCKS_PER_SM blocks per SM. With all 40 resident warps of an SM contending for its FP64
// pipe, the warps that lose the arbitration keep their first group for the whole launch and
// finish it alone at the end; 20 warps keep the pipe as busy with a shorter tail (1% faster at
// 1,048,576 bodies than 40, 0.2% faster than 24 or 16).
constexpr int LANE_BLOCKS_PER_SM = 5;

template <int MODE>
nb_status launch_lane(nb_ctx* ctx, const nb_bh_tree* t, const double* x, const double* y,
                      const double* z, double* ax, double* ay, double* az, double G, double eps2,
                      cudaStream_t s) {
    int ps = 0;
    NB_TRY(lane_per_sm<MODE>(&ps));
    ps = std::min(ps, LANE_BLOCKS_PER_SM);
    int grid = nb::ceil_div(t->n, TR_THREADS);
    if (grid > ctx->sm_count * ps) grid = ctx->sm_count * ps;
    NB_CUDA_TRY(cudaMemsetAsync(t->work + 1, 0, sizeof(uint32_t), s));
    const uint32_t* order = nullptr;
    NB_TRY(walk_order(t, s, &order));
    bh_theta_lane_kernel<MODE><<<grid, TR_THREADS, 0, s>>>(
        t->rec32, t->rec64, t->info, t->ids, x, y, z, t->box, t->n, t->params.theta, eps2, G, ax,
        ay, az, t->work + 1, order, t->walk_len);
    NB_TRY(nb::check_launch(MODE == IEEE64 ? "bh_theta_lane_kernel<ieee>" : "bh_theta_lane_kernel"));
    t->walk_n = t->n;
    return NB_OK;
}

}  // namespace

namespace nb {
nb_status launch_learned(nb_ctx* ctx, const nb_bh_tree* t, const double* x, const double* y,
                         const double* z, double* ax, double* ay, double* az, double eps2,
                         unsigned long long* counters, cudaStream_t s);
nb_status learned_per_sm(int* out);
}

extern "C" {

nb_status nb_bh_set_schedule(int lockstep) {
    g_lockstep = lockstep ? 1 : 0;
    return NB_OK;
}

nb_status nb_bh_accel(nb_ctx* ctx, const nb_bh_tree* t, const double* x, const double* y,
                      const double* z, double* ax, double* ay, double* az, double G, double eps2,
                      nb_opening opening, nb_precision prec, nb_stream_t stream_) {
    NB_CHECK_CTX(ctx);
    if (!t) return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_accel: null tree");
    if (!t->built) return nb::set_error(NB_ERR_NOT_BUILT, "nb_bh_accel: tree not built");
    if (!x || !y || !z || !ax || !ay || !az)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_accel: null array");
    cudaStream_t s = (cudaStream_t)stream_;
    const uint32_t n = t->n;
    const int grid = nb::ceil_div(n, TR_THREADS);
    const double theta = t->params.theta;
    if (opening == NB_OPEN_THETA) {
        switch (prec) {
            case NB_F64_IEEE:
                NB_TRY(nb_need_records(t, NB_REC_FP64, "nb_bh_accel"));
                if (g_lockstep) {
                    bh_theta_f64_kernel<IEEE64><<<grid, TR_THREADS, 0, s>>>(
                        t->rec64, t->info, t->ids, x, y, z, n, theta, eps2, G, ax, ay, az);
                    return nb::check_launch("bh_theta_f64_kernel<ieee>");
                }
                return launch_lane<IEEE64>(ctx, t, x, y, z, ax, ay, az, G, eps2, s);
            case NB_F64:
                NB_TRY(nb_need_records(t, NB_REC_FP64, "nb_bh_accel"));
                if (g_lockstep) {
                    bh_theta_f64_kernel<FAST64><<<grid, TR_THREADS, 0, s>>>(
                        t->rec64, t->info, t->ids, x, y, z, n, theta, eps2, G, ax, ay, az);
                    return nb::check_launch("bh_theta_f64_kernel");
                }
                return launch_lane<FAST64>(ctx, t, x, y, z, ax, ay, az, G, eps2, s);
            case NB_DF64:
                NB_TRY(nb_need_records(t, NB_REC_FP64 | NB_REC_DF, "nb_bh_accel"));
                if (t->G == 0)
                    return nb::set_error(NB_ERR_INVALID_ARG,
                                         "nb_bh_accel: NB_DF64 needs a build with G != 0");
            {
                const uint32_t* order = nullptr;
                NB_TRY(walk_order(t, s, &order));
                bh_theta_df_kernel<<<grid, TR_THREADS, 0, s>>>(
                    t->rec32, t->rec32lo, t->rec32lo2, t->rec64, t->info, t->ids, x, y, z, t->box,
                    n, theta, eps2, G / t->G, ax, ay, az, order, t->walk_len);
                NB_TRY(nb::check_launch("bh_theta_df_kernel"));
                t->walk_n = t->n;
                return NB_OK;
            }
            case NB_F32C:
                if (G != t->G)
                    return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_accel: G differs from the build's");
                bh_theta_f32_kernel<<<grid, TR_THREADS, 0, s>>>(t->rec32, t->info, t->ids, x, y, z,
                                                                t->box, n, (float)theta,
                                                                (float)eps2, ax, ay, az);
                return nb::check_launch("bh_theta_f32_kernel");
            default:
                break;
        }
    } else if (opening == NB_OPEN_THETA_GROUP) {
        switch (prec) {
            case NB_F64_IEEE:
            case NB_F64:
                NB_TRY(nb_need_records(t, NB_REC_FP64, "nb_bh_accel"));
                bh_group_f64_kernel<<<grid, TR_THREADS, 0, s>>>(t->rec64, t->info, t->ids, x, y, z,
                                                                n, theta, eps2, G, ax, ay, az);
                return nb::check_launch("bh_group_f64_kernel");
            case NB_F32C:
                if (G != t->G)
                    return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_accel: G differs from the build's");
                bh_group_f32_kernel<<<grid, TR_THREADS, 0, s>>>(t->rec32, t->info, t->ids, x, y, z,
                                                                t->box, n, (float)theta,
                                                                (float)eps2, ax, ay, az);
                return nb::check_launch("bh_group_f32_kernel");
            default:
                break;
        }
    } else if (opening == NB_OPEN_LEARNED) {
        if (prec != NB_F32C)
            return nb::set_error(NB_ERR_UNSUPPORTED, "nb_bh_accel: NB_OPEN_LEARNED runs in NB_F32C");
        if (G != t->G)
            return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_accel: G differs from the build's");
        NB_TRY(nb_need_records(t, NB_REC_LEARNED, "nb_bh_accel"));
        return nb::launch_learned(ctx, t, x, y, z, ax, ay, az, eps2, nullptr, s);
    }
    return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_accel: unknown opening %d / precision %d",
                         (int)opening, (int)prec);
}

nb_status nb_bh_count_interactions(nb_ctx* ctx, const nb_bh_tree* t, const double* x,
                                   const double* y, const double* z, nb_opening opening,
                                   unsigned long long* out_dev, nb_stream_t stream_) {
    NB_CHECK_CTX(ctx);
    if (!t || !t->built) return nb::set_error(NB_ERR_NOT_BUILT, "nb_bh_count_interactions: tree not built");
    if (!x || !y || !z || !out_dev) return nb::set_error(NB_ERR_INVALID_ARG, "null pointer");
    if (opening != NB_OPEN_THETA && opening != NB_OPEN_THETA_GROUP)
        return nb::set_error(NB_ERR_UNSUPPORTED, "nb_bh_count_interactions: theta rules only");
    NB_TRY(nb_need_records(t, NB_REC_FP64, "nb_bh_count_interactions"));
    cudaStream_t s = (cudaStream_t)stream_;
    NB_CUDA_TRY(cudaMemsetAsync(out_dev, 0, 2 * sizeof(unsigned long long), s));
    bh_count_kernel<<<nb::ceil_div(t->n, TR_THREADS), TR_THREADS, 0, s>>>(
        t->rec64, t->info, t->ids, x, y, z, t->n, t->params.theta,
        opening == NB_OPEN_THETA_GROUP ? 1 : 0, out_dev);
    return nb::check_launch("bh_count_kernel");
}

nb_status nb_bh_accel_learned_counted(nb_ctx* ctx, const nb_bh_tree* t, const double* x,
                                     const double* y, const double* z, double* ax, double* ay,
                                     double* az, double eps2, unsigned long long* counters_dev,
                                     nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (!t || !t->built) return nb::set_error(NB_ERR_NOT_BUILT, "tree not built");
    if (!counters_dev) return nb::set_error(NB_ERR_INVALID_ARG, "null counters");
    NB_TRY(nb_need_records(t, NB_REC_LEARNED, "nb_bh_accel_learned_counted"));
    NB_CUDA_TRY(cudaMemsetAsync(counters_dev, 0, 2 * sizeof(unsigned long long), (cudaStream_t)stream));
    return nb::launch_learned(ctx, t, x, y, z, ax, ay, az, eps2, counters_dev, (cudaStream_t)stream);
}

nb_status nb_bh_graph_create(nb_ctx* ctx, nb_bh_tree* t, const double* m, double* x, double* y,
                             double* z, double* vx, double* vy, double* vz, double* vhx,
                             double* vhy, double* vhz, double* ax, double* ay, double* az,
                             uint32_t n, double G, double eps2, double dt, int steps,
                             nb_opening opening, nb_precision prec, nb_graph** out) {
    NB_CHECK_CTX(ctx);
    if (!t || !out || steps < 1)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_graph_create: bad arguments");
    if (t->phase_timing)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_graph_create: phase timing is on");
    *out = nullptr;
    int ps = 0;  // one-time queries happen here, outside the capture
    NB_TRY(lane_per_sm<IEEE64>(&ps));
    NB_TRY(lane_per_sm<FAST64>(&ps));
    NB_TRY(nb::learned_per_sm(&ps));
    cudaStream_t s;
    NB_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        return nb::cuda_error(e, "cudaStreamBeginCapture");
    }
    nb_status st = NB_OK;
    const nb_stream_t ns = (nb_stream_t)s;
    for (int k = 0; k < steps && st == NB_OK; ++k) {
        st = nb_leapfrog_kick_drift(ctx, vhx, vhy, vhz, vx, vy, vz, x, y, z, ax, ay, az, n, dt, ns);
        if (st == NB_OK) st = nb_bh_build(ctx, t, m, x, y, z, n, G, ns);
        if (st == NB_OK) st = nb_bh_accel(ctx, t, x, y, z, ax, ay, az, G, eps2, opening, prec, ns);
        if (st == NB_OK) st = nb_leapfrog_kick(ctx, vx, vy, vz, vhx, vhy, vhz, ax, ay, az, n, dt, ns);
    }
    return nb_finish_capture(s, st, steps, out);
}

}  // extern "C"
