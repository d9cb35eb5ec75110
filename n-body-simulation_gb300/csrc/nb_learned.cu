// nb_learned.cu -- learned opening policy for the Barnes-Hut traversal.
//
// A small MLP (8 -> 32 -> 32 -> 1, ReLU) predicts, for a group of 32 bodies adjacent in tree
// order and a cell, y = log10(max over the group of |F_exact - F_monopole| / |a_body|) / 5: the
// worst relative force error that accepting the cell's monopole would add to the group. The
// traversal accepts the cell when y < log10(tau)/5.
//
//  * Labels come from the method itself (nb_bh_generate_pairs): a theta-rule walk samples
//    (group, cell) pairs, and for each pair one warp computes the exact cell force on its 32
//    bodies by direct summation over the cell's bodies (contiguous in tree order) against the
//    cell's monopole.
//  * Training (nb_mlp_loss_grad, nb_mlp_adam): FP32 forward/backward kernels, MSE loss, Adam.
//  * Inference (nb_bh_accel with NB_OPEN_LEARNED): each warp keeps a stack of cells in shared
//    memory, pops up to 32 at a time and scores the network's cells with BF16 tensor-core
//    mma.sync.m16n8k16 (FP32 accumulate, one or two 16-row blocks); each layer's accumulator
//    fragments are reused in registers as the next layer's A fragments. Body leaves are always
//    accepted, cells that may overlap the group are always opened, cells whose analytic monopole
//    error bound is below tau are accepted without the network, and cells with more bodies than
//    the training range fall back to the group theta rule. Accepted monopoles and the bodies of
//    small opened cells go to a per-warp interaction list summed by all lanes. Groups whose walk
//    cost at least twice the mean in the previous launch are walked first.
#include <cuda_bf16.h>

#include "nb_bh.cuh"

namespace {

// parameter layout (FP32): W1[8][32], b1[32], W2[32][32], b2[32], w3[32], b3
constexpr int P_W1 = 0, P_B1 = 256, P_W2 = 288, P_B2 = 1312, P_W3 = 1344, P_B3 = 1376;
constexpr int P_COUNT = 1377;
constexpr int NF = 8;
constexpr float SQRT3 = 1.7320508f;

struct GroupGeo {
    float cx, cy, cz, r, a_ref, lg_aref;  // box centre, radius, weakest |a|, log2(a_ref)
};

__device__ __forceinline__ float warp_min(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Group geometry from the lanes' FP32 positions (relative to the box centre): bounding-box
// centre, radius, and the weakest previous acceleration of the group.
__device__ GroupGeo group_geo(bool valid, float px, float py, float pz, float a_prev) {
    const float inf = __int_as_float(0x7f800000);
    GroupGeo g;
    const float lx = warp_min(valid ? px : inf), hx = warp_max(valid ? px : -inf);
    const float ly = warp_min(valid ? py : inf), hy = warp_max(valid ? py : -inf);
    const float lz = warp_min(valid ? pz : inf), hz = warp_max(valid ? pz : -inf);
    g.cx = 0.5f * (lx + hx);
    g.cy = 0.5f * (ly + hy);
    g.cz = 0.5f * (lz + hz);
    const float dx = px - g.cx, dy = py - g.cy, dz = pz - g.cz;
    g.r = warp_max(valid ? sqrtf(dx * dx + dy * dy + dz * dz) : 0.f);
    g.a_ref = fmaxf(warp_min(valid ? a_prev : inf), 1e-30f);
    g.lg_aref = __log2f(g.a_ref);
    return g;
}

// FP32 box edge and its base-2 logarithm, for the cell edges: a cell of level L has edge
// box_edge * 2^-L, exact in FP32 (the edges the records held), formed by exponent arithmetic
// while the result stays a normal number.
struct BoxScale {
    float e0, lg_e0;
    bool bits;
    BoxScale() = default;
    __device__ explicit BoxScale(double box_edge) {
        e0 = (float)box_edge;
        lg_e0 = e0 > 0.f ? __log2f(e0) : -128.f;
        bits = e0 >= 1e-20f;
    }
    __device__ __forceinline__ float edge(uint32_t level) const {
        return bits ? __int_as_float(__float_as_int(e0) - ((int)level << 23))
                    : ldexpf(e0, -(int)level);
    }
};

// The class of a (group, cell) pair: 1 = body leaf (accept), 2 = may overlap the group (gap <=
// sqrt(3) * edge: open), 3 = outside the training range (theta rule), 0 = for the policy. m2 =
// squared gap, the smallest squared distance from a member of the group to the cell's centre of
// mass.
__device__ __forceinline__ int cell_class(const NodeRec32& r, const NodeAux& x, float m2,
                                          uint32_t count_cap) {
    if (r.body != NB_NONE) return 1;
    if (m2 <= 3.f * r.edge2) return 2;
    return x.count > count_cap ? 3 : 0;
}

// The 8 features of a (group, cell) pair and its class (cell_class, plus 4 = provably accurate
// enough: accept). d = distance from the group's box centre to the cell's centre of mass. The
// per-cell terms (spread / edge, log2 of G * mass) come from the build; logarithms are the fast
// base-2 logarithm (features only steer the policy; labels and training use the same function).
//
// Class 4 (only when bound_tau > 0): the cell's bodies lie within b = sqrt(3) * edge of its
// centre of mass, so for a body at distance R >= gap the monopole's force error is at most
// G M / R^2 * sum_{l>=2} (l+1) (b/R)^l = G M / R^2 * rho^2 (3 - 2 rho) / (1 - rho)^2, rho = b / gap
// (the multipole series of the potential with a vanishing dipole). When that bound relative to
// the group's smallest |a| is below bound_tau the cell is accepted; the test is multiplied out,
// G M b^2 (3 gap - 2 b) < bound_tau a_ref gap^3 (gap - b)^2, so it needs no division.
__device__ __forceinline__ int cell_features(const NodeRec32& r, const NodeAux& x,
                                             const GroupGeo& g, const BoxScale& bs, float m2,
                                             uint32_t count_cap, float* f, float bound_tau = 0.f) {
    if (r.body != NB_NONE) return 1;
    if (m2 <= 3.f * r.edge2) return 2;
    const float e = bs.edge(r.level);
    const float inv_gap = rsqrtf(m2), gap = m2 * inv_gap;
    if (bound_tau > 0.f) {
        const float b = SQRT3 * e, gb = gap - b;
        if (r.gm * (b * b) * fmaf(3.f, gap, -2.f * b) <
            bound_tau * g.a_ref * (gap * gap) * gap * (gb * gb))
            return 4;
    }
    if (x.count > count_cap) return 3;
    const float dx = r.cx - g.cx, dy = r.cy - g.cy, dz = r.cz - g.cz;
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float lg_e = bs.lg_e0 - (float)r.level;
    const float lg_m2 = __log2f(m2);
    f[0] = (0.5f * __log2f(d2) - lg_e) * 0.25f;
    f[1] = x.spread_rel;
    f[2] = __log2f((float)x.count) * 0.0625f;
    f[3] = (float)r.level * 0.0625f;
    f[4] = g.r * rsqrtf(d2);
    // log10(G m / (gap^2 a_ref)) / 4
    f[5] = (x.lg_gm - lg_m2 - g.lg_aref) * (0.30103f * 0.25f);
    f[6] = (0.5f * lg_m2 - lg_e) * 0.25f;
    f[7] = x.spread_rel * e * inv_gap;
    return 0;
}

// Smallest squared distance from a valid lane's body to (cx, cy, cz), over the whole warp.
__device__ __forceinline__ float warp_min_dist2(bool valid, float px, float py, float pz,
                                                float cx, float cy, float cz) {
    const float dx = cx - px, dy = cy - py, dz = cz - pz;
    const float inf = __int_as_float(0x7f800000);
    return warp_min(valid ? fmaf(dx, dx, fmaf(dy, dy, dz * dz)) : inf);
}

// ---------------------------------------------------------------------------------------------
// BF16 tensor-core MLP over 16 cells (mma.sync.m16n8k16, FP32 accumulate)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// max(lo, 0), max(hi, 0) as a BF16 pair in one instruction (the ReLU commutes with the rounding).
__device__ __forceinline__ uint32_t pack_bf16_relu(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

__device__ __forceinline__ void mma16816(float* c, uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Weight fragments of one lane (g = lane/4, t = lane%4), flat:
//  w[nt]                      layer 1, n-tile nt: W1[2t..2t+1][nt*8+g] (k rows 8..15 are zero)
//  w[4 + (ks*4 + nt)*2 + j]   layer 2, k-step ks, n-tile nt, register j
//  w[20 + ks*2 + j]           layer 3 (output column 0 only: lanes with g == 0)
//  b[nt*2 + j], b[8 + nt*2 + j], b[16]: biases of layers 1, 2 and 3 for the lane's columns.
// They live in shared memory, shared by the block's warps, [lane][index] with row strides of 28
// and 20 words, so that a layer's fragments come in 16-byte loads (6 for the weights, 5 for the
// biases) and the 8 lanes of each load phase hit disjoint banks.
constexpr int MF_W = 24, MF_B = 17;    // weight fragments and biases per lane
constexpr int MF_WS = 28, MF_BS = 20;  // per-lane strides (words)
static_assert(MF_WS >= MF_W && MF_BS >= MF_B && MF_WS % 4 == 0 && MF_BS % 4 == 0,
              "a lane's fragments fit its 16-byte-aligned row");
struct MlpFragsSmem {
    const uint32_t* ws;  // this lane's weight fragments
    const float* bs;     // this lane's biases
    __device__ __forceinline__ uint4 w4(int k) const {
        return reinterpret_cast<const uint4*>(ws)[k];
    }
    __device__ __forceinline__ float4 b4(int k) const {
        return reinterpret_cast<const float4*>(bs)[k];
    }
    // layer 1: weights w[0..3], biases b[0..7]
    __device__ __forceinline__ void layer1(uint32_t* w, float* b) const {
        const uint4 a = w4(0);
        const float4 p = b4(0), q = b4(1);
        w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w;
        b[0] = p.x; b[1] = p.y; b[2] = p.z; b[3] = p.w;
        b[4] = q.x; b[5] = q.y; b[6] = q.z; b[7] = q.w;
    }
    // layer 2: weights w[4..19] (as w[0..15]), biases b[8..15] (as b[0..7])
    __device__ __forceinline__ void layer2(uint32_t* w, float* b) const {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint4 a = w4(1 + k);
            w[4 * k] = a.x; w[4 * k + 1] = a.y; w[4 * k + 2] = a.z; w[4 * k + 3] = a.w;
        }
        const float4 p = b4(2), q = b4(3);
        b[0] = p.x; b[1] = p.y; b[2] = p.z; b[3] = p.w;
        b[4] = q.x; b[5] = q.y; b[6] = q.z; b[7] = q.w;
    }
    // layer 3: weights w[20..23] (as w[0..3]), bias b[16]
    __device__ __forceinline__ void layer3(uint32_t* w, float& b) const {
        const uint4 a = w4(5);
        w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w;
        b = b4(4).x;
    }
};

__device__ void load_frags(const float* __restrict__ P, int lane, uint32_t* w, float* b,
                           int stride) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        const int o = nt * 8 + g;
        w[nt * stride] = pack_bf16(P[P_W1 + (2 * t) * 32 + o], P[P_W1 + (2 * t + 1) * 32 + o]);
        b[(nt * 2) * stride] = P[P_B1 + nt * 8 + 2 * t];
        b[(nt * 2 + 1) * stride] = P[P_B1 + nt * 8 + 2 * t + 1];
        b[(8 + nt * 2) * stride] = P[P_B2 + nt * 8 + 2 * t];
        b[(8 + nt * 2 + 1) * stride] = P[P_B2 + nt * 8 + 2 * t + 1];
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            const int k0 = ks * 16 + 2 * t;
            w[(4 + (ks * 4 + nt) * 2) * stride] =
                pack_bf16(P[P_W2 + k0 * 32 + o], P[P_W2 + (k0 + 1) * 32 + o]);
            w[(4 + (ks * 4 + nt) * 2 + 1) * stride] =
                pack_bf16(P[P_W2 + (k0 + 8) * 32 + o], P[P_W2 + (k0 + 9) * 32 + o]);
        }
    }
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        const int k0 = ks * 16 + 2 * t;
        w[(20 + ks * 2) * stride] = g == 0 ? pack_bf16(P[P_W3 + k0], P[P_W3 + k0 + 1]) : 0u;
        w[(20 + ks * 2 + 1) * stride] = g == 0 ? pack_bf16(P[P_W3 + k0 + 8], P[P_W3 + k0 + 9]) : 0u;
    }
    b[16 * stride] = P[P_B3];
}

// Scores of the 16 feature rows in smem (row-major [16][16] bf16, columns 8..15 zero); returns
// the score of row (lane & 15).
template <class Frags>
__device__ float mlp16(const __nv_bfloat16* __restrict__ feat, int lane, const Frags& F) {
    const int g = lane >> 2, t = lane & 3;
    const uint32_t* row = reinterpret_cast<const uint32_t*>(feat);  // 8 u32 per row
    const uint32_t a0 = row[g * 8 + t], a1 = row[(g + 8) * 8 + t];
    uint32_t w1[4], w2[16], w3[4];
    float b1[8], b2[8], b3;
    F.layer1(w1, b1);
    float c1[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        c1[nt][0] = b1[nt * 2 + 0];
        c1[nt][1] = b1[nt * 2 + 1];
        c1[nt][2] = b1[nt * 2 + 0];
        c1[nt][3] = b1[nt * 2 + 1];
        mma16816(c1[nt], a0, a1, 0u, 0u, w1[nt], 0u);
    }
    F.layer2(w2, b2);
    uint32_t h1[2][4];
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        h1[ks][0] = pack_bf16_relu(c1[2 * ks][0], c1[2 * ks][1]);
        h1[ks][1] = pack_bf16_relu(c1[2 * ks][2], c1[2 * ks][3]);
        h1[ks][2] = pack_bf16_relu(c1[2 * ks + 1][0], c1[2 * ks + 1][1]);
        h1[ks][3] = pack_bf16_relu(c1[2 * ks + 1][2], c1[2 * ks + 1][3]);
    }
    float c2[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        c2[nt][0] = b2[nt * 2 + 0];
        c2[nt][1] = b2[nt * 2 + 1];
        c2[nt][2] = b2[nt * 2 + 0];
        c2[nt][3] = b2[nt * 2 + 1];
#pragma unroll
        for (int ks = 0; ks < 2; ++ks)
            mma16816(c2[nt], h1[ks][0], h1[ks][1], h1[ks][2], h1[ks][3], w2[(ks * 4 + nt) * 2],
                     w2[(ks * 4 + nt) * 2 + 1]);
    }
    F.layer3(w3, b3);
    uint32_t h2[2][4];
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        h2[ks][0] = pack_bf16_relu(c2[2 * ks][0], c2[2 * ks][1]);
        h2[ks][1] = pack_bf16_relu(c2[2 * ks][2], c2[2 * ks][3]);
        h2[ks][2] = pack_bf16_relu(c2[2 * ks + 1][0], c2[2 * ks + 1][1]);
        h2[ks][3] = pack_bf16_relu(c2[2 * ks + 1][2], c2[2 * ks + 1][3]);
    }
    float c3[4] = {b3, b3, b3, b3};
#pragma unroll
    for (int ks = 0; ks < 2; ++ks)
        mma16816(c3, h2[ks][0], h2[ks][1], h2[ks][2], h2[ks][3], w3[ks * 2], w3[ks * 2 + 1]);
    // row r's score sits in lane 4*(r%8): c3[0] for r < 8, c3[2] for r >= 8
    const int r = lane & 15;
    const float v0 = __shfl_sync(0xffffffffu, c3[0], 4 * (r & 7));
    const float v2 = __shfl_sync(0xffffffffu, c3[2], 4 * (r & 7));
    return r < 8 ? v0 : v2;
}

// Scores of 32 feature rows in smem (row-major [32][16] bf16, columns 8..15 zero): the two 16-row
// blocks go through each layer together, so their mma chains overlap. Returns the score of row
// `lane`.
template <class Frags>
__device__ float mlp32(const __nv_bfloat16* __restrict__ feat, int lane, const Frags& F) {
    const int g = lane >> 2, t = lane & 3;
    const uint32_t* row = reinterpret_cast<const uint32_t*>(feat);  // 8 u32 per row
    uint32_t a0[2], a1[2];
#pragma unroll
    for (int b = 0; b < 2; ++b) {
        a0[b] = row[(16 * b + g) * 8 + t];
        a1[b] = row[(16 * b + g + 8) * 8 + t];
    }
    uint32_t w1[4], w2[16], w3[4];
    float b1[8], b2[8], b3;
    F.layer1(w1, b1);
    float c1[2][4][4];
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            c1[b][nt][0] = b1[nt * 2 + 0];
            c1[b][nt][1] = b1[nt * 2 + 1];
            c1[b][nt][2] = b1[nt * 2 + 0];
            c1[b][nt][3] = b1[nt * 2 + 1];
            mma16816(c1[b][nt], a0[b], a1[b], 0u, 0u, w1[nt], 0u);
        }
    F.layer2(w2, b2);
    uint32_t h[2][2][4];
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            h[b][ks][0] = pack_bf16_relu(c1[b][2 * ks][0], c1[b][2 * ks][1]);
            h[b][ks][1] = pack_bf16_relu(c1[b][2 * ks][2], c1[b][2 * ks][3]);
            h[b][ks][2] = pack_bf16_relu(c1[b][2 * ks + 1][0], c1[b][2 * ks + 1][1]);
            h[b][ks][3] = pack_bf16_relu(c1[b][2 * ks + 1][2], c1[b][2 * ks + 1][3]);
        }
    float c2[2][4][4];
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            c2[b][nt][0] = b2[nt * 2 + 0];
            c2[b][nt][1] = b2[nt * 2 + 1];
            c2[b][nt][2] = b2[nt * 2 + 0];
            c2[b][nt][3] = b2[nt * 2 + 1];
        }
#pragma unroll
    for (int ks = 0; ks < 2; ++ks)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
                mma16816(c2[b][nt], h[b][ks][0], h[b][ks][1], h[b][ks][2], h[b][ks][3],
                         w2[(ks * 4 + nt) * 2], w2[(ks * 4 + nt) * 2 + 1]);
    F.layer3(w3, b3);
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            h[b][ks][0] = pack_bf16_relu(c2[b][2 * ks][0], c2[b][2 * ks][1]);
            h[b][ks][1] = pack_bf16_relu(c2[b][2 * ks][2], c2[b][2 * ks][3]);
            h[b][ks][2] = pack_bf16_relu(c2[b][2 * ks + 1][0], c2[b][2 * ks + 1][1]);
            h[b][ks][3] = pack_bf16_relu(c2[b][2 * ks + 1][2], c2[b][2 * ks + 1][3]);
        }
    float c3[2][4];
#pragma unroll
    for (int b = 0; b < 2; ++b) {
        c3[b][0] = c3[b][1] = c3[b][2] = c3[b][3] = b3;
    }
#pragma unroll
    for (int ks = 0; ks < 2; ++ks)
#pragma unroll
        for (int b = 0; b < 2; ++b)
            mma16816(c3[b], h[b][ks][0], h[b][ks][1], h[b][ks][2], h[b][ks][3], w3[ks * 2], w3[ks * 2 + 1]);
    // row r of block b sits in lane 4*(r%8): c3[b][0] for r < 8, c3[b][2] for r >= 8
    const int r = lane & 15, src = 4 * (r & 7);
    const float v00 = __shfl_sync(0xffffffffu, c3[0][0], src);
    const float v02 = __shfl_sync(0xffffffffu, c3[0][2], src);
    const float v10 = __shfl_sync(0xffffffffu, c3[1][0], src);
    const float v12 = __shfl_sync(0xffffffffu, c3[1][2], src);
    return lane < 16 ? (r < 8 ? v00 : v02) : (r < 8 ? v10 : v12);
}

// ---------------------------------------------------------------------------------------------
// Learned traversal
// ---------------------------------------------------------------------------------------------
constexpr int LT_WARPS = 4;
constexpr int LT_THREADS = LT_WARPS * 32;
constexpr int LT_CAP = (int)NB_LEARNED_STACK_CAP;  // stack entries per warp
constexpr int LT_RESERVE = 7 * NB_MAX_TREE_DEPTH + 8;  // headroom of single-cell steps
constexpr int LT_BATCH = 32;        // cells popped per step (one per lane)
constexpr uint32_t LT_DIRECT = 12;  // opened cells up to this many bodies: direct sums (12
                                    // measured 2.5% faster than 8 for the learned walk, 1% for the
                                    // theta rule; 6 slower for both)
constexpr int LT_LIST = 384;        // interaction list entries per warp (a full step fits: a lane
                                    // adds at most max(LT_DIRECT, 1) entries per step)
static_assert(LT_LIST >= LT_BATCH * LT_DIRECT, "one step must fit in an empty list");

// Sum of the interactions in list[0..count) for one body; 4 independent accumulators. 1/r is
// capped at 1e12: an entry at zero distance (the body itself) then contributes exactly 0 even
// without softening, and with eps^2 >= 1e-24 the cap never binds.
__device__ __forceinline__ void pair_term(const float4 e, float px, float py, float pz,
                                          float eps2, float& ax, float& ay, float& az) {
    const float dx = e.x - px, dy = e.y - py, dz = e.z - pz;
    const float inv = fminf(nb_rsqrt_f32(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)))), 1e12f);
    const float w = e.w * inv * inv * inv;
    ax = fmaf(dx, w, ax);
    ay = fmaf(dy, w, ay);
    az = fmaf(dz, w, az);
}

__device__ __forceinline__ void flush_list(const float4* __restrict__ list, int count, float px,
                                           float py, float pz, float eps2, float& ox, float& oy,
                                           float& oz) {
    float ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0}, az[4] = {0, 0, 0, 0};
    int j = 0;
    for (; j + 4 <= count; j += 4) {
#pragma unroll
        for (int u = 0; u < 4; ++u) pair_term(list[j + u], px, py, pz, eps2, ax[u], ay[u], az[u]);
    }
    for (; j < count; ++j) pair_term(list[j], px, py, pz, eps2, ax[0], ay[0], az[0]);
    ox = (ax[0] + ax[1]) + (ax[2] + ax[3]);
    oy = (ay[0] + ay[1]) + (ay[2] + ay[3]);
    oz = (az[0] + az[1]) + (az[2] + az[3]);
}

__device__ __forceinline__ void two_sum_add(float& h, float& l, float v) {
    const float s = h + v, bp = s - h;
    l += (h - (s - bp)) + (v - bp);
    h = s;
}

// One warp per group of 32 bodies adjacent in tree order. Each step pops up to 32 cells (one per
// lane) with their records, extra data and child lists, computes the exact smallest distance
// from the group to each cell's centre of mass, scores the network's cells with two 16-row BF16
// mma passes, and then (i) appends accepted monopoles, body leaves and the bodies of small opened
// cells to the warp's interaction list and (ii) pushes the children of the other opened cells.
// Interaction-list positions are relative to the group's first body and built from two-float
// (FP32 value + FP32 residual) coordinates, so nearby pairs keep their full FP32 precision. With
// params == nullptr the network's cells use the group theta rule instead (same walk, no network).
// Groups are taken in tree order; when sched[0] equals the group count, the sched[1] groups of
// `first` (the costliest of the previous launch, flagged in the bit mask `skip`) are taken before
// all others and skipped in the tree-order pass. Each group is walked once either way, so the
// results do not depend on the schedule. Each group's cost (2 per cell visited + 1 per list entry)
// goes to cost[] for the next launch's schedule. NET = false is the theta-rule walk (params ==
// nullptr), compiled without the network.
template <bool COUNTED, bool NET>
__global__ void __launch_bounds__(LT_THREADS, 4)
bh_learned_kernel(const NodeRec32* __restrict__ rec, const NodeAux* __restrict__ aux,
                  const uint32_t* __restrict__ children, const float4* __restrict__ sorted4,
                  const float4* __restrict__ sorted4lo, uint32_t n,
                  const float* __restrict__ params, float log_tau_scaled, float bound_tau,
                  float theta2, uint32_t count_cap, float eps2, const uint32_t* __restrict__ ids,
                  double* __restrict__ ax, double* __restrict__ ay, double* __restrict__ az,
                  unsigned long long* __restrict__ counters, uint32_t* __restrict__ err_word,
                  uint32_t* __restrict__ next_group, int cap, const double* __restrict__ box,
                  const uint32_t* __restrict__ first, const uint32_t* __restrict__ skip,
                  const uint32_t* __restrict__ sched, uint32_t* __restrict__ cost,
                  unsigned long long* __restrict__ cost_total) {
    // cap <= LT_CAP: the stack entries a walk may use (LT_CAP except in the failure-path tests)
    __shared__ uint32_t stack[LT_WARPS][LT_CAP];
    __shared__ __align__(16) __nv_bfloat16 feat[LT_WARPS][LT_BATCH][16];
    // the group's positions as packed pairs (bodies 2j, 2j+1) per axis, for the gap loop
    __shared__ nb_f2 gpx[LT_WARPS][16], gpy[LT_WARPS][16], gpz[LT_WARPS][16];
    __shared__ float4 ilist[LT_WARPS][LT_LIST];
    // per step: the lane whose cell fills each new list slot (0xff: a monopole, written by its lane)
    __shared__ uint8_t slot_lane[LT_WARPS][LT_BATCH * LT_DIRECT];
    __shared__ __align__(16) uint32_t wfrag[32 * MF_WS];
    __shared__ __align__(16) float bfrag[32 * MF_BS];
    __shared__ BoxScale bs;  // in shared memory: no registers held through the walk
    __shared__ uint32_t n_first;  // groups of the priority list (0: tree order only)
    __shared__ uint32_t wcost[LT_WARPS];  // cost of each warp's current group (no register)
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const uint32_t n_groups = (n + 31) / 32;
    if (threadIdx.x == 0) {
        bs = BoxScale(box[6]);
        n_first = sched[0] == n_groups ? min(sched[1], n_groups) : 0u;
    }
    if (NET && wi == 0) load_frags(params, lane, wfrag + lane * MF_WS, bfrag + lane * MF_BS, 1);
    __syncthreads();  // before any warp leaves
    unsigned long long t_acc = 0, t_mlp = 0, t_cells = 0, t_steps = 0;
    bool listed = n_first > 0;  // lane 0: still taking groups from the priority list
    // persistent warps: each takes the next group until none are left (no warp idles while its
    // block's other warps finish long walks)
    for (;;) {
        uint32_t gw = 0;
        if (lane == 0) {
            if (listed) {
                const uint32_t k = atomicAdd(next_group + 2, 1u);
                if (k < n_first) gw = first[k];
                else listed = false;
            }
            if (!listed) {
                do {
                    gw = atomicAdd(next_group, 1u);
                } while (n_first > 0 && gw < n_groups && ((skip[gw >> 5] >> (gw & 31)) & 1u));
            }
        }
        gw = __shfl_sync(0xffffffffu, gw, 0);
        if (gw >= n_groups) break;
        const uint32_t p = gw * 32 + lane;
        const bool valid = p < n;
        const uint32_t me = valid ? ids[p] : NB_NONE;
        // own position: box-centre relative (features), group-relative (forces)
        float4 ph = make_float4(0.f, 0.f, 0.f, 0.f), pl = ph;
        float a_prev = 0.f;
        if (valid) {
            ph = sorted4[p];
            pl = sorted4lo[p];
            const double a2 = ax[me] * ax[me] + ay[me] * ay[me] + az[me] * az[me];
            a_prev = (float)sqrt(a2);
        }
        const float ghx = __shfl_sync(0xffffffffu, ph.x, 0), ghy = __shfl_sync(0xffffffffu, ph.y, 0),
                    ghz = __shfl_sync(0xffffffffu, ph.z, 0);
        const float glx = __shfl_sync(0xffffffffu, pl.x, 0), gly = __shfl_sync(0xffffffffu, pl.y, 0),
                    glz = __shfl_sync(0xffffffffu, pl.z, 0);
        const float px = (ph.x - ghx) + (pl.x - glx), py = (ph.y - ghy) + (pl.y - gly),
                    pz = (ph.z - ghz) + (pl.z - glz);
        const GroupGeo G = group_geo(valid, ph.x, ph.y, ph.z, a_prev);
        const float inf = __int_as_float(0x7f800000);
        reinterpret_cast<float*>(gpx[wi])[lane] = valid ? ph.x : inf;
        reinterpret_cast<float*>(gpy[wi])[lane] = valid ? ph.y : inf;
        reinterpret_cast<float*>(gpz[wi])[lane] = valid ? ph.z : inf;
        constexpr bool use_net = NET;
        const MlpFragsSmem F{wfrag + lane * MF_WS, bfrag + lane * MF_BS};
        uint32_t* st = stack[wi];
        __nv_bfloat16* fm = &feat[wi][0][0];
        for (int k = lane; k < LT_BATCH * 16; k += 32) fm[k] = __float2bfloat16(0.f);
        if (lane == 0) st[0] = 0;
        int top = 1;
        float hx = 0, hy = 0, hz = 0, lx = 0, ly = 0, lz = 0;
        int list_n = 0;
        uint32_t n_acc = 0, n_mlp = 0, n_cells = 0, n_steps = 0;  // COUNTED only
        if (lane == 0) wcost[wi] = 0;
        NodeRec32 r{};
        NodeAux xa{};
        uint4 c0, c1;
        // Pops the next step's cells and issues their loads. Wide steps keep top <= cap -
        // LT_RESERVE; single-cell steps are a plain depth-first walk, which adds at most 7 entries
        // per tree level, so with cap = LT_CAP they stay below it. A step whose pushes could pass
        // cap (only with a smaller cap) is not taken: the walk stops with the stack bit.
        auto pop_and_load = [&]() -> int {
            __syncwarp();
            int nb = top > 0 ? min(min(LT_BATCH, top), max(1, (cap - LT_RESERVE - top) / 7)) : 0;
            if (nb > 0 && top + 7 * nb > cap) {  // unreachable for cap = LT_CAP; report, stop
                if (lane == 0) atomicOr(err_word, NB_DEVERR_STACK);
                nb = 0;
            }
            c0 = make_uint4(NB_NONE, NB_NONE, NB_NONE, NB_NONE);
            c1 = c0;
            if (lane < nb) {
                const uint32_t node = st[top - 1 - lane];
                r = rec[node];
                xa = aux[node];
                const uint4* cl = reinterpret_cast<const uint4*>(children + (size_t)node * 8);
                c0 = cl[0];
                c1 = cl[1];
            }
            __syncwarp();
            top -= nb;
            return nb;
        };
        int B = pop_and_load();
        while (B > 0) {
            const bool live = lane < B;
            if (COUNTED) {
                n_cells += (unsigned)B;
                ++n_steps;
            }
            float m2 = inf;
            if (live) {  // packed: two group bodies per f32x2 operation
                const nb_f2 cx2 = f2_pack(r.cx, r.cx), cy2 = f2_pack(r.cy, r.cy),
                            cz2 = f2_pack(r.cz, r.cz);
    #pragma unroll 8
                for (int j = 0; j < 16; ++j) {
                    const nb_f2 dx = f2_sub(gpx[wi][j], cx2), dy = f2_sub(gpy[wi][j], cy2),
                                dz = f2_sub(gpz[wi][j], cz2);
                    float d0, d1;
                    f2_unpack(f2_fma(dx, dx, f2_fma(dy, dy, f2_mul(dz, dz))), d0, d1);
                    m2 = fminf(m2, fminf(d0, d1));
                }
            }
            int cls = 1;
            uint4 fv = make_uint4(0u, 0u, 0u, 0u);  // the features as BF16 pairs
            if (live) {
                if (use_net) {
                    float f[NF];
                    cls = cell_features(r, xa, G, bs, m2, count_cap, f, bound_tau);
                    fv = make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]),
                                    pack_bf16(f[4], f[5]), pack_bf16(f[6], f[7]));
                } else {  // the theta rule needs the class only
                    cls = cell_class(r, xa, m2, count_cap);
                }
            }
            // the network's cells are packed into the first rows of the feature tile
            const unsigned net_mask = __ballot_sync(0xffffffffu, live && cls == 0);
            const int row = __popc(net_mask & ((1u << lane) - 1u));
            const int rows = __popc(net_mask);
            float score = 0.f;
            if (use_net && rows) {
                if (live && cls == 0) *reinterpret_cast<uint4*>(fm + row * 16) = fv;
                __syncwarp();
                const float v = rows > 16 ? mlp32(fm, lane, F) : mlp16(fm, lane, F);
                score = __shfl_sync(0xffffffffu, v, row & 31);
                __syncwarp();
            }
            if (COUNTED) n_mlp += rows;
            bool accept = false;
            if (live) {
                if (cls == 1 || cls == 4) accept = true;
                else if (cls == 0 && use_net) accept = score < log_tau_scaled;
                else if (cls != 2)  // group theta rule on the smallest distance
                    accept = m2 > 0.f && r.edge2 < theta2 * m2;
            }
            // body leaves and small opened cells: their bodies; other accepted cells: the monopole
            const bool body_leaf = live && cls == 1;
            const bool direct = body_leaf || (live && !accept && xa.count <= LT_DIRECT);
            const bool mono = live && accept && !body_leaf;
            const bool open = live && !accept && !direct;
            // push the children of opened cells (8-entry child lists, NB_NONE padded) and place the
            // step's list entries: one warp scan of both counts (each <= 8 per lane, so the packed
            // 16-bit halves cannot carry into each other)
            uint32_t nchild = 0;
            if (open) {
                const uint32_t v[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
    #pragma unroll
                for (int q = 0; q < 8; ++q) nchild += v[q] != NB_NONE;
            }
            const uint32_t d_first = xa.first, d_count = direct ? xa.count : 0u;
            const uint32_t slots = direct ? d_count : (mono ? 1u : 0u);
            uint32_t scan = nchild | (slots << 16);
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, scan, o);
                if (lane >= o) scan += v;
            }
            const uint32_t totals = __shfl_sync(0xffffffffu, scan, 31);
            {
                const uint32_t off = (scan & 0xffffu) - nchild;
                if (nchild) {
                    const uint32_t v[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
    #pragma unroll
                    for (int q = 0; q < 8; ++q)
                        if (q < (int)nchild) st[top + off + q] = v[q];
                }
                top += (int)(totals & 0xffffu);
            }
            // what the interaction list needs from this step, before the next step's loads land
            const float4 mono_e = make_float4((r.cx - ghx) - glx, (r.cy - ghy) - gly,
                                              (r.cz - ghz) - glz, r.gm);
            const uint32_t step_total = totals >> 16;
            const uint32_t pos = (scan >> 16) - slots;
            if (lane == 0) wcost[wi] += 2u * (uint32_t)B + step_total;
            B = pop_and_load();  // next step's cells are in flight during the list work below
            if (list_n + (int)step_total > LT_LIST) {  // make room: sum the list so far
                float fx, fy, fz;
                flush_list(ilist[wi], list_n, px, py, pz, eps2, fx, fy, fz);
                if (valid) {
                    two_sum_add(hx, lx, fx);
                    two_sum_add(hy, ly, fy);
                    two_sum_add(hz, lz, fz);
                }
                list_n = 0;
                __syncwarp();
            }
            // the step's entries: monopoles from their lanes' registers; the bodies of body leaves
            // and small opened cells loaded by the whole warp, one slot per lane and pass, so the
            // loads of all cells are in flight together
            float4* L = ilist[wi] + list_n;
            uint8_t* owner = slot_lane[wi];
            if (mono) {
                L[pos] = mono_e;
                owner[pos] = 0xffu;
            }
            for (uint32_t j = 0; j < d_count; ++j) owner[pos + j] = (uint8_t)lane;
            __syncwarp();
            for (uint32_t e0 = 0; e0 < step_total; e0 += 32) {  // warp-uniform trip count
                const uint32_t e = e0 + lane;
                const uint32_t o = e < step_total ? owner[e] : 0xffu;
                const int src = o == 0xffu ? 0 : (int)o;
                const uint32_t f = __shfl_sync(0xffffffffu, d_first, src);
                const uint32_t p0 = __shfl_sync(0xffffffffu, pos, src);
                if (o != 0xffu) {
                    const uint32_t b = f + (e - p0);
                    const float4 h = sorted4[b], l = sorted4lo[b];
                    L[e] = make_float4((h.x - ghx) + (l.x - glx), (h.y - ghy) + (l.y - gly),
                                       (h.z - ghz) + (l.z - glz), h.w);
                }
            }
            list_n += (int)step_total;
            if (COUNTED) n_acc += step_total;
            __syncwarp();
        }
        __syncwarp();
        float fx, fy, fz;
        flush_list(ilist[wi], list_n, px, py, pz, eps2, fx, fy, fz);
        if (valid) {
            ax[me] = ((double)hx + (double)lx) + (double)fx;
            ay[me] = ((double)hy + (double)ly) + (double)fy;
            az[me] = ((double)hz + (double)lz) + (double)fz;
        }
        if (lane == 0) {
            cost[gw] = wcost[wi];
            atomicAdd(cost_total, (unsigned long long)wcost[wi]);
        }
        const unsigned valid_lanes = __popc(__ballot_sync(0xffffffffu, valid));
        if (COUNTED) {
            t_acc += n_acc * (unsigned long long)valid_lanes;
            t_mlp += n_mlp;
            t_cells += n_cells;
            t_steps += n_steps;
        }
        __syncwarp();
    }
    if (COUNTED && lane == 0) {
        atomicAdd(&counters[0], t_acc);
        atomicAdd(&counters[1], t_mlp);
        atomicAdd(&counters[2], t_cells);
        atomicAdd(&counters[3], t_steps);
    }
}

// Schedule of the next learned traversal from this one's group costs: the groups costing at least
// twice the mean go to the priority list (taken first, so that the long walks do not end the
// launch alone) and are flagged in the skip mask; all others keep tree order, which keeps the walks
// of neighbouring groups together in the caches.
__global__ void sched_kernel(const uint32_t* __restrict__ cost, uint32_t n_groups,
                             uint32_t* __restrict__ sched, uint32_t* __restrict__ first,
                             uint32_t* __restrict__ skip) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const unsigned long long total = *reinterpret_cast<const unsigned long long*>(sched + 18);
    // cost >= 2 * total / n_groups, in integers
    const bool costly = g < n_groups && total > 0 &&
                        (unsigned long long)cost[g] * n_groups >= 2ull * total;
    const unsigned m = __ballot_sync(0xffffffffu, costly);
    if (lane == 0 && g < n_groups) skip[g >> 5] = m;
    if (m) {
        const int leader = __ffs(m) - 1;
        uint32_t at = 0;
        if (lane == leader) at = atomicAdd(&sched[1], (uint32_t)__popc(m));
        at = __shfl_sync(0xffffffffu, at, leader);
        if (costly) first[at + __popc(m & ((1u << lane) - 1u))] = g;
    }
    if (g == 0) sched[0] = n_groups;  // read by the next traversal, after this kernel
}

// ---------------------------------------------------------------------------------------------
// Label generation
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t hash32(uint32_t a) {
    a ^= a >> 16;
    a *= 0x7feb352dU;
    a ^= a >> 15;
    a *= 0x846ca68bU;
    a ^= a >> 16;
    return a;
}

// Group-rule walk with theta_gen; records sampled (group, cell) pairs of the network's class 0.
__global__ void __launch_bounds__(128)
pairs_collect_kernel(const NodeRec32* __restrict__ rec, const NodeAux* __restrict__ aux,
                     const uint32_t* __restrict__ info, const uint32_t* __restrict__ ids,
                     const double* __restrict__ x, const double* __restrict__ y,
                     const double* __restrict__ z, const double* __restrict__ ax,
                     const double* __restrict__ ay, const double* __restrict__ az,
                     const double* __restrict__ box, uint32_t n, float theta2, uint32_t count_cap,
                     uint32_t threshold, uint32_t seed, uint2* __restrict__ out,
                     uint32_t max_pairs, unsigned int* __restrict__ counter) {
    const int lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (gw * 32 >= n) return;
    const uint32_t p = gw * 32 + lane;
    const bool valid = p < n;
    const uint32_t me = valid ? ids[p] : NB_NONE;
    const double ox = box[0] + box[6] / 2, oy = box[1] + box[6] / 2, oz = box[2] + box[6] / 2;
    float px = 0, py = 0, pz = 0, a_prev = 0;
    if (valid) {
        px = (float)(x[me] - ox);
        py = (float)(y[me] - oy);
        pz = (float)(z[me] - oz);
        a_prev = (float)sqrt(ax[me] * ax[me] + ay[me] * ay[me] + az[me] * az[me]);
    }
    const GroupGeo G = group_geo(valid, px, py, pz, a_prev);
    const uint32_t nn = info[0];
    uint32_t k = 0;
    while (k < nn) {
        const NodeRec32 r = rec[k];
        if (r.body != NB_NONE) {
            k = r.skip;
            continue;
        }
        const NodeAux xa = aux[k];
        const float m2 = warp_min_dist2(valid, px, py, pz, r.cx, r.cy, r.cz);
        const int cls = cell_class(r, xa, m2, count_cap);
        if (cls == 0 && lane == 0 && hash32(k * 2654435761u ^ gw ^ seed) < threshold) {
            const unsigned int slot = atomicAdd(counter, 1u);
            if (slot < max_pairs) out[slot] = make_uint2(gw, k);
        }
        const bool open = cls == 2 || !(m2 > 0 && r.edge2 < theta2 * m2);
        k = open ? k + 1 : r.skip;
    }
}

// One warp per recorded pair: features, and the label from an exact direct sum over the cell.
__global__ void __launch_bounds__(128)
pairs_label_kernel(const NodeRec32* __restrict__ rec, const NodeRec64* __restrict__ rec64,
                   const NodeAux* __restrict__ aux, const uint32_t* __restrict__ ids,
                   const double* __restrict__ m, const double* __restrict__ x,
                   const double* __restrict__ y, const double* __restrict__ z,
                   const double* __restrict__ ax, const double* __restrict__ ay,
                   const double* __restrict__ az, const double* __restrict__ box, uint32_t n,
                   double G, float eps2, uint32_t count_cap, const uint2* __restrict__ pairs,
                   const unsigned int* __restrict__ counter, uint32_t max_pairs,
                   float* __restrict__ features, float* __restrict__ labels) {
    __shared__ float4 chunk[4][32];
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const uint32_t total = min(*counter, max_pairs);
    for (uint32_t q = blockIdx.x * 4 + wi; q < total; q += gridDim.x * 4) {
        const uint2 pr = pairs[q];
        const uint32_t p = pr.x * 32 + lane;
        const bool valid = p < n;
        const uint32_t me = valid ? ids[p] : NB_NONE;
        const double ox = box[0] + box[6] / 2, oy = box[1] + box[6] / 2, oz = box[2] + box[6] / 2;
        double bx = 0, by = 0, bz = 0;
        float px = 0, py = 0, pz = 0, a_b = 0;
        if (valid) {
            bx = x[me];
            by = y[me];
            bz = z[me];
            px = (float)(bx - ox);
            py = (float)(by - oy);
            pz = (float)(bz - oz);
            a_b = (float)sqrt(ax[me] * ax[me] + ay[me] * ay[me] + az[me] * az[me]);
        }
        const GroupGeo Gg = group_geo(valid, px, py, pz, a_b);
        const NodeRec32 r = rec[pr.y];
        const NodeAux xa = aux[pr.y];
        const float m2 = warp_min_dist2(valid, px, py, pz, r.cx, r.cy, r.cz);
        float f[NF];
        cell_features(r, xa, Gg, BoxScale(box[6]), m2, count_cap, f);
        // exact cell force on each lane's body; positions relative to the group's first valid
        // body in FP64 before rounding, so close pairs keep their digits
        const double gx = __shfl_sync(0xffffffffu, bx, 0), gy = __shfl_sync(0xffffffffu, by, 0),
                     gz = __shfl_sync(0xffffffffu, bz, 0);
        const float qx = (float)(bx - gx), qy = (float)(by - gy), qz = (float)(bz - gz);
        float fx = 0, fy = 0, fz = 0;
        for (uint32_t base = 0; base < xa.count; base += 32) {
            const uint32_t j = base + lane;
            if (j < xa.count) {
                const uint32_t b = ids[xa.first + j];
                chunk[wi][lane] = make_float4((float)(x[b] - gx), (float)(y[b] - gy),
                                              (float)(z[b] - gz), (float)(G * m[b]));
            }
            __syncwarp();
            const uint32_t cnt = min(32u, xa.count - base);
            float cxs = 0, cys = 0, czs = 0;
            for (uint32_t jj = 0; jj < cnt; ++jj) {
                const float4 s = chunk[wi][jj];
                const float dx = s.x - qx, dy = s.y - qy, dz = s.z - qz;
                const float inv = rsqrtf(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2))));
                const float w = s.w * inv * inv * inv;
                cxs = fmaf(dx, w, cxs);
                cys = fmaf(dy, w, cys);
                czs = fmaf(dz, w, czs);
            }
            fx += cxs;
            fy += cys;
            fz += czs;
            __syncwarp();
        }
        const NodeRec64 c = rec64[pr.y];
        const float mx = (float)(c.cx - gx) - qx, my = (float)(c.cy - gy) - qy,
                    mz = (float)(c.cz - gz) - qz;
        const float inv = rsqrtf(fmaf(mx, mx, fmaf(my, my, fmaf(mz, mz, eps2))));
        const float w = (float)(G * c.mass) * inv * inv * inv;
        const float ex = fx - mx * w, ey = fy - my * w, ez = fz - mz * w;
        float rel = valid ? sqrtf(ex * ex + ey * ey + ez * ez) / fmaxf(a_b, 1e-30f) : 0.f;
        rel = warp_max(rel);
        if (lane < NF) features[(size_t)q * NF + lane] = f[lane];
        if (lane == 0) labels[q] = fminf(fmaxf(__log10f(fmaxf(rel, 1e-30f)), -12.f), 2.f) * 0.2f;
    }
}

// ---------------------------------------------------------------------------------------------
// Training: FP32 forward / backward of the MLP (MSE loss), Adam
// ---------------------------------------------------------------------------------------------
constexpr int TR_BLOCK = 256;
constexpr int TR_CHUNK = 64;

__global__ void __launch_bounds__(TR_BLOCK)
mlp_grad_kernel(const float* __restrict__ P, const float* __restrict__ X,
                const float* __restrict__ Y, const uint32_t* __restrict__ idx, uint32_t n,
                float* __restrict__ grad, float* __restrict__ loss) {
    __shared__ float w[P_COUNT];
    __shared__ float sx[TR_CHUNK][NF], sh1[TR_CHUNK][32], sh2[TR_CHUNK][32];
    __shared__ float sd1[TR_CHUNK][32], sd2[TR_CHUNK][32], sdo[TR_CHUNK];
    for (int k = threadIdx.x; k < P_COUNT; k += TR_BLOCK) w[k] = P[k];
    float acc[6] = {0, 0, 0, 0, 0, 0};  // gradient entries threadIdx.x + i*TR_BLOCK
    float lsum = 0;
    const float inv_n = 1.0f / (float)n;
    const uint32_t per_block = (n + gridDim.x - 1) / gridDim.x;
    const uint32_t s0 = blockIdx.x * per_block, s1 = min(n, s0 + per_block);
    __syncthreads();
    for (uint32_t c0 = s0; c0 < s1; c0 += TR_CHUNK) {
        const uint32_t cnt = min((uint32_t)TR_CHUNK, s1 - c0);
        if (threadIdx.x < TR_CHUNK) {
            const int s = threadIdx.x;
            float xv[NF] = {0, 0, 0, 0, 0, 0, 0, 0}, h1[32], h2[32], d1[32], d2[32], dout = 0;
            if ((uint32_t)s < cnt) {
                const uint32_t row = idx ? idx[c0 + s] : c0 + s;
                for (int i = 0; i < NF; ++i) xv[i] = X[(size_t)row * NF + i];
                for (int o = 0; o < 32; ++o) {
                    float a = w[P_B1 + o];
                    for (int i = 0; i < NF; ++i) a = fmaf(xv[i], w[P_W1 + i * 32 + o], a);
                    h1[o] = fmaxf(a, 0.f);
                }
                float out = w[P_B3];
                for (int o = 0; o < 32; ++o) {
                    float a = w[P_B2 + o];
                    for (int i = 0; i < 32; ++i) a = fmaf(h1[i], w[P_W2 + i * 32 + o], a);
                    h2[o] = fmaxf(a, 0.f);
                    out = fmaf(h2[o], w[P_W3 + o], out);
                }
                const float e = out - Y[row];
                lsum += e * e;
                dout = 2.f * e * inv_n;
                for (int o = 0; o < 32; ++o) d2[o] = h2[o] > 0.f ? dout * w[P_W3 + o] : 0.f;
                for (int i = 0; i < 32; ++i) {
                    float a = 0;
                    for (int o = 0; o < 32; ++o) a = fmaf(d2[o], w[P_W2 + i * 32 + o], a);
                    d1[i] = h1[i] > 0.f ? a : 0.f;
                }
            } else {
                for (int o = 0; o < 32; ++o) h1[o] = h2[o] = d1[o] = d2[o] = 0.f;
            }
            for (int i = 0; i < NF; ++i) sx[s][i] = xv[i];
            for (int o = 0; o < 32; ++o) {
                sh1[s][o] = h1[o];
                sh2[s][o] = h2[o];
                sd1[s][o] = d1[o];
                sd2[s][o] = d2[o];
            }
            sdo[s] = dout;
        }
        __syncthreads();
        for (int i = 0; i < 6; ++i) {
            const int e = threadIdx.x + i * TR_BLOCK;
            if (e >= P_COUNT) break;
            float a = 0;
            if (e < P_B1) {  // W1[in][out]
                const int in = e / 32, o = e % 32;
                for (uint32_t s = 0; s < cnt; ++s) a = fmaf(sx[s][in], sd1[s][o], a);
            } else if (e < P_W2) {
                const int o = e - P_B1;
                for (uint32_t s = 0; s < cnt; ++s) a += sd1[s][o];
            } else if (e < P_B2) {
                const int in = (e - P_W2) / 32, o = (e - P_W2) % 32;
                for (uint32_t s = 0; s < cnt; ++s) a = fmaf(sh1[s][in], sd2[s][o], a);
            } else if (e < P_W3) {
                const int o = e - P_B2;
                for (uint32_t s = 0; s < cnt; ++s) a += sd2[s][o];
            } else if (e < P_B3) {
                const int in = e - P_W3;
                for (uint32_t s = 0; s < cnt; ++s) a = fmaf(sh2[s][in], sdo[s], a);
            } else {
                for (uint32_t s = 0; s < cnt; ++s) a += sdo[s];
            }
            acc[i] += a;
        }
        __syncthreads();
    }
    for (int i = 0; i < 6; ++i) {
        const int e = threadIdx.x + i * TR_BLOCK;
        if (e < P_COUNT) atomicAdd(&grad[e], acc[i]);
    }
    if (threadIdx.x < TR_CHUNK) atomicAdd(loss, lsum * inv_n);
}

__global__ void mlp_adam_kernel(float* __restrict__ P, float* __restrict__ M, float* __restrict__ V,
                                const float* __restrict__ grad, float lr, float b1, float b2,
                                float eps, float c1, float c2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P_COUNT) return;
    const float g = grad[k];
    const float m = b1 * M[k] + (1.f - b1) * g;
    const float v = b2 * V[k] + (1.f - b2) * g * g;
    M[k] = m;
    V[k] = v;
    P[k] -= lr * (m * c1) / (sqrtf(v * c2) + eps);
}

__global__ void mlp_predict_kernel(const float* __restrict__ P, const float* __restrict__ X,
                                   uint32_t n, float* __restrict__ out) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float xv[NF], h1[32];
    for (int i = 0; i < NF; ++i) xv[i] = X[(size_t)s * NF + i];
    for (int o = 0; o < 32; ++o) {
        float a = P[P_B1 + o];
        for (int i = 0; i < NF; ++i) a = fmaf(xv[i], P[P_W1 + i * 32 + o], a);
        h1[o] = fmaxf(a, 0.f);
    }
    float res = P[P_B3];
    for (int o = 0; o < 32; ++o) {
        float a = P[P_B2 + o];
        for (int i = 0; i < 32; ++i) a = fmaf(h1[i], P[P_W2 + i * 32 + o], a);
        res = fmaf(fmaxf(a, 0.f), P[P_W3 + o], res);
    }
    out[s] = res;
}

// BF16 tensor-core inference of the same network as the traversal runs it (weight fragments in
// shared memory, 32 rows per warp step through mlp32, a last step of at most 16 rows through
// mlp16), for validating both against the FP32 network.
__global__ void __launch_bounds__(128)
mlp_predict_bf16_kernel(const float* __restrict__ P, const float* __restrict__ X, uint32_t n,
                        float* __restrict__ out) {
    __shared__ __align__(16) __nv_bfloat16 feat[4][32][16];
    __shared__ __align__(16) uint32_t wsm[32 * MF_WS];
    __shared__ __align__(16) float bsm[32 * MF_BS];
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    if (wi == 0) load_frags(P, lane, wsm + lane * MF_WS, bsm + lane * MF_BS, 1);
    __syncthreads();
    const MlpFragsSmem F{wsm + lane * MF_WS, bsm + lane * MF_BS};
    __nv_bfloat16* fm = &feat[wi][0][0];
    for (uint32_t base = (blockIdx.x * 4 + wi) * 32; base < n; base += gridDim.x * 4 * 32) {
        for (int k = lane; k < 512; k += 32) {
            const uint32_t r = base + k / 16;
            const int c = k % 16;
            fm[k] = __float2bfloat16(c < NF && r < n ? X[(size_t)r * NF + c] : 0.f);
        }
        __syncwarp();
        const float v = n - base > 16 ? mlp32(fm, lane, F) : mlp16(fm, lane, F);
        if (base + lane < n && (n - base > 16 || lane < 16)) out[base + lane] = v;
        __syncwarp();
    }
}

}  // namespace

extern "C" {

nb_status nb_mlp_param_count(uint32_t* out) {
    if (!out) return nb::set_error(NB_ERR_INVALID_ARG, "null output");
    *out = P_COUNT;
    return NB_OK;
}

nb_status nb_mlp_loss_grad(nb_ctx* ctx, const float* params, const float* X, const float* Y,
                           const uint32_t* idx, uint32_t n, float* grad, float* loss,
                           nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (!params || !X || !Y || !grad || !loss || n == 0)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_mlp_loss_grad: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    NB_CUDA_TRY(cudaMemsetAsync(grad, 0, P_COUNT * sizeof(float), s));
    NB_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(float), s));
    int blocks = nb::ceil_div(n, TR_CHUNK * 4);
    if (blocks > ctx->sm_count * 2) blocks = ctx->sm_count * 2;
    mlp_grad_kernel<<<blocks, TR_BLOCK, 0, s>>>(params, X, Y, idx, n, grad, loss);
    return nb::check_launch("mlp_grad_kernel");
}

nb_status nb_mlp_adam(nb_ctx* ctx, float* params, float* m, float* v, const float* grad,
                      float lr, float beta1, float beta2, float eps, int step,
                      nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (!params || !m || !v || !grad || step < 1)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_mlp_adam: bad arguments");
    const float c1 = 1.f / (1.f - powf(beta1, (float)step));
    const float c2 = 1.f / (1.f - powf(beta2, (float)step));
    mlp_adam_kernel<<<nb::ceil_div(P_COUNT, 256), 256, 0, (cudaStream_t)stream>>>(
        params, m, v, grad, lr, beta1, beta2, eps, c1, c2);
    return nb::check_launch("mlp_adam_kernel");
}

nb_status nb_mlp_predict(nb_ctx* ctx, const float* params, const float* X, uint32_t n,
                         float* out, int bf16_tensor_cores, nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (!params || !X || !out) return nb::set_error(NB_ERR_INVALID_ARG, "nb_mlp_predict: null");
    if (n == 0) return NB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (bf16_tensor_cores) {
        int blocks = nb::ceil_div(n, 128);
        if (blocks > ctx->sm_count * 8) blocks = ctx->sm_count * 8;
        mlp_predict_bf16_kernel<<<blocks, 128, 0, s>>>(params, X, n, out);
        return nb::check_launch("mlp_predict_bf16_kernel");
    }
    mlp_predict_kernel<<<nb::ceil_div(n, 128), 128, 0, s>>>(params, X, n, out);
    return nb::check_launch("mlp_predict_kernel");
}

nb_status nb_bh_set_policy(nb_bh_tree* t, const float* params_dev, float log10_tau,
                           double theta_fallback, uint32_t count_cap, uint32_t flags) {
    if (!t) return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_set_policy: null tree");
    if (flags & ~(uint32_t)NB_POLICY_BOUND_ACCEPT)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_set_policy: unknown flags 0x%x", flags);
    t->policy_flags = flags;
    t->policy = params_dev;
    t->policy_set = true;
    t->policy_log_tau = log10_tau;
    t->policy_theta = (float)theta_fallback;
    t->policy_count_cap = count_cap;
    return NB_OK;
}

nb_status nb_bh_generate_pairs(nb_ctx* ctx, const nb_bh_tree* t, const double* m,
                               const double* x, const double* y, const double* z,
                               const double* ax, const double* ay, const double* az, double G,
                               double eps2, double theta_gen, double sample_fraction,
                               uint32_t seed, uint32_t count_cap, uint32_t max_pairs,
                               float* features, float* labels, uint32_t* count_dev,
                               uint32_t* pairs_out, nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (!t || !t->built) return nb::set_error(NB_ERR_NOT_BUILT, "nb_bh_generate_pairs: tree not built");
    NB_TRY(nb_need_records(t, NB_REC_FP64 | NB_REC_LEARNED, "nb_bh_generate_pairs"));
    if (!m || !x || !y || !z || !ax || !ay || !az || !features || !labels || !count_dev ||
        max_pairs == 0 || !(sample_fraction > 0) || sample_fraction > 1)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_generate_pairs: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    void* buf = nullptr;
    NB_TRY(nb::scratch(ctx, NB_SCRATCH_LABELS, (size_t)max_pairs * sizeof(uint2), &buf));
    NB_CUDA_TRY(cudaMemsetAsync(count_dev, 0, sizeof(uint32_t), s));
    const uint32_t warps = (t->n + 31) / 32;
    const uint32_t threshold = (uint32_t)(sample_fraction * 4294967295.0);
    pairs_collect_kernel<<<nb::ceil_div((long long)warps * 32, 128), 128, 0, s>>>(
        t->rec32, t->aux, t->info, t->ids, x, y, z, ax, ay, az, t->box, t->n,
        (float)(theta_gen * theta_gen), count_cap, threshold, seed, (uint2*)buf, max_pairs,
        (unsigned int*)count_dev);
    NB_TRY(nb::check_launch("pairs_collect_kernel"));
    pairs_label_kernel<<<ctx->sm_count * 8, 128, 0, s>>>(
        t->rec32, t->rec64, t->aux, t->ids, m, x, y, z, ax, ay, az, t->box, t->n, G, (float)eps2,
        count_cap, (const uint2*)buf, (const unsigned int*)count_dev, max_pairs, features, labels);
    NB_TRY(nb::check_launch("pairs_label_kernel"));
    if (pairs_out)
        NB_CUDA_TRY(cudaMemcpyAsync(pairs_out, buf, (size_t)max_pairs * sizeof(uint2),
                                    cudaMemcpyDeviceToDevice, s));
    return NB_OK;
}

}  // extern "C"

namespace nb {

// Resident blocks per SM of the learned traversal (queried once; also called before stream
// captures so that no query happens inside one).
nb_status learned_per_sm(int* out) {
    static int per_sm = 0;
    if (per_sm == 0) {
        NB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, bh_learned_kernel<false, true>, LT_THREADS, 0));
        if (per_sm < 1) per_sm = 1;
    }
    *out = per_sm;
    return NB_OK;
}

nb_status launch_learned(nb_ctx* ctx, const nb_bh_tree* t, const double* x, const double* y,
                         const double* z, double* ax, double* ay, double* az, double eps2,
                         unsigned long long* counters, cudaStream_t s) {
    if (!t->policy_set)
        return set_error(NB_ERR_INVALID_ARG, "nb_bh_accel: NB_OPEN_LEARNED needs nb_bh_set_policy");
    const uint32_t warps = (t->n + 31) / 32;
    int blocks = ceil_div(warps, LT_WARPS);
    int per_sm = 0;
    NB_TRY(learned_per_sm(&per_sm));
    if (blocks > ctx->sm_count * per_sm) blocks = ctx->sm_count * per_sm;
    // group counters (tree order, priority list) and the cost total; the schedule the previous
    // launch left in sched[0..1], first[] and skip[] stays for this one
    NB_CUDA_TRY(cudaMemsetAsync(t->work, 0, 3 * sizeof(uint32_t), s));
    NB_CUDA_TRY(cudaMemsetAsync(t->sched + 18, 0, sizeof(unsigned long long), s));
    const bool net = t->policy != nullptr;
    auto kernel = counters ? (net ? bh_learned_kernel<true, true> : bh_learned_kernel<true, false>)
                           : (net ? bh_learned_kernel<false, true> : bh_learned_kernel<false, false>);
    kernel<<<blocks, LT_THREADS, 0, s>>>(
        t->rec32, t->aux, t->children, t->sorted4, t->sorted4lo, t->n, t->policy,
        t->policy_log_tau * 0.2f,
        (t->policy_flags & NB_POLICY_BOUND_ACCEPT) ? exp10f(t->policy_log_tau) : 0.f,
        t->policy_theta * t->policy_theta, t->policy_count_cap,
        (float)eps2, t->ids, ax, ay, az, counters, ctx->dev_error, t->work,
        ctx->learned_stack_cap ? (int)ctx->learned_stack_cap : LT_CAP, t->box, t->group_first,
        t->group_skip, t->sched, t->group_cost,
        reinterpret_cast<unsigned long long*>(t->sched + 18));
    NB_TRY(check_launch("bh_learned_kernel"));
    NB_CUDA_TRY(cudaMemsetAsync(t->sched + 1, 0, sizeof(uint32_t), s));
    sched_kernel<<<ceil_div((int)warps, 256), 256, 0, s>>>(t->group_cost, warps, t->sched,
                                                           t->group_first, t->group_skip);
    return check_launch("sched_kernel");
}

}  // namespace nb
