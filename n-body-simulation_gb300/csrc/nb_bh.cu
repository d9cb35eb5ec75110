// nb_bh.cu -- Barnes-Hut octree build on the GPU (replaces BarnesHutOctree::buildOctree,
// ParallelOctreeTopDownSubtrees.cpp:15-93, and its AABB / centre-of-mass / sortBodies passes).
//
// Pipeline (all on one stream, no host round trip):
//  1. AABB with the reference's conventions (nb_integrate.cu).
//  2. keys: per body the octant digit of every level from the reference's FP64 recurrence
//     (mid = min + edge/2, strict compares, z below the midpoint selects bit 0; child min corner =
//     parent min + child edge), mapped to the visit rank so that ascending keys are the
//     reference's DFS pop order; read off a 52-bit fixed-point position wherever the body is
//     provably far enough from every midpoint for the recurrence's rounding not to matter.
//  3. stable LSD radix sort of (key, body id).
//  4. bodies whose first 21 digits collide get their next 21 digits and are re-sorted in place.
//  5. splits: adjacent sorted bodies share a prefix of L digits; the split belongs to the cell at
//     level L containing both. Its cell range comes from galloping searches over the keys; the
//     leftmost split of each cell ("first split") stands for the cell.
//  6. DFS numbering: each sorted position p starts popc(mask[p]) internal cells plus its leaf;
//     an exclusive scan gives every node its DFS pre-order index and skip link.
//  7. bottom-up centre of mass: leaves one thread each, cells by blocks over chunks of 4,096
//     sorted positions (deepest level first), the cells reaching past their chunk (at most one
//     per level) by tiers of blocks over 64 chunks each; children summed in octant order 0..7
//     (bit-identical to BarnesHutOctree.cpp:304-311), node records written with the sums.
#include <algorithm>

#include "nb_bh.cuh"
#include "nb_sort.cuh"

namespace nb {
nb_status launch_aabb(nb_ctx* ctx, const double* x, const double* y, const double* z, uint32_t n,
                      double* out_dev, cudaStream_t stream);
}

namespace {

constexpr int BH_THREADS = 256;
constexpr uint32_t RUN_LIMIT = 1u << 14;  // longest run of equal first key words we re-sort

// Order-preserving map of an FP64 value (no NaN, -0 already turned into +0) to uint64: the
// strict comparisons of the recurrence become integer comparisons (ALU instead of FP64 pipe).
__device__ __forceinline__ uint64_t ordered_bits(double v) {
    const uint64_t u = (uint64_t)__double_as_longlong(v);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// The edge halvings of the recurrence: exponent decrements while they stay exact (the normal,
// positive edges of <= 42 levels), otherwise (a zero or tiny box) FP64 divisions by 2.
struct Halving {
    double e;
    uint64_t e_bits;
    bool bits;
    __device__ explicit Halving(double edge) : e(edge) {
        e_bits = (uint64_t)__double_as_longlong(edge);
        bits = (e_bits >> 52) > 64 && (e_bits >> 52) < 0x7ff;
    }
    // edge / 2 of the next level
    __device__ double next() {
        if (bits) {
            e_bits -= 1ull << 52;
            return __longlong_as_double((long long)e_bits);
        }
        e = e / 2;
        return e;
    }
};

// Octant digits of levels [L0, last) appended to `key` for a body (ordered bits ox, oy, oz of
// its coordinates), from the cell mins entering level L0: the reference's FP64 recurrence
// (mid = min + edge/2 rounded as FP64, strict compares, child min = mid or min). Only the three
// midpoint additions per level run on the FP64 pipe: the compares are integer compares of
// order-preserving bit patterns (exact: a midpoint is never -0 since edge/2 > 0, and the body's
// -0 coordinates are taken as +0, which compares equal). Digits of levels below `first` are not
// appended.
__device__ uint64_t key_levels(Halving h, uint64_t ox, uint64_t oy, uint64_t oz, double mnx,
                               double mny, double mnz, int L0, int first, int last,
                               uint64_t key) {
    for (int L = L0; L < last; ++L) {
        const double ce = h.next();
        const double midx = __dadd_rn(mnx, ce);
        const double midy = __dadd_rn(mny, ce);
        const double midz = __dadd_rn(mnz, ce);
        const bool up = oy > ordered_bits(midy), rt = ox > ordered_bits(midx),
                   bk = oz < ordered_bits(midz);
        if (L >= first)
            key = (key << 3) |
                  nb_visit_of_octant((uint32_t)up * 4u + (uint32_t)rt * 2u + (uint32_t)bk);
        if (rt) mnx = midx;
        if (up) mny = midy;
        if (!bk) mnz = midz;
    }
    return key;
}

__device__ __forceinline__ uint64_t ordered_coord(double v) {
    return ordered_bits(v == 0.0 ? 0.0 : v);
}

// Octant digits of levels [word*21, word*21+21) for a body, from the root.
__device__ uint64_t key_word(const double* __restrict__ box, double px, double py, double pz,
                             int word) {
    const int first = word * NB_KEY_LEVELS;
    return key_levels(Halving(box[6]), ordered_coord(px), ordered_coord(py), ordered_coord(pz),
                      box[0], box[1], box[2], 0, first, first + NB_KEY_LEVELS, 0);
}

// Quantized keys (NB_BUILD_QUANTIZED_KEYS): every coordinate as a 42-bit fraction of the box,
// floor((v - min) * 2^42 / edge), one bit per level. Bodies fall into the cells of the
// reference's recurrence except within FP64 rounding of a cell midpoint (there the quantized
// rule puts them in the upper half). Bits interleave with the usual 3-way spread, the digits
// already in visit order: visit rank = 4 * (y upper) + 2 * (z lower) + (x lower).
__device__ __forceinline__ uint64_t spread3(uint64_t v) {  // bit i -> bit 3i, i < 21
    v &= 0x1fffffull;
    v = (v | v << 32) & 0x1f00000000ffffull;
    v = (v | v << 16) & 0x1f0000ff0000ffull;
    v = (v | v << 8) & 0x100f00f00f00f00full;
    v = (v | v << 4) & 0x10c30c30c30c30c3ull;
    v = (v | v << 2) & 0x1249249249249249ull;
    return v;
}

__device__ __forceinline__ uint64_t quantize42(double v, double mn, double scale) {
    const double q = (v - mn) * scale;
    const uint64_t top = (1ull << 42) - 1;
    if (!(q > 0.0)) return 0;
    const uint64_t u = __double2ull_rz(q);
    return u > top ? top : u;
}

__device__ uint64_t key_word_quantized(const double* __restrict__ box, double px, double py,
                                       double pz, int word) {
    const double scale = box[6] > 0.0 ? 4398046511104.0 / box[6] : 0.0;  // 2^42 / edge
    const uint64_t ix = quantize42(px, box[0], scale), iy = quantize42(py, box[1], scale),
                   iz = quantize42(pz, box[2], scale);
    const int shift = word == 0 ? NB_KEY_LEVELS : 0;
    const uint64_t m = 0x1fffffull;
    const uint64_t hx = (ix >> shift) & m, hy = (iy >> shift) & m, hz = (iz >> shift) & m;
    return (spread3(hy) << 2) | (spread3(~hz & m) << 1) | spread3(~hx & m);
}

__global__ void keys_quantized_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                      const double* __restrict__ z, uint32_t n,
                                      double* __restrict__ box, uint64_t* __restrict__ key0,
                                      uint32_t* __restrict__ ids) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 3) box[7 + i] = box[i] + box[6] / 2;  // box centre, for the node records
    if (i >= n) return;
    key0[i] = key_word_quantized(box, x[i], y[i], z[i], 0);
    ids[i] = i;
}

// First key word of every body, the digits of key_word bit for bit, mostly without the FP64
// recurrence. The recurrence's midpoints differ from the dyadic grid min + (2j + 1) edge /
// 2^(L+1) only by the rounding of its additions (the halvings are exact): after L + 1 of them by
// at most (L + 1) 2^-53 R, R = |min| + edge bounding every midpoint, i.e. (L + 1) R / (2 edge)
// units of edge / 2^52. A coordinate as a 52-bit fraction of the edge, U = floor((v - min) 2^52 /
// edge), is within 1.5 units of the exact value (three roundings), so when U is more than
// m = 10.5 R / edge + 4 units from every multiple of 2^31 (the grid boundaries of levels 0..20),
// the digits of those levels are bits 51..31 of U. Bodies inside a margin, and boxes whose edge
// the recurrence does not halve by exponent arithmetic, take the recurrence itself.
struct FixedGrid {
    double scale;  // 2^52 / edge
    long long margin[3];
    bool ok;
};

__device__ FixedGrid fixed_grid(const double* __restrict__ box) {
    FixedGrid g;
    const double e = box[6];
    const uint64_t eb = (uint64_t)__double_as_longlong(e);
    g.ok = (eb >> 52) > 64 && (eb >> 52) < 0x7ff;  // Halving's exponent mode: positive, normal
    g.scale = g.ok ? 4503599627370496.0 / e : 0.0;
    g.ok = g.ok && g.scale < 1e308;
#pragma unroll
    for (int a = 0; a < 3; ++a) {  // R / edge = |min| * scale / 2^52 + 1
        const double m = 10.5 * fma(fabs(box[a]), g.scale * 0x1p-52, 1.0) * (1.0 + 0x1p-30) + 4.0;
        g.ok = g.ok && m < 0x1p29;  // false for NaN as well
        g.margin[a] = g.ok ? (long long)m + 1 : 0;
    }
    return g;
}

// Bits 51..31 of U for one axis, or -1 when U lies within the margin of a grid boundary (or the
// coordinate is outside the box or NaN).
__device__ __forceinline__ long long fixed_digits(double v, double mn, double scale, long long m) {
    const double u = __dmul_rn(__dsub_rn(v, mn), scale);
    if (!(u >= 0.0 && u <= 4503599627370496.0)) return -1;
    const long long U = (long long)u;
    const long long hi = (U + m) >> 31, lo = (U - m - 1) >> 31;
    return hi == lo ? hi : -1;
}

__global__ void __launch_bounds__(BH_THREADS)
keys_kernel(const double* __restrict__ x, const double* __restrict__ y,
            const double* __restrict__ z, uint32_t n, double* __restrict__ box,
            uint64_t* __restrict__ key0, uint32_t* __restrict__ ids) {
    __shared__ FixedGrid grid_s;  // once per block: it takes an FP64 division
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 3) box[7 + i] = box[i] + box[6] / 2;  // box centre, for the node records
    if (threadIdx.x == 0) grid_s = fixed_grid(box);
    __syncthreads();
    if (i >= n) return;
    const FixedGrid g = grid_s;
    const double px = x[i], py = y[i], pz = z[i];
    long long hx = -1, hy = -1, hz = -1;
    if (g.ok) {
        hx = fixed_digits(px, box[0], g.scale, g.margin[0]);
        hy = fixed_digits(py, box[1], g.scale, g.margin[1]);
        hz = fixed_digits(pz, box[2], g.scale, g.margin[2]);
    }
    uint64_t key;
    if ((hx | hy | hz) >= 0) {  // visit rank = 4 (y upper) + 2 (z lower) + (x lower)
        const uint64_t m = 0x1fffffull;
        key = (spread3((uint64_t)hy) << 2) | (spread3(~(uint64_t)hz & m) << 1) |
              spread3(~(uint64_t)hx & m);
    } else {
        key = key_word(box, px, py, pz, 0);
    }
    key0[i] = key;
    ids[i] = i;
}

// Runs of equal first words: compute the second word and insertion-sort the run (stable).
__global__ void runs_fixup_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                  const double* __restrict__ z, uint32_t n,
                                  const double* __restrict__ box, const uint64_t* __restrict__ key0,
                                  uint64_t* __restrict__ key1, uint32_t* __restrict__ ids,
                                  uint32_t* __restrict__ err, int quantized) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p + 1 >= n) return;
    const uint64_t k = key0[p];
    if (key0[p + 1] != k) return;
    if (p > 0 && key0[p - 1] == k) return;
    uint32_t r = 2;
    while (p + r < n && key0[p + r] == k && r < RUN_LIMIT) ++r;
    if (p + r < n && key0[p + r] == k) {
        atomicOr(err, NB_DEVERR_DEPTH);
        return;
    }
    for (uint32_t q = p; q < p + r; ++q) {
        const uint32_t b = ids[q];
        key1[q] = quantized ? key_word_quantized(box, x[b], y[b], z[b], 1)
                            : key_word(box, x[b], y[b], z[b], 1);
    }
    for (uint32_t q = p + 1; q < p + r; ++q) {  // insertion sort, stable
        const uint64_t kk = key1[q];
        const uint32_t bb = ids[q];
        uint32_t s = q;
        while (s > p && key1[s - 1] > kk) {
            key1[s] = key1[s - 1];
            ids[s] = ids[s - 1];
            --s;
        }
        key1[s] = kk;
        ids[s] = bb;
    }
}

// Number of leading octal digits two sorted positions share (0 .. 42).
__device__ __forceinline__ int shared_digits(const uint64_t* __restrict__ key0,
                                             const uint64_t* __restrict__ key1, uint32_t p,
                                             uint32_t q) {
    const uint64_t a = key0[p], b = key0[q];
    if (a != b) return (__clzll((long long)(a ^ b)) - 1) / 3;
    const uint64_t c = key1[p], d = key1[q];
    if (c != d) return NB_KEY_LEVELS + (__clzll((long long)(c ^ d)) - 1) / 3;
    return 2 * NB_KEY_LEVELS;
}

__global__ void splits_kernel(const uint64_t* __restrict__ key0, const uint64_t* __restrict__ key1,
                              uint32_t n, uint8_t* __restrict__ split_level,
                              uint32_t* __restrict__ split_start, uint32_t* __restrict__ split_end,
                              unsigned long long* __restrict__ mask, uint32_t* __restrict__ err) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j + 1 >= n) return;
    int L = shared_digits(key0, key1, j, j + 1);
    if (L >= 2 * NB_KEY_LEVELS) {
        atomicOr(err, NB_DEVERR_DEPTH);
        L = 2 * NB_KEY_LEVELS - 1;
    }
    split_level[j] = (uint8_t)L;
    // leftmost a <= j with shared_digits(a, j) >= L (galloping, then bisection)
    long long good = j, bad = -1;
    for (long long step = 1;; step <<= 1) {
        const long long c = good - step;
        if (c < 0) break;
        if (shared_digits(key0, key1, (uint32_t)c, j) >= L) {
            good = c;
        } else {
            bad = c;
            break;
        }
    }
    while (good - bad > 1) {
        const long long mid = bad + (good - bad) / 2;
        if (shared_digits(key0, key1, (uint32_t)mid, j) >= L) good = mid; else bad = mid;
    }
    const uint32_t a = (uint32_t)good;
    split_start[j] = a;
    const bool first = (a == j) || shared_digits(key0, key1, a, j) > L;
    if (!first) {
        split_end[j] = NB_NONE;
        return;
    }
    // rightmost b >= j+1 with shared_digits(j, b) >= L
    long long g2 = j + 1, b2 = n;
    for (long long step = 1;; step <<= 1) {
        const long long c = g2 + step;
        if (c >= (long long)n) break;
        if (shared_digits(key0, key1, j, (uint32_t)c) >= L) {
            g2 = c;
        } else {
            b2 = c;
            break;
        }
    }
    while (b2 - g2 > 1) {
        const long long mid = g2 + (b2 - g2) / 2;
        if (shared_digits(key0, key1, j, (uint32_t)mid) >= L) g2 = mid; else b2 = mid;
    }
    split_end[j] = (uint32_t)g2;
    atomicOr(&mask[a], 1ull << L);
}

__global__ void count_kernel(const unsigned long long* __restrict__ mask, uint32_t n,
                             uint32_t* __restrict__ cnt) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) cnt[p] = __popcll(mask[p]) + 1;
}

__device__ __forceinline__ uint32_t node_index(const uint32_t* __restrict__ base,
                                               const unsigned long long* __restrict__ mask,
                                               uint32_t start, int level) {
    return base[start] + __popcll(mask[start] & ((1ull << level) - 1ull));
}

// Parent of the node covering sorted positions [a, b]: the cell at level max(dl, dr) holding the
// neighbouring split (dl = level of split a-1, dr = level of split b, -1 when absent).
__device__ __forceinline__ uint32_t parent_of(uint32_t a, uint32_t b, int dl, int dr,
                                              const uint8_t* __restrict__ split_level,
                                              const uint32_t* __restrict__ split_start,
                                              const uint32_t* __restrict__ base,
                                              const unsigned long long* __restrict__ mask) {
    if (dl < 0 && dr < 0) return NB_NONE;
    const uint32_t s = dl >= dr ? a - 1 : b;
    return node_index(base, mask, split_start[s], split_level[s]);
}

__device__ __forceinline__ uint32_t digit_at(const uint64_t* __restrict__ key0,
                                             const uint64_t* __restrict__ key1, uint32_t q, int L) {
    if (L < NB_KEY_LEVELS) return (uint32_t)(key0[q] >> (60 - 3 * L)) & 7u;
    return (uint32_t)(key1[q] >> (60 - 3 * (L - NB_KEY_LEVELS))) & 7u;
}

__global__ void emit_kernel(uint32_t n, const uint32_t* __restrict__ ids,
                            const uint8_t* __restrict__ split_level,
                            const uint32_t* __restrict__ split_start,
                            const uint32_t* __restrict__ split_end,
                            const unsigned long long* __restrict__ mask,
                            const uint32_t* __restrict__ base, uint8_t* __restrict__ node_level,
                            uint32_t* __restrict__ node_first, uint32_t* __restrict__ node_last,
                            uint32_t* __restrict__ node_skip, uint32_t* __restrict__ node_parent,
                            uint32_t* __restrict__ node_body,
                            uint32_t* __restrict__ info, const uint64_t* __restrict__ key0,
                            const uint64_t* __restrict__ key1, uint32_t* __restrict__ children) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    if (p == 0) info[0] = base[n];
    {  // leaf of the body at sorted position p
        const int dl = p > 0 ? (int)split_level[p - 1] : -1;
        const int dr = p + 1 < n ? (int)split_level[p] : -1;
        const uint32_t idx = base[p] + __popcll(mask[p]);
        node_level[idx] = (uint8_t)(max(dl, dr) + 1);
        node_first[idx] = p;
        node_last[idx] = p;
        node_skip[idx] = base[p + 1];
        node_body[idx] = ids[p];
        const uint32_t par = parent_of(p, p, dl, dr, split_level, split_start, base, mask);
        node_parent[idx] = par;
        if (par != NB_NONE) {
            // the parent's level is the deeper boundary split; slot = visit rank there
            children[(size_t)par * 8 + digit_at(key0, key1, p, max(dl, dr))] = idx;
        }
    }
    if (p + 1 < n && split_end[p] != NB_NONE) {  // internal cell whose first split is p
        const uint32_t a = split_start[p], b = split_end[p];
        const int L = split_level[p];
        const uint32_t idx = node_index(base, mask, a, L);
        node_level[idx] = (uint8_t)L;
        node_first[idx] = a;
        node_last[idx] = b;
        node_skip[idx] = base[b + 1];
        node_body[idx] = NB_NONE;
        const int dl = a > 0 ? (int)split_level[a - 1] : -1;
        const int dr = b + 1 < n ? (int)split_level[b] : -1;
        const uint32_t par = parent_of(a, b, dl, dr, split_level, split_start, base, mask);
        node_parent[idx] = par;
        if (par != NB_NONE) {
            children[(size_t)par * 8 + digit_at(key0, key1, a, max(dl, dr))] = idx;
        }
    }
}

struct ComArgs {
    uint32_t n;
    uint32_t* err;  // device error word

    uint32_t records;  // NB_REC_* sets to compute
    const double *m, *x, *y, *z;
    const double* box;
    double G;
    const uint64_t *key0, *key1;
    const uint32_t* ids;
    const unsigned long long* mask;
    const uint32_t* base;
    const uint8_t* node_level;
    const uint32_t *node_first, *node_last, *node_skip, *node_parent, *node_body;
    uint32_t* node_count;
    double *comx, *comy, *comz, *mass, *q;
    NodeRec64* rec64;
    NodeRec32* rec32;
    float4* rec32lo;
    float4* rec32lo2;
    NodeAux* aux;
    const uint32_t* node_first_pos;
    uint32_t* children;
    float4* sorted4;
    float4* sorted4lo;
};

// Edge of a cell of the given level: box edge * 2^-level by exponent arithmetic (exact, and no
// FP64 instructions) while the result stays a normal number, else ldexp.
__device__ __forceinline__ double cell_edge64(double box_edge, int level) {
    const long long bits = __double_as_longlong(box_edge);
    const int biased = (int)((bits >> 52) & 0x7ff);
    if (biased > level + 1 && biased < 0x7ff)
        return __longlong_as_double(bits - ((long long)level << 52));
    return ldexp(box_edge, -level);
}

// RN(c / m) for the rounded product c = RN(x * m) of a leaf (its centre-of-mass numerator over its
// mass): that quotient is x itself whenever |c / m - x| < ulp(x) / 2, and the difference is known
// exactly, since the rounding error x * m - c of a product is exact in one FMA. So
// |x * m - c| * 2^(53 - e(x)) < m (a power-of-two scaling, exact) decides it without a division;
// the IEEE division remains for the rest (x a power of two, zero, subnormal or extreme, or the
// quotient rounding to a neighbour of x).
__device__ __forceinline__ double leaf_quotient(double x, double m, double c) {
    const long long xb = __double_as_longlong(x);
    const int biased = (int)((xb >> 52) & 0x7ff);
    const int s = 1023 + 53 - (biased - 1023);  // biased exponent of 2^(53 - e(x))
    const bool pow2 = (xb & 0xfffffffffffffll) == 0;
    if (biased == 0 || biased == 0x7ff || pow2 || s < 1 || s > 2046 || !(m > 0.0))
        return __ddiv_rn(c, m);
    const double err = fma(x, m, -c);
    if (fabs(err) * __longlong_as_double((long long)s << 52) < m) return x;
    return __ddiv_rn(c, m);
}

__device__ void write_records(const ComArgs& A, uint32_t idx, double cx, double cy, double cz,
                              double sm, double qsum, uint32_t count, int level, uint32_t skip,
                              uint32_t body) {
    const double edge = cell_edge64(A.box[6], level);
    const double ox = A.box[7], oy = A.box[8], oz = A.box[9];  // box centre
    // centre = sums / mass: the IEEE quotients when the FP64 records are built (the reference's
    // values, also behind the FP32 pre-test's proven margin), else from one reciprocal (the FP32
    // records round it); massless cells get a finite centre (never used)
    double rcx = 0.0, rcy = 0.0, rcz = 0.0, inv = 0.0;
    if (sm != 0) {
        // 1/M from the hardware estimate and one Newton step (~2^-44: ample for the FP32
        // centres and the spread)
        asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(inv) : "d"(sm));
        inv = inv * fma(-sm, inv, 2.0);
        if (A.records & NB_REC_FP64) {
            rcx = __ddiv_rn(cx, sm);
            rcy = __ddiv_rn(cy, sm);
            rcz = __ddiv_rn(cz, sm);
        } else {
            rcx = cx * inv;
            rcy = cy * inv;
            rcz = cz * inv;
        }
    }
    if (A.records & NB_REC_FP64) {
        NodeRec64 r;
        r.cx = rcx;
        r.cy = rcy;
        r.cz = rcz;
        r.mass = sm;
        r.edge = edge;
        r.skip = skip;
        r.body = body;
        A.rec64[idx] = r;
    }
    NodeRec32 q;
    const double gx = rcx - ox, gy = rcy - oy, gz = rcz - oz;
    if (sm != 0) {
        q.cx = (float)gx;
        q.cy = (float)gy;
        q.cz = (float)gz;
    } else {  // massless cell: far away, contributes exactly 0
        q.cx = q.cy = q.cz = 1e30f;
    }
    q.gm = (float)(A.G * sm);
    q.edge2 = (float)(edge * edge);
    q.skip = skip;
    q.body = body;
    q.level = (uint32_t)level;
    A.rec32[idx] = q;
    if (A.records & NB_REC_DF) {
        // further FP32 terms: the centre minus the box centre, exactly, as a triple-float (rec32,
        // rec32lo, rec32lo2 .xyz) and G*mass as a double-float (rec32.gm, rec32lo.w)
        float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), lo2 = lo;
        if (sm != 0) {
            float hx, hy, hz;  // equal to q.cx, q.cy, q.cz (both round the same FP64 difference)
            tf_split_diff(rcx, ox, hx, lo.x, lo2.x);
            tf_split_diff(rcy, oy, hy, lo.y, lo2.y);
            tf_split_diff(rcz, oz, hz, lo.z, lo2.z);
            lo.w = (float)(A.G * sm - (double)q.gm);
        }
        A.rec32lo[idx] = lo;
        A.rec32lo2[idx] = lo2;
    }
    if (A.records & NB_REC_LEARNED) {
        // spread^2 = sum m |x-o|^2 / M - |c-o|^2 (o = box centre, which keeps both terms small);
        // the spread is a feature of the learned policy, not a sum of the reference: 1/M from the
        // reciprocal, the root in FP32
        NodeAux x;
        x.spread_rel = 0.f;
        x.lg_gm = __log2f(fmaxf(q.gm, 1e-37f));
        if (sm != 0) {
            const double s2 = qsum * inv - (gx * gx + gy * gy + gz * gz);
            const float e = (float)edge;
            if (e > 0.f) x.spread_rel = sqrtf((float)(s2 > 0 ? s2 : 0.0)) / e;
        }
        x.count = count;
        x.first = A.node_first_pos[idx];
        A.aux[idx] = x;
    }
}

// Sums of internal node `idx` from its children (the reference's octant order 0..7, FP64 adds:
// bit-identical to BarnesHutOctree.cpp:304-311), its records, and its child list rewritten as the
// compacted visit-order list the learned traversal reads (emit_kernel wrote it by visit rank).
// c0, c1: the cell's child list as emit_kernel wrote it (loaded by the caller, possibly earlier).
__device__ void sum_children(const ComArgs& A, uint32_t idx, bool records, uint4 c0, uint4 c1) {
    uint4* cl = reinterpret_cast<uint4*>(A.children + (size_t)idx * 8);
    const uint32_t vs[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
    const bool learned = (A.records & NB_REC_LEARNED) != 0;
    // every child's sums requested before the first is used (one round trip, not eight)
    double cx[8], cy[8], cz[8], cm[8], cq[8];
    uint32_t cc[8];
#pragma unroll
    for (int o = 0; o < 8; ++o) {  // the reference's octant order 0..7
        const uint32_t ch = vs[nb_visit_of_octant(o)];
        cx[o] = cy[o] = cz[o] = cm[o] = cq[o] = 0.0;
        cc[o] = 0;
        if (ch != NB_NONE) {
            cx[o] = __ldcg(&A.comx[ch]);
            cy[o] = __ldcg(&A.comy[ch]);
            cz[o] = __ldcg(&A.comz[ch]);
            cm[o] = __ldcg(&A.mass[ch]);
            if (learned) cq[o] = __ldcg(&A.q[ch]);
            cc[o] = __ldcg(&A.node_count[ch]);
        }
    }
    // the compacted visit-order child list the learned traversal reads
    uint32_t list[8];
    int nch = 0;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        list[t] = NB_NONE;
        if (vs[t] != NB_NONE) list[nch++] = vs[t];
    }
    cl[0] = make_uint4(list[0], list[1], list[2], list[3]);
    cl[1] = make_uint4(list[4], list[5], list[6], list[7]);
    double sx = 0, sy = 0, sz = 0, sm = 0, sq = 0;
    uint32_t count = 0;
#pragma unroll
    for (int o = 0; o < 8; ++o) {
        if (vs[nb_visit_of_octant(o)] == NB_NONE) continue;  // absent children add nothing
        sx = __dadd_rn(sx, cx[o]);
        sy = __dadd_rn(sy, cy[o]);
        sz = __dadd_rn(sz, cz[o]);
        sm = __dadd_rn(sm, cm[o]);
        if (learned) sq += cq[o];
        count += cc[o];
    }
    A.comx[idx] = sx;
    A.comy[idx] = sy;
    A.comz[idx] = sz;
    A.mass[idx] = sm;
    if (learned) A.q[idx] = sq;
    A.node_count[idx] = count;
    if (records)
        write_records(A, idx, sx, sy, sz, sm, sq, count, A.node_level[idx], A.node_skip[idx],
                      NB_NONE);
}

// Records of internal node `idx` from its final sums (written earlier by sum_children).
__device__ void cell_records(const ComArgs& A, uint32_t idx) {
    const bool learned = (A.records & NB_REC_LEARNED) != 0;
    write_records(A, idx, __ldcg(&A.comx[idx]), __ldcg(&A.comy[idx]), __ldcg(&A.comz[idx]),
                  __ldcg(&A.mass[idx]), learned ? __ldcg(&A.q[idx]) : 0.0,
                  __ldcg(&A.node_count[idx]), A.node_level[idx], A.node_skip[idx], NB_NONE);
}

// Sums and records of the leaf `idx` (body b at sorted position p). A leaf's centre of mass is
// its body: the FP64 records keep the reference's quotient (c / m, mostly decided without a
// division by leaf_quotient), the FP32 records take the body position itself (within their own
// rounding of that quotient), and the spread of a single body is 0.
__device__ void leaf_sums(const ComArgs& A, uint32_t idx, uint32_t p, uint32_t b) {
    const double mb = A.m[b];
    const double bx = A.x[b], by = A.y[b], bz = A.z[b];
    const double cx = __dmul_rn(bx, mb), cy = __dmul_rn(by, mb), cz = __dmul_rn(bz, mb);
    A.comx[idx] = cx;
    A.comy[idx] = cy;
    A.comz[idx] = cz;
    A.mass[idx] = mb;
    A.node_count[idx] = 1;
    const int level = A.node_level[idx];
    const uint32_t skip = A.node_skip[idx];
    const double edge = cell_edge64(A.box[6], level);
    const double ox = A.box[7], oy = A.box[8], oz = A.box[9];
    const bool fp64 = (A.records & NB_REC_FP64) != 0;
    double rcx = bx, rcy = by, rcz = bz;
    if (fp64 && mb != 0) {
        rcx = leaf_quotient(bx, mb, cx);
        rcy = leaf_quotient(by, mb, cy);
        rcz = leaf_quotient(bz, mb, cz);
    }
    if (fp64) {
        NodeRec64 r;
        r.cx = mb != 0 ? rcx : 0.0;
        r.cy = mb != 0 ? rcy : 0.0;
        r.cz = mb != 0 ? rcz : 0.0;
        r.mass = mb;
        r.edge = edge;
        r.skip = skip;
        r.body = b;
        A.rec64[idx] = r;
    }
    const double gx = rcx - ox, gy = rcy - oy, gz = rcz - oz;
    NodeRec32 q;
    q.cx = mb != 0 ? (float)gx : 1e30f;  // a massless body: far away, contributes exactly 0
    q.cy = mb != 0 ? (float)gy : 1e30f;
    q.cz = mb != 0 ? (float)gz : 1e30f;
    q.gm = (float)(A.G * mb);
    q.edge2 = (float)(edge * edge);
    q.skip = skip;
    q.body = b;
    q.level = (uint32_t)level;
    A.rec32[idx] = q;
    if (A.records & NB_REC_DF) {
        float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), lo2 = lo;
        if (mb != 0) {
            float hx, hy, hz;
            tf_split_diff(rcx, ox, hx, lo.x, lo2.x);
            tf_split_diff(rcy, oy, hy, lo.y, lo2.y);
            tf_split_diff(rcz, oz, hz, lo.z, lo2.z);
            lo.w = (float)(A.G * mb - (double)q.gm);
        }
        A.rec32lo[idx] = lo;
        A.rec32lo2[idx] = lo2;
    }
    if (A.records & NB_REC_LEARNED) {  // spread sums and the FP32 body copies of the policy
        const double rx = bx - ox, ry = by - oy, rz = bz - oz;
        A.q[idx] = mb * (rx * rx + ry * ry + rz * rz);
        const float hx = (float)rx, hy = (float)ry, hz = (float)rz;
        A.sorted4[p] = make_float4(hx, hy, hz, q.gm);
        A.sorted4lo[p] = make_float4((float)(rx - (double)hx), (float)(ry - (double)hy),
                                     (float)(rz - (double)hz), 0.f);
        NodeAux x;
        x.spread_rel = 0.f;
        x.count = 1;
        x.first = p;
        x.lg_gm = __log2f(fmaxf(q.gm, 1e-37f));
        A.aux[idx] = x;
    }
}

// Centre of mass and records, bottom-up, in chunks of CW consecutive sorted positions. The nodes
// starting in a chunk are the DFS indices [base[P], base[P + CW]); the ones that also end in it
// ("local": all leaves and most cells) are summed by the chunk's block. A cell that starts in a
// chunk and reaches past its end holds the chunk's last body and the next one, so there is at
// most one such cell per level: each chunk lists them (<= CM_LEVELS) for the next tier, whose
// blocks cover CM_FAN chunks each and sum the listed cells that end inside their span, passing
// the rest up again, until one block spans all bodies. Every sum has its children's sums final
// before it starts (kernel order, then levels deepest first within a block), so no thread waits
// on another, and the FP64 work is spread over all SMs at every tier.
//  * com_leaf_kernel: one thread per sorted position sums its leaf and writes its records;
//  * com_cells_kernel: one block per chunk sums the chunk's local cells level by level, then
//    writes their records in one sweep over the compacted cell list (FP64 work with full warps:
//    on this part an FP64 warp instruction costs the FP64 pipe the same time however few of its
//    lanes are active);
//  * com_tier_kernel: one block per span of CM_FAN lower-tier chunks, same scheme on the listed
//    cells.
constexpr int CW = 4096;                          // sorted positions per chunk
constexpr int CM_LEVELS = 2 * NB_KEY_LEVELS + 1;  // node levels 0..42
constexpr int CM_FAN = 64;                        // lower-tier chunks per upper-tier chunk
constexpr int CM_TIER_MAX = CM_LEVELS * CM_FAN;   // listed cells one upper-tier block reads
constexpr int CM_TIERS = 5;                       // 2048 * 64^4 > 2^27 bodies
constexpr int CC_THREADS = 256;                   // threads per block of the cell kernels
constexpr int CC_BATCH = 4;  // node-table entries each thread loads together in the scan

__global__ void __launch_bounds__(256, 5) com_leaf_kernel(ComArgs A) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= A.n) return;
    leaf_sums(A, A.base[p] + __popcll(A.mask[p]), p, A.ids[p]);
}

// Sums the `nf` cells found[k] (level flev[k]) level by level, deepest first, then writes their
// records. Block-wide; smem arrays given by the caller.
__device__ void sum_by_level(const ComArgs& A, const uint32_t* found, const uint8_t* flev,
                             uint32_t nf, uint32_t* nodes, uint32_t* cnt, uint32_t* off,
                             uint32_t* fill) {
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int l = 0; l < CM_LEVELS; ++l) {
            off[l] = run;
            run += cnt[l];
        }
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < nf; k += blockDim.x) {
        const uint32_t l = flev[k];
        nodes[off[l] + atomicAdd(&fill[l], 1u)] = found[k];
    }
    __syncthreads();
    // deepest level first; each thread's first cell of the next level has its child list loaded
    // before the barrier (a list only changes when its own cell is summed), so a level costs one
    // round trip to the children's sums instead of two
    const uint4 none4 = make_uint4(NB_NONE, NB_NONE, NB_NONE, NB_NONE);
    auto list_of = [&](uint32_t idx, uint4& c0, uint4& c1) {
        const uint4* cl = reinterpret_cast<const uint4*>(A.children + (size_t)idx * 8);
        c0 = __ldcg(cl);
        c1 = __ldcg(cl + 1);
    };
    int l = CM_LEVELS - 1;
    while (l >= 0 && cnt[l] == 0) --l;  // uniform across the block
    uint4 p0 = none4, p1 = none4;
    if (l >= 0 && threadIdx.x < cnt[l]) list_of(nodes[off[l] + threadIdx.x], p0, p1);
    while (l >= 0) {
        const uint32_t c = cnt[l];
        int next = l - 1;
        while (next >= 0 && cnt[next] == 0) --next;
        for (uint32_t k = threadIdx.x; k < c; k += blockDim.x) {
            const uint32_t idx = nodes[off[l] + k];
            uint4 c0 = p0, c1 = p1;
            if (k != threadIdx.x) list_of(idx, c0, c1);
            sum_children(A, idx, false, c0, c1);
        }
        if (next >= 0 && threadIdx.x < cnt[next]) list_of(nodes[off[next] + threadIdx.x], p0, p1);
        __syncthreads();
        l = next;
    }
    for (uint32_t k = threadIdx.x; k < nf; k += blockDim.x) cell_records(A, nodes[k]);
}

__global__ void __launch_bounds__(CC_THREADS) com_cells_kernel(ComArgs A, uint2* up,
                                                               uint32_t* up_count) {
    __shared__ uint32_t found[CW];  // the chunk's local cells as found
    __shared__ uint8_t flev[CW];    // and their levels
    __shared__ uint32_t nodes[CW];  // the same cells, grouped by level
    __shared__ uint32_t cnt[CM_LEVELS], off[CM_LEVELS], fill[CM_LEVELS];
    __shared__ uint32_t n_found, n_up;
    const uint32_t P = blockIdx.x * CW;
    if (P >= A.n) return;
    const uint32_t Pend = min(P + (uint32_t)CW, A.n);
    const uint32_t d0 = A.base[P], d1 = A.base[Pend];
    for (int l = threadIdx.x; l < CM_LEVELS; l += CC_THREADS) cnt[l] = fill[l] = 0;
    if (threadIdx.x == 0) n_found = n_up = 0;
    __syncthreads();
    // one scan of the chunk's node range, CC_BATCH entries per thread in flight together
    for (uint32_t i0 = d0 + threadIdx.x; i0 < d1; i0 += CC_THREADS * CC_BATCH) {
        uint32_t body[CC_BATCH], last[CC_BATCH];
        uint8_t lvl[CC_BATCH];
#pragma unroll
        for (int k = 0; k < CC_BATCH; ++k) {
            const uint32_t idx = i0 + k * CC_THREADS;
            body[k] = idx < d1 ? A.node_body[idx] : 0u;
            last[k] = idx < d1 ? A.node_last[idx] : 0u;
            lvl[k] = idx < d1 ? A.node_level[idx] : 0;
        }
#pragma unroll
        for (int k = 0; k < CC_BATCH; ++k) {
            const uint32_t idx = i0 + k * CC_THREADS;
            if (idx >= d1 || body[k] != NB_NONE) continue;  // past the range, or a leaf
            const int l = min((int)lvl[k], CM_LEVELS - 1);
            if (last[k] >= Pend) {  // reaches past the chunk: for the next tier
                const uint32_t g = atomicAdd(&n_up, 1u);
                if (g < (uint32_t)CM_LEVELS)
                    up[(size_t)blockIdx.x * CM_LEVELS + g] = make_uint2(idx, (uint32_t)l);
                else
                    atomicOr(A.err, NB_DEVERR_DEPTH);  // more than one per level: inconsistent
                continue;
            }
            atomicAdd(&cnt[l], 1u);
            const uint32_t slot = atomicAdd(&n_found, 1u);
            if (slot < (uint32_t)CW) {
                found[slot] = idx;
                flev[slot] = (uint8_t)l;
            } else {
                atomicOr(A.err, NB_DEVERR_DEPTH);  // a consistent tree never gets here
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) up_count[blockIdx.x] = min(n_up, (uint32_t)CM_LEVELS);
    // more local cells than a chunk's bodies allow: only an inconsistent tree (error bit set);
    // stop here, before any index beyond what the scan recorded is used
    if (n_found > (uint32_t)CW) return;
    sum_by_level(A, found, flev, n_found, nodes, cnt, off, fill);
}

// Tier of `span` sorted positions per block (span = CW * CM_FAN^t): the cells listed by the
// CM_FAN lower-tier chunks of the span (in[c * CM_LEVELS + k], k < in_count[c]) that end inside
// it are summed here; the others go to up[] for the next tier (up == nullptr: the last tier,
// whose single block spans all bodies).
__global__ void __launch_bounds__(CC_THREADS)
com_tier_kernel(ComArgs A, uint32_t span, const uint2* __restrict__ in,
                const uint32_t* __restrict__ in_count, uint32_t in_chunks, uint2* up,
                uint32_t* up_count) {
    __shared__ uint32_t found[CM_TIER_MAX];
    __shared__ uint8_t flev[CM_TIER_MAX];
    __shared__ uint32_t nodes[CM_TIER_MAX];
    __shared__ uint32_t cnt[CM_LEVELS], off[CM_LEVELS], fill[CM_LEVELS];
    __shared__ uint32_t n_found, n_up;
    const uint32_t P = blockIdx.x * span;
    if (P >= A.n) return;
    const uint32_t Pend = (uint32_t)min((uint64_t)P + span, (uint64_t)A.n);
    for (int l = threadIdx.x; l < CM_LEVELS; l += CC_THREADS) cnt[l] = fill[l] = 0;
    if (threadIdx.x == 0) n_found = n_up = 0;
    __syncthreads();
    const uint32_t c0 = blockIdx.x * CM_FAN, c1 = min(c0 + (uint32_t)CM_FAN, in_chunks);
    for (uint32_t e = threadIdx.x; e < (c1 - c0) * CM_LEVELS; e += CC_THREADS) {
        const uint32_t c = c0 + e / CM_LEVELS, k = e % CM_LEVELS;
        if (k >= in_count[c]) continue;
        const uint2 g = in[(size_t)c * CM_LEVELS + k];
        if (up != nullptr && A.node_last[g.x] >= Pend) {
            const uint32_t u = atomicAdd(&n_up, 1u);
            if (u < (uint32_t)CM_LEVELS) up[(size_t)blockIdx.x * CM_LEVELS + u] = g;
            else atomicOr(A.err, NB_DEVERR_DEPTH);
            continue;
        }
        atomicAdd(&cnt[g.y], 1u);
        const uint32_t slot = atomicAdd(&n_found, 1u);
        if (slot < (uint32_t)CM_TIER_MAX) {
            found[slot] = g.x;
            flev[slot] = (uint8_t)g.y;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && up_count != nullptr) up_count[blockIdx.x] = min(n_up, (uint32_t)CM_LEVELS);
    if (n_found > (uint32_t)CM_TIER_MAX) return;  // cannot happen: <= CM_LEVELS per chunk
    sum_by_level(A, found, flev, n_found, nodes, cnt, off, fill);
}

// ---------------------------------------------------------------------------------------------
// allocation
// ---------------------------------------------------------------------------------------------
struct Carver {
    char* base = nullptr;
    size_t off = 0;
    template <typename T>
    T* take(size_t count) {
        off = (off + 255) & ~(size_t)255;
        T* p = (T*)(base + off);
        off += count * sizeof(T);
        return p;
    }
};

void carve(nb_bh_tree* t, Carver& c) {
    const size_t n = t->n_max, cap = t->node_cap;
    t->box = c.take<double>(16);
    t->info = c.take<uint32_t>(16);
    t->work = c.take<uint32_t>(16);
    t->sched = c.take<uint32_t>(32);
    t->group_cost = c.take<uint32_t>(n / 32 + 1);
    t->group_first = c.take<uint32_t>(n / 32 + 1);
    t->group_skip = c.take<uint32_t>(n / 1024 + 1);
    t->walk_len = c.take<uint32_t>(n);
    t->walk_ids = c.take<uint32_t>(n);
    t->key0 = c.take<uint64_t>(n);
    t->key1 = c.take<uint64_t>(n);
    t->key_alt = c.take<uint64_t>(n);
    t->ids = c.take<uint32_t>(n);
    t->ids_alt = c.take<uint32_t>(n);
    t->split_level = c.take<uint8_t>(n);
    t->split_start = c.take<uint32_t>(n);
    t->split_end = c.take<uint32_t>(n);
    t->mask = c.take<uint64_t>(n);
    t->cnt = c.take<uint32_t>(n + 1);
    t->base = c.take<uint32_t>(n + 1);
    t->sort_temp = c.take<char>(nb::radix_temp_bytes((uint32_t)n));
    t->scan_temp = c.take<uint32_t>(nb::scan_temp_bytes((uint32_t)n + 1) / 4 + 16);
    t->node_level = c.take<uint8_t>(cap);
    t->node_first = c.take<uint32_t>(cap);
    t->node_last = c.take<uint32_t>(cap);
    t->node_skip = c.take<uint32_t>(cap);
    t->node_parent = c.take<uint32_t>(cap);
    t->node_body = c.take<uint32_t>(cap);
    t->node_count = c.take<uint32_t>(cap);
    t->node_comx = c.take<double>(cap);
    t->node_comy = c.take<double>(cap);
    t->node_comz = c.take<double>(cap);
    t->node_mass = c.take<double>(cap);
    t->rec64 = c.take<NodeRec64>(cap);
    t->rec32 = c.take<NodeRec32>(cap);
    t->rec32lo = c.take<float4>(cap);
    t->rec32lo2 = c.take<float4>(cap);
    t->node_q = c.take<double>(cap);
    t->aux = c.take<NodeAux>(cap);
    t->children = c.take<uint32_t>(cap * 8);
    t->sorted4 = c.take<float4>(n);
    t->sorted4lo = c.take<float4>(n);
    // per tier, CM_LEVELS listed cells and a count per chunk (two lists, used in turn)
    const size_t chunks = (n + CW - 1) / CW;
    for (int k = 0; k < 2; ++k) {
        t->tier_cells[k] = c.take<uint2>(chunks * CM_LEVELS);
        t->tier_count[k] = c.take<uint32_t>(chunks);
    }
}

}  // namespace

extern "C" {

nb_status nb_bh_params_default(nb_bh_params* out) {
    if (!out) return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_params_default: null pointer");
    out->theta = 1.05;  // Configuration.cpp:18
    out->storage_size_param = 16;
    out->stack_size_param = 16;
    out->max_build_level = 7;
    out->sort_bodies = 1;
    return NB_OK;
}

nb_status nb_bh_tree_create(nb_ctx* ctx, uint32_t n_max, const nb_bh_params* params,
                            nb_bh_tree** out) {
    NB_CHECK_CTX(ctx);
    if (!out) return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_tree_create: null output");
    if (n_max == 0 || n_max > (1u << 27))
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_tree_create: n_max = %u out of range", n_max);
    nb_bh_tree* t = new nb_bh_tree();
    t->n_max = n_max;
    t->node_cap = 2 * n_max;
    t->device = ctx->device;
    if (params) {
        t->params = *params;
    } else {
        nb_bh_params_default(&t->params);
    }
    NB_TRY(nb::radix_prepare());  // before any capture of a build
    Carver sizing;
    carve(t, sizing);
    void* mem = nullptr;
    cudaError_t e = cudaMalloc(&mem, sizing.off + 256);
    if (e != cudaSuccess) {
        delete t;
        return nb::cuda_error(e, "nb_bh_tree_create");
    }
    Carver real;
    real.base = (char*)mem;
    carve(t, real);
    e = cudaMemset(t->sched, 0, 32 * sizeof(uint32_t));  // no group order yet
    if (e != cudaSuccess) {
        cudaFree(mem);
        delete t;
        return nb::cuda_error(e, "nb_bh_tree_create");
    }
    // the carve order puts box first: its address is the allocation base (freed in destroy)
    *out = t;
    return NB_OK;
}

nb_status nb_bh_tree_destroy(nb_bh_tree* t) {
    if (!t) return NB_OK;
    if (t->phase_timing)
        for (auto& e : t->phase_ev) cudaEventDestroy(e);
    if (t->box) cudaFree(t->box);
    delete t;
    return NB_OK;
}

nb_status nb_bh_set_phase_timing(nb_bh_tree* t, int enable) {
    if (!t) return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_set_phase_timing: null tree");
    NB_CUDA_TRY(cudaSetDevice(t->device));
    if (enable && !t->phase_timing) {
        for (auto& e : t->phase_ev) NB_CUDA_TRY(cudaEventCreate(&e));
    } else if (!enable && t->phase_timing) {
        for (auto& e : t->phase_ev) {
            cudaEventDestroy(e);
            e = nullptr;
        }
    }
    t->phase_timing = enable != 0;
    return NB_OK;
}

nb_status nb_bh_build_phase_ms(nb_bh_tree* t, float* ms) {
    if (!t || !ms) return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_build_phase_ms: null argument");
    if (!t->phase_timing)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_build_phase_ms: phase timing is off");
    if (!t->built) return nb::set_error(NB_ERR_NOT_BUILT, "nb_bh_build_phase_ms: tree not built");
    NB_CUDA_TRY(cudaEventSynchronize(t->phase_ev[5]));
    for (int k = 0; k < 5; ++k)
        NB_CUDA_TRY(cudaEventElapsedTime(&ms[k], t->phase_ev[k], t->phase_ev[k + 1]));
    return NB_OK;
}

nb_status nb_bh_tree_set_theta(nb_bh_tree* t, double theta) {
    if (!t) return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_tree_set_theta: null tree");
    if (!(theta >= 0)) return nb::set_error(NB_ERR_INVALID_ARG, "theta must be >= 0");
    t->params.theta = theta;
    return NB_OK;
}

nb_status nb_bh_build(nb_ctx* ctx, nb_bh_tree* t, const double* m, const double* x,
                      const double* y, const double* z, uint32_t n, double G,
                      nb_stream_t stream_) {
    NB_CHECK_CTX(ctx);
    if (!t) return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_build: null tree");
    if (!m || !x || !y || !z) return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_build: null array");
    if (n == 0 || n > t->n_max)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_build: n = %u (tree capacity %u)", n, t->n_max);
    cudaStream_t s = (cudaStream_t)stream_;
    t->built = false;
    t->n = n;
    t->G = G;
    const int grid = nb::ceil_div(n, BH_THREADS);
    auto mark = [&](int phase) -> nb_status {
        if (t->phase_timing) NB_CUDA_TRY(cudaEventRecord(t->phase_ev[phase], s));
        return NB_OK;
    };
    NB_TRY(mark(0));
    NB_TRY(nb::launch_aabb(ctx, x, y, z, n, t->box, s));
    NB_TRY(mark(1));
    const bool quantized = (t->records & NB_BUILD_QUANTIZED_KEYS) != 0;
    if (quantized) {
        keys_quantized_kernel<<<grid, BH_THREADS, 0, s>>>(x, y, z, n, t->box, t->key0, t->ids);
    } else {
        keys_kernel<<<grid, BH_THREADS, 0, s>>>(x, y, z, n, t->box, t->key0, t->ids);
    }
    NB_TRY(nb::check_launch("keys_kernel"));
    NB_TRY(mark(2));
    int in_alt = 0;
    NB_TRY(nb::radix_sort_pairs(t->key0, t->ids, t->key_alt, t->ids_alt, n, 0, 3 * NB_KEY_LEVELS,
                                t->sort_temp, ctx->dev_error, s, &in_alt));
    if (in_alt) {  // an odd number of passes leaves the result in the alternate buffers
        NB_CUDA_TRY(cudaMemcpyAsync(t->key0, t->key_alt, (size_t)n * 8, cudaMemcpyDeviceToDevice, s));
        NB_CUDA_TRY(cudaMemcpyAsync(t->ids, t->ids_alt, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    }
    NB_TRY(mark(3));
    NB_CUDA_TRY(cudaMemsetAsync(t->key1, 0, (size_t)n * 8, s));
    runs_fixup_kernel<<<grid, BH_THREADS, 0, s>>>(x, y, z, n, t->box, t->key0, t->key1, t->ids,
                                                  ctx->dev_error, quantized ? 1 : 0);
    NB_TRY(nb::check_launch("runs_fixup_kernel"));
    NB_CUDA_TRY(cudaMemsetAsync(t->mask, 0, (size_t)n * 8, s));
    splits_kernel<<<grid, BH_THREADS, 0, s>>>(t->key0, t->key1, n, t->split_level, t->split_start,
                                              t->split_end, (unsigned long long*)t->mask,
                                              ctx->dev_error);
    NB_TRY(nb::check_launch("splits_kernel"));
    count_kernel<<<grid, BH_THREADS, 0, s>>>((const unsigned long long*)t->mask, n, t->cnt);
    NB_TRY(nb::check_launch("count_kernel"));
    NB_TRY(nb::exclusive_scan_u32(t->cnt, t->base, n, 1, t->scan_temp, s));
    const size_t nodes_max = 2 * (size_t)n;
    NB_CUDA_TRY(cudaMemsetAsync(t->children, 0xff, nodes_max * 8 * 4, s));  // NB_NONE
    emit_kernel<<<grid, BH_THREADS, 0, s>>>(n, t->ids, t->split_level, t->split_start, t->split_end,
                                            (const unsigned long long*)t->mask, t->base,
                                            t->node_level, t->node_first, t->node_last, t->node_skip,
                                            t->node_parent, t->node_body, t->info,
                                            t->key0, t->key1, t->children);
    NB_TRY(nb::check_launch("emit_kernel"));
    NB_TRY(mark(4));
    ComArgs A;
    A.n = n;
    A.records = t->records;
    A.m = m;
    A.x = x;
    A.y = y;
    A.z = z;
    A.box = t->box;
    A.G = G;
    A.key0 = t->key0;
    A.key1 = t->key1;
    A.ids = t->ids;
    A.mask = (const unsigned long long*)t->mask;
    A.base = t->base;
    A.node_level = t->node_level;
    A.node_first = t->node_first;
    A.node_last = t->node_last;
    A.node_skip = t->node_skip;
    A.err = ctx->dev_error;

    A.node_parent = t->node_parent;
    A.node_body = t->node_body;
    A.node_count = t->node_count;
    A.comx = t->node_comx;
    A.comy = t->node_comy;
    A.comz = t->node_comz;
    A.mass = t->node_mass;
    A.rec64 = t->rec64;
    A.rec32 = t->rec32;
    A.rec32lo = t->rec32lo;
    A.rec32lo2 = t->rec32lo2;
    A.q = t->node_q;
    A.aux = t->aux;
    A.node_first_pos = t->node_first;
    A.children = t->children;
    A.sorted4 = t->sorted4;
    A.sorted4lo = t->sorted4lo;
    com_leaf_kernel<<<grid, BH_THREADS, 0, s>>>(A);
    NB_TRY(nb::check_launch("com_leaf_kernel"));
    {
        uint32_t chunks = (uint32_t)nb::ceil_div(n, CW);
        com_cells_kernel<<<chunks, CC_THREADS, 0, s>>>(A, t->tier_cells[0], t->tier_count[0]);
        NB_TRY(nb::check_launch("com_cells_kernel"));
        uint64_t span = CW;
        int in = 0;
        for (int tier = 1; tier <= CM_TIERS; ++tier) {
            span *= CM_FAN;
            const uint32_t blocks = (uint32_t)((n + span - 1) / span);
            const bool last = blocks == 1;
            com_tier_kernel<<<blocks, CC_THREADS, 0, s>>>(
                A, (uint32_t)std::min<uint64_t>(span, 0xffffffffu), t->tier_cells[in],
                t->tier_count[in], chunks, last ? nullptr : t->tier_cells[1 - in],
                last ? nullptr : t->tier_count[1 - in]);
            NB_TRY(nb::check_launch("com_tier_kernel"));
            if (last) break;
            chunks = blocks;
            in = 1 - in;
        }
    }
    NB_TRY(mark(5));
    t->built = true;
    t->built_records = t->records;
    return NB_OK;
}

nb_status nb_bh_set_records(nb_bh_tree* t, unsigned int mask) {
    if (!t) return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_set_records: null tree");
    if (mask & ~(NB_REC_ALL | NB_BUILD_QUANTIZED_KEYS))
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_set_records: unknown bits 0x%x", mask);
    t->records = mask;
    return NB_OK;
}

}  // extern "C"
