// nbody_oracle.cpp -- CPU ORACLE (test infrastructure only).
//
// A C++17/OpenMP restatement of TimThuering/N-Body-Simulation's two force paths, used as the
// parity reference for the CUDA library and as the timed CPU baseline. It is never linked into, loaded by,
// or called from the product path (the CUDA library and the host driver); only tests/, the smoke
// check and bench.py's CPU legs load it.
//
// Every function follows the reference's operation order and conventions (file:line cited at
// each function). The reference itself cannot be compiled here: it needs a SYCL 2020 compiler
// (AdaptiveCpp or DPC++) and FetchContent downloads (CMakeLists.txt:10-29,58-115), none of which
// exist on either machine.
//
// Pinning: the AABB, octree node table, subtree preparation, subtree body sort, root mass and
// in-order body sort are pinned against the known answers in the reference's
// tests/BarnesHutTest.cpp (fixture tests/golden/reference_kats.json). Force, centre-of-mass
// (beyond the root mass), leapfrog and energy VALUES are not covered by any reference test:
// for those the oracle is "parity unpinned" -- a restatement checked only by review against
// the cited lines, plus property tests (momentum conservation, symmetry, N=2 closed form).
//
// SYCL -> OpenMP mapping: parallel_for over bodies -> `omp parallel for`; the single-work-group
// lock-based insertions run sequentially in body order (which reproduces the node ids the
// reference's tests expect); `atomic_ref::fetch_add` on nextFreeNodeID -> std::atomic when the
// subtrees are built in parallel (node ids then depend on thread timing, exactly as on a GPU).

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum : int {
    ORC_OK = 0,
    ORC_ERR_INVALID_ARG = 1,
    ORC_ERR_POOL_OVERFLOW = 4,
    ORC_ERR_STACK_OVERFLOW = 6,
};

int resolve_threads(int threads) {
#ifdef _OPENMP
    return threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

// sycl::rsqrt on the host: 1/sqrt with two IEEE roundings.
inline double rsqrt_ref(double v) { return 1.0 / std::sqrt(v); }

}  // namespace

extern "C" {

// ------------------------------------------------------------------------------------------
// Naive all-pairs acceleration.
// Follows NaiveAlgorithm.cpp:262-360 (opt_2). opt_0 (:362-417) and opt_1 (:419-482) evaluate
// the identical per-body sum: j ascending from 0 to N-1, the self pair included (it contributes
// exactly 0 because r = 0), G applied once at the end. The local-memory tiling of opt_2 does not
// change the j order of any body's sum, so all three stages give bit-identical results here.
// ------------------------------------------------------------------------------------------
int orc_naive_accel(const double* m, const double* x, const double* y, const double* z,
                    double* ax, double* ay, double* az, uint32_t n, double G, double eps2,
                    int threads) {
    if (n == 0) return ORC_OK;
    if (!m || !x || !y || !z || !ax || !ay || !az) return ORC_ERR_INVALID_ARG;
    const int T = resolve_threads(threads);
#pragma omp parallel for schedule(static) num_threads(T)
    for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
        const uint32_t i = (uint32_t)ii;
        const double px = x[i], py = y[i], pz = z[i];
        double acc_x = 0, acc_y = 0, acc_z = 0;
        for (uint32_t j = 0; j < n; ++j) {  // NaiveAlgorithm.cpp:318-346
            double r_x = x[j] - px;
            double r_y = y[j] - py;
            double r_z = z[j] - pz;
            double den = (r_x * r_x) + (r_y * r_y) + (r_z * r_z) + eps2;  // :336
            den = den * den * den;                                          // :337
            den = rsqrt_ref(den);                                           // :338
            acc_x += m[j] * (r_x * den);                                    // :340-342
            acc_y += m[j] * (r_y * den);
            acc_z += m[j] * (r_z * den);
        }
        ax[i] = acc_x * G;  // :348-351
        ay[i] = acc_y * G;
        az[i] = acc_z * G;
    }
    return ORC_OK;
}

// Naive acceleration for a subset of target bodies (sampled-body error checks at large N).
int orc_naive_accel_subset(const double* m, const double* x, const double* y, const double* z,
                           uint32_t n, const uint32_t* targets, uint32_t n_targets,
                           double* ax, double* ay, double* az, double G, double eps2,
                           int threads) {
    if (!m || !x || !y || !z || !targets || !ax || !ay || !az) return ORC_ERR_INVALID_ARG;
    const int T = resolve_threads(threads);
#pragma omp parallel for schedule(static) num_threads(T)
    for (int64_t t = 0; t < (int64_t)n_targets; ++t) {
        const uint32_t i = targets[t];
        const double px = x[i], py = y[i], pz = z[i];
        double acc_x = 0, acc_y = 0, acc_z = 0;
        for (uint32_t j = 0; j < n; ++j) {
            double r_x = x[j] - px, r_y = y[j] - py, r_z = z[j] - pz;
            double den = (r_x * r_x) + (r_y * r_y) + (r_z * r_z) + eps2;
            den = den * den * den;
            den = rsqrt_ref(den);
            acc_x += m[j] * (r_x * den);
            acc_y += m[j] * (r_y * den);
            acc_z += m[j] * (r_z * den);
        }
        ax[t] = acc_x * G;
        ay[t] = acc_y * G;
        az[t] = acc_z * G;
    }
    return ORC_OK;
}

// ------------------------------------------------------------------------------------------
// Leapfrog kick-drift-kick. NaiveAlgorithm.cpp:154-163 / BarnesHutAlgorithm.cpp:171-181 (part 1)
// and NaiveAlgorithm.cpp:217-221 / BarnesHutAlgorithm.cpp:234-238 (part 2).
// ------------------------------------------------------------------------------------------
void orc_leapfrog_part1(double* vhx, double* vhy, double* vhz, const double* vx, const double* vy,
                        const double* vz, double* px, double* py, double* pz, const double* ax,
                        const double* ay, const double* az, uint32_t n, double dt) {
    for (uint32_t i = 0; i < n; ++i) {
        vhx[i] = vx[i] + ax[i] * (dt / 2.0);
        vhy[i] = vy[i] + ay[i] * (dt / 2.0);
        vhz[i] = vz[i] + az[i] * (dt / 2.0);
        px[i] = px[i] + vhx[i] * dt;
        py[i] = py[i] + vhy[i] * dt;
        pz[i] = pz[i] + vhz[i] * dt;
    }
}

void orc_leapfrog_part2(double* vx, double* vy, double* vz, const double* vhx, const double* vhy,
                        const double* vhz, const double* ax, const double* ay, const double* az,
                        uint32_t n, double dt) {
    for (uint32_t i = 0; i < n; ++i) {
        vx[i] = vhx[i] + ax[i] * (dt / 2.0);
        vy[i] = vhy[i] + ay[i] * (dt / 2.0);
        vz[i] = vhz[i] + az[i] * (dt / 2.0);
    }
}

// ------------------------------------------------------------------------------------------
// Energy. nBodyAlgorithm.cpp:11-86: per body j the kinetic energy 0.5*m*v^2 and the potential
// sum over i < j of G*m_i*m_j/r WITHOUT softening; host sums in body order; U negated; virial
// 2K/|U|. out = {E_kin, E_pot, E_total, virial}.
// ------------------------------------------------------------------------------------------
void orc_energy(const double* m, const double* x, const double* y, const double* z,
                const double* vx, const double* vy, const double* vz, uint32_t n, double G,
                double* out, int threads) {
    std::vector<double> ekin(n), epot(n);
    const int T = resolve_threads(threads);
#pragma omp parallel for schedule(dynamic, 16) num_threads(T)
    for (int64_t jj = 0; jj < (int64_t)n; ++jj) {
        const uint32_t j = (uint32_t)jj;
        double v = vx[j] * vx[j] + vy[j] * vy[j] + vz[j] * vz[j];  // :49-51
        ekin[j] = 0.5 * m[j] * v;                                   // :52
        double ep = 0;
        for (uint32_t i = 0; i < j; ++i) {  // :55-63
            double r_x = x[j] - x[i];
            double r_y = y[j] - y[i];
            double r_z = z[j] - z[i];
            double r = std::sqrt(r_x * r_x + r_y * r_y + r_z * r_z);
            ep += G * m[i] * m[j] / r;
        }
        epot[j] = ep;
    }
    double ek = 0, ep = 0;
    for (uint32_t i = 0; i < n; ++i) {  // :71-74
        ek += ekin[i];
        ep += epot[i];
    }
    ep *= -1;  // :77
    out[0] = ek;
    out[1] = ep;
    out[2] = ek + ep;
    out[3] = (2.0 * ek) / std::abs(ep);  // :85
}

// nBodyAlgorithm.cpp:104-127: subtracts the mass-weighted mean velocity (used only for the
// step-0 output velocities; the integration starts from the unadjusted input velocities).
void orc_adjust_velocities(const double* m, double* vx, double* vy, double* vz, uint32_t n) {
    double sm = 0, sx = 0, sy = 0, sz = 0;
    for (uint32_t i = 0; i < n; ++i) {
        sm += m[i];
        sx += m[i] * vx[i];
        sy += m[i] * vy[i];
        sz += m[i] * vz[i];
    }
    double ux = sx / sm, uy = sy / sm, uz = sz / sm;
    for (uint32_t i = 0; i < n; ++i) {
        vx[i] -= ux;
        vy[i] -= uy;
        vz[i] -= uz;
    }
}

// ------------------------------------------------------------------------------------------
// AABB. BarnesHutOctree.cpp:45-191. `work_items` partial min/max accumulators over contiguous
// chunks of ceil(N/work_items) bodies. The accumulators start at 0.0 (value-initialised
// std::vector, :58-72), so every partial -- and therefore the box -- contains the origin.
// Host reduction over partials i < N (:122-159), then the cube rule: the longest axis wins with
// ties resolved x, then y, then z, and the shorter axes are padded equally on both sides
// (:161-190). out = {min_x, min_y, min_z, max_x, max_y, max_z, edge}.
// ------------------------------------------------------------------------------------------
int orc_aabb(const double* x, const double* y, const double* z, uint32_t n, int work_items,
             double* out) {
    if (work_items <= 0) return ORC_ERR_INVALID_ARG;
    double min_x = std::numeric_limits<double>::infinity();
    double min_y = min_x, min_z = min_x;
    double max_x = std::numeric_limits<double>::lowest();
    double max_y = max_x, max_z = max_x;
    const int per = (int)std::ceil((double)n / (double)work_items);
    std::vector<double> lmin_x(work_items, 0.0), lmin_y(work_items, 0.0), lmin_z(work_items, 0.0);
    std::vector<double> lmax_x(work_items, 0.0), lmax_y(work_items, 0.0), lmax_z(work_items, 0.0);
    for (int w = 0; w < work_items; ++w) {  // :91-111
        for (int64_t i = (int64_t)per * w; i < (int64_t)per * w + per; ++i) {
            if (i < (int64_t)n) {
                lmin_x[w] = std::min(lmin_x[w], x[i]);
                lmin_y[w] = std::min(lmin_y[w], y[i]);
                lmin_z[w] = std::min(lmin_z[w], z[i]);
                lmax_x[w] = std::max(lmax_x[w], x[i]);
                lmax_y[w] = std::max(lmax_y[w], y[i]);
                lmax_z[w] = std::max(lmax_z[w], z[i]);
            }
        }
    }
    for (int w = 0; w < work_items; ++w) {  // :122-159
        if ((uint32_t)w < n) {
            if (lmin_x[w] < min_x) min_x = lmin_x[w];
            if (lmin_y[w] < min_y) min_y = lmin_y[w];
            if (lmin_z[w] < min_z) min_z = lmin_z[w];
            if (lmax_x[w] > max_x) max_x = lmax_x[w];
            if (lmax_y[w] > max_y) max_y = lmax_y[w];
            if (lmax_z[w] > max_z) max_z = lmax_z[w];
        }
    }
    double x_len = std::abs(max_x - min_x);  // :162-165
    double y_len = std::abs(max_y - min_y);
    double z_len = std::abs(max_z - min_z);
    double edge = std::max(x_len, std::max(y_len, z_len));
    if (edge == x_len) {  // :168-188
        min_z = min_z - ((edge - z_len) / 2);
        min_y = min_y - ((edge - y_len) / 2);
        max_z = max_z + ((edge - z_len) / 2);
        max_y = max_y + ((edge - y_len) / 2);
    } else if (edge == y_len) {
        min_x = min_x - ((edge - x_len) / 2);
        min_z = min_z - ((edge - z_len) / 2);
        max_x = max_x + ((edge - x_len) / 2);
        max_z = max_z + ((edge - z_len) / 2);
    } else if (edge == z_len) {
        min_x = min_x - ((edge - x_len) / 2);
        min_y = min_y - ((edge - y_len) / 2);
        max_x = max_x + ((edge - x_len) / 2);
        max_y = max_y + ((edge - y_len) / 2);
    } else {
        return ORC_ERR_INVALID_ARG;  // :187 throws std::invalid_argument (NaN input)
    }
    out[0] = min_x; out[1] = min_y; out[2] = min_z;
    out[3] = max_x; out[4] = max_y; out[5] = max_z;
    out[6] = edge;
    return ORC_OK;
}

// ------------------------------------------------------------------------------------------
// Linearised octree (BarnesHutOctree.hpp:33-95, ctor BarnesHutOctree.cpp:5-43).
// ------------------------------------------------------------------------------------------
struct orc_tree {
    uint32_t n = 0;
    uint32_t S = 0;  // storageSizeParameter * N nodes
    std::vector<uint32_t> octants;       // 8 * S, octants[o*S + node]
    std::vector<double> edge, min_x, min_y, min_z;
    std::vector<uint32_t> body_of_node;  // N = empty or internal
    std::vector<int> node_is_leaf;
    std::vector<double> sum_masses, com_x, com_y, com_z;  // com = mass-weighted numerators
    std::vector<uint32_t> body_count;
    std::vector<uint32_t> sorted_bodies;  // sortedBodiesInOrder
    std::vector<uint32_t> subtree_of_body;
    uint32_t next_free = 0;
    double aabb[7] = {0, 0, 0, 0, 0, 0, 0};
};

struct orc_tree_view {
    uint32_t n, S, node_count, pad;
    const uint32_t* octants;
    const double *edge, *min_x, *min_y, *min_z;
    const uint32_t* body_of_node;
    const int* node_is_leaf;
    const double *sum_masses, *com_x, *com_y, *com_z;
    const uint32_t* body_count;
    const uint32_t* sorted_bodies;
    const uint32_t* subtree_of_body;
    double aabb[7];
};

orc_tree* orc_tree_create(uint32_t n, uint32_t storage_size_param) {
    orc_tree* t = new orc_tree();
    t->n = n;
    t->S = storage_size_param * n;
    const size_t S = t->S;
    t->octants.assign(8 * S, 0);
    t->edge.assign(S, 0.0);
    t->min_x.assign(S, 0.0);
    t->min_y.assign(S, 0.0);
    t->min_z.assign(S, 0.0);
    t->body_of_node.assign(S, n);
    t->node_is_leaf.assign(S, 1);
    t->sum_masses.assign(S, 0.0);
    t->com_x.assign(S, 0.0);
    t->com_y.assign(S, 0.0);
    t->com_z.assign(S, 0.0);
    t->body_count.assign(S, 0);
    t->sorted_bodies.assign(n, n);
    t->subtree_of_body.assign(n, 0);
    return t;
}

void orc_tree_destroy(orc_tree* t) { delete t; }

void orc_tree_view_get(const orc_tree* t, orc_tree_view* v) {
    v->n = t->n;
    v->S = t->S;
    v->node_count = t->next_free;
    v->pad = 0;
    v->octants = t->octants.data();
    v->edge = t->edge.data();
    v->min_x = t->min_x.data();
    v->min_y = t->min_y.data();
    v->min_z = t->min_z.data();
    v->body_of_node = t->body_of_node.data();
    v->node_is_leaf = t->node_is_leaf.data();
    v->sum_masses = t->sum_masses.data();
    v->com_x = t->com_x.data();
    v->com_y = t->com_y.data();
    v->com_z = t->com_z.data();
    v->body_count = t->body_count.data();
    v->sorted_bodies = t->sorted_bodies.data();
    v->subtree_of_body = t->subtree_of_body.data();
    std::memcpy(v->aabb, t->aabb, sizeof(v->aabb));
}

}  // extern "C"

namespace {

// Octant rule (ParallelOctreeTopDownSubtrees.cpp:400-414): strict compares against
// min + edge/2; y selects 4, x selects 2, z BELOW the midpoint selects 1.
inline uint32_t octant_of(const orc_tree& t, uint32_t node, double px, double py, double pz) {
    const double pmx = t.min_x[node], pmy = t.min_y[node], pmz = t.min_z[node];
    const double pe = t.edge[node];
    bool upper = py > pmy + (pe / 2.0);
    bool right = px > pmx + (pe / 2.0);
    bool back = pz < pmz + (pe / 2.0);
    return (uint32_t)upper * 4u + (uint32_t)right * 2u + (uint32_t)back * 1u;
}

inline uint32_t child_of(const orc_tree& t, uint32_t node, uint32_t octant) {
    return t.octants[(size_t)octant * t.S + node];
}

// Resets node `idx` to an empty leaf (ParallelOctreeTopDownSubtrees.cpp:321-339).
inline void init_empty_leaf(orc_tree& t, uint32_t idx) {
    for (int o = 0; o < 8; ++o) t.octants[(size_t)o * t.S + idx] = 0;
    t.body_of_node[idx] = t.n;
    t.body_count[idx] = 0;
    t.node_is_leaf[idx] = 1;
    t.com_x[idx] = 0;
    t.com_y[idx] = 0;
    t.com_z[idx] = 0;
    t.sum_masses[idx] = 0;
}

// Splits leaf `node` holding a body: allocates 8 children at `first`, children slots
// first+0..7 hold octants 5,7,4,6,1,3,0,2 with the child min corners of
// ParallelOctreeTopDownSubtrees.cpp:256-315, moves the old body into its octant (:342-369).
// Returns the child the old body moved to.
uint32_t split_leaf(orc_tree& t, uint32_t node, uint32_t first, const double* x, const double* y,
                    const double* z) {
    const uint32_t old_body = t.body_of_node[node];
    const double ce = t.edge[node] / 2;
    const double pmx = t.min_x[node], pmy = t.min_y[node], pmz = t.min_z[node];
    for (uint32_t k = 0; k < 8; ++k) t.edge[first + k] = ce;
    static const uint32_t slot_octant[8] = {5, 7, 4, 6, 1, 3, 0, 2};
    for (uint32_t k = 0; k < 8; ++k) t.octants[(size_t)slot_octant[k] * t.S + node] = first + k;
    // slot k -> (dx, dy, dz) offsets in units of ce
    static const int off[8][3] = {{0, 1, 0}, {1, 1, 0}, {0, 1, 1}, {1, 1, 1},
                                  {0, 0, 0}, {1, 0, 0}, {0, 0, 1}, {1, 0, 1}};
    for (uint32_t k = 0; k < 8; ++k) {
        t.min_x[first + k] = off[k][0] ? pmx + ce : pmx;
        t.min_y[first + k] = off[k][1] ? pmy + ce : pmy;
        t.min_z[first + k] = off[k][2] ? pmz + ce : pmz;
    }
    for (uint32_t k = 0; k < 8; ++k) init_empty_leaf(t, first + k);
    const uint32_t oct = octant_of(t, node, x[old_body], y[old_body], z[old_body]);
    const uint32_t child = child_of(t, node, oct);
    t.body_of_node[child] = old_body;
    t.body_of_node[node] = t.n;
    return child;
}

void init_root(orc_tree& t) {  // ParallelOctreeTopDownSubtrees.cpp:135-163
    t.edge[0] = t.aabb[6];
    t.min_x[0] = t.aabb[0];
    t.min_y[0] = t.aabb[1];
    t.min_z[0] = t.aabb[2];
    for (int o = 0; o < 8; ++o) t.octants[(size_t)o * t.S] = 0;
    t.next_free = 1;
    t.node_is_leaf[0] = 1;
    t.body_count[0] = 0;
    t.sum_masses[0] = 0;
    t.com_x[0] = t.com_y[0] = t.com_z[0] = 0;
    t.body_of_node[0] = t.n;
}

// Inserts body i starting at `node`/`depth`; with max_level >= 0 the insertion stops at depth
// max_level and records the subtree root (buildOctreeToLevel); with max_level < 0 it inserts to
// the bottom (buildSubtrees / synchronized builder). `next_free` is shared between threads when
// subtrees are built in parallel.
int insert_body(orc_tree& t, uint32_t i, uint32_t node, int depth, int max_level,
                std::atomic<uint32_t>& next_free, const double* x, const double* y,
                const double* z) {
    for (;;) {
        if (max_level >= 0 && depth >= max_level) {  // :420-427
            t.subtree_of_body[i] = node;
            return ORC_OK;
        }
        if (t.node_is_leaf[node] == 1) {
            if (t.body_of_node[node] == t.n) {  // :240-246
                t.body_of_node[node] = i;
                return ORC_OK;
            }
            const uint32_t first = next_free.fetch_add(8);  // :254
            if ((uint64_t)first + 8 > t.S) return ORC_ERR_POOL_OVERFLOW;
            const uint32_t old_body = t.body_of_node[node];
            const uint32_t child = split_leaf(t, node, first, x, y, z);
            if (max_level >= 0 && depth == max_level - 1) {  // :371-376
                t.body_of_node[child] = t.n;
                t.subtree_of_body[old_body] = child;
            }
            t.node_is_leaf[node] = 0;  // :380
        } else {  // :390-418
            const uint32_t oct = octant_of(t, node, x[i], y[i], z[i]);
            node = child_of(t, node, oct);
            depth += 1;
        }
    }
}

}  // namespace

extern "C" {

// ParallelOctreeTopDownSubtrees.cpp:436-476 (prepareSubtrees): histogram of subtreeOfBody,
// then a serial scan over nodes 1..nodeCount-1 collecting referenced subtree roots.
void orc_prepare_subtrees(const uint32_t* subtree_of_body, uint32_t n, uint32_t node_count,
                          uint32_t* body_count_subtree, uint32_t* subtrees,
                          uint32_t* subtree_count) {
    for (uint32_t k = 0; k < node_count; ++k) body_count_subtree[k] = 0;
    for (uint32_t i = 0; i < n; ++i) body_count_subtree[subtree_of_body[i]] += 1;
    uint32_t next = 0;
    for (uint32_t k = 1; k < node_count; ++k) {
        if (body_count_subtree[k] > 0) subtrees[next++] = k;
    }
    *subtree_count = next;
}

// ParallelOctreeTopDownSubtrees.cpp:478-534 (sortBodiesForSubtrees): start index of subtree s =
// bodies of all lower subtrees; bodies scattered into their subtree's range in ascending body id
// (the reference's order within a subtree follows its atomic counter; ascending is what a
// sequential run produces and what its test expects).
void orc_sort_bodies_for_subtrees(const uint32_t* subtree_of_body, uint32_t n,
                                  const uint32_t* body_count_subtree, const uint32_t* subtrees,
                                  uint32_t num_subtrees, uint32_t* start_index,
                                  uint32_t* sorted_bodies) {
    std::vector<uint32_t> next(num_subtrees);
    uint32_t acc = 0;
    for (uint32_t s = 0; s < num_subtrees; ++s) {
        start_index[s] = acc;
        next[s] = acc;
        acc += body_count_subtree[subtrees[s]];
    }
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t root = subtree_of_body[i];
        for (uint32_t s = 0; s < num_subtrees; ++s) {
            if (subtrees[s] == root) {
                sorted_bodies[next[s]++] = i;
                break;
            }
        }
    }
}

}  // extern "C"

namespace {

// BarnesHutOctree.cpp:193-229 (prepareCenterOfMass) + :231-548 (bottom-up). Children always
// have larger node ids than their parent (they are allocated when the parent splits), so one
// sweep in decreasing id order finishes every child before its parent; each internal node sums
// its children in octant order 0..7 (:304-311), which is the order the reference uses
// regardless of its work distribution.
void compute_center_of_mass(orc_tree& t, const double* m, const double* x, const double* y,
                            const double* z) {
    const uint32_t nodes = t.next_free;
    for (uint32_t k = 0; k < nodes; ++k) {
        const uint32_t b = t.body_of_node[k];
        if (t.node_is_leaf[k] == 1 && b != t.n) {
            t.com_x[k] = x[b] * m[b];
            t.com_y[k] = y[b] * m[b];
            t.com_z[k] = z[b] * m[b];
            t.sum_masses[k] = m[b];
            t.body_count[k] = 1;
        }
    }
    for (int64_t k = (int64_t)nodes - 1; k >= 0; --k) {
        if (t.node_is_leaf[k] != 0) continue;
        double sm = 0, cx = 0, cy = 0, cz = 0;
        uint32_t cnt = 0;
        for (int o = 0; o < 8; ++o) {
            const uint32_t c = t.octants[(size_t)o * t.S + k];
            cx += t.com_x[c];
            cy += t.com_y[c];
            cz += t.com_z[c];
            sm += t.sum_masses[c];
            cnt += t.body_count[c];
        }
        t.body_count[k] = cnt;
        t.com_x[k] = cx;
        t.com_y[k] = cy;
        t.com_z[k] = cz;
        t.sum_masses[k] = sm;
    }
}

// BarnesHutOctree.cpp:550-613 (sortBodies): rank of body i = sum of the body counts of all
// lower-octant siblings on its root-to-leaf path.
void sort_bodies(orc_tree& t, const double* x, const double* y, const double* z, int T) {
#pragma omp parallel for schedule(static) num_threads(T)
    for (int64_t ii = 0; ii < (int64_t)t.n; ++ii) {
        const uint32_t i = (uint32_t)ii;
        uint32_t idx = 0, node = 0;
        while (!t.node_is_leaf[node]) {
            const uint32_t oct = octant_of(t, node, x[i], y[i], z[i]);
            for (uint32_t j = 0; j < oct; ++j) idx += t.body_count[child_of(t, node, j)];
            node = child_of(t, node, oct);
        }
        t.sorted_bodies[idx] = i;
    }
}

}  // namespace

extern "C" {

// ParallelOctreeTopDownSubtrees::buildOctree (ParallelOctreeTopDownSubtrees.cpp:15-93):
// AABB -> top of the tree to max_level -> prepareSubtrees -> sortBodiesForSubtrees ->
// buildSubtrees (subtrees in parallel when threads != 1) -> centre of mass -> body sort.
int orc_tree_build_subtrees(orc_tree* t, const double* m, const double* x, const double* y,
                            const double* z, int max_level, int aabb_work_items, int sort,
                            int threads) {
    if (!t || max_level < 1) return ORC_ERR_INVALID_ARG;
    const uint32_t n = t->n;
    const int T = resolve_threads(threads);
    int rc = orc_aabb(x, y, z, n, aabb_work_items, t->aabb);
    if (rc) return rc;
    init_root(*t);
    std::atomic<uint32_t> next_free(t->next_free);
    for (uint32_t i = 0; i < n; ++i) {  // buildOctreeToLevel, :202-431
        t->subtree_of_body[i] = 0;
        rc = insert_body(*t, i, 0, 0, max_level, next_free, x, y, z);
        if (rc) return rc;
    }
    const uint32_t node_count = next_free.load();
    std::vector<uint32_t> count_subtree(node_count), subtrees(node_count);
    uint32_t num_subtrees = 0;
    orc_prepare_subtrees(t->subtree_of_body.data(), n, node_count, count_subtree.data(),
                         subtrees.data(), &num_subtrees);
    std::vector<uint32_t> start(num_subtrees), sorted(n);
    orc_sort_bodies_for_subtrees(t->subtree_of_body.data(), n, count_subtree.data(),
                                 subtrees.data(), num_subtrees, start.data(), sorted.data());
    std::atomic<int> err(ORC_OK);
#pragma omp parallel for schedule(dynamic, 1) num_threads(T)
    for (int64_t s = 0; s < (int64_t)num_subtrees; ++s) {  // buildSubtrees, :586-811
        const uint32_t root = subtrees[s];
        const uint32_t cnt = count_subtree[root];
        for (uint32_t k = 0; k < cnt; ++k) {
            if (err.load(std::memory_order_relaxed)) break;
            int r = insert_body(*t, sorted[start[s] + k], root, max_level, -1, next_free, x, y, z);
            if (r) err.store(r);
        }
    }
    if (err.load()) return err.load();
    t->next_free = next_free.load();
    compute_center_of_mass(*t, m, x, y, z);
    if (sort) sort_bodies(*t, x, y, z, T);
    return ORC_OK;
}

// ParallelOctreeTopDownSynchronized::buildOctree (ParallelOctreeTopDownSynchronized.cpp:10-388):
// AABB -> every body inserted from the root without a depth limit -> centre of mass -> sort.
int orc_tree_build_sync(orc_tree* t, const double* m, const double* x, const double* y,
                        const double* z, int aabb_work_items, int sort, int threads) {
    if (!t) return ORC_ERR_INVALID_ARG;
    const int T = resolve_threads(threads);
    int rc = orc_aabb(x, y, z, t->n, aabb_work_items, t->aabb);
    if (rc) return rc;
    init_root(*t);
    std::atomic<uint32_t> next_free(t->next_free);
    for (uint32_t i = 0; i < t->n; ++i) {
        rc = insert_body(*t, i, 0, 0, -1, next_free, x, y, z);
        if (rc) return rc;
    }
    t->next_free = next_free.load();
    compute_center_of_mass(*t, m, x, y, z);
    if (sort) sort_bodies(*t, x, y, z, T);
    return ORC_OK;
}

// BarnesHutAlgorithm::computeAccelerations (BarnesHutAlgorithm.cpp:280-401). Per body a DFS
// with an explicit stack of capacity stack_size-1 (the reference's per-body slice of
// nodesOnStack, :340-344): skip empty nodes and the body's own leaf (:349); d = com/sum - x_i
// (:351-353); accept if edge*rsqrt(d^2) < theta or the node is a body leaf (:355-359) with the
// monopole sum*d*rsqrt((d^2+eps2)^3) (:361-367); otherwise push children 5,7,4,6,1,3,0,2
// (:370-385). The reference does not check the stack bound; the oracle reports an overflow.
int orc_bh_accel(const orc_tree* t, const double* x, const double* y, const double* z,
                 double* ax, double* ay, double* az, double G, double eps2, double theta,
                 uint32_t stack_size, int sorted, int threads) {
    if (!t || stack_size < 2) return ORC_ERR_INVALID_ARG;
    const uint32_t N = t->n;
    const size_t S = t->S;
    const int T = resolve_threads(threads);
    std::atomic<int> err(ORC_OK);
#pragma omp parallel num_threads(T)
    {
        std::vector<uint32_t> stack(stack_size);
#pragma omp for schedule(dynamic, 64)
        for (int64_t id = 0; id < (int64_t)N; ++id) {
            const uint32_t i = sorted ? t->sorted_bodies[id] : (uint32_t)id;
            const double px = x[i], py = y[i], pz = z[i];
            double acc_x = 0, acc_y = 0, acc_z = 0;
            uint32_t top = 1;
            stack[top] = 0;
            bool overflow = false;
            while (top != 0) {
                const uint32_t node = stack[top];
                top -= 1;
                const double sm = t->sum_masses[node];
                if (sm != 0 && t->body_of_node[node] != i) {
                    double d_x = (t->com_x[node] / sm) - px;
                    double d_y = (t->com_y[node] / sm) - py;
                    double d_z = (t->com_z[node] / sm) - pz;
                    double d = rsqrt_ref(d_x * d_x + d_y * d_y + d_z * d_z);
                    double cur = t->edge[node] * d;
                    if ((cur < theta) || t->body_of_node[node] != N) {
                        double den = (d_x * d_x) + (d_y * d_y) + (d_z * d_z) + eps2;
                        den = den * den * den;
                        den = rsqrt_ref(den);
                        acc_x += sm * (d_x * den);
                        acc_y += sm * (d_y * den);
                        acc_z += sm * (d_z * den);
                    } else {
                        if (top + 8 > stack_size - 1) {
                            overflow = true;
                            break;
                        }
                        static const uint32_t push_order[8] = {5, 7, 4, 6, 1, 3, 0, 2};
                        for (int k = 0; k < 8; ++k) stack[++top] = t->octants[push_order[k] * S + node];
                    }
                }
            }
            if (overflow) err.store(ORC_ERR_STACK_OVERFLOW);
            ax[i] = acc_x * G;
            ay[i] = acc_y * G;
            az[i] = acc_z * G;
        }
    }
    return err.load();
}

// Same traversal for a subset of target bodies (bounded CPU samples at large N); results are
// written to ax[t] for targets[t].
int orc_bh_accel_subset(const orc_tree* t, const double* x, const double* y, const double* z,
                        const uint32_t* targets, uint32_t n_targets, double* ax, double* ay,
                        double* az, double G, double eps2, double theta, uint32_t stack_size,
                        int threads) {
    if (!t || stack_size < 2 || !targets) return ORC_ERR_INVALID_ARG;
    const uint32_t N = t->n;
    const size_t S = t->S;
    const int T = resolve_threads(threads);
    std::atomic<int> err(ORC_OK);
#pragma omp parallel num_threads(T)
    {
        std::vector<uint32_t> stack(stack_size);
#pragma omp for schedule(dynamic, 64)
        for (int64_t q = 0; q < (int64_t)n_targets; ++q) {
            const uint32_t i = targets[q];
            const double px = x[i], py = y[i], pz = z[i];
            double acc_x = 0, acc_y = 0, acc_z = 0;
            uint32_t top = 1;
            stack[top] = 0;
            while (top != 0) {
                const uint32_t node = stack[top--];
                const double sm = t->sum_masses[node];
                if (sm != 0 && t->body_of_node[node] != i) {
                    double d_x = (t->com_x[node] / sm) - px;
                    double d_y = (t->com_y[node] / sm) - py;
                    double d_z = (t->com_z[node] / sm) - pz;
                    double d = rsqrt_ref(d_x * d_x + d_y * d_y + d_z * d_z);
                    if ((t->edge[node] * d < theta) || t->body_of_node[node] != N) {
                        double den = (d_x * d_x) + (d_y * d_y) + (d_z * d_z) + eps2;
                        den = den * den * den;
                        den = rsqrt_ref(den);
                        acc_x += sm * (d_x * den);
                        acc_y += sm * (d_y * den);
                        acc_z += sm * (d_z * den);
                    } else {
                        if (top + 8 > stack_size - 1) {
                            err.store(ORC_ERR_STACK_OVERFLOW);
                            break;
                        }
                        static const uint32_t push_order[8] = {5, 7, 4, 6, 1, 3, 0, 2};
                        for (int k = 0; k < 8; ++k) stack[++top] = t->octants[push_order[k] * S + node];
                    }
                }
            }
            ax[q] = acc_x * G;
            ay[q] = acc_y * G;
            az[q] = acc_z * G;
        }
    }
    return err.load();
}

// Per-body count of accepted nodes and opened nodes for the reference traversal (work model).
int orc_bh_interaction_counts(const orc_tree* t, const double* x, const double* y,
                              const double* z, double theta, uint32_t stack_size,
                              uint64_t* accepted, uint64_t* opened, int threads) {
    if (!t || stack_size < 2) return ORC_ERR_INVALID_ARG;
    const uint32_t N = t->n;
    const size_t S = t->S;
    const int T = resolve_threads(threads);
    uint64_t acc_total = 0, open_total = 0;
#pragma omp parallel num_threads(T) reduction(+ : acc_total, open_total)
    {
        std::vector<uint32_t> stack(stack_size);
#pragma omp for schedule(dynamic, 64)
        for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
            const uint32_t i = (uint32_t)ii;
            uint32_t top = 1;
            stack[top] = 0;
            while (top != 0) {
                const uint32_t node = stack[top--];
                const double sm = t->sum_masses[node];
                if (sm != 0 && t->body_of_node[node] != i) {
                    double d_x = (t->com_x[node] / sm) - x[i];
                    double d_y = (t->com_y[node] / sm) - y[i];
                    double d_z = (t->com_z[node] / sm) - z[i];
                    double cur = t->edge[node] * rsqrt_ref(d_x * d_x + d_y * d_y + d_z * d_z);
                    if ((cur < theta) || t->body_of_node[node] != N) {
                        acc_total += 1;
                    } else {
                        open_total += 1;
                        if (top + 8 > stack_size - 1) break;
                        static const uint32_t push_order[8] = {5, 7, 4, 6, 1, 3, 0, 2};
                        for (int k = 0; k < 8; ++k) stack[++top] = t->octants[push_order[k] * S + node];
                    }
                }
            }
        }
    }
    *accepted = acc_total;
    *opened = open_total;
    return ORC_OK;
}

// Stack size rule of configuration::initializeConfigValues (Configuration.cpp:24-33).
uint32_t orc_stack_size(uint32_t n, uint32_t stack_size_param) {
    const uint32_t lg = (uint32_t)std::ceil(std::log2((double)n));
    return n < 15000 ? stack_size_param * lg + 500 : stack_size_param * lg;
}

}  // extern "C"
