/*
 * nbody.h -- C ABI of libnbody_cuda.so, the GB300 (sm_103a) implementation of the naive all-pairs
 * and Barnes-Hut force paths of TimThuering/N-Body-Simulation.
 *
 * Conventions (all entry points):
 *  - Every function returns nb_status (0 = NB_OK). nb_last_error_string() describes the last
 *    failure of the calling thread. Nothing throws across this boundary.
 *  - Body data are caller-owned DEVICE pointers in structure-of-arrays form (FP64), exactly the
 *    reference's SimulationData / SYCL buffer layout (SimulationData.hpp:13-27). Counts are
 *    uint32_t like the reference's d_type::int_t (Configuration.hpp:8-10).
 *  - Work is enqueued on the given stream (NULL = legacy default stream) and nothing
 *    synchronises implicitly, except where a function's comment says "synchronous".
 *  - Masses are in kg and G in AU^3 kg^-1 d^-2 for the reference's units
 *    (nBodyAlgorithm.hpp:55-61); any consistent unit system works since G is a parameter.
 *  - A context owns the scratch memory of its calls; calls on one context must not overlap in
 *    time on different streams.
 */
#ifndef NBODY_GB300_H
#define NBODY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* nb_stream_t; /* identical to cudaStream_t */

typedef enum nb_status {
    NB_OK = 0,
    NB_ERR_INVALID_ARG = 1,     /* bad pointer, size or parameter */
    NB_ERR_CUDA = 2,            /* a CUDA runtime call or kernel launch failed */
    NB_ERR_OOM = 3,             /* device allocation failed */
    NB_ERR_POOL_OVERFLOW = 4,   /* octree node pool (storage_size_param * N) too small */
    NB_ERR_DEPTH_OVERFLOW = 5,  /* bodies too close to separate within NB_MAX_TREE_DEPTH levels
                                   (e.g. coincident bodies; the reference splits forever) */
    NB_ERR_STACK_OVERFLOW = 6,  /* traversal stack capacity exceeded */
    NB_ERR_TIMEOUT = 7,         /* a bounded device-side wait ran out */
    NB_ERR_UNSUPPORTED = 8,     /* combination of options not implemented */
    NB_ERR_NOT_BUILT = 9        /* tree used before nb_bh_build succeeded */
} nb_status;

/* Arithmetic of the pair interactions. Positions, velocities, integration, AABB and energy sums
 * are FP64 in every mode. */
typedef enum nb_precision {
    NB_F64 = 0,       /* FP64 pair math with fused multiply-adds and a Newton-refined rsqrt
                         (relative difference to the reference's FP64 sum ~1e-15) */
    NB_F64_IEEE = 1,  /* FP64, every operation separately and correctly rounded in the reference's
                         order (1/sqrt for sycl::rsqrt): bit-identical to a host FP64 evaluation
                         of the reference's formula */
    NB_F32C = 2,      /* FP32 pair math, compensated (TwoSum) per-body accumulation */
    NB_DF64 = 3       /* FP64-accurate double-float (pairs of FP32, ~2^-48 per operation) on the
                         FP32 pipe: naive all-pairs, and the Barnes-Hut per-body rule (same
                         accepted cells as NB_F64) */
} nb_precision;

#define NB_MAX_TREE_DEPTH 42

typedef struct nb_ctx nb_ctx;

nb_status nb_ctx_create(int device, nb_ctx** out);
nb_status nb_ctx_destroy(nb_ctx* ctx);
/* Blocks until all work of `stream` has finished and reports any device-side error word. */
nb_status nb_sync(nb_ctx* ctx, nb_stream_t stream);
const char* nb_last_error_string(void);
const char* nb_version(void);

/* Failure-path hooks for tests (no reference counterpart: the reference's device waits and its
 * traversal stack are unchecked, BarnesHutOctree.cpp:263-384, BarnesHutAlgorithm.cpp:340-388).
 * They act on later launches of this context only and make a failure happen without faulting
 * the GPU:
 *  - wait_limit: polls of every bounded device-side wait before it gives up and sets the
 *    timeout bit (nb_sync then returns NB_ERR_TIMEOUT); negative = the default (2^22); 0 = no
 *    waiting at all (a tile wait gives up without polling, a look-back gives up at the first
 *    count not yet published). Honoured by the pair kernels' tile waits (nb_naive_accel,
 *    nb_naive_accel_range, nb_batch_naive_accel) and the radix look-back of
 *    nb_util_radix_sort_pairs; the octree build keeps the default. A CTA
 *    whose wait ran out still drains its own copies in flight with the default limit before it
 *    leaves (should that drain run out too, nb_sync reports it and the context refuses all
 *    further calls, since copies may still land in shared memory after the CTA left).
 *  - flags NB_FAULT_DROP_LOOKBACK: nb_util_radix_sort_pairs drops the first tile's published
 *    count in every digit pass, so later tiles wait for a word that nothing writes.
 *  - learned_stack_cap: cells the NB_OPEN_LEARNED traversal's per-warp stack may hold, 1 ..
 *    NB_LEARNED_STACK_CAP (0 = all); a walk that would exceed it stops and sets the stack bit
 *    (nb_sync returns NB_ERR_STACK_OVERFLOW).
 * Results of a launch that hit a limit are undefined; the context stays usable. */
#define NB_FAULT_DROP_LOOKBACK 1u
#define NB_LEARNED_STACK_CAP 1024u
nb_status nb_ctx_set_fault_hooks(nb_ctx* ctx, long long wait_limit, unsigned int flags,
                                 unsigned int learned_stack_cap);

/* ---------------------------------------------------------------------------------------------
 * Naive all-pairs acceleration.
 * Replaces NaiveAlgorithm::computeAccelerations_opt_{0,1,2} (NaiveAlgorithm.hpp:31-53,
 * NaiveAlgorithm.cpp:262-482): a_i = G * sum_j m_j r_ij / (|r_ij|^2 + eps2)^{3/2}, self pair
 * included, j ascending per body, G applied once at the end.
 * block_size: the reference's --block_size (j-tile and work-group size). It is a tuning hint
 * only here (0 = automatic); results do not depend on it.
 * ------------------------------------------------------------------------------------------- */
nb_status nb_naive_accel(nb_ctx* ctx, const double* m, const double* x, const double* y,
                         const double* z, double* ax, double* ay, double* az, uint32_t n,
                         double G, double eps2, nb_precision prec, int block_size,
                         nb_stream_t stream);

/* Same, for target bodies [i_begin, i_end) only (sharding hook: each GPU of a replicated run
 * computes its own range against all n sources). */
nb_status nb_naive_accel_range(nb_ctx* ctx, const double* m, const double* x, const double* y,
                               const double* z, double* ax, double* ay, double* az, uint32_t n,
                               uint32_t i_begin, uint32_t i_end, double G, double eps2,
                               nb_precision prec, nb_stream_t stream);

/* FP64 accelerations of listed target bodies: ax[t] for body targets[t] (all DEVICE arrays); the
 * FP64 GPU oracle for sampled-body force errors at large N. */
nb_status nb_naive_accel_targets(nb_ctx* ctx, const double* m, const double* x, const double* y,
                                 const double* z, uint32_t n, const uint32_t* targets,
                                 uint32_t n_targets, double* ax, double* ay, double* az, double G,
                                 double eps2, nb_stream_t stream);

/* Tile configuration of the FP32-compensated pair kernel used by nb_naive_accel (process-wide;
 * 0..NB_PAIR_CONFIG_COUNT-1, see nb_batch_info for the shapes; 0 = default). */
#define NB_PAIR_CONFIG_COUNT 8
nb_status nb_naive_set_pair_config(int config);

/* Symmetric pair kernel for nb_naive_accel (NB_F32C, NB_F64 and NB_DF64) over all bodies of a
 * system (no reference counterpart; the reference evaluates every ordered pair,
 * NaiveAlgorithm.cpp:318-346): each unordered pair is evaluated once and added to both bodies,
 * per-body sums combined in a fixed order (deterministic; FP32 sums compensated). mode: 0 = never
 * (always the one-sided kernels), 1 = automatic (default: systems large enough to fill the GPU,
 * partial buffers of at most 4 GiB), 2 = always for full ranges. Tile shapes (warps, bodies per
 * lane, j-tile): config_f32 0..NB_SYM_CONFIG_COUNT-1 = (8,12,128) (default), (4,12,256),
 * (4,12,128), (4,16,128), (8,8,256), (4,8,256), (8,6,256), (2,12,128); config_f64
 * 0..NB_SYM64_CONFIG_COUNT-1 = (4,2,64), (4,4,64), (8,2,64), (4,2,128); config_df
 * 0..NB_SYMDF_CONFIG_COUNT-1 = (4,2,64), (4,4,64). In mode 1 the FP64 and double-float shapes
 * are chosen by the library (FP64: the larger I-block when it still fills the GPU; double-float:
 * the faster (4,2,64) unless its partials exceed the cap). Process-wide; nb_naive_accel_range
 * with a partial range always uses the one-sided kernels. */
#define NB_SYM_CONFIG_COUNT 8
#define NB_SYM64_CONFIG_COUNT 4
#define NB_SYMDF_CONFIG_COUNT 2
nb_status nb_naive_set_symmetric(int mode, int config_f32, int config_f64, int config_df);

/* ---------------------------------------------------------------------------------------------
 * Batched ensembles (the batching form of the method; the reference simulates one system).
 * Many independent systems of uneven size in concatenated FP64 arrays (system s owns bodies
 * [sum(counts[0..s)), +counts[s])). Forces use FP32 pair math with compensated accumulation, one
 * persistent stream-K launch for all systems; integration stays FP64 (nb_leapfrog_* over all
 * bodies). The batch owns every buffer its launches need, so steps can be captured in a graph.
 * ------------------------------------------------------------------------------------------- */
typedef struct nb_batch nb_batch;
typedef struct nb_graph nb_graph;
nb_status nb_batch_create(nb_ctx* ctx, uint32_t n_systems, const uint32_t* counts_host,
                          nb_batch** out);
nb_status nb_batch_destroy(nb_batch* batch);
/* Batch tile configurations: 0..NB_PAIR_CONFIG_COUNT-1 run the one-sided pair kernel (every
 * ordered pair), NB_PAIR_CONFIG_COUNT.. NB_BATCH_CONFIG_COUNT-1 the symmetric kernel's shapes
 * (each unordered pair once, added to both bodies; same order as nb_naive_set_symmetric). */
#define NB_BATCH_CONFIG_COUNT 16
/* Total bodies and the current tile configuration: CTA threads, targets (bodies) per thread,
 * j-tile. */
nb_status nb_batch_info(const nb_batch* batch, uint32_t* n_total, int* config, int* threads,
                        int* targets_per_thread, int* j_tile);
nb_status nb_batch_set_config(nb_ctx* ctx, nb_batch* batch, int config);
nb_status nb_batch_naive_accel(nb_ctx* ctx, nb_batch* batch, const double* m, const double* x,
                               const double* y, const double* z, double* ax, double* ay,
                               double* az, double G, double eps2, nb_stream_t stream);
/* Autotuner (synchronous): times every tile configuration of both kernels on these arrays (reps
 * launches each, CUDA events), keeps the fastest; ms_per_config (host, NB_BATCH_CONFIG_COUNT
 * entries) optional. */
nb_status nb_batch_autotune(nb_ctx* ctx, nb_batch* batch, const double* m, const double* x,
                            const double* y, const double* z, double* ax, double* ay, double* az,
                            double G, double eps2, int reps, float* ms_per_config, int* chosen);
/* Captures `steps` leapfrog steps (kick-drift, batch accelerations, kick) of the batch into a
 * CUDA graph; nb_graph_launch replays them on a stream. */
nb_status nb_batch_graph_create(nb_ctx* ctx, nb_batch* batch, const double* m, double* x,
                                double* y, double* z, double* vx, double* vy, double* vz,
                                double* vhx, double* vhy, double* vhz, double* ax, double* ay,
                                double* az, double G, double eps2, double dt, int steps,
                                nb_graph** out);
nb_status nb_graph_launch(nb_graph* graph, nb_stream_t stream);
nb_status nb_graph_destroy(nb_graph* graph);

/* ---------------------------------------------------------------------------------------------
 * Leapfrog kick-drift-kick.
 * nb_leapfrog_kick_drift replaces "leapfrog integration part 1" (NaiveAlgorithm.cpp:140-164,
 * BarnesHutAlgorithm.cpp:157-182): v_half = v + a*(dt/2); x = x + v_half*dt.
 * nb_leapfrog_kick replaces "part 2" (NaiveAlgorithm.cpp:206-222, BarnesHutAlgorithm.cpp:223-239):
 * v = v_half + a*(dt/2).
 * nb_leapfrog_kick_kick_drift fuses part 2 of one step with part 1 of the next (identical
 * results, one pass over memory).
 * ------------------------------------------------------------------------------------------- */
nb_status nb_leapfrog_kick_drift(nb_ctx* ctx, double* vhx, double* vhy, double* vhz,
                                 const double* vx, const double* vy, const double* vz, double* x,
                                 double* y, double* z, const double* ax, const double* ay,
                                 const double* az, uint32_t n, double dt, nb_stream_t stream);
nb_status nb_leapfrog_kick(nb_ctx* ctx, double* vx, double* vy, double* vz, const double* vhx,
                           const double* vhy, const double* vhz, const double* ax,
                           const double* ay, const double* az, uint32_t n, double dt,
                           nb_stream_t stream);
nb_status nb_leapfrog_kick_kick_drift(nb_ctx* ctx, double* vx, double* vy, double* vz,
                                      double* vhx, double* vhy, double* vhz, double* x, double* y,
                                      double* z, const double* ax, const double* ay,
                                      const double* az, uint32_t n, double dt,
                                      nb_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * Energy. Replaces nBodyAlgorithm::computeEnergy (nBodyAlgorithm.cpp:11-86): kinetic
 * sum 0.5 m v^2, potential -sum_{i<j} G m_i m_j / r WITHOUT softening, in FP64.
 * out_dev: DEVICE pointer to 4 doubles {kinetic, potential, total, virial = 2K/|U|}.
 * ------------------------------------------------------------------------------------------- */
nb_status nb_energy(nb_ctx* ctx, const double* m, const double* x, const double* y,
                    const double* z, const double* vx, const double* vy, const double* vz,
                    uint32_t n, double G, double* out_dev, nb_stream_t stream);

/* Energy for callers that cannot let the library allocate device memory (no counterpart in the
 * reference). Same result as nb_energy, but needs no context and never calls cudaMalloc,
 * cudaFree or any allocating routine: the per-block partial sums live in a fixed 128 KiB
 * file-scope device array, present on every GPU that loads the library until the process exits.
 * Limit: n <= NB_ENERGY_NOALLOC_MAX_N bodies (larger n returns NB_ERR_INVALID_ARG).
 * Runs on the current device. Its first call on each device looks up that array's device
 * address (cudaGetSymbolAddress); with CUDA's lazy module loading that lookup is also what loads
 * the library's device code on that device, and loading it is when the driver allocates the
 * fixed array. So make one call per device during initialisation, before any stream capture and
 * before the caller's memory pool takes the device's memory; later calls allocate nothing. The
 * address is kept for the life of the process: a cudaDeviceReset (or anything else that tears
 * down the device's primary context) invalidates it, and the entry point must not be called on
 * that device afterwards. All calls share the array: calls that overlap on the GPU race, so
 * serialise them (one stream at a time). out_dev: DEVICE pointer to 4 doubles {kinetic,
 * potential, total, virial}. */
#define NB_ENERGY_NOALLOC_MAX_N 1048576u
nb_status nb_energy_noalloc(const double* m, const double* x, const double* y, const double* z,
                            const double* vx, const double* vy, const double* vz, uint32_t n,
                            double G, double* out_dev, nb_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * AABB. Replaces BarnesHutOctree::computeMinMaxValuesAABB (BarnesHutOctree.cpp:45-191),
 * including its conventions: the box always contains the origin (the reference's partial
 * accumulators start at 0.0) and is made a cube by padding the shorter axes equally, ties
 * resolved x, y, z. out_dev: DEVICE pointer to 7 doubles {min_x, min_y, min_z, max_x, max_y,
 * max_z, edge}; bit-identical to the reference's host arithmetic.
 * ------------------------------------------------------------------------------------------- */
nb_status nb_aabb(nb_ctx* ctx, const double* x, const double* y, const double* z, uint32_t n,
                  double* out_dev, nb_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * Barnes-Hut.
 * The tree is the reference's point-region octree over the cube AABB (one body per leaf, the
 * octant rule of ParallelOctreeTopDownSubtrees.cpp:400-414 with its FP64 midpoint recurrence,
 * so every body lands in the same octant at every level), stored compressed (no empty children,
 * single-child chains folded into their deepest cell, which the reference's traversal accepts
 * or opens identically) in DFS pre-order with skip links. Node sums are the reference's: children
 * summed in octant order 0..7 in FP64 (BarnesHutOctree.cpp:304-311).
 * ------------------------------------------------------------------------------------------- */
typedef struct nb_bh_params {
    double theta;                 /* opening angle: a cell is accepted when edge/d < theta
                                     (reference --theta, default 1.05) */
    uint32_t storage_size_param;  /* reference --storage_size_param (default 16). The reference
                                     needs storage_size_param*N node slots; this tree needs at
                                     most 2N-1 and reports the reference's count in stats */
    uint32_t stack_size_param;    /* reference --stack_size_param (default 16); the traversal
                                     here is stackless, the value is recorded only */
    int max_build_level;          /* reference --max_level_top_octree (default 7); the tree shape
                                     and all results are independent of it */
    int sort_bodies;              /* reference --sort_bodies (default 1): bodies are traversed in
                                     tree order; results are independent of it */
} nb_bh_params;

typedef enum nb_opening {
    NB_OPEN_THETA = 0,        /* the reference's per-body rule (BarnesHutAlgorithm.cpp:355-359):
                                 accept if edge*rsqrt(d^2) < theta or the node is a body leaf;
                                 contributions summed in the reference's DFS order */
    NB_OPEN_THETA_GROUP = 1,  /* per group of 32 bodies adjacent in tree order: a cell is opened
                                 for the whole group when any member's rule would open it
                                 (never less accurate than NB_OPEN_THETA) */
    NB_OPEN_LEARNED = 2       /* per (32-body group, cell) decision of a trained MLP, with the
                                 group theta rule as fallback */
} nb_opening;

typedef struct nb_bh_tree nb_bh_tree;

typedef struct nb_bh_stats {
    uint32_t n;                   /* bodies of the last build */
    uint32_t node_count;          /* nodes of the compressed tree (<= 2n-1) */
    uint32_t max_depth;           /* deepest leaf level (root = 0) */
    uint32_t ref_node_count;      /* nodes the reference's linearised octree holds for the same
                                     bodies (nextFreeNodeID: 1 + 8 * internal cells) */
    double aabb[7];               /* min x,y,z, max x,y,z, edge */
} nb_bh_stats;

/* Reference-layout export for parity checks (BarnesHutOctree.hpp:33-95). Caller-owned HOST
 * arrays of capacity `capacity` nodes (octants: 8*capacity, plane o at octants[o*capacity]) and
 * n bodies (sorted_bodies). Node ids: root 0, the 8 children of a split cell allocated together
 * in the reference's slot order (octants 5,7,4,6,1,3,0,2), cells numbered breadth-first. */
typedef struct nb_bh_ref_layout {
    uint32_t capacity;
    uint32_t node_count;          /* out */
    uint32_t* octants;
    double *edge, *min_x, *min_y, *min_z;
    uint32_t* body_of_node;       /* n = empty or internal */
    int* node_is_leaf;
    double *sum_masses, *com_x, *com_y, *com_z;  /* com = mass-weighted numerators */
    uint32_t* body_count;
    uint32_t* sorted_bodies;      /* sortedBodiesInOrder (BarnesHutOctree.cpp:550-613) */
} nb_bh_ref_layout;

nb_status nb_bh_params_default(nb_bh_params* out);
/* Allocates a tree for up to n_max bodies (device memory, ~0.5 KB per body). */
nb_status nb_bh_tree_create(nb_ctx* ctx, uint32_t n_max, const nb_bh_params* params,
                            nb_bh_tree** out);
nb_status nb_bh_tree_destroy(nb_bh_tree* tree);
nb_status nb_bh_tree_set_theta(nb_bh_tree* tree, double theta);

/* Node records later builds compute (no reference counterpart: the reference keeps only the
 * sums). The FP32 records (centres relative to the box centre, G*mass, edge^2) are always built;
 * further sets by bit:
 *   NB_REC_FP64    FP64 centres (the IEEE quotients of the reference's sums), masses, edges: the
 *                  per-body rule in NB_F64_IEEE, NB_F64 and NB_DF64, the FP64 group rule,
 *                  nb_bh_count_interactions and nb_bh_generate_pairs;
 *   NB_REC_DF      the further FP32 terms of centres and G*mass (exact triple-floats): NB_DF64;
 *   NB_REC_LEARNED per-node spread, count and first body, FP32 body copies in tree order:
 *                  NB_OPEN_LEARNED and nb_bh_generate_pairs.
 * Default NB_REC_ALL. Without NB_REC_FP64 the FP32 centres come from a reciprocal instead of the
 * IEEE quotients (within an FP32 rounding of them). A call whose records the last build did not
 * compute fails with NB_ERR_INVALID_ARG.
 * NB_BUILD_QUANTIZED_KEYS (same mask; for runs whose forces need no reference-exact cells, such
 * as the FP32 and learned rules): bodies are placed by 42-bit quantized coordinates instead of
 * the reference's FP64 midpoint recurrence (BarnesHutOctree.cpp, ParallelOctreeTopDownSubtrees
 * .cpp:219-428); the cells then differ from the reference's only for bodies within FP64 rounding
 * of a cell midpoint. Off by default. */
#define NB_REC_FP64 1u
#define NB_REC_DF 2u
#define NB_REC_LEARNED 4u
#define NB_REC_ALL 7u
#define NB_BUILD_QUANTIZED_KEYS 8u
nb_status nb_bh_set_records(nb_bh_tree* tree, unsigned int mask);

/* Replaces BarnesHutOctree::buildOctree (BarnesHutOctree.hpp:102-103;
 * ParallelOctreeTopDownSubtrees.cpp:15-93): AABB, octree, centre of mass, body order.
 * G only scales the FP32 traversal records (masses stay in the caller's units). */
nb_status nb_bh_build(nb_ctx* ctx, nb_bh_tree* tree, const double* m, const double* x,
                      const double* y, const double* z, uint32_t n, double G,
                      nb_stream_t stream);
/* Captures `steps` Barnes-Hut leapfrog steps (kick-drift, nb_bh_build, nb_bh_accel with the
 * given opening rule and precision, kick) of n bodies into a CUDA graph; nb_graph_launch replays
 * them (one launch for all of a step's kernels), nb_graph_destroy frees it. The arrays, the tree
 * and its policy are bound at capture time. Phase timing must be off. */
nb_status nb_bh_graph_create(nb_ctx* ctx, nb_bh_tree* tree, const double* m, double* x, double* y,
                             double* z, double* vx, double* vy, double* vz, double* vhx,
                             double* vhy, double* vhz, double* ax, double* ay, double* az,
                             uint32_t n, double G, double eps2, double dt, int steps,
                             nb_opening opening, nb_precision prec, nb_graph** out);

/* Phase timing of nb_bh_build (for measurements): when enabled, each build records CUDA events at
 * its phase boundaries; nb_bh_build_phase_ms (synchronous) returns the last build's durations
 * in ms: [0] AABB, [1] keys, [2] radix sort, [3] cells (runs, splits, counts, scan, emit),
 * [4] centre of mass and node records. */
nb_status nb_bh_set_phase_timing(nb_bh_tree* tree, int enable);
nb_status nb_bh_build_phase_ms(nb_bh_tree* tree, float* ms5);

/* Replaces BarnesHutAlgorithm::computeAccelerations (BarnesHutAlgorithm.hpp:43-46,
 * BarnesHutAlgorithm.cpp:280-401) for the bodies of the last build (same x, y, z). The tree holds
 * the persistent traversals' work counters, each body's walk length from the last per-body
 * traversal (NB_OPEN_THETA with NB_F64, NB_F64_IEEE or NB_DF64), from which the next one of the
 * same bodies groups its bodies, and for NB_OPEN_LEARNED the cost of each group of 32 bodies from
 * the last learned traversal, from which the next one takes its costliest groups first; the
 * results do not depend on either order. Calls on one tree therefore run one after another (on one
 * stream, or ordered by events), never concurrently. */
nb_status nb_bh_accel(nb_ctx* ctx, const nb_bh_tree* tree, const double* x, const double* y,
                      const double* z, double* ax, double* ay, double* az, double G, double eps2,
                      nb_opening opening, nb_precision prec, nb_stream_t stream);

/* Execution schedule of the per-body FP64 traversal (process-wide): 0 (default) = every lane
 * walks its own body's DFS sequence with an FP32 pre-test of the opening rule; 1 = the warp walks
 * the union of its 32 sequences in lockstep. Results are identical; this exists for comparison. */
nb_status nb_bh_set_schedule(int lockstep);

/* Synchronous. */
nb_status nb_bh_tree_stats(nb_bh_tree* tree, nb_bh_stats* out);
nb_status nb_bh_export_ref_layout(nb_bh_tree* tree, nb_bh_ref_layout* out);
/* Per node in DFS order (HOST arrays of node_count entries, any may be NULL): first sorted position
 * of its bodies, body count, level, body id (NB leaves) or 0xffffffff. */
nb_status nb_bh_export_node_ranges(nb_bh_tree* tree, uint32_t* first, uint32_t* count,
                                   uint32_t* level, uint32_t* body);
/* Sorted body ids (tree DFS order) and per-body leaf depth, HOST arrays of n entries. */
nb_status nb_bh_export_order(nb_bh_tree* tree, uint32_t* ids_in_dfs_order, uint32_t* leaf_level);

/* Work model of a traversal: total cells accepted (interactions) into out_dev[0] and opened into
 * out_dev[1] (DEVICE pointer to 2 uint64) under the per-body or the group theta rule. */
nb_status nb_bh_count_interactions(nb_ctx* ctx, const nb_bh_tree* tree, const double* x,
                                   const double* y, const double* z, nb_opening opening,
                                   unsigned long long* out_dev, nb_stream_t stream);

/* Synchronous FMA-throughput probe of the current GPU: FP64 (fp64 = 1) or FP32 flop/s (2 per FMA).
 * The measured pipe peaks the pair and traversal kernels are reported against. */
nb_status nb_util_fma_peak(nb_ctx* ctx, int fp64, double* flops_per_s);

/* ---------------------------------------------------------------------------------------------
 * Learned opening policy (the learned form of the method; no reference counterpart).
 * Network: 8 features -> 32 -> 32 -> 1 (ReLU), NB_MLP_PARAMS FP32 parameters in the layout
 * W1[8][32], b1[32], W2[32][32], b2[32], w3[32], b3 (all DEVICE arrays). It predicts
 * y = log10(worst relative force error of accepting a cell for a 32-body group) / 5.
 * ------------------------------------------------------------------------------------------- */
#define NB_MLP_PARAMS 1377
#define NB_MLP_FEATURES 8
nb_status nb_mlp_param_count(uint32_t* out);
/* Mean-squared-error loss and its gradient over rows idx[0..n) (idx NULL: rows 0..n) of X [n][8]
 * and Y [n]; grad (NB_MLP_PARAMS floats) and loss (1 float) are overwritten. FP32. */
nb_status nb_mlp_loss_grad(nb_ctx* ctx, const float* params, const float* X, const float* Y,
                           const uint32_t* idx, uint32_t n, float* grad, float* loss,
                           nb_stream_t stream);
/* One Adam step (step = 1, 2, ...) on params with moment buffers m, v (NB_MLP_PARAMS each). */
nb_status nb_mlp_adam(nb_ctx* ctx, float* params, float* m, float* v, const float* grad,
                      float lr, float beta1, float beta2, float eps, int step, nb_stream_t stream);
/* Network outputs for X [n][8]: FP32 CUDA cores, or (bf16_tensor_cores = 1) the BF16 mma.sync
 * path the traversal uses. */
nb_status nb_mlp_predict(nb_ctx* ctx, const float* params, const float* X, uint32_t n,
                         float* out, int bf16_tensor_cores, nb_stream_t stream);
/* Labelled training pairs from a built tree: a group theta_gen walk samples (32-body group, cell)
 * pairs (fraction sample_fraction, seeded); for each, features and the label log10(max over the
 * group of |exact cell force - monopole| / |a_body|) / 5, with |a_body| from ax, ay, az
 * (reference accelerations). Writes at most max_pairs rows; *count_dev (DEVICE) = pairs found
 * (may exceed max_pairs). Cells with more than count_cap bodies are not sampled. pairs_out
 * (optional DEVICE, 2*max_pairs u32) receives each row's (group = first sorted position / 32,
 * node in DFS order). */
nb_status nb_bh_generate_pairs(nb_ctx* ctx, const nb_bh_tree* tree, const double* m,
                               const double* x, const double* y, const double* z,
                               const double* ax, const double* ay, const double* az, double G,
                               double eps2, double theta_gen, double sample_fraction,
                               uint32_t seed, uint32_t count_cap, uint32_t max_pairs,
                               float* features, float* labels, uint32_t* count_dev,
                               uint32_t* pairs_out, nb_stream_t stream);
/* Policy of NB_OPEN_LEARNED: accept a cell when the network predicts an error below tau;
 * cells with more than count_cap bodies use the group theta rule with theta_fallback. The
 * traversal reads |a| of the previous step from the ax, ay, az arrays it then overwrites.
 * params_dev NULL selects the same walk with the group theta rule (theta_fallback) in place of
 * the network: the method without it.
 * flags: NB_POLICY_BOUND_ACCEPT accepts, before the network is asked, every cell whose analytic
 * monopole error bound (multipole series, bodies within sqrt(3) * edge of the centre of mass)
 * relative to the group's smallest |a| is below tau. */
#define NB_POLICY_BOUND_ACCEPT 1u
nb_status nb_bh_set_policy(nb_bh_tree* tree, const float* params_dev, float log10_tau,
                           double theta_fallback, uint32_t count_cap, uint32_t flags);
/* Opening-policy files (host-side, synchronous): a trained network (NB_MLP_PARAMS FP32 values in
 * HOST memory, the layout above) with the nb_bh_set_policy settings it was tuned for. Text
 * format, one item per line: "nbody-gb300 opening policy 1", "network 8 32 32 1 relu",
 * "log10_tau <v>", "theta_fallback <v>", "count_cap <v>", "flags <v>", "params 1377", then the
 * 1377 parameters (9 significant digits: FP32 values round-trip exactly). nb_policy_load rejects
 * any other shape or a malformed file with NB_ERR_INVALID_ARG. The host driver reads these files
 * (nbody_sim --opening=learned --policy=<file>). */
nb_status nb_policy_save(const char* path, const float* params_host, float log10_tau,
                         double theta_fallback, uint32_t count_cap, uint32_t flags);
nb_status nb_policy_load(const char* path, float* params_host, float* log10_tau,
                         double* theta_fallback, uint32_t* count_cap, uint32_t* flags);
/* NB_OPEN_LEARNED traversal that also counts, into 4 DEVICE uint64: body-cell interactions
 * (counters_dev[0]), cells decided by the policy (network, or theta rule when the policy has no
 * network) ([1]), cells visited ([2]) and walk steps of up to 32 cells ([3]), summed over
 * groups. */
nb_status nb_bh_accel_learned_counted(nb_ctx* ctx, const nb_bh_tree* tree, const double* x,
                                      const double* y, const double* z, double* ax, double* ay,
                                      double* az, double eps2, unsigned long long* counters_dev,
                                      nb_stream_t stream);

/* Building blocks exposed for tests: stable radix sort of (u64, u32) device pairs on bits
 * [begin_bit, end_bit) and an exclusive scan of u32 device data (out has n+1 entries). These two
 * allocate their temporaries with cudaMallocAsync on the stream. */
nb_status nb_util_radix_sort_pairs(nb_ctx* ctx, uint64_t* keys, uint32_t* vals, uint32_t n,
                                   int begin_bit, int end_bit, nb_stream_t stream);
nb_status nb_util_exclusive_scan_u32(nb_ctx* ctx, const uint32_t* in, uint32_t* out, uint32_t n,
                                     nb_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* NBODY_GB300_H */
