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
    NB_F32C = 2       /* FP32 pair math, compensated (TwoSum) per-body accumulation */
} nb_precision;

#define NB_MAX_TREE_DEPTH 42

typedef struct nb_ctx nb_ctx;

nb_status nb_ctx_create(int device, nb_ctx** out);
nb_status nb_ctx_destroy(nb_ctx* ctx);
/* Blocks until all work of `stream` has finished and reports any device-side error word. */
nb_status nb_sync(nb_ctx* ctx, nb_stream_t stream);
const char* nb_last_error_string(void);
const char* nb_version(void);

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

/* ---------------------------------------------------------------------------------------------
 * AABB. Replaces BarnesHutOctree::computeMinMaxValuesAABB (BarnesHutOctree.cpp:45-191),
 * including its conventions: the box always contains the origin (the reference's partial
 * accumulators start at 0.0) and is made a cube by padding the shorter axes equally, ties
 * resolved x, y, z. out_dev: DEVICE pointer to 7 doubles {min_x, min_y, min_z, max_x, max_y,
 * max_z, edge}; bit-identical to the reference's host arithmetic.
 * ------------------------------------------------------------------------------------------- */
nb_status nb_aabb(nb_ctx* ctx, const double* x, const double* y, const double* z, uint32_t n,
                  double* out_dev, nb_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* NBODY_GB300_H */
