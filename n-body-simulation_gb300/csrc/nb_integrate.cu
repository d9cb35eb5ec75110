// nb_integrate.cu -- leapfrog kick-drift-kick, energy and AABB kernels (all FP64).
#include <mutex>

#include "nb_internal.cuh"

namespace {

constexpr int EW_THREADS = 256;

// NaiveAlgorithm.cpp:154-163 / BarnesHutAlgorithm.cpp:171-181. Each statement is a separately
// rounded multiply and add, exactly as the reference writes it.
__global__ void kick_drift_kernel(double* __restrict__ vhx, double* __restrict__ vhy,
                                  double* __restrict__ vhz, const double* __restrict__ vx,
                                  const double* __restrict__ vy, const double* __restrict__ vz,
                                  double* __restrict__ x, double* __restrict__ y,
                                  double* __restrict__ z, const double* __restrict__ ax,
                                  const double* __restrict__ ay, const double* __restrict__ az,
                                  uint32_t n, double dt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double h = dt / 2.0;
    const double hx = __dadd_rn(vx[i], __dmul_rn(ax[i], h));
    const double hy = __dadd_rn(vy[i], __dmul_rn(ay[i], h));
    const double hz = __dadd_rn(vz[i], __dmul_rn(az[i], h));
    vhx[i] = hx;
    vhy[i] = hy;
    vhz[i] = hz;
    x[i] = __dadd_rn(x[i], __dmul_rn(hx, dt));
    y[i] = __dadd_rn(y[i], __dmul_rn(hy, dt));
    z[i] = __dadd_rn(z[i], __dmul_rn(hz, dt));
}

// NaiveAlgorithm.cpp:217-221 / BarnesHutAlgorithm.cpp:234-238.
__global__ void kick_kernel(double* __restrict__ vx, double* __restrict__ vy,
                            double* __restrict__ vz, const double* __restrict__ vhx,
                            const double* __restrict__ vhy, const double* __restrict__ vhz,
                            const double* __restrict__ ax, const double* __restrict__ ay,
                            const double* __restrict__ az, uint32_t n, double dt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double h = dt / 2.0;
    vx[i] = __dadd_rn(vhx[i], __dmul_rn(ax[i], h));
    vy[i] = __dadd_rn(vhy[i], __dmul_rn(ay[i], h));
    vz[i] = __dadd_rn(vhz[i], __dmul_rn(az[i], h));
}

// Part 2 of one step followed by part 1 of the next: v = vh + a*dt/2; vh = v + a*dt/2;
// x += vh*dt. The same roundings as running the two kernels back to back.
__global__ void kick_kick_drift_kernel(double* __restrict__ vx, double* __restrict__ vy,
                                       double* __restrict__ vz, double* __restrict__ vhx,
                                       double* __restrict__ vhy, double* __restrict__ vhz,
                                       double* __restrict__ x, double* __restrict__ y,
                                       double* __restrict__ z, const double* __restrict__ ax,
                                       const double* __restrict__ ay,
                                       const double* __restrict__ az, uint32_t n, double dt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double h = dt / 2.0;
    const double kx = __dmul_rn(ax[i], h), ky = __dmul_rn(ay[i], h), kz = __dmul_rn(az[i], h);
    const double nvx = __dadd_rn(vhx[i], kx), nvy = __dadd_rn(vhy[i], ky),
                 nvz = __dadd_rn(vhz[i], kz);
    vx[i] = nvx;
    vy[i] = nvy;
    vz[i] = nvz;
    const double hx = __dadd_rn(nvx, kx), hy = __dadd_rn(nvy, ky), hz = __dadd_rn(nvz, kz);
    vhx[i] = hx;
    vhy[i] = hy;
    vhz[i] = hz;
    x[i] = __dadd_rn(x[i], __dmul_rn(hx, dt));
    y[i] = __dadd_rn(y[i], __dmul_rn(hy, dt));
    z[i] = __dadd_rn(z[i], __dmul_rn(hz, dt));
}

// ---------------------------------------------------------------------------------------------
// Energy: per target body j the kinetic term and the potential sum over sources i < j
// (nBodyAlgorithm.cpp:48-64), then a fixed-order reduction (deterministic).
// ---------------------------------------------------------------------------------------------
constexpr int EN_THREADS = 128;

__global__ void __launch_bounds__(EN_THREADS)
energy_kernel(const double* __restrict__ m, const double* __restrict__ x,
              const double* __restrict__ y, const double* __restrict__ z,
              const double* __restrict__ vx, const double* __restrict__ vy,
              const double* __restrict__ vz, uint32_t n, double G, double2* __restrict__ part) {
    __shared__ double sx[EN_THREADS], sy[EN_THREADS], sz[EN_THREADS], sm[EN_THREADS];
    __shared__ double red_k[EN_THREADS / 32], red_p[EN_THREADS / 32];
    // blocks in reverse so the longest triangles start first
    const uint32_t blk = gridDim.x - 1 - blockIdx.x;
    const uint32_t j = blk * EN_THREADS + threadIdx.x;
    const bool active = j < n;
    double px = 0, py = 0, pz = 0, mj = 0, ek = 0, ep = 0;
    if (active) {
        px = x[j];
        py = y[j];
        pz = z[j];
        mj = m[j];
        const double v = vx[j] * vx[j] + vy[j] * vy[j] + vz[j] * vz[j];
        ek = 0.5 * mj * v;
    }
    const uint32_t j_last = min(n, (blk + 1) * EN_THREADS);
    for (uint32_t k = 0; k < j_last; k += EN_THREADS) {
        const uint32_t i = k + threadIdx.x;
        if (i < n) {
            sx[threadIdx.x] = x[i];
            sy[threadIdx.x] = y[i];
            sz[threadIdx.x] = z[i];
            sm[threadIdx.x] = m[i];
        }
        __syncthreads();
        if (active) {
            const uint32_t cnt = min((uint32_t)EN_THREADS, j > k ? j - k : 0u);
            for (uint32_t ii = 0; ii < cnt; ++ii) {
                const double rx = px - sx[ii], ry = py - sy[ii], rz = pz - sz[ii];
                const double r2 = fma(rx, rx, fma(ry, ry, rz * rz));
                ep = fma(G * sm[ii] * mj, nb_rsqrt_f64(r2), ep);
            }
        }
        __syncthreads();
    }
    // block reduction in a fixed order
    for (int off = 16; off > 0; off >>= 1) {
        ek += __shfl_down_sync(0xffffffffu, ek, off);
        ep += __shfl_down_sync(0xffffffffu, ep, off);
    }
    if ((threadIdx.x & 31) == 0) {
        red_k[threadIdx.x >> 5] = ek;
        red_p[threadIdx.x >> 5] = ep;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double k2 = 0, p2 = 0;
        for (int w = 0; w < EN_THREADS / 32; ++w) {
            k2 += red_k[w];
            p2 += red_p[w];
        }
        part[blk] = make_double2(k2, p2);
    }
}

__global__ void energy_finalize(const double2* __restrict__ part, uint32_t nparts,
                                double* __restrict__ out) {
    __shared__ double sk[256], sp[256];
    double k = 0, p = 0;
    for (uint32_t b = threadIdx.x; b < nparts; b += 256) {
        k += part[b].x;
        p += part[b].y;
    }
    sk[threadIdx.x] = k;
    sp[threadIdx.x] = p;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sk[threadIdx.x] += sk[threadIdx.x + s];
            sp[threadIdx.x] += sp[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double ek = sk[0], ep = -sp[0];
        out[0] = ek;
        out[1] = ep;
        out[2] = ek + ep;
        out[3] = (2.0 * ek) / fabs(ep);
    }
}

// ---------------------------------------------------------------------------------------------
// AABB: order-preserving integer images of the doubles make min/max integer-pipe work; every
// accumulator starts at the image of 0.0 (the reference's zero-initialised partials), the last
// block to finish reduces the per-block partials in a fixed order and applies the cube rule of
// BarnesHutOctree.cpp:161-190 with separately rounded IEEE operations.
// ---------------------------------------------------------------------------------------------
constexpr int AABB_THREADS = 256;

__device__ __forceinline__ long long ord_of(double v) {
    const long long b = __double_as_longlong(v);
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double val_of(long long o) {
    return __longlong_as_double(o >= 0 ? o : (o ^ 0x7fffffffffffffffLL));
}

struct MinMax6 {
    long long v[6];  // min x, y, z (as ordered ints), max x, y, z
};

__device__ void cube_rule(double min_x, double min_y, double min_z, double max_x, double max_y,
                          double max_z, double* out) {
    const double x_len = fabs(__dsub_rn(max_x, min_x));
    const double y_len = fabs(__dsub_rn(max_y, min_y));
    const double z_len = fabs(__dsub_rn(max_z, min_z));
    const double edge = fmax(x_len, fmax(y_len, z_len));
    if (edge == x_len) {
        min_z = __dsub_rn(min_z, __dsub_rn(edge, z_len) / 2);
        min_y = __dsub_rn(min_y, __dsub_rn(edge, y_len) / 2);
        max_z = __dadd_rn(max_z, __dsub_rn(edge, z_len) / 2);
        max_y = __dadd_rn(max_y, __dsub_rn(edge, y_len) / 2);
    } else if (edge == y_len) {
        min_x = __dsub_rn(min_x, __dsub_rn(edge, x_len) / 2);
        min_z = __dsub_rn(min_z, __dsub_rn(edge, z_len) / 2);
        max_x = __dadd_rn(max_x, __dsub_rn(edge, x_len) / 2);
        max_z = __dadd_rn(max_z, __dsub_rn(edge, z_len) / 2);
    } else {
        min_x = __dsub_rn(min_x, __dsub_rn(edge, x_len) / 2);
        min_y = __dsub_rn(min_y, __dsub_rn(edge, y_len) / 2);
        max_x = __dadd_rn(max_x, __dsub_rn(edge, x_len) / 2);
        max_y = __dadd_rn(max_y, __dsub_rn(edge, y_len) / 2);
    }
    out[0] = min_x;
    out[1] = min_y;
    out[2] = min_z;
    out[3] = max_x;
    out[4] = max_y;
    out[5] = max_z;
    out[6] = edge;
}

__global__ void __launch_bounds__(AABB_THREADS)
aabb_kernel(const double* __restrict__ x, const double* __restrict__ y,
            const double* __restrict__ z, uint32_t n, MinMax6* __restrict__ part,
            unsigned int* __restrict__ counter, double* __restrict__ out) {
    const long long zero = ord_of(0.0);
    long long mn[3] = {zero, zero, zero}, mx[3] = {zero, zero, zero};
    const double* p[3] = {x, y, z};
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const long long o = ord_of(p[a][i]);
            mn[a] = min(mn[a], o);
            mx[a] = max(mx[a], o);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        for (int off = 16; off > 0; off >>= 1) {
            mn[a] = min(mn[a], __shfl_down_sync(0xffffffffu, mn[a], off));
            mx[a] = max(mx[a], __shfl_down_sync(0xffffffffu, mx[a], off));
        }
    }
    __shared__ MinMax6 warp_part[AABB_THREADS / 32];
    __shared__ bool last;
    if ((threadIdx.x & 31) == 0) {
        for (int a = 0; a < 3; ++a) {
            warp_part[threadIdx.x >> 5].v[a] = mn[a];
            warp_part[threadIdx.x >> 5].v[3 + a] = mx[a];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        MinMax6 r = warp_part[0];
        for (int w = 1; w < AABB_THREADS / 32; ++w)
            for (int a = 0; a < 3; ++a) {
                r.v[a] = min(r.v[a], warp_part[w].v[a]);
                r.v[3 + a] = max(r.v[3 + a], warp_part[w].v[3 + a]);
            }
        part[blockIdx.x] = r;
        __threadfence();
        const unsigned int done = atomicAdd(counter, 1u);
        last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    // the last block reduces all blocks' partials with all its threads
    __threadfence();
    for (int a = 0; a < 3; ++a) {
        mn[a] = zero;
        mx[a] = zero;
    }
    for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
        const MinMax6 q = part[b];
        for (int a = 0; a < 3; ++a) {
            mn[a] = min(mn[a], q.v[a]);
            mx[a] = max(mx[a], q.v[3 + a]);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        for (int off = 16; off > 0; off >>= 1) {
            mn[a] = min(mn[a], __shfl_down_sync(0xffffffffu, mn[a], off));
            mx[a] = max(mx[a], __shfl_down_sync(0xffffffffu, mx[a], off));
        }
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        for (int a = 0; a < 3; ++a) {
            warp_part[threadIdx.x >> 5].v[a] = mn[a];
            warp_part[threadIdx.x >> 5].v[3 + a] = mx[a];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        MinMax6 r = warp_part[0];
        for (int w = 1; w < AABB_THREADS / 32; ++w)
            for (int a = 0; a < 3; ++a) {
                r.v[a] = min(r.v[a], warp_part[w].v[a]);
                r.v[3 + a] = max(r.v[3 + a], warp_part[w].v[3 + a]);
            }
        cube_rule(val_of(r.v[0]), val_of(r.v[1]), val_of(r.v[2]), val_of(r.v[3]),
                  val_of(r.v[4]), val_of(r.v[5]), out);
        *counter = 0;  // ready for the next launch on this context
    }
}

}  // namespace

namespace nb {

// Enqueues the AABB of (x, y, z) into out_dev[7]. Used by nb_aabb and the tree build.
nb_status launch_aabb(nb_ctx* ctx, const double* x, const double* y, const double* z,
                      uint32_t n, double* out_dev, cudaStream_t stream) {
    int blocks = nb::ceil_div(n, AABB_THREADS * 8);
    if (blocks > ctx->sm_count * 4) blocks = ctx->sm_count * 4;
    if (blocks < 1) blocks = 1;
    void* part = nullptr;
    NB_TRY(nb::scratch(ctx, NB_SCRATCH_AABB, (size_t)blocks * sizeof(MinMax6), &part));
    aabb_kernel<<<blocks, AABB_THREADS, 0, stream>>>(x, y, z, n, (MinMax6*)part,
                                                     ctx->dev_counter + 0, out_dev);
    return nb::check_launch("aabb_kernel");
}

}  // namespace nb

extern "C" {

nb_status nb_leapfrog_kick_drift(nb_ctx* ctx, double* vhx, double* vhy, double* vhz,
                                 const double* vx, const double* vy, const double* vz, double* x,
                                 double* y, double* z, const double* ax, const double* ay,
                                 const double* az, uint32_t n, double dt, nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (n == 0) return NB_OK;
    if (!vhx || !vhy || !vhz || !vx || !vy || !vz || !x || !y || !z || !ax || !ay || !az)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_leapfrog_kick_drift: null array pointer");
    kick_drift_kernel<<<nb::ceil_div(n, EW_THREADS), EW_THREADS, 0, (cudaStream_t)stream>>>(
        vhx, vhy, vhz, vx, vy, vz, x, y, z, ax, ay, az, n, dt);
    return nb::check_launch("kick_drift_kernel");
}

nb_status nb_leapfrog_kick(nb_ctx* ctx, double* vx, double* vy, double* vz, const double* vhx,
                           const double* vhy, const double* vhz, const double* ax,
                           const double* ay, const double* az, uint32_t n, double dt,
                           nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (n == 0) return NB_OK;
    if (!vhx || !vhy || !vhz || !vx || !vy || !vz || !ax || !ay || !az)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_leapfrog_kick: null array pointer");
    kick_kernel<<<nb::ceil_div(n, EW_THREADS), EW_THREADS, 0, (cudaStream_t)stream>>>(
        vx, vy, vz, vhx, vhy, vhz, ax, ay, az, n, dt);
    return nb::check_launch("kick_kernel");
}

nb_status nb_leapfrog_kick_kick_drift(nb_ctx* ctx, double* vx, double* vy, double* vz,
                                      double* vhx, double* vhy, double* vhz, double* x, double* y,
                                      double* z, const double* ax, const double* ay,
                                      const double* az, uint32_t n, double dt,
                                      nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (n == 0) return NB_OK;
    if (!vhx || !vhy || !vhz || !vx || !vy || !vz || !x || !y || !z || !ax || !ay || !az)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_leapfrog_kick_kick_drift: null pointer");
    kick_kick_drift_kernel<<<nb::ceil_div(n, EW_THREADS), EW_THREADS, 0, (cudaStream_t)stream>>>(
        vx, vy, vz, vhx, vhy, vhz, x, y, z, ax, ay, az, n, dt);
    return nb::check_launch("kick_kick_drift_kernel");
}

nb_status nb_energy(nb_ctx* ctx, const double* m, const double* x, const double* y,
                    const double* z, const double* vx, const double* vy, const double* vz,
                    uint32_t n, double G, double* out_dev, nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (!m || !x || !y || !z || !vx || !vy || !vz || !out_dev)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_energy: null pointer");
    if (n == 0) return nb::set_error(NB_ERR_INVALID_ARG, "nb_energy: n == 0");
    const int blocks = nb::ceil_div(n, EN_THREADS);
    void* part = nullptr;
    NB_TRY(nb::scratch(ctx, NB_SCRATCH_ENERGY, (size_t)blocks * sizeof(double2), &part));
    energy_kernel<<<blocks, EN_THREADS, 0, (cudaStream_t)stream>>>(m, x, y, z, vx, vy, vz, n, G,
                                                                 (double2*)part);
    NB_TRY(nb::check_launch("energy_kernel"));
    energy_finalize<<<1, 256, 0, (cudaStream_t)stream>>>((const double2*)part, blocks, out_dev);
    return nb::check_launch("energy_finalize");
}

nb_status nb_aabb(nb_ctx* ctx, const double* x, const double* y, const double* z, uint32_t n,
                  double* out_dev, nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (!x || !y || !z || !out_dev) return nb::set_error(NB_ERR_INVALID_ARG, "nb_aabb: null pointer");
    return nb::launch_aabb(ctx, x, y, z, n, out_dev, (cudaStream_t)stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Energy without any allocation.
//
// Some callers cannot let this library allocate device memory: an application that reserves the
// GPU's memory up front for its own pool and forbids later cudaMalloc calls, or a time-critical
// loop that cannot pay for cudaMalloc's device-wide synchronisation and unpredictable latency.
// nb_energy needs a context (whose creation allocates) and grows per-block scratch on demand;
// nb_energy_noalloc runs the same two kernels with their per-block partial sums in the fixed
// array below instead. Nothing in the array needs clearing between calls: every call writes each
// partial it later reads. All calls share the array, so calls that overlap on the GPU (two
// streams, two host threads) race and must be serialised by the caller.
// ---------------------------------------------------------------------------------------------
namespace {

constexpr uint32_t NOALLOC_MAX_BLOCKS = 8192;  // 8192 * 16 B = 128 KiB of scratch per device
static_assert(NB_ENERGY_NOALLOC_MAX_N == NOALLOC_MAX_BLOCKS * EN_THREADS, "size mismatch");

// Per-block (kinetic, potential) partials. Every GPU that loads the library holds this array
// until the process exits. Host code must not pass the symbol itself to a kernel: its host-side
// name is only a stand-in, so the device address is looked up once per device below.
static __device__ __align__(256) double2 g_energy_noalloc_partials[NOALLOC_MAX_BLOCKS];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};

// Device address of the partials array on the current device (looked up on first use).
nb_status noalloc_partials(double2** out) {
    int dev = -1;
    NB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return nb::set_error(NB_ERR_UNSUPPORTED, "nb_energy_noalloc: device %d not supported", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_energy_noalloc_partials);
        if (e != cudaSuccess) return nb::cuda_error(e, "nb_energy_noalloc: cudaGetSymbolAddress");
        g_noalloc_addr[dev] = p;
    }
    *out = (double2*)g_noalloc_addr[dev];
    return NB_OK;
}

}  // namespace

extern "C" {

nb_status nb_energy_noalloc(const double* m, const double* x, const double* y, const double* z,
                            const double* vx, const double* vy, const double* vz, uint32_t n,
                            double G, double* out_dev, nb_stream_t stream) {
    if (!m || !x || !y || !z || !vx || !vy || !vz || !out_dev)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_energy_noalloc: null pointer");
    if (n == 0) return nb::set_error(NB_ERR_INVALID_ARG, "nb_energy_noalloc: n == 0");
    if (n > NB_ENERGY_NOALLOC_MAX_N)
        return nb::set_error(NB_ERR_INVALID_ARG,
                             "nb_energy_noalloc: n = %u exceeds the fixed scratch limit of %u "
                             "bodies; use nb_energy", n, (unsigned)NB_ENERGY_NOALLOC_MAX_N);
    double2* part = nullptr;
    NB_TRY(noalloc_partials(&part));
    const uint32_t blocks = (n + EN_THREADS - 1) / EN_THREADS;
    energy_kernel<<<blocks, EN_THREADS, 0, (cudaStream_t)stream>>>(m, x, y, z, vx, vy, vz, n, G,
                                                                  part);
    NB_TRY(nb::check_launch("energy_kernel (noalloc)"));
    energy_finalize<<<1, 256, 0, (cudaStream_t)stream>>>(part, blocks, out_dev);
    return nb::check_launch("energy_finalize (noalloc)");
}

}  // extern "C"
