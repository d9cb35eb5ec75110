// nb_sort.cu -- device-wide exclusive scan (u32) and stable LSD radix sort of (u64 key, u32 value)
// pairs, used by the octree build. Deterministic: no result depends on thread timing.
#include "nb_sort.cuh"

namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// Block-wide exclusive scan of one value per thread; returns the block total in *total.
__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t block_total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        uint32_t ws = lane < nw ? warp_sums[lane] : 0;
        uint32_t wi = ws;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, off);
            if (lane >= off) wi += t;
        }
        if (lane < nw) warp_sums[lane] = wi - ws;
        if (lane == nw - 1) block_total = wi;
    }
    __syncthreads();
    const uint32_t res = warp_sums[warp] + incl - v;
    const uint32_t tot = block_total;
    __syncthreads();
    *total = tot;
    return res;
}

__global__ void __launch_bounds__(SCAN_THREADS)
scan_reduce_kernel(const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ sums) {
    const uint32_t base = blockIdx.x * SCAN_TILE;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const uint32_t i = base + k * SCAN_THREADS + threadIdx.x;
        if (i < n) s += in[i];
    }
    uint32_t total;
    block_exclusive_scan(s, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Exclusive scan of sums[0..nb) in place by one block; sums[nb] = grand total.
__global__ void __launch_bounds__(SCAN_THREADS)
scan_sums_kernel(uint32_t* __restrict__ sums, uint32_t nb) {
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nb; base += SCAN_THREADS) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < nb ? sums[i] : 0;
        uint32_t total;
        const uint32_t ex = block_exclusive_scan(v, &total);
        if (i < nb) sums[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void __launch_bounds__(SCAN_THREADS)
scan_apply_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint32_t n,
                  const uint32_t* __restrict__ sums, int write_total) {
    const uint32_t base = blockIdx.x * SCAN_TILE;
    // blocked arrangement: thread t owns items base + t*ITEMS .. +ITEMS-1
    uint32_t v[SCAN_ITEMS];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const uint32_t i = base + threadIdx.x * SCAN_ITEMS + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(s, &total) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const uint32_t i = base + threadIdx.x * SCAN_ITEMS + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (write_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = sums[gridDim.x];
}

// ---------------------------------------------------------------------------------------------
// Radix sort: 8-bit digits, tiles of 2048 keys (256 threads x 8 items).
// ---------------------------------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_BINS = 256;

__global__ void __launch_bounds__(RS_THREADS)
radix_hist_kernel(const uint64_t* __restrict__ keys, uint32_t n, int shift,
                  uint32_t* __restrict__ hist, uint32_t n_tiles) {
    __shared__ uint32_t h[RS_BINS];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * RS_TILE;
#pragma unroll
    for (int k = 0; k < RS_ITEMS; ++k) {
        const uint32_t i = base + k * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[(uint32_t)(keys[i] >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * n_tiles + blockIdx.x] = h[threadIdx.x];  // digit-major
}

__global__ void __launch_bounds__(RS_THREADS)
radix_scatter_kernel(const uint64_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                     uint64_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint32_t n,
                     int shift, const uint32_t* __restrict__ offsets, uint32_t n_tiles) {
    __shared__ uint32_t wcnt[RS_WARPS][RS_BINS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int b = threadIdx.x; b < RS_WARPS * RS_BINS; b += RS_THREADS) (&wcnt[0][0])[b] = 0;
    __syncthreads();
    // warp-striped: warp w owns tile positions [w*256, w*256+256); item k, lane l -> w*256+k*32+l
    const uint32_t base = blockIdx.x * RS_TILE + warp * (RS_ITEMS * 32);
    uint64_t key[RS_ITEMS];
    uint32_t val[RS_ITEMS], digit[RS_ITEMS], rank[RS_ITEMS];
    const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < RS_ITEMS; ++k) {
        const uint32_t i = base + k * 32 + lane;
        const bool valid = i < n;
        key[k] = valid ? keys_in[i] : 0;
        val[k] = valid ? vals_in[i] : 0;
        digit[k] = valid ? ((uint32_t)(key[k] >> shift) & 0xffu) : RS_BINS;
        const uint32_t peers = __match_any_sync(0xffffffffu, digit[k]);
        const int leader = __ffs(peers) - 1;
        uint32_t prev = 0;
        if (valid) prev = wcnt[warp][digit[k]];
        __syncwarp();
        if (valid && lane == leader) wcnt[warp][digit[k]] = prev + __popc(peers);
        __syncwarp();
        rank[k] = prev + __popc(peers & lt_mask);
    }
    __syncthreads();
    // exclusive prefix over warps per digit; thread t owns digit t
    {
        uint32_t run = 0;
        for (int w = 0; w < RS_WARPS; ++w) {
            const uint32_t c = wcnt[w][threadIdx.x];
            wcnt[w][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < RS_ITEMS; ++k) {
        if (digit[k] < RS_BINS) {
            const uint32_t dst =
                offsets[digit[k] * n_tiles + blockIdx.x] + wcnt[warp][digit[k]] + rank[k];
            keys_out[dst] = key[k];
            vals_out[dst] = val[k];
        }
    }
}

}  // namespace

namespace nb {

size_t scan_temp_bytes(uint32_t n) {
    const uint32_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    return ((size_t)nb + 1) * sizeof(uint32_t);
}

nb_status exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, int write_total,
                             uint32_t* temp, cudaStream_t stream) {
    if (n == 0) {
        if (write_total) NB_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(uint32_t), stream));
        return NB_OK;
    }
    const uint32_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb > 64u * SCAN_THREADS)
        return set_error(NB_ERR_INVALID_ARG, "exclusive_scan_u32: n = %u too large", n);
    scan_reduce_kernel<<<nb, SCAN_THREADS, 0, stream>>>(in, n, temp);
    NB_TRY(check_launch("scan_reduce_kernel"));
    scan_sums_kernel<<<1, SCAN_THREADS, 0, stream>>>(temp, nb);
    NB_TRY(check_launch("scan_sums_kernel"));
    scan_apply_kernel<<<nb, SCAN_THREADS, 0, stream>>>(in, out, n, temp, write_total);
    return check_launch("scan_apply_kernel");
}

size_t radix_temp_bytes(uint32_t n) {
    const uint32_t tiles = (n + RS_TILE - 1) / RS_TILE;
    const size_t hist = (size_t)tiles * RS_BINS;
    return (2 * hist + 1) * sizeof(uint32_t) + scan_temp_bytes((uint32_t)hist) + 256;
}

nb_status radix_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt,
                           uint32_t* vals_alt, uint32_t n, int begin_bit, int end_bit,
                           void* temp, cudaStream_t stream, int* result_in_alt) {
    *result_in_alt = 0;
    if (n <= 1) return NB_OK;
    const uint32_t tiles = (n + RS_TILE - 1) / RS_TILE;
    const uint32_t hist_n = tiles * RS_BINS;
    uint32_t* hist = (uint32_t*)temp;
    uint32_t* offs = hist + hist_n;
    uint32_t* scan_tmp = offs + hist_n + 1;
    uint64_t* kin = keys;
    uint32_t* vin = vals;
    uint64_t* kout = keys_alt;
    uint32_t* vout = vals_alt;
    int flips = 0;
    for (int shift = begin_bit; shift < end_bit; shift += 8) {
        radix_hist_kernel<<<tiles, RS_THREADS, 0, stream>>>(kin, n, shift, hist, tiles);
        NB_TRY(check_launch("radix_hist_kernel"));
        NB_TRY(exclusive_scan_u32(hist, offs, hist_n, 0, scan_tmp, stream));
        radix_scatter_kernel<<<tiles, RS_THREADS, 0, stream>>>(kin, vin, kout, vout, n, shift, offs,
                                                              tiles);
        NB_TRY(check_launch("radix_scatter_kernel"));
        uint64_t* tk = kin;
        kin = kout;
        kout = tk;
        uint32_t* tv = vin;
        vin = vout;
        vout = tv;
        flips ^= 1;
    }
    *result_in_alt = flips;
    return NB_OK;
}

}  // namespace nb

extern "C" {

// Test hooks for the sort and scan building blocks (DEVICE pointers; results as documented in
// include/nbody.h).
nb_status nb_util_radix_sort_pairs(nb_ctx* ctx, uint64_t* keys, uint32_t* vals, uint32_t n,
                                   int begin_bit, int end_bit, nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (begin_bit < 0 || end_bit > 64 || begin_bit >= end_bit)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_util_radix_sort_pairs: bad bit range");
    if (n <= 1) return NB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t* ka = nullptr;
    uint32_t* va = nullptr;
    void* tmp = nullptr;
    NB_CUDA_TRY(cudaMallocAsync(&ka, (size_t)n * 8, s));
    NB_CUDA_TRY(cudaMallocAsync(&va, (size_t)n * 4, s));
    NB_CUDA_TRY(cudaMallocAsync(&tmp, nb::radix_temp_bytes(n), s));
    int in_alt = 0;
    nb_status st = nb::radix_sort_pairs(keys, vals, ka, va, n, begin_bit, end_bit, tmp, s, &in_alt);
    if (st == NB_OK && in_alt) {
        cudaMemcpyAsync(keys, ka, (size_t)n * 8, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(vals, va, (size_t)n * 4, cudaMemcpyDeviceToDevice, s);
    }
    cudaFreeAsync(ka, s);
    cudaFreeAsync(va, s);
    cudaFreeAsync(tmp, s);
    if (st != NB_OK) return st;
    return nb::check_launch("nb_util_radix_sort_pairs");
}

nb_status nb_util_exclusive_scan_u32(nb_ctx* ctx, const uint32_t* in, uint32_t* out, uint32_t n,
                                     nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t* tmp = nullptr;
    NB_CUDA_TRY(cudaMallocAsync(&tmp, nb::scan_temp_bytes(n) + 64, s));
    nb_status st = nb::exclusive_scan_u32(in, out, n, 1, tmp, s);
    cudaFreeAsync(tmp, s);
    return st;
}

}  // extern "C"
