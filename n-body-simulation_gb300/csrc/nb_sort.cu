// nb_sort.cu -- device-wide exclusive scan (u32) and stable LSD radix sort of (u64 key, u32 value)
// pairs, used by the octree build. Deterministic: no result depends on thread timing.
#include <algorithm>

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
// Radix sort: 8-bit digits, tiles of 2048 keys (256 threads x 8 items), one launch per digit
// pass. The digit histograms of all passes come from one read of the keys up front; within a
// pass each tile finds the keys of its digit in earlier tiles by decoupled look-back (Merrill and
// Garland, "Single-pass parallel prefix scan with decoupled look-back", NVIDIA TR 2016; the
// radix-sort use as in Adinets and Merrill, "Onesweep", 2022): a tile publishes its per-digit
// count, then the running total up to and including it, and reads its predecessors' words until
// it meets a total. Tiles take their position from an atomic ticket in the order they start, so
// a tile only waits for tiles that are already running; every wait is bounded (on timeout the
// error word gets the timeout bit and the pass goes on). Deterministic and stable: the offsets
// depend on the counts only.
// ---------------------------------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_BINS = 256;
constexpr int RS_MAX_PASSES = 8;
// look-back words: 2 flag bits over a 30-bit count (tile counts <= 4096, totals <= n < 2^30)
constexpr uint32_t LB_AGGREGATE = 1u << 30;
constexpr uint32_t LB_TOTAL = 2u << 30;
constexpr uint32_t LB_VALUE = (1u << 30) - 1u;
constexpr int LB_WINDOW = 8;  // predecessor words read per look-back round trip
static_assert(RS_THREADS == RS_BINS, "the look-back and the digit scan run one thread per digit");

// hist[p][d]: keys whose digit of pass p is d, for all passes in one read.
__global__ void __launch_bounds__(RS_THREADS)
radix_hist_all_kernel(const uint64_t* __restrict__ keys, uint32_t n, int begin_bit, int passes,
                      uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[RS_MAX_PASSES][RS_BINS];
    for (int e = threadIdx.x; e < RS_MAX_PASSES * RS_BINS; e += RS_THREADS) (&h[0][0])[e] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * RS_THREADS + threadIdx.x; i < n; i += gridDim.x * RS_THREADS) {
        const uint64_t k = keys[i] >> begin_bit;
        for (int p = 0; p < passes; ++p) atomicAdd(&h[p][(uint32_t)(k >> (8 * p)) & 0xffu], 1u);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < passes * RS_BINS; e += RS_THREADS) {
        const uint32_t v = (&h[0][0])[e];
        if (v) atomicAdd(&hist[e], v);
    }
}

// hist[p][d] -> exclusive prefix over d (block p, thread d).
__global__ void __launch_bounds__(RS_BINS) radix_offsets_kernel(uint32_t* __restrict__ hist) {
    uint32_t total;
    uint32_t* h = hist + blockIdx.x * RS_BINS;
    h[threadIdx.x] = block_exclusive_scan(h[threadIdx.x], &total);
}

__device__ __forceinline__ void lb_store(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t lb_load(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// The tile's keys and values reordered by digit (dynamic shared memory: above the static limit).
constexpr int RS_REORDER_BYTES = RS_TILE * (int)(sizeof(uint64_t) + sizeof(uint32_t));

// One digit pass: keys of tile `ticket` in, ranked within the tile (warp-striped, stable),
// placed at digit offset + keys of the digit in earlier tiles + rank.
__global__ void __launch_bounds__(RS_THREADS)
radix_pass_kernel(const uint64_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                  uint64_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint32_t n,
                  int shift, const uint32_t* __restrict__ digit_off, uint32_t* __restrict__ lb,
                  uint32_t* __restrict__ ticket, uint32_t* __restrict__ err,
                  unsigned long long wait_limit, int drop_first) {
    __shared__ uint32_t wcnt[RS_WARPS][RS_BINS];
    __shared__ uint32_t tile_base[RS_BINS];   // first output position of the tile's digit d
    __shared__ uint32_t digit_local[RS_BINS];  // first tile position of digit d after the reorder
    extern __shared__ __align__(16) unsigned char rs_reorder[];  // RS_REORDER_BYTES
    uint64_t* skeys = reinterpret_cast<uint64_t*>(rs_reorder);
    uint32_t* svals = reinterpret_cast<uint32_t*>(rs_reorder + RS_TILE * sizeof(uint64_t));
    __shared__ uint32_t tile_s;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) tile_s = atomicAdd(ticket, 1u);
    for (int b = threadIdx.x; b < RS_WARPS * RS_BINS; b += RS_THREADS) (&wcnt[0][0])[b] = 0;
    __syncthreads();
    const uint32_t tile = tile_s;
    // warp-striped: warp w owns tile positions [w*512, w*512+512); item k, lane l -> w*512+k*32+l
    const uint32_t base = tile * RS_TILE + warp * (RS_ITEMS * 32);
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
    {
        // thread d owns digit d: exclusive prefix over warps, the tile's count, then look-back
        const uint32_t d = threadIdx.x;
        uint32_t run = 0;
        for (int w = 0; w < RS_WARPS; ++w) {
            const uint32_t c = wcnt[w][d];
            wcnt[w][d] = run;
            run += c;
        }
        uint32_t* mine = lb + (size_t)tile * RS_BINS + d;
        uint32_t before = 0;
        if (tile == 0) {
            // drop_first (failure-path test hook): the first tile's count is never published,
            // so the tiles after it wait for a word that nothing writes
            if (!drop_first) lb_store(mine, LB_TOTAL | run);
        } else {
            lb_store(mine, LB_AGGREGATE | run);
            // walk back in windows of LB_WINDOW predecessors, their words loaded together (one
            // round trip per window), up to the nearest published total (tile 0 always has one)
            bool timed_out = false, done = false;
            for (int t0 = (int)tile - 1; !done && t0 >= 0; t0 -= LB_WINDOW) {
                uint32_t v[LB_WINDOW];
#pragma unroll
                for (int j = 0; j < LB_WINDOW; ++j)
                    v[j] = t0 - j >= 0 ? lb_load(lb + (size_t)(t0 - j) * RS_BINS + d) : 0u;
#pragma unroll
                for (int j = 0; j < LB_WINDOW; ++j) {
                    if (done || t0 - j < 0) break;
                    const uint32_t* w = lb + (size_t)(t0 - j) * RS_BINS + d;
                    for (unsigned long long it = 0; (v[j] & (LB_AGGREGATE | LB_TOTAL)) == 0; ++it) {
                        if (it >= wait_limit) {
                            timed_out = true;
                            break;
                        }
                        __nanosleep(32);
                        v[j] = lb_load(w);
                    }
                    if (timed_out) {
                        done = true;
                        break;
                    }
                    before += v[j] & LB_VALUE;
                    if (v[j] & LB_TOTAL) done = true;
                }
            }
            if (timed_out) atomicOr(err, NB_DEVERR_TIMEOUT);
            lb_store(mine, LB_TOTAL | (before + run));
        }
        tile_base[d] = digit_off[d] + before;
        uint32_t tile_total;
        digit_local[d] = block_exclusive_scan(run, &tile_total);  // one digit per thread
    }
    __syncthreads();
    // reorder the tile by digit in shared memory, then write each digit's run of keys to
    // consecutive output positions (coalesced instead of one scattered store per key)
#pragma unroll
    for (int k = 0; k < RS_ITEMS; ++k) {
        if (digit[k] < RS_BINS) {
            const uint32_t q = digit_local[digit[k]] + wcnt[warp][digit[k]] + rank[k];
            skeys[q] = key[k];
            svals[q] = val[k];
        }
    }
    __syncthreads();
    const uint32_t tile_n = min((uint32_t)RS_TILE, n - tile * RS_TILE);
    for (uint32_t q = threadIdx.x; q < tile_n; q += RS_THREADS) {
        const uint64_t kk = skeys[q];
        const uint32_t d = (uint32_t)(kk >> shift) & 0xffu;
        const uint32_t dst = tile_base[d] + (q - digit_local[d]);
        keys_out[dst] = kk;
        vals_out[dst] = svals[q];
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

nb_status radix_prepare() {
    static bool done[64] = {};
    int dev = 0;
    NB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64 || done[dev]) return NB_OK;
    NB_CUDA_TRY(cudaFuncSetAttribute(radix_pass_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     RS_REORDER_BYTES));
    done[dev] = true;
    return NB_OK;
}

// Temporary storage of radix_sort_pairs: digit offsets and tickets of all passes, then one
// look-back word per (pass, tile, digit).
size_t radix_temp_bytes(uint32_t n) {
    const size_t tiles = (n + RS_TILE - 1) / RS_TILE;
    return ((size_t)RS_MAX_PASSES * RS_BINS + 64 + (size_t)RS_MAX_PASSES * tiles * RS_BINS) *
           sizeof(uint32_t);
}

nb_status radix_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt,
                           uint32_t* vals_alt, uint32_t n, int begin_bit, int end_bit,
                           void* temp, uint32_t* err, cudaStream_t stream, int* result_in_alt,
                           unsigned long long wait_limit, int drop_first) {
    *result_in_alt = 0;
    if (n <= 1) return NB_OK;
    if (n > LB_VALUE)  // look-back words count keys in 30 bits
        return set_error(NB_ERR_INVALID_ARG, "radix_sort_pairs: n = %u above 2^30 - 1", n);
    const int passes = (end_bit - begin_bit + 7) / 8;
    if (passes < 1 || passes > RS_MAX_PASSES)
        return set_error(NB_ERR_INVALID_ARG, "radix_sort_pairs: bit range [%d, %d)", begin_bit,
                         end_bit);
    NB_TRY(radix_prepare());
    const uint32_t tiles = (n + RS_TILE - 1) / RS_TILE;
    uint32_t* offs = (uint32_t*)temp;                   // [passes][256]
    uint32_t* tickets = offs + RS_MAX_PASSES * RS_BINS;  // [passes]
    uint32_t* lb = tickets + 64;                         // [passes][tiles][256]
    NB_CUDA_TRY(cudaMemsetAsync(temp, 0, radix_temp_bytes(n), stream));
    const int hist_blocks = (int)std::min<uint32_t>(tiles, 1024u);
    radix_hist_all_kernel<<<hist_blocks, RS_THREADS, 0, stream>>>(keys, n, begin_bit, passes, offs);
    NB_TRY(check_launch("radix_hist_all_kernel"));
    radix_offsets_kernel<<<passes, RS_BINS, 0, stream>>>(offs);
    NB_TRY(check_launch("radix_offsets_kernel"));
    uint64_t* kin = keys;
    uint32_t* vin = vals;
    uint64_t* kout = keys_alt;
    uint32_t* vout = vals_alt;
    int flips = 0;
    for (int p = 0; p < passes; ++p) {
        radix_pass_kernel<<<tiles, RS_THREADS, RS_REORDER_BYTES, stream>>>(
            kin, vin, kout, vout, n, begin_bit + 8 * p, offs + p * RS_BINS,
            lb + (size_t)p * tiles * RS_BINS, tickets + p, err, wait_limit, drop_first);
        NB_TRY(check_launch("radix_pass_kernel"));
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
    nb_status st = nb::radix_sort_pairs(keys, vals, ka, va, n, begin_bit, end_bit, tmp,
                                        ctx->dev_error, s, &in_alt, ctx->wait_limit,
                                        (ctx->fault_flags & NB_FAULT_DROP_LOOKBACK) ? 1 : 0);
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
