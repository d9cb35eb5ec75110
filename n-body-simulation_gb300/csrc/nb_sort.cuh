// nb_sort.cuh -- device-wide scan and radix sort used by the octree build.
#pragma once
#include "nb_internal.cuh"

namespace nb {

// Bytes of temporary storage exclusive_scan_u32 needs for n elements.
size_t scan_temp_bytes(uint32_t n);
// out[i] = sum(in[0..i)); with write_total, out[n] = sum(in[0..n)). In-place allowed.
nb_status exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, int write_total,
                             uint32_t* temp, cudaStream_t stream);

size_t radix_temp_bytes(uint32_t n);
// One-time set-up of the sort's kernels on the current device (their dynamic shared memory);
// radix_sort_pairs calls it, and so do callers that may sort inside a stream capture, earlier.
nb_status radix_prepare();
// Stable LSD sort of (keys, vals) on bits [begin_bit, end_bit) (at most 64) in 8-bit digits, one
// launch per digit pass after one histogram launch, ping-ponging with (keys_alt, vals_alt);
// *result_in_alt says which pair holds the result. A look-back wait that runs out (after
// wait_limit polls) sets NB_DEVERR_TIMEOUT in *err (device word); every output position then
// still lies inside [0, n), since a partial look-back only undercounts the keys before a tile.
// drop_first (failure-path tests only) withholds the first tile's published count.
nb_status radix_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt,
                           uint32_t* vals_alt, uint32_t n, int begin_bit, int end_bit,
                           void* temp, uint32_t* err, cudaStream_t stream, int* result_in_alt,
                           unsigned long long wait_limit = NB_WAIT_LIMIT_DEFAULT,
                           int drop_first = 0);

}  // namespace nb
