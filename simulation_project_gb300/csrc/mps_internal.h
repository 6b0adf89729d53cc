// mps_internal.h - declarations shared between the translation units of the library.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/mps_types.h"

namespace mps {

// radix sort (sort.cu).  Scratch: alternate key and value arrays, the digit counts
// of every tile (digit-major), 8 spare words and per-pass digit totals.
constexpr int kRadixSortTile = 2048;
constexpr int kRadixBuckets = 256;
constexpr int kRadixMaxPasses = 4;
constexpr size_t radix_scratch_bytes_for(long long n) {
    return sizeof(int) * 2 * (size_t)(n > 0 ? n : 0) +
           sizeof(unsigned) * ((size_t)kRadixBuckets * (size_t)(((n > 0 ? n : 1) + kRadixSortTile - 1) / kRadixSortTile) +
                               8 + (size_t)kRadixMaxPasses * kRadixBuckets) +
           256;
}
size_t radix_scratch_bytes(int n);
int radix_passes(unsigned range);
cudaError_t radix_sort_pairs(int n, int* keys, int* vals, int kmin, int passes, void* scratch, cudaStream_t st);
// the same with the key range (min, max) in device memory (key_minmax): no host wait
cudaError_t radix_sort_pairs_range(int n, int* keys, int* vals, const int* mm_dev, void* scratch, cudaStream_t st);
cudaError_t key_minmax(int n, const int* keys, int* mm_dev, cudaStream_t st);
// in-place exclusive scan of len unsigned values, total to *total_dev (if not NULL);
// tile_sums (scan_tile_sums_capacity() values, or NULL: single-CTA scan) lets it
// run on many CTAs
cudaError_t scan_exclusive(unsigned* a, int len, unsigned* total_dev, cudaStream_t st, unsigned* tile_sums = nullptr);
size_t scan_tile_sums_capacity();

// library-owned scratch for the reference-named entry points, which take no scratch
// argument (runtime.cu).  Grows on demand; one buffer per slot.
void* scratch_get(int slot, size_t bytes);
// records "where: CUDA error string" for mps_last_error()
void note_error(const char* where, cudaError_t e);
// records a message of the library's own for mps_last_error()
void note_message(const char* msg);

// Kernel launches issued by this library since load (every launch site is written as
// MPS_COUNT_LAUNCH k<<<...>>>(...); read by mps_kernel_launches()).
extern unsigned long long g_kernel_launches;
#define MPS_COUNT_LAUNCH __atomic_fetch_add(&::mps::g_kernel_launches, 1ull, __ATOMIC_RELAXED),
void scratch_release_all();

inline CCTStatusType cuda_status(cudaError_t e) { return e == cudaSuccess ? CCT_NOERR : CCT_CUDAERR; }

}  // namespace mps

#define MPS_CUDA_TRY(expr)                                  \
    do {                                                    \
        cudaError_t _e = (expr);                            \
        if (_e != cudaSuccess) return CCT_CUDAERR;          \
    } while (0)
