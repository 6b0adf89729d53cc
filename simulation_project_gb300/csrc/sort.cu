// sort.cu - stable LSD radix sort of (int key, int value) pairs on the GPU.
//
// Replaces the reference's thrust::sort_by_key call (SortUsingThrust,
// radix/SPVSOLVER/MultiGPUSolver/DeviceProcess.cu:207-220).  For int keys Thrust's
// sort is a stable radix sort, so the result is uniquely the stable order; this sort
// produces exactly that order.
//
// Per 8-bit digit pass:
//   k_digit_hist : each 2048-key tile counts its digits (warp-aggregated with
//                  __match_any_sync, then shared-memory adds); counts stored
//                  digit-major: counts[d * tiles + tile]
//                  and adds its per-digit totals to dtot[pass][d]
//   k_scan_digits: CTA per digit d: base(d) = sum of the totals of the smaller
//                  digits, then the exclusive scan of counts[d][0..tiles) from base(d)
//   k_scatter    : each tile re-reads its keys in index order (warp w owns keys
//                  [w*256, w*256+256) of the tile, 32 per round), ranks them stably
//                  with __match_any_sync + per-warp running digit counters, and
//                  writes key and value to offset[d][tile] + warp prefix + rank.
// Keys are sorted as unsigned offsets (key - kmin), so negative keys sort correctly
// and a pass runs only for the digits the key range actually spans.  With the range in
// device memory (radix_sort_pairs_range) the host launches the largest number of passes
// and each pass's kernels read the range and return at once past the passes it needs,
// so the caller does not wait for the key range on the host.
#include "mps_common.cuh"
#include "mps_internal.h"

namespace mps {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kRadix = kRadixBuckets;
static_assert(kSortTile == kRadixSortTile, "tile size of the scratch formula");

__device__ __forceinline__ unsigned digit_of(int key, int kmin, int shift) {
    return (((unsigned)key - (unsigned)kmin) >> shift) & 255u;
}
// 8-bit passes a key range needs (radix_passes on the device)
__device__ __forceinline__ int range_passes(unsigned range) { return range == 0u ? 0 : (39 - __clz((int)range)) / 8; }
// with the key range (min, max) in device memory: the pass's kmin, false when the pass
// is past the ones the range needs
__device__ __forceinline__ bool pass_live(const int* __restrict__ mm, int shift, int& kmin) {
    if (!mm) return true;
    kmin = mm[0];
    return shift / 8 < range_passes((unsigned)mm[1] - (unsigned)mm[0]);
}

__global__ void __launch_bounds__(kSortThreads) k_digit_hist(const int* __restrict__ keys, int n, int kmin, int shift,
                                                            int tiles, unsigned* __restrict__ counts,
                                                            unsigned* __restrict__ dtot, const int* __restrict__ mm) {
    if (!pass_live(mm, shift, kmin)) return;
    __shared__ unsigned h[kRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int base = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = base + r * kSortThreads + threadIdx.x;
        const bool ok = idx < n;
        const unsigned d = ok ? digit_of(keys[idx], kmin, shift) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (ok && (peers & ((1u << lane) - 1u)) == 0) atomicAdd(&h[d], (unsigned)__popc(peers));
    }
    __syncthreads();
    counts[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
    if (h[threadIdx.x]) atomicAdd(&dtot[threadIdx.x], h[threadIdx.x]);
}

// Exclusive scan of len unsigned values, in place, by one CTA of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan_excl(unsigned* __restrict__ a, int len, unsigned* __restrict__ total) {
    __shared__ unsigned wsum[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int per = (len + 1023) / 1024;
    const int b = min(len, tid * per), e = min(len, b + per);
    unsigned s = 0;
    for (int i = b; i < e; ++i) s += a[i];
    unsigned inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    if (w == 0) {
        const unsigned x = wsum[lane];
        unsigned xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned v = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi += v;
        }
        wsum[lane] = xi - x;
        if (lane == 31 && total) *total = xi;
    }
    __syncthreads();
    unsigned run = inc - s + wsum[w];
    for (int i = b; i < e; ++i) {
        const unsigned c = a[i];
        a[i] = run;
        run += c;
    }
}

// Multi-CTA exclusive scan (scan_exclusive with a tile-sum buffer): tiles of
// kScanTile elements loaded coalesced into shared memory; k_scan_tile_sums writes
// each tile's sum, k_scan_tiles scans one tile (4 contiguous items per thread plus
// a block scan of the thread sums) starting from the tile's offset.  The tile sums
// are scanned in place by k_scan_tiles as a single tile.
constexpr int kScanThreads = 1024;
constexpr int kScanTile = 4 * kScanThreads;

__device__ __forceinline__ unsigned block_exclusive(unsigned v, unsigned* ws, unsigned& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        unsigned s = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        ws[lane] = s;
    }
    __syncthreads();
    const unsigned ex = x - v + (w > 0 ? ws[w - 1] : 0u);
    total = ws[31];
    return ex;
}

// CTA per digit: offsets[d][t] = base(d) + sum of counts[d][t' < t], in place
__global__ void __launch_bounds__(kScanThreads) k_scan_digits(unsigned* __restrict__ counts, int tiles,
                                                              const unsigned* __restrict__ dtot,
                                                              const int* __restrict__ mm, int shift) {
    int kmin_unused = 0;
    if (!pass_live(mm, shift, kmin_unused)) return;
    __shared__ unsigned ws[32];
    __shared__ unsigned carry;
    const int d = blockIdx.x;
    unsigned v = threadIdx.x < (unsigned)d ? dtot[threadIdx.x] : 0u;   // d < 256 <= blockDim
    unsigned base;
    (void)block_exclusive(v, ws, base);
    if (threadIdx.x == 0) carry = base;
    __syncthreads();
    unsigned* row = counts + (size_t)d * tiles;
    for (int c0 = 0; c0 < tiles; c0 += 4 * kScanThreads) {
        const int o4 = c0 + 4 * threadIdx.x;
        const unsigned v0 = o4 < tiles ? row[o4] : 0u, v1 = o4 + 1 < tiles ? row[o4 + 1] : 0u;
        const unsigned v2 = o4 + 2 < tiles ? row[o4 + 2] : 0u, v3 = o4 + 3 < tiles ? row[o4 + 3] : 0u;
        unsigned total;
        const unsigned ex = block_exclusive(v0 + v1 + v2 + v3, ws, total) + carry;
        if (o4 < tiles) row[o4] = ex;
        if (o4 + 1 < tiles) row[o4 + 1] = ex + v0;
        if (o4 + 2 < tiles) row[o4 + 2] = ex + v0 + v1;
        if (o4 + 3 < tiles) row[o4 + 3] = ex + v0 + v1 + v2;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tile_sums(const unsigned* __restrict__ a, int len,
                                                                 unsigned* __restrict__ sums) {
    __shared__ unsigned ws[32];
    const int base = blockIdx.x * kScanTile;
    unsigned s = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = base + q * kScanThreads + threadIdx.x;
        if (i < len) s += a[i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned t = ws[threadIdx.x];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) sums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(unsigned* __restrict__ a, int len,
                                                             const unsigned* __restrict__ offsets,
                                                             unsigned* __restrict__ total_dev) {
    __shared__ unsigned t[kScanTile];
    __shared__ unsigned ws[32];
    const int base = blockIdx.x * kScanTile;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = base + q * kScanThreads + threadIdx.x;
        t[q * kScanThreads + threadIdx.x] = i < len ? a[i] : 0u;
    }
    __syncthreads();
    const int o4 = 4 * threadIdx.x;
    const unsigned v0 = t[o4], v1 = t[o4 + 1], v2 = t[o4 + 2], v3 = t[o4 + 3];
    unsigned total;
    const unsigned off = (offsets ? offsets[blockIdx.x] : 0u);
    const unsigned ex = block_exclusive(v0 + v1 + v2 + v3, ws, total) + off;
    t[o4] = ex;
    t[o4 + 1] = ex + v0;
    t[o4 + 2] = ex + v0 + v1;
    t[o4 + 3] = ex + v0 + v1 + v2;
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = base + q * kScanThreads + threadIdx.x;
        if (i < len) a[i] = t[q * kScanThreads + threadIdx.x];
    }
    if (total_dev && threadIdx.x == 0 && blockIdx.x == gridDim.x - 1) *total_dev = off + total;
}

__global__ void __launch_bounds__(kSortThreads) k_scatter(const int* __restrict__ kin, const int* __restrict__ vin,
                                                         int* __restrict__ kout, int* __restrict__ vout, int n,
                                                         int kmin, int shift, int tiles,
                                                         const unsigned* __restrict__ offsets,
                                                         const int* __restrict__ mm) {
    if (!pass_live(mm, shift, kmin)) return;
    __shared__ unsigned wcount[kSortThreads / 32][kRadix];
    __shared__ unsigned toff[kRadix];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < (kSortThreads / 32) * kRadix; i += kSortThreads) (&wcount[0][0])[i] = 0;
    toff[threadIdx.x] = offsets[threadIdx.x * tiles + blockIdx.x];
    __syncthreads();
    const int base = blockIdx.x * kSortTile + w * (32 * kSortItems);
    int key[kSortItems], val[kSortItems];
    unsigned dig[kSortItems], rank[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int idx = base + r * 32 + lane;
        const bool ok = idx < n;
        key[r] = ok ? kin[idx] : 0;
        val[r] = ok ? vin[idx] : 0;
        const unsigned d = ok ? digit_of(key[r], kmin, shift) : 256u;
        dig[r] = d;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned lt = peers & ((1u << lane) - 1u);
        const unsigned before = ok ? wcount[w][d] : 0u;
        __syncwarp();
        if (ok && lt == 0) wcount[w][d] = before + (unsigned)__popc(peers);
        __syncwarp();
        rank[r] = before + (unsigned)__popc(lt);
    }
    __syncthreads();
    {
        unsigned run = 0;
        for (int ww = 0; ww < kSortThreads / 32; ++ww) {
            const unsigned c = wcount[ww][threadIdx.x];
            wcount[ww][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const unsigned d = dig[r];
        if (d < 256u) {
            const unsigned dst = toff[d] + wcount[w][d] + rank[r];
            kout[dst] = key[r];
            vout[dst] = val[r];
        }
    }
}

__global__ void k_minmax(const int* __restrict__ keys, int n, int* __restrict__ mm) {
    int lo = INT_MAX, hi = INT_MIN;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int k = keys[i];
        lo = min(lo, k);
        hi = max(hi, k);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&mm[0], lo);
        atomicMax(&mm[1], hi);
    }
}

// after the passes of radix_sort_pairs_range: an odd number of passes left the pairs
// in the scratch arrays; copy them back
__global__ void k_copy_back_odd(const int* __restrict__ mm, int n, const int* __restrict__ ka,
                                const int* __restrict__ va, int* __restrict__ keys, int* __restrict__ vals) {
    if ((range_passes((unsigned)mm[1] - (unsigned)mm[0]) & 1) == 0) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        keys[i] = ka[i];
        vals[i] = va[i];
    }
}

__global__ void k_minmax_init(int* mm) {
    mm[0] = INT_MAX;
    mm[1] = INT_MIN;
}

size_t radix_scratch_bytes(int n) { return radix_scratch_bytes_for(n); }

int radix_passes(unsigned range) {
    int bits = 0;
    while (bits < 32 && (range >> bits) != 0u) ++bits;
    return (bits + 7) / 8;
}

cudaError_t radix_sort_pairs(int n, int* keys, int* vals, int kmin, int passes, void* scratch, cudaStream_t st) {
    if (n <= 1 || passes <= 0) return cudaSuccess;
    const int tiles = div_up(n, kSortTile);
    char* p = (char*)scratch;
    int* kalt = (int*)p;
    p += sizeof(int) * (size_t)n;
    int* valt = (int*)p;
    p += sizeof(int) * (size_t)n;
    unsigned* counts = (unsigned*)p;
    unsigned* dtot = counts + (size_t)kRadix * tiles + 8;   // [kRadixMaxPasses][kRadix]
    if (passes > kRadixMaxPasses) return cudaErrorInvalidValue;
    cudaMemsetAsync(dtot, 0, sizeof(unsigned) * kRadix * passes, st);
    int* ka = keys;
    int* va = vals;
    int* kb = kalt;
    int* vb = valt;
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = pass * 8;
        unsigned* dt = dtot + (size_t)kRadix * pass;
        MPS_COUNT_LAUNCH k_digit_hist<<<tiles, kSortThreads, 0, st>>>(ka, n, kmin, shift, tiles, counts, dt, nullptr);
        MPS_COUNT_LAUNCH k_scan_digits<<<kRadix, kScanThreads, 0, st>>>(counts, tiles, dt, nullptr, shift);
        MPS_COUNT_LAUNCH k_scatter<<<tiles, kSortThreads, 0, st>>>(ka, va, kb, vb, n, kmin, shift, tiles, counts,
                                                                   nullptr);
        int* t = ka; ka = kb; kb = t;
        t = va; va = vb; vb = t;
    }
    if (ka != keys) {
        cudaMemcpyAsync(keys, ka, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(vals, va, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, st);
    }
    return cudaGetLastError();
}

cudaError_t radix_sort_pairs_range(int n, int* keys, int* vals, const int* mm_dev, void* scratch, cudaStream_t st) {
    if (n <= 1) return cudaSuccess;
    const int tiles = div_up(n, kSortTile);
    char* p = (char*)scratch;
    int* kalt = (int*)p;
    p += sizeof(int) * (size_t)n;
    int* valt = (int*)p;
    p += sizeof(int) * (size_t)n;
    unsigned* counts = (unsigned*)p;
    unsigned* dtot = counts + (size_t)kRadix * tiles + 8;   // [kRadixMaxPasses][kRadix]
    cudaMemsetAsync(dtot, 0, sizeof(unsigned) * kRadix * kRadixMaxPasses, st);
    int* ka = keys;
    int* va = vals;
    int* kb = kalt;
    int* vb = valt;
    for (int pass = 0; pass < kRadixMaxPasses; ++pass) {
        const int shift = pass * 8;
        unsigned* dt = dtot + (size_t)kRadix * pass;
        MPS_COUNT_LAUNCH k_digit_hist<<<tiles, kSortThreads, 0, st>>>(ka, n, 0, shift, tiles, counts, dt, mm_dev);
        MPS_COUNT_LAUNCH k_scan_digits<<<kRadix, kScanThreads, 0, st>>>(counts, tiles, dt, mm_dev, shift);
        MPS_COUNT_LAUNCH k_scatter<<<tiles, kSortThreads, 0, st>>>(ka, va, kb, vb, n, 0, shift, tiles, counts, mm_dev);
        int* t = ka; ka = kb; kb = t;
        t = va; va = vb; vb = t;
    }
    // passes 0, 2 read the caller's arrays and 1, 3 the scratch: after the passes the
    // range needed, the pairs sit in the scratch arrays when that number is odd
    MPS_COUNT_LAUNCH k_copy_back_odd<<<min(div_up(n, 256), 152 * 8), 256, 0, st>>>(mm_dev, n, kalt, valt, keys, vals);
    return cudaGetLastError();
}

cudaError_t key_minmax(int n, const int* keys, int* mm_dev, cudaStream_t st) {
    MPS_COUNT_LAUNCH k_minmax_init<<<1, 1, 0, st>>>(mm_dev);
    const int blocks = min(div_up(n, 1024), 152 * 4);
    if (n > 0) MPS_COUNT_LAUNCH k_minmax<<<blocks, 1024, 0, st>>>(keys, n, mm_dev);
    return cudaGetLastError();
}

cudaError_t scan_exclusive(unsigned* a, int len, unsigned* total_dev, cudaStream_t st, unsigned* tile_sums) {
    if (len <= 0) return cudaSuccess;
    const int tiles = (len + kScanTile - 1) / kScanTile;
    if (tiles == 1) {
        MPS_COUNT_LAUNCH k_scan_tiles<<<1, kScanThreads, 0, st>>>(a, len, nullptr, total_dev);
    } else if (tile_sums && tiles <= kScanTile) {
        MPS_COUNT_LAUNCH k_scan_tile_sums<<<tiles, kScanThreads, 0, st>>>(a, len, tile_sums);
        MPS_COUNT_LAUNCH k_scan_tiles<<<1, kScanThreads, 0, st>>>(tile_sums, tiles, nullptr, nullptr);
        MPS_COUNT_LAUNCH k_scan_tiles<<<tiles, kScanThreads, 0, st>>>(a, len, tile_sums, total_dev);
    } else {
        MPS_COUNT_LAUNCH k_scan_excl<<<1, 1024, 0, st>>>(a, len, total_dev);
    }
    return cudaGetLastError();
}

size_t scan_tile_sums_capacity() { return (size_t)kScanTile; }

}  // namespace mps
