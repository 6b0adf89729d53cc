// sort_noalloc.cu - SortUsingThrustNoAlloc: the stable (key, index) radix sort of
// SortUsingThrust for callers that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is not allowed or not wanted -- inside
// an allocator hook or a memory-pool callback (allocating would recurse), in a process
// whose device memory is pre-reserved and fenced by a host framework, or on a
// real-time path where a driver allocation (and its implicit synchronisation) is not
// acceptable.  SortUsingThrust takes no scratch argument and grows library-owned
// buffers with cudaMalloc; this variant uses one file-scope __device__ array instead.
//
// Limits and rules:
//   * at most kNoAllocMaxKeys = 262,144 keys per call; larger n returns CCT_PARAMERR
//     (mps_last_error() says why) without touching the arrays;
//   * the array (2,232,864 bytes, about 2.1 MiB) lives in every GPU that loads the
//     library, until the process exits;
//   * every call looks up the array's device address on the current device with
//     cudaGetSymbolAddress (no allocation; nothing is cached, so a device reset or a
//     re-created context cannot leave a stale address behind, and concurrent first
//     calls from several host threads share no unsynchronised state); the first call
//     on a device also makes the runtime load the library's module there, so make that
//     first call before any stream capture;
//   * every call shares the array, and it keeps the last call's contents: the sort
//     writes each scratch word before it reads it (min/max re-initialised, histograms
//     fully rewritten per pass), so nothing is stale -- but calls that overlap on the
//     GPU (from several host threads or streams) race on it and must be serialised;
//   * like SortUsingThrust it runs on the legacy default stream and returns after the
//     sort has finished.
#include <stdio.h>

#include "mps_common.cuh"
#include "mps_internal.h"
#include "../../include/mps_device_process.h"

namespace mps {
namespace {

constexpr int kNoAllocMaxKeys = 1 << 18;
constexpr size_t kNoAllocHeader = 256;  // min/max words, padded to the array alignment
constexpr size_t kNoAllocSortBytes = radix_scratch_bytes_for(kNoAllocMaxKeys);
constexpr size_t kNoAllocBytes = kNoAllocHeader + kNoAllocSortBytes;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// device address of the array on the current device, looked up on every call: the
// host-side symbol g_noalloc_scratch is only a stand-in for it and must never reach a
// kernel
CCTStatusType noalloc_scratch(void** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        note_error("SortUsingThrustNoAlloc: cudaGetSymbolAddress", e);
        return CCT_CUDAERR;
    }
    *out = p;
    return CCT_NOERR;
}

}  // namespace
}  // namespace mps

using namespace mps;

extern "C" CCTStatusType SortUsingThrustNoAlloc(Integer MaxParticleNum, Integer* daNumberHash, Integer* daNumberIndex) {
    const int n = MaxParticleNum;
    if (n > kNoAllocMaxKeys) {
        note_error("SortUsingThrustNoAlloc: more keys than the 262144 its static scratch holds", cudaErrorInvalidValue);
        return CCT_PARAMERR;
    }
    if (n <= 1) return CCT_NOERR;
    if (radix_scratch_bytes(n) > kNoAllocSortBytes) return CCT_PARAMERR;
    void* base = nullptr;
    CCTStatusType rc = noalloc_scratch(&base);
    if (rc != CCT_NOERR) return rc;
    int* mm = (int*)base;
    void* scr = (char*)base + kNoAllocHeader;
    cudaStream_t st = 0;
    MPS_CUDA_TRY(key_minmax(n, daNumberHash, mm, st));
    int h[2];
    MPS_CUDA_TRY(cudaMemcpyAsync(h, mm, sizeof(h), cudaMemcpyDeviceToHost, st));
    MPS_CUDA_TRY(cudaStreamSynchronize(st));
    const int passes = radix_passes((unsigned)h[1] - (unsigned)h[0]);
    MPS_CUDA_TRY(radix_sort_pairs(n, daNumberHash, daNumberIndex, h[0], passes, scr, st));
    MPS_CUDA_TRY(cudaStreamSynchronize(st));
    return cuda_status(cudaGetLastError());
}
