// runtime.cu - device memory / stream / event helpers (include/mps_runtime.h) and the
// library-owned scratch buffers used by the reference-named entry points.
#include <stdio.h>
#include <string.h>

#include "mps_internal.h"
#include "../../include/mps_runtime.h"

namespace mps {

namespace {
struct Slot {
    void* ptr = nullptr;
    size_t bytes = 0;
};
constexpr int kSlots = 16;
Slot g_slots[kSlots];
thread_local char g_err[256] = "no error";

CCTStatusType rec(cudaError_t e) {
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof(g_err), "%s", cudaGetErrorString(e));
        return CCT_CUDAERR;
    }
    return CCT_NOERR;
}
}  // namespace

unsigned long long g_kernel_launches = 0;

void note_error(const char* where, cudaError_t e) {
    snprintf(g_err, sizeof(g_err), "%s: %s", where, cudaGetErrorString(e));
}
void note_message(const char* msg) { snprintf(g_err, sizeof(g_err), "%s", msg); }

void* scratch_get(int slot, size_t bytes) {
    if (slot < 0 || slot >= kSlots) return nullptr;
    Slot& s = g_slots[slot];
    if (s.bytes >= bytes && s.ptr) return s.ptr;
    if (s.ptr) {
        cudaDeviceSynchronize();
        cudaFree(s.ptr);
        s.ptr = nullptr;
        s.bytes = 0;
    }
    size_t want = bytes + bytes / 4 + 256;
    if (cudaMalloc(&s.ptr, want) != cudaSuccess) {
        s.ptr = nullptr;
        return nullptr;
    }
    s.bytes = want;
    return s.ptr;
}

void scratch_release_all() {
    for (auto& s : g_slots) {
        if (s.ptr) cudaFree(s.ptr);
        s.ptr = nullptr;
        s.bytes = 0;
    }
}

}  // namespace mps

using mps::rec;

extern "C" {

CCTStatusType mps_device_count(int* count) { return rec(cudaGetDeviceCount(count)); }
CCTStatusType mps_device_sm_count(int* count) {
    if (!count) return CCT_PARAMERR;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(count, cudaDevAttrMultiProcessorCount, dev);
    return rec(e);
}
CCTStatusType mps_set_device(int device) { return rec(cudaSetDevice(device)); }
CCTStatusType mps_malloc(void** ptr, size_t bytes) { return rec(cudaMalloc(ptr, bytes ? bytes : 1)); }
CCTStatusType mps_free(void* ptr) { return rec(cudaFree(ptr)); }
CCTStatusType mps_memset(void* ptr, int value, size_t bytes) { return rec(cudaMemset(ptr, value, bytes)); }
CCTStatusType mps_memcpy_htod(void* dst, const void* src, size_t bytes) {
    return rec(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
}
CCTStatusType mps_memcpy_dtoh(void* dst, const void* src, size_t bytes) {
    return rec(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
}
CCTStatusType mps_memcpy_dtod(void* dst, const void* src, size_t bytes) {
    return rec(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToDevice));
}
CCTStatusType mps_host_alloc_pinned(void** ptr, size_t bytes) { return rec(cudaMallocHost(ptr, bytes ? bytes : 1)); }
CCTStatusType mps_host_free_pinned(void* ptr) { return rec(cudaFreeHost(ptr)); }
CCTStatusType mps_stream_create(void** stream) {
    return rec(cudaStreamCreateWithFlags((cudaStream_t*)stream, cudaStreamNonBlocking));
}
CCTStatusType mps_stream_destroy(void* stream) { return rec(cudaStreamDestroy((cudaStream_t)stream)); }
CCTStatusType mps_stream_sync(void* stream) { return rec(cudaStreamSynchronize((cudaStream_t)stream)); }
CCTStatusType mps_device_sync(void) { return rec(cudaDeviceSynchronize()); }
CCTStatusType mps_event_create(void** event) { return rec(cudaEventCreate((cudaEvent_t*)event)); }
CCTStatusType mps_event_destroy(void* event) { return rec(cudaEventDestroy((cudaEvent_t)event)); }
CCTStatusType mps_event_record(void* event, void* stream) {
    return rec(cudaEventRecord((cudaEvent_t)event, (cudaStream_t)stream));
}
CCTStatusType mps_event_elapsed_ms(void* start, void* stop, float* ms) {
    return rec(cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)stop));
}
const char* mps_last_error(void) {
    // a failing runtime call also leaves its error pending: keep the message that names
    // the failing step and append what is pending, if it is not already part of it
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        const char* what = cudaGetErrorString(e);
        if (strcmp(mps::g_err, "no error") == 0) {
            snprintf(mps::g_err, sizeof(mps::g_err), "%s", what);
        } else if (!strstr(mps::g_err, what)) {
            const size_t len = strlen(mps::g_err);
            snprintf(mps::g_err + len, sizeof(mps::g_err) - len, " (pending: %s)", what);
        }
    }
    return mps::g_err;
}
void mps_clear_error(void) {
    cudaGetLastError();
    snprintf(mps::g_err, sizeof(mps::g_err), "no error");
}
size_t mps_scratch_bytes(void) {
    size_t s = 0;
    for (auto& x : mps::g_slots) s += x.bytes;
    return s;
}
const char* mps_build_info(void) { return "gb300-mps 0.1 sm_103a"; }

unsigned long long mps_kernel_launches(void) { return __atomic_load_n(&mps::g_kernel_launches, __ATOMIC_RELAXED); }

}  // extern "C"
