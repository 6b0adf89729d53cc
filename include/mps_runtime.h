/*
 * mps_runtime.h - small device-memory, stream and timing helpers of the library.
 *
 * No counterpart in the reference (its host code calls the CUDA runtime directly).
 * They let a caller without CUDA headers (ctypes, a cgo/JNI shim) allocate the
 * device arrays the launcher API binds, move data, and time launches with CUDA
 * events on the launching stream.  All return CCT_NOERR or CCT_CUDAERR.
 */
#ifndef MPS_RUNTIME_H
#define MPS_RUNTIME_H

#include <stddef.h>
#include <stdint.h>

#include "mps_types.h"

#ifdef __cplusplus
extern "C" {
#endif

CCTStatusType mps_device_count(int* count);
/* streaming multiprocessors of the current device */
CCTStatusType mps_device_sm_count(int* count);
CCTStatusType mps_set_device(int device);
CCTStatusType mps_malloc(void** ptr, size_t bytes);
CCTStatusType mps_free(void* ptr);
CCTStatusType mps_memset(void* ptr, int value, size_t bytes);
CCTStatusType mps_memcpy_htod(void* dst, const void* src, size_t bytes);
CCTStatusType mps_memcpy_dtoh(void* dst, const void* src, size_t bytes);
CCTStatusType mps_memcpy_dtod(void* dst, const void* src, size_t bytes);
CCTStatusType mps_host_alloc_pinned(void** ptr, size_t bytes);
CCTStatusType mps_host_free_pinned(void* ptr);
CCTStatusType mps_stream_create(void** stream);   /* cudaStream_t written to *stream */
CCTStatusType mps_stream_destroy(void* stream);
CCTStatusType mps_stream_sync(void* stream);
CCTStatusType mps_device_sync(void);
CCTStatusType mps_event_create(void** event);
CCTStatusType mps_event_destroy(void* event);
CCTStatusType mps_event_record(void* event, void* stream);
CCTStatusType mps_event_elapsed_ms(void* start, void* stop, float* ms);
/* last CUDA error string of the calling thread (never NULL) */
const char* mps_last_error(void);
/* resets the recorded error and the CUDA runtime's last (non-sticky) error */
void mps_clear_error(void);
/* bytes of library-owned scratch currently held by the reference-named entry points */
size_t mps_scratch_bytes(void);
/* build identification: "sm_103a" and the library version */
const char* mps_build_info(void);
/* kernels this library has launched since it was loaded (all threads, all devices) */
unsigned long long mps_kernel_launches(void);

#ifdef __cplusplus
}
#endif

#endif
