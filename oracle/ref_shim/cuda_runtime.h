/* Host stand-in for <cuda_runtime.h> used only when oracle/ref_harness.cpp compiles
 * the reference's kernel header for the CPU: the vector types and the few runtime
 * names that header mentions.  Test infrastructure only. */
#pragma once
struct float3 { float x, y, z; };
struct double3 { double x, y, z; };
struct int3 { int x, y, z; };
typedef int cudaError_t;
typedef void* cudaStream_t;
#define cudaSuccess 0
#define cudaErrorInvalidValue 1
static inline const char* cudaGetErrorString(int) { return ""; }
static inline float3 make_float3(float x, float y, float z) { float3 t; t.x = x; t.y = y; t.z = z; return t; }
static inline int3 make_int3(int x, int y, int z) { int3 t; t.x = x; t.y = y; t.z = z; return t; }
