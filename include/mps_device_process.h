/*
 * mps_device_process.h - the reference-named kernel launcher API (drop-in boundary).
 *
 * Replaces radix/SPVSOLVER/MultiGPUSolver/DeviceProcess.h:78-120 (implemented there
 * in DeviceProcess.cu:49-409).  Same names, argument order and meaning; every call
 * returns a CCTStatusType (CCT_NOERR on success, CCT_CUDAERR when a launch fails,
 * CCT_PARAMERR for a feature this library does not implement) and returns CCT_NOERR
 * without work for counts <= 0.  The caller owns every device array
 * (CGPUCellSet.cpp:487-635 allocates them); the binding calls record the pointers
 * once, like the reference's __constant__ symbols, and each launcher uses them.
 *
 * cudaStream_t& is a C++ reference: the ABI passes the address of the caller's
 * cudaStream_t variable (a C or ctypes caller passes a pointer to a stream handle).
 *
 * Semantics are the reference's, bit for bit in float, with these documented
 * differences (all on inputs the reference would mis-handle):
 *   - every kernel checks its index against the count (CalcSTLDistance_Kernel,
 *     DeviceProcess_Kernel.h:857-860, has that check commented out);
 *   - cell bounds ignore keys outside [0, CellNum) (the reference writes out of bounds
 *     there, and reads gridParticleHash[-1], DeviceProcess_Kernel.h:75);
 *   - RegisterTriangleTopology lists a cell's triangles in ascending triangle id (the
 *     reference's atomics give an arbitrary order); the set and the 100-entry
 *     capacity are the reference's;
 *   - SortUsingThrust runs a stable LSD radix sort (the order thrust::sort_by_key
 *     produces for int keys) and synchronises the legacy default stream;
 *   - CheckParticleOutsideComputeZone performs on the GPU the compaction the reference
 *     does on the host (CGPUCellSet.cpp:1160-1202), in the same order; ParticleNum is a
 *     HOST pointer (in: count, out: remaining count) and the call synchronises Stream.
 *     It works on the output-order arrays bound by InitializeDeviceConstOutPutParticles.
 *   - CalcTemperatureFactor (DeviceProcess_Kernel.h:705-852) and CalcTurbulenceViscosity
 *     (:1273-1476) run whatever the parameter's switches say, as the reference's
 *     launchers do; the caller calls them only when bUpdateTemperature / bTurbulance
 *     is on.  CalcTurbulenceViscosity and a turbulent CalcExplicitly need the last two
 *     arrays of InitializeDeviceConstInputParticles (CCT_PARAMERR when they are null).
 *   - CalcExplicitPressureGradient returns CCT_PARAMERR when bNegativePressure is on.
 */
#ifndef MPS_DEVICE_PROCESS_H
#define MPS_DEVICE_PROCESS_H

#include <cuda_runtime.h>

#include "mps_types.h"

#ifdef __cplusplus
extern "C" {
#define MPS_STREAM_REF cudaStream_t&
#else
#define MPS_STREAM_REF cudaStream_t*
#endif

/* per-step launchers */
CCTStatusType CalcTurbulenceViscosity(MPS_STREAM_REF Stream, Integer ComputeParticleNum);
CCTStatusType CheckParticleOutsideComputeZone(MPS_STREAM_REF Stream, Integer* ParticleNum);
CCTStatusType CalcDragEffect(MPS_STREAM_REF Stream, Integer ComputeParticleNum);
CCTStatusType CalcExplicitly(MPS_STREAM_REF Stream, Integer ParticleNum);
CCTStatusType CalcExplicitPressure(MPS_STREAM_REF Stream, Integer ComputeParticleNum);
CCTStatusType CalcExplicitPressureGradient(MPS_STREAM_REF Stream, Integer ComputeParticleNum);
CCTStatusType CalcTemperatureFactor(MPS_STREAM_REF Stream, Integer ComputeParticleNum);
CCTStatusType RegisterTriangleTopology(MPS_STREAM_REF Stream, CTriangle* daTriangle, Integer TriangleNum, CCell* daCell,
                                       Integer CellNum);
CCTStatusType ResetTriangleTopology(MPS_STREAM_REF Stream, Integer CellNum, CCell* aCell);
CCTStatusType ResetWallPosition(MPS_STREAM_REF Stream, const Integer TriangleNum, const Integer AnalysisStep,
                                const CTriangle* daTriangles);
CCTStatusType UpdateTrianglePosition(MPS_STREAM_REF Stream, const Integer TriangleNum, CTriangle* daTriangles);
CCTStatusType RotateTrianglePosition(MPS_STREAM_REF Stream, const Integer TriangleNum, CTriangle* daTriangles,
                                     const Integer analysisStep);
CCTStatusType CalcSTLDistance(MPS_STREAM_REF Stream, Integer ComputeParticleNum);
CCTStatusType CaculateCellIDandInitializeHash(MPS_STREAM_REF Stream, Integer ParticleNum, Integer CellNum,
                                              int* dGridParticleHash, int* dGridParticleIndex,
                                              Scalar3* particlePosition);
CCTStatusType reorderDataAndFindCellStart(MPS_STREAM_REF Stream, Integer numParticles, Integer numCells,
                                          int* gridParticleHash, int* gridParticleIndex, int* cellStart,
                                          int* cellEnd);
CCTStatusType SortUsingThrust(Integer MaxParticleNum, Integer* daNumberHash, Integer* daNumberIndex);
CCTStatusType StableSortUsingThrust(Integer MaxParticleNum, Integer* daNumberHash, Integer* daNumberIndex);
/* No counterpart in the reference.  SortUsingThrust for callers that cannot allocate
 * device memory (an allocator hook, a pre-reserved memory pool, a real-time path):
 * same result, but its scratch is one static __device__ array of about 2.1 MiB held by
 * every GPU that loads the library.  At most 262,144 keys (more: CCT_PARAMERR, arrays
 * untouched).  Every call looks up the array's device address on the current device
 * (nothing cached, so a device reset leaves no stale address); the first call on a device
 * also loads the library's module there: make it before any stream capture.  Calls share
 * the array: calls that overlap on the GPU race. */
CCTStatusType SortUsingThrustNoAlloc(Integer MaxParticleNum, Integer* daNumberHash, Integer* daNumberIndex);

/* one-time binding calls */
CCTStatusType InitializeDeviceMemConst(CParameter Parameter, Integer ParticleNum, CTriangle* Triangles,
                                       Integer TriangleNum, CTriangleParameters* TriangleParameters,
                                       Integer MaxParticleNum, CDistance* STLDistance, Integer* StlID, CCell* Cell,
                                       Integer CellNum, Integer* CellStart, Integer* CellEnd,
                                       Integer* GridParticleIndex, CGridBox BoundingBox);
CCTStatusType InitializeDeviceConstOutPutParticles(Integer* OutputParticleID, Scalar3* OutputParticlePosition,
                                                   Scalar3* OutputParticleVelocity, Scalar* OutputParticlePressure,
                                                   Scalar* OutputParticleDensity, Scalar* OutputParticleTemperature,
                                                   Scalar* OutputParticleKineticViscosity,
                                                   Scalar* OutputParticleSolidPhaseRate,
                                                   ParticleType* OutputParticleType);
CCTStatusType InitializeDeviceConstInputParticles(Integer* InputParticleID, Scalar3* InputParticlePosition,
                                                  Scalar3* InputParticleVelocity, Scalar* InputParticlePressure,
                                                  Scalar* InputParticleDensity, Scalar* InputParticleTemperature,
                                                  Scalar* InputParticleKineticViscosity,
                                                  Scalar* InputParticleSolidPhaseRate, ParticleType* InputParticleType,
                                                  Scalar* ParticleTurbulaceViscosity,
                                                  Scalar* ParticleStrainTensorProduct);
CCTStatusType ParticleNumberToConst(Integer ParticleNum);
CCTStatusType DragParametersToConst(DragParameter* InputDragParameter, Scalar3* InputDragAcc,
                                    Scalar* InputDragTemperature, Integer DragTriangleNum, Integer* MagnifierCount,
                                    CDragTriangle* DragTriangles);

#ifdef __cplusplus
}
#endif
#undef MPS_STREAM_REF

#endif
