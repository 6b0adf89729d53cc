/*
 * ref_gpu_harness.cu - runs the reference solver's own particle kernels on the GPU.
 *
 * TEST INFRASTRUCTURE ONLY (the second baseline: the reference's kernels compiled for
 * sm_103a on the same GB300).  This file contains no solver arithmetic of its own: it
 * includes the reference's kernel header (DeviceProcess_Kernel.h with the DataType.h /
 * Constant.h / Utility_Inline.h it includes, decoded by oracle/build_ref.py into
 * oracle/_ref/src/), binds the reference's __constant__ symbols from a bindings record
 * with the layout of oracle/mps_oracle.h's OrcBindings (device pointers here), and
 * launches five of its __global__ kernels with the reference's own launch geometry
 * (CThreadScaler, DeviceProcess.cu: blocks of min(256, N) threads, ceil(N / 256)
 * blocks).  oracle/build_ref.py compiles it twice: with nvcc's default contraction of
 * multiply-adds (as the reference's project builds it; timing) and with -fmad=false
 * (bit-for-bit comparison with the library's reference-named launchers).
 *
 * Kernels: CalcSTLDistance_Kernel (DeviceProcess_Kernel.h:853-919), CalcDragEffect_Kernel
 * (:309-389), CalcExplicitly_Kernel (:390-582), CalcExplicitPressure_Kernel
 * (:921-1054), CalcExplicitPressureGradient_Kernel (:1056-1271).  Memory safety, read
 * from the kernel source: the last four return for thread indices >= N; the STL kernel
 * has no such guard, so its threads up to the grid's end read the sorted positions and
 * write the distance and triangle-ID arrays at their own index: the caller allocates
 * those arrays with room for the whole grid (N rounded up to 256).  Every other index
 * the kernels form comes from the cell tables, the sorted-to-original map and the
 * per-cell triangle lists, which the caller builds with the library's launchers (the
 * reference's own hash/reorder reads hash[-1] and its triangle binning races on the
 * per-cell counts; neither runs here).
 */
#include <cuda_runtime.h>

#include "DeviceProcess_Kernel.h"

struct HarnessBindings {
    CParameter param;
    CGridBox box;
    int particle_num;
    int max_particle_num;
    Integer* id;
    Scalar3* pos;
    Scalar3* vel;
    Scalar* pressure;
    Scalar* density;
    Scalar* temperature;
    Scalar* kin_visc;
    Scalar* solid_rate;
    ParticleType* type;
    Integer* out_id;
    Scalar3* out_pos;
    Scalar3* out_vel;
    Scalar* out_pressure;
    Scalar* out_density;
    Scalar* out_temperature;
    Scalar* out_kin_visc;
    Scalar* out_solid_rate;
    ParticleType* out_type;
    CTriangle* triangles;
    int triangle_num;
    CTriangleParameters* tri_params;
    CDistance* stl_distance;
    Integer* stl_id;
    CCell* cells;
    int cell_num;
    int* cell_start;
    int* cell_end;
    DragParameter* drag_params;
    int drag_num;
    Scalar3* drag_acc;
    Scalar* drag_temperature;
    Integer* magnifier_count;
    Scalar* turb_visc;
    Scalar* strain;
};

#define HARNESS_SET(sym, val)                                                   \
    do {                                                                       \
        const auto v_ = (val);                                                 \
        const cudaError_t e_ = cudaMemcpyToSymbol(sym, &v_, sizeof(v_));        \
        if (e_ != cudaSuccess) return (int)e_;                                 \
    } while (0)

extern "C" {

/* the reference's __constant__ symbols (InitializeDeviceMemConst,
 * InitializeDeviceConst{Input,OutPut}Particles, DragParametersToConst,
 * ParticleNumberToConst; DeviceProcess.cu:284-408) from device pointers */
int refgpu_bind(const HarnessBindings* b) {
    HARNESS_SET(CONSTANT_PARAMETER, b->param);
    HARNESS_SET(CONSTANT_BOUNDINGBOX, b->box);
    HARNESS_SET(c_ParticleNum, (Integer)b->particle_num);
    HARNESS_SET(c_MaxParticleNum, (Integer)b->max_particle_num);
    HARNESS_SET(c_daParticleID, b->id);
    HARNESS_SET(c_daParticlePosition, b->pos);
    HARNESS_SET(c_daParticleVelocity, b->vel);
    HARNESS_SET(c_daParticlePressure, b->pressure);
    HARNESS_SET(c_daParticleDensity, b->density);
    HARNESS_SET(c_daParticleTemperature, b->temperature);
    HARNESS_SET(c_daParticleKineticViscosity, b->kin_visc);
    HARNESS_SET(c_daParticleSolidPhaseRate, b->solid_rate);
    HARNESS_SET(c_daParticleType, b->type);
    HARNESS_SET(c_daOutputParticleID, b->out_id);
    HARNESS_SET(c_daOutputParticlePosition, b->out_pos);
    HARNESS_SET(c_daOutputParticleVelocity, b->out_vel);
    HARNESS_SET(c_daOutputParticlePressure, b->out_pressure);
    HARNESS_SET(c_daOutputParticleDensity, b->out_density);
    HARNESS_SET(c_daOutputParticleTemperature, b->out_temperature);
    HARNESS_SET(c_daOutputParticleKineticViscosity, b->out_kin_visc);
    HARNESS_SET(c_daOutputParticleSolidPhaseRate, b->out_solid_rate);
    HARNESS_SET(c_daOutputParticleType, b->out_type);
    HARNESS_SET(c_daTriangles, b->triangles);
    HARNESS_SET(c_TriangleNum, (Integer)b->triangle_num);
    HARNESS_SET(c_daTrianglesParameters, b->tri_params);
    HARNESS_SET(c_daSTLDistance, b->stl_distance);
    HARNESS_SET(c_daSTLID, b->stl_id);
    HARNESS_SET(c_daCell, b->cells);
    HARNESS_SET(c_CellNum, (Integer)b->cell_num);
    HARNESS_SET(c_cellStart, b->cell_start);
    HARNESS_SET(c_cellEnd, b->cell_end);
    HARNESS_SET(c_daSTLDragParameter, b->drag_params);
    HARNESS_SET(c_DragTriangleNum, (Integer)b->drag_num);
    HARNESS_SET(c_daDragAcc, b->drag_acc);
    HARNESS_SET(c_daDragTemperature, b->drag_temperature);
    HARNESS_SET(c_daMagnifierCount, b->magnifier_count);
    HARNESS_SET(c_daParticleTurbulaceViscosity, b->turb_visc);
    HARNESS_SET(c_daParticleStrainTensorProduct, b->strain);
    return 0;
}

/* layout probe: the bindings record's size, checked against the tests' OrcBindings */
int refgpu_sizeof_bindings(void) { return (int)sizeof(HarnessBindings); }

/* c_ParticleNum after a compaction (ParticleNumberToConst) */
int refgpu_particle_num(int n) {
    HARNESS_SET(c_ParticleNum, (Integer)n);
    return 0;
}

/* grid size the STL kernel's caller must allocate its per-particle arrays for */
int refgpu_grid_items(int n) {
    if (n <= 0) return 0;
    const int db = n < BLOCK_MAX_DIM ? n : BLOCK_MAX_DIM;
    return (n + db - 1) / db * db;
}

enum { REFGPU_STL = 0, REFGPU_DRAG = 1, REFGPU_EXPLICITLY = 2, REFGPU_PRESSURE = 3, REFGPU_GRADIENT = 4 };

/* one kernel over n particles on the stream, launched as the reference launches it */
int refgpu_launch(int kernel, cudaStream_t stream, int n) {
    if (n <= 0) return 0;
    const int db = n < BLOCK_MAX_DIM ? n : BLOCK_MAX_DIM;
    const int dg = (n + db - 1) / db;
    switch (kernel) {
        case REFGPU_STL: CalcSTLDistance_Kernel<<<dg, db, 0, stream>>>(n); break;
        case REFGPU_DRAG: CalcDragEffect_Kernel<<<dg, db, 0, stream>>>(n); break;
        case REFGPU_EXPLICITLY: CalcExplicitly_Kernel<<<dg, db, 0, stream>>>(n); break;
        case REFGPU_PRESSURE: CalcExplicitPressure_Kernel<<<dg, db, 0, stream>>>(n); break;
        case REFGPU_GRADIENT: CalcExplicitPressureGradient_Kernel<<<dg, db, 0, stream>>>(n); break;
        default: return (int)cudaErrorInvalidValue;
    }
    return (int)cudaGetLastError();
}

}  // extern "C"
