/*
 * ref_harness.cpp - runs the reference solver's own kernel code on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  This file contains no solver arithmetic of its own:
 * it includes the reference's kernel header (DeviceProcess_Kernel.h and the
 * DataType.h / Constant.h / Utility_Inline.h it includes, decoded from UTF-16 by
 * oracle/build_ref.py into oracle/_ref/src/), maps the CUDA keywords to host C++,
 * binds the reference's __constant__ pointer symbols from an OrcBindings struct and
 * runs each __global__ kernel serially over its thread index.  The result is
 * oracle/_ref/libref.so, exporting the same orc_* names as oracle/liborc.so, which
 * tests/test_oracle_pin.py uses to pin the oracle restatement bit for bit.
 *
 * Serial execution is a valid schedule of every kernel used here: the particle
 * kernels are one-thread-per-item without inter-thread communication, triangle
 * binning's atomics become plain read-modify-writes executed in triangle-id
 * order, and reorderDataAndFindCellStartD's shared-memory halo works when the
 * threads of one block run in index order.
 *
 * Entry points whose reference code is host code that does not build here
 * (compaction in CGPUCellSet.cpp, the lambda table in MultiGPUHandler.cpp, the
 * Thrust sort) are not exported.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "cuda_runtime.h"

struct HarnessDim3 { unsigned x, y, z; };
static thread_local HarnessDim3 blockIdx, threadIdx, blockDim, gridDim;
#define __global__
#define __constant__ static
#define __shared__
#define __device__
#define __host__
#define __inline__ inline
#define __CUDACC__ 1
static int sharedHash[(1 << 22) + 1];
static inline unsigned atomicCAS(unsigned* a, unsigned cmp, unsigned val) {
    unsigned old = *a;
    if (old == cmp) *a = val;
    return old;
}
static inline unsigned atomicInc(unsigned* a, unsigned lim) {
    unsigned old = *a;
    *a = (old >= lim) ? 0 : old + 1;
    return old;
}
static inline void __syncthreads() {}
using std::isfinite;
using std::max;
using std::min;
/* device code's abs(float) and sqrt(float) are the float overloads: the same here
 * (the C library's ::abs(int) and ::sqrt(double) would convert) */
using std::abs;
using std::sqrt;

#include "DataType.h"
#include "DeviceProcess_Kernel.h"

/* Same layout as OrcBindings in oracle/mps_oracle.h, spelled with the reference's
 * own type names. */
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

/* Equivalent of InitializeDeviceMemConst / InitializeDeviceConst{Input,OutPut}
 * Particles / DragParametersToConst (DeviceProcess.cu:284-408). */
static void bind(const HarnessBindings* b) {
    CONSTANT_PARAMETER = b->param;
    CONSTANT_BOUNDINGBOX = b->box;
    c_ParticleNum = b->particle_num;
    c_MaxParticleNum = b->max_particle_num;
    c_daParticleID = b->id;
    c_daParticlePosition = b->pos;
    c_daParticleVelocity = b->vel;
    c_daParticlePressure = b->pressure;
    c_daParticleDensity = b->density;
    c_daParticleTemperature = b->temperature;
    c_daParticleKineticViscosity = b->kin_visc;
    c_daParticleSolidPhaseRate = b->solid_rate;
    c_daParticleType = b->type;
    c_daOutputParticleID = b->out_id;
    c_daOutputParticlePosition = b->out_pos;
    c_daOutputParticleVelocity = b->out_vel;
    c_daOutputParticlePressure = b->out_pressure;
    c_daOutputParticleDensity = b->out_density;
    c_daOutputParticleTemperature = b->out_temperature;
    c_daOutputParticleKineticViscosity = b->out_kin_visc;
    c_daOutputParticleSolidPhaseRate = b->out_solid_rate;
    c_daOutputParticleType = b->out_type;
    c_daTriangles = b->triangles;
    c_TriangleNum = b->triangle_num;
    c_daTrianglesParameters = b->tri_params;
    c_daSTLDistance = b->stl_distance;
    c_daSTLID = b->stl_id;
    c_daCell = b->cells;
    c_CellNum = b->cell_num;
    c_cellStart = b->cell_start;
    c_cellEnd = b->cell_end;
    c_daSTLDragParameter = b->drag_params;
    c_DragTriangleNum = b->drag_num;
    c_daDragAcc = b->drag_acc;
    c_daDragTemperature = b->drag_temperature;
    c_daMagnifierCount = b->magnifier_count;
    c_daParticleTurbulaceViscosity = b->turb_visc;
    c_daParticleStrainTensorProduct = b->strain;
}

/* Run a one-thread-per-item kernel: block size 1, block index = item.  Items are
 * independent in every kernel run this way, so they are spread over OpenMP threads
 * (the CUDA index variables above are thread-local). */
template <class K>
static void run_items(int n, K k) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; ++i) {
        blockDim.x = 1;
        threadIdx.x = 0;
        blockIdx.x = (unsigned)i;
        k();
    }
}
template <class K>
static void run_items_serial(int n, K k) {
    blockDim.x = 1;
    threadIdx.x = 0;
    for (int i = 0; i < n; ++i) {
        blockIdx.x = (unsigned)i;
        k();
    }
}

extern "C" {

float orc_sqrt_utility(float x) { return sqrt_utility(x); }
float orc_calc_distance(const Scalar3* a, const Scalar3* b) { return CalcDistance(a, b); }
float orc_get_weight(float re, float r) { return GetWeight(re, r); }
float orc_zgrad(float r, float l0) { return GetZValueFunctionGradient(r, l0); }
float orc_zlap(float r, float l0) { return GetZValueFunctionLaplacian(r, l0); }
float orc_zgrad2d(float r, float l0) { return GetZValueFunctionGradient2D(r, l0); }
float orc_zlap2d(float r, float l0) { return GetZValueFunctionLaplacian2D(r, l0); }
float orc_triangle_distance(const CTriangle* t, const Scalar3* p, Scalar3* dir) { return CalcDistance(t, p, dir); }
int orc_cell_id(const CGridBox* box, const Scalar3* p, int* i, int* j, int* k) { return GetCellID(box, p, *i, *j, *k); }
int orc_is_include(const CGridBox* box, const Scalar3* p, float tol) { return IsInclude(box, p, tol) ? 1 : 0; }
void orc_correct_velocity(const CParameter* param, Scalar3* v) {
    CParameter p = *param;
    CorrectVelocity(&p, *v);
}

int orc_calc_hash(const HarnessBindings* b, int n, int* hash, int* index, Scalar3* pos) {
    bind(b);
    run_items(n, [&] { calcHashD(n, hash, index, pos); });
    return CCT_NOERR;
}

int orc_reorder_find_cell_start(HarnessBindings* b, int n, int cells, const int* hash, const int* index,
                                int* cs, int* ce) {
    if (n <= 0) return CCT_NOERR;
    if (n > (1 << 22)) return CCT_PARAMERR;
    bind(b);
    std::memset(cs, 0xff, sizeof(int) * cells);
    std::memset(ce, 0xff, sizeof(int) * cells);
    /* one block of n threads run in index order; the kernel reads hash[index-1]
     * at index 0, so hand it a copy with one leading pad element. */
    std::vector<int> h(n + 1);
    h[0] = 0;
    std::memcpy(h.data() + 1, hash, sizeof(int) * n);
    std::vector<int> idx(index, index + n);
    blockDim.x = (unsigned)n;
    blockIdx.x = 0;
    for (int t = 0; t < n; ++t) {
        threadIdx.x = (unsigned)t;
        reorderDataAndFindCellStartD(n, cells, h.data() + 1, idx.data(), cs, ce);
    }
    return CCT_NOERR;
}

int orc_reset_triangle_topology(int cells, CCell* cell) {
    c_daCell = cell;
    run_items(cells, [&] { ResetTriangleTopology_Kernel(cells, cell); });
    return CCT_NOERR;
}

int orc_register_triangle_topology(HarnessBindings* b, const CTriangle* tri, int t, CCell* cell, int cells) {
    bind(b);
    run_items_serial(t, [&] { RegisterTriangleTopology_Kernel(tri, t, cell, cells); });
    return CCT_NOERR;
}

int orc_update_triangle_position(HarnessBindings* b, int t) {
    bind(b);
    run_items(t, [&] { UpdateTrianglePosition_Kernel(t, b->triangles); });
    return CCT_NOERR;
}

int orc_rotate_triangle_position(HarnessBindings* b, int t, int step) {
    bind(b);
    run_items(t, [&] { RotateTrianglePosition_Kernel(t, b->triangles, step); });
    return CCT_NOERR;
}

int orc_reset_wall_position(HarnessBindings* b, int t, int step, const CTriangle* orig) {
    bind(b);
    run_items(t, [&] { ResetWallPosition_Kernel(t, step, orig); });
    return CCT_NOERR;
}

int orc_calc_stl_distance(HarnessBindings* b, int n) {
    bind(b);
    for (int i = 0; i < n; ++i) b->stl_id[i] = -1;
    run_items(n, [&] { CalcSTLDistance_Kernel(n); });
    return CCT_NOERR;
}

int orc_calc_drag_effect(HarnessBindings* b, int n) {
    bind(b);
    run_items(n, [&] { CalcDragEffect_Kernel(n); });
    return CCT_NOERR;
}

int orc_calc_explicitly(HarnessBindings* b, int n) {
    bind(b);
    run_items(n, [&] { CalcExplicitly_Kernel(n); });
    return CCT_NOERR;
}

int orc_calc_temperature_factor(HarnessBindings* b, int n) {
    bind(b);
    run_items(n, [&] { CalcTemperatureFactor_Kernel(n); });
    return CCT_NOERR;
}

int orc_calc_turbulence_viscosity(HarnessBindings* b, int n) {
    bind(b);
    run_items(n, [&] { CalcTurbulenceViscosity_Kernel(n); });
    return CCT_NOERR;
}

int orc_calc_explicit_pressure(HarnessBindings* b, int n) {
    bind(b);
    run_items(n, [&] { CalcExplicitPressure_Kernel(n); });
    return CCT_NOERR;
}

int orc_calc_explicit_pressure_gradient(HarnessBindings* b, int n) {
    bind(b);
    run_items(n, [&] { CalcExplicitPressureGradient_Kernel(n); });
    return CCT_NOERR;
}

/* Layout probes for the types test. */
int ref_sizeof_cparameter(void) { return (int)sizeof(CParameter); }
int ref_sizeof_ctriangle_parameters(void) { return (int)sizeof(CTriangleParameters); }
int ref_sizeof_cgridbox(void) { return (int)sizeof(CGridBox); }
int ref_sizeof_drag_parameter(void) { return (int)sizeof(DragParameter); }

}  // extern "C"
