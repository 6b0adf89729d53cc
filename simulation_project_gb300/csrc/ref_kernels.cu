// ref_kernels.cu - the reference solver's explicit-schedule kernels, GB300 build, and
// the reference-named C-ABI that a caller of the reference's launcher API binds.
//
// Boundary: radix/SPVSOLVER/MultiGPUSolver/DeviceProcess.h:78-120 (declarations) and
// DeviceProcess.cu:49-409 (launchers).  The reference binds every device array once
// through __constant__ pointer symbols (Constant.h:4-76, filled by
// InitializeDeviceMemConst & co.); here the same binding calls fill one host-side
// RefBind record that every launch passes to its kernel as a __grid_constant__
// parameter (it lands in the same constant bank, without cudaMemcpyToSymbol).
//
// This translation unit is compiled with -fmad=false: the float arithmetic below is
// written in the reference's operation order, so each kernel produces the reference's
// results bit for bit (checked against the oracle, which is itself pinned to the
// reference's kernel code).  Deviations, all on invalid inputs: every kernel checks
// its thread index against the item count (CalcSTLDistance_Kernel does not), cell
// bounds skip keys outside [0, cells) instead of writing out of bounds, and a cell's
// triangle list is filled in ascending triangle id (the reference's atomics give an
// arbitrary order).
#include <cfloat>
#include <stdio.h>

#include "mps_common.cuh"
#include "mps_internal.h"
#include "../../include/mps_device_process.h"

namespace mps {

struct RefBind {
    CParameter param;
    CGridBox box;
    int particle_num;
    int max_particle_num;
    int* id;
    Scalar3* pos;
    Scalar3* vel;
    float* pressure;
    float* density;
    float* temperature;
    float* kin_visc;
    float* solid_rate;
    int* type;
    int* out_id;
    Scalar3* out_pos;
    Scalar3* out_vel;
    float* out_pressure;
    float* out_density;
    float* out_temperature;
    float* out_kin_visc;
    float* out_solid_rate;
    int* out_type;
    CTriangle* triangles;
    int triangle_num;
    CTriangleParameters* tri_params;
    CDistance* stl_distance;
    int* stl_id;
    CCell* cells;
    int cell_num;
    int* cell_start;
    int* cell_end;
    int* grid_index;
    DragParameter* drag_params;
    int drag_num;
    Scalar3* drag_acc;
    float* drag_temperature;
    int* magnifier_count;
    CDragTriangle* drag_triangles;
    float* turb_visc;   // c_daParticleTurbulaceViscosity (sorted order)
    float* strain;      // c_daParticleStrainTensorProduct (sorted order)
};

static RefBind g_bind;

// ---------------------------------------------------------------------------
// grid
// ---------------------------------------------------------------------------
// calcHashD (DeviceProcess_Kernel.h:39-50)
__global__ void k_ref_hash(int n, const __grid_constant__ CGridBox box, const Scalar3* __restrict__ pos,
                           int* __restrict__ hash, int* __restrict__ index) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int a, b, c;
    hash[i] = ref_cell(box, pos[i], a, b, c);
    index[i] = i;
}

// reorderDataAndFindCellStartD (DeviceProcess_Kernel.h:54-124): cell bounds from
// key changes along the sorted keys, and the gather of the nine particle arrays.
__global__ void k_ref_reorder(int n, int cells, const int* __restrict__ hash, const int* __restrict__ index,
                              int* __restrict__ cs, int* __restrict__ ce, const __grid_constant__ RefBind b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int h = hash[i];
    const bool ok = h >= 0 && h < cells;
    if (i == 0 || h != hash[i - 1]) {
        if (ok) cs[h] = i;
        if (i > 0) {
            const int hp = hash[i - 1];
            if (hp >= 0 && hp < cells) ce[hp] = i;
        }
    }
    if (i == n - 1 && ok) ce[h] = i + 1;
    const int s = index[i];
    b.pos[i] = b.out_pos[s];
    b.vel[i] = b.out_vel[s];
    b.pressure[i] = b.out_pressure[s];
    b.density[i] = b.out_density[s];
    b.temperature[i] = b.out_temperature[s];
    b.kin_visc[i] = b.out_kin_visc[s];
    b.solid_rate[i] = b.out_solid_rate[s];
    b.type[i] = b.out_type[s];
    b.id[i] = s;
}

// Compaction with the order of CCellSet::CheckParticleOutsideComputeZone
// (CGPUCellSet.cpp:1160-1202): the j-th out-of-zone slot i (j = 1, 2, ...) takes the
// particle at N0 - j while i <= N0 - j; the taken particles are not re-checked.
// Sources are never earlier destinations, so one gather kernel suffices.
__global__ void k_ref_outside_flags(int n, const __grid_constant__ RefBind b, unsigned* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Scalar3 p = b.out_pos[i];
    flag[i] = in_zone<float>(b.box, p.x, p.y, p.z, b.param.Tolerance) ? 0u : 1u;
}
__global__ void k_ref_compact(int n, const __grid_constant__ RefBind b, const unsigned* __restrict__ flag,
                              const unsigned* __restrict__ rank, int* __restrict__ removed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    const int j = (int)rank[i] + 1;
    if (i > n - j) return;
    atomicAdd(removed, 1);
    const int s = n - j;
    if (s == i) return;
    b.out_pos[i] = b.out_pos[s];
    b.out_vel[i] = b.out_vel[s];
    b.out_pressure[i] = b.out_pressure[s];
    b.out_density[i] = b.out_density[s];
    b.out_temperature[i] = b.out_temperature[s];
    b.out_kin_visc[i] = b.out_kin_visc[s];
    b.out_solid_rate[i] = b.out_solid_rate[s];
    b.out_type[i] = b.out_type[s];
    b.out_id[i] = b.out_id[s];
}

// ---------------------------------------------------------------------------
// walls
// ---------------------------------------------------------------------------
// SegmentRatio / CalcDistanceVectorLine / CalcNormalDistance / CalcDistance(triangle)
// (Utility_Inline.h:56-232), reference arithmetic.
__device__ __forceinline__ float ref_segment_ratio(const Scalar3& p1, const Scalar3& p2, const Scalar3& p3) {
    const Scalar3 d = s3sub(p2, p1);
    float den = d.x * d.x + d.y * d.y + d.z * d.z;
    if (den == 0.0f) den = (float)1e-5;
    return (p3.x - p1.x) * (p2.x - p1.x) + (p3.y - p1.y) * (p2.y - p1.y) + (p3.z - p1.z) * (p2.z - p1.z) / den;
}
__device__ __forceinline__ Scalar3 ref_line(const Scalar3& l0, const Scalar3& l1, const Scalar3& p) {
    const float u = ref_segment_ratio(l0, l1, p);
    Scalar3 dv = s3(0, 0, 0);
    if (u >= 0 && u <= 1) {
        const Scalar3 v = s3sub(l1, l0);
        dv = s3sub(p, s3(l0.x + u * v.x, l0.y + u * v.y, l0.z + u * v.z));
    }
    if (u < 0) dv = s3sub(l1, p);
    if (u > 1) dv = s3sub(l0, p);
    return dv;
}
__device__ __forceinline__ float ref_tri_distance(const CTriangle& T, const Scalar3& p, Scalar3& dir) {
    const Scalar3 n = T.Normal;
    Scalar3 c;
    c.x = (float)((double)(T.Vertex[0].x + T.Vertex[1].x + T.Vertex[2].x) / 3.0);
    c.y = (float)((double)(T.Vertex[0].y + T.Vertex[1].y + T.Vertex[2].y) / 3.0);
    c.z = (float)((double)(T.Vertex[0].z + T.Vertex[1].z + T.Vertex[2].z) / 3.0);
    const float sd = ref_sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
    Scalar3 dv = s3(0, 0, 0);
    if (sd != 0.0f) {
        const float coef = ((n.x * p.x + n.y * p.y + n.z * p.z) - (n.x * c.x + n.y * c.y + n.z * c.z)) / sd;
        dv = s3(coef / sd * n.x, coef / sd * n.y, coef / sd * n.z);
    }
    const Scalar3 P = s3(p.x - dv.x, p.y - dv.y, p.z - dv.z);
    const Scalar3 v0 = s3sub(T.Vertex[2], T.Vertex[0]);
    const Scalar3 v1 = s3sub(T.Vertex[1], T.Vertex[0]);
    const Scalar3 v2 = s3sub(P, T.Vertex[0]);
    const float d00 = ref_dot(v0, v0), d01 = ref_dot(v0, v1), d02 = ref_dot(v0, v2);
    const float d11 = ref_dot(v1, v1), d12 = ref_dot(v1, v2);
    const float inv = 1.0f / (d00 * d11 - d01 * d01);
    const float u = (d11 * d02 - d01 * d12) * inv;
    const float v = (d00 * d12 - d01 * d02) * inv;
    if (u >= 0 && v >= 0 && u + v > 1) dv = ref_line(T.Vertex[1], T.Vertex[2], p);
    if (u < 0) dv = ref_line(T.Vertex[0], T.Vertex[1], p);
    if (v < 0) dv = ref_line(T.Vertex[0], T.Vertex[2], p);
    dir = dv;
    return ref_mag(dv);
}

// RegisterLine / RegisterTriangle (Utility_Inline.h:1745-1855): walk the three edges
// in cell-size steps, shrink the triangle toward its interior by one cell, repeat.
// Visit(cell) is called for every sample point inside the grid.
template <class Visit>
__device__ void ref_walk_line(const CGridBox& B, Scalar3 v, Scalar3 d, float m, int cells, Visit& visit) {
    float tab = 0.0f;
    int guard = 0;
    do {
        const Scalar3 t = s3(v.x + tab * d.x, v.y + tab * d.y, v.z + tab * d.z);
        int i, j, k;
        const int cid = ref_cell(B, t, i, j, k);
        if (cid >= 0 && cid < cells) visit(cid);
        tab += B.m_CellSize;
    } while (tab <= m && ++guard < 100000);
}
template <class Visit>
__device__ void ref_walk_triangle(const CGridBox& B, const CTriangle& T, int cells, Visit& visit) {
    Scalar3 A = T.Vertex[0], Bv = T.Vertex[1], C = T.Vertex[2];
    const float cs = B.m_CellSize;
    float mbc, mab, mca;
    int guard = 0;
    do {
        const Scalar3 ab = s3sub(Bv, A), ba = s3sub(A, Bv), bc = s3sub(C, Bv), cb = s3sub(Bv, C), ca = s3sub(A, C),
                      ac = s3sub(C, A);
        mbc = ref_mag(bc);
        mab = ref_mag(ab);
        mca = ref_mag(ca);
        if (mab > 0.0f) ref_walk_line(B, A, s3(ab.x / mab, ab.y / mab, ab.z / mab), mab, cells, visit);
        if (mbc > 0.0f) ref_walk_line(B, Bv, s3(bc.x / mbc, bc.y / mbc, bc.z / mbc), mbc, cells, visit);
        if (mca > 0.0f) ref_walk_line(B, C, s3(ca.x / mca, ca.y / mca, ca.z / mca), mca, cells, visit);
        Scalar3 am = s3add(ab, ac), bm = s3add(ba, bc), cm = s3add(ca, cb);
        const float mam = ref_mag(am), mbm = ref_mag(bm), mcm = ref_mag(cm);
        if (mam > 0.0f) {
            am.x /= mam; am.y /= mam; am.z /= mam;
            A.x += am.x * cs; A.y += am.y * cs; A.z += am.z * cs;
        }
        if (mbm > 0.0f) {
            bm.x /= mbm; bm.y /= mbm; bm.z /= mbm;
            Bv.x += bm.x * cs; Bv.y += bm.y * cs; Bv.z += bm.z * cs;
        }
        if (mcm > 0.0f) {
            cm.x /= mcm; cm.y /= mcm; cm.z /= mcm;
            C.x += cm.x * cs; C.y += cm.y * cs; C.z += cm.z * cs;
        }
    } while (mbc >= cs && mab >= cs && mca >= cs && ++guard < 100000);
}

struct CountVisit {
    int n = 0;
    __device__ void operator()(int) { ++n; }
};
struct StoreVisit {
    int* cell;
    int* tri;
    int t;
    int k = 0;
    __device__ void operator()(int c) { cell[k] = c; tri[k] = t; ++k; }
};

__global__ void k_tri_count(int t, const CTriangle* __restrict__ tri, const __grid_constant__ CGridBox box, int cells,
                            unsigned* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= t) return;
    CountVisit v;
    const CTriangle T = tri[i];
    ref_walk_triangle(box, T, cells, v);
    count[i] = (unsigned)v.n;
}
__global__ void k_tri_fill(int t, const CTriangle* __restrict__ tri, const __grid_constant__ CGridBox box, int cells,
                           const unsigned* __restrict__ off, int* __restrict__ vcell, int* __restrict__ vtri) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= t) return;
    StoreVisit v;
    v.cell = vcell + off[i];
    v.tri = vtri + off[i];
    v.t = i;
    const CTriangle T = tri[i];
    ref_walk_triangle(box, T, cells, v);
}
// visits sorted (stably) by cell: unique triangle ids per cell, ascending, first 100
__global__ void k_tri_bounds(int nv, const int* __restrict__ vcell, int* __restrict__ vs, int* __restrict__ ve) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int c = vcell[i];
    if (i == 0 || c != vcell[i - 1]) {
        vs[c] = i;
        if (i > 0) ve[vcell[i - 1]] = i;
    }
    if (i == nv - 1) ve[c] = i + 1;
}
__global__ void k_tri_cells(int cells, const int* __restrict__ vs, const int* __restrict__ ve,
                            const int* __restrict__ vtri, CCell* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    const int s = vs[c];
    if (s < 0) return;
    const int e = ve[c];
    unsigned cnt = out[c].m_TriangleNum;
    int last = -1;
    for (int i = s; i < e; ++i) {
        const int t = vtri[i];
        if (t == last) continue;
        last = t;
        bool have = false;
        for (unsigned l = 0; l < cnt; ++l)
            if (out[c].m_TriangleID[l] == t) { have = true; break; }
        if (!have && cnt < CELLMAXTRIANGLENUM) out[c].m_TriangleID[cnt++] = t;
    }
    out[c].m_TriangleNum = cnt;
}

// ResetTriangleTopology_Kernel (DeviceProcess_Kernel.h:594-602)
__global__ void k_tri_reset(int cells, CCell* __restrict__ cell) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < cells) cell[c].m_TriangleNum = 0;
}

// UpdateTrianglePosition_Kernel (DeviceProcess_Kernel.h:603-621)
__global__ void k_tri_translate(int t, CTriangle* __restrict__ tri, const __grid_constant__ RefBind b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= t) return;
    Scalar3 v = b.tri_params[tri[i].ModelIDNumber].Velocity;
    const float dt = b.param.Dt;
    v.x = v.x * dt; v.y = v.y * dt; v.z = v.z * dt;
    for (int q = 0; q < 3; ++q) tri[i].Vertex[q] = s3add(tri[i].Vertex[q], v);
}

// RotateTrianglePosition_Kernel (DeviceProcess_Kernel.h:622-689)
__global__ void k_tri_rotate(int t, CTriangle* __restrict__ tri, int step, const __grid_constant__ RefBind b) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= t) return;
    CTriangle& T = tri[id];
    const CTriangleParameters tp = b.tri_params[T.ModelIDNumber];
    if (!tp.RotatingOrNot) return;
    const float dt = b.param.Dt;
    if ((step * dt) < tp.RotationStartTime) return;
    float ang = 0.0f;
    const int req = (int)((tp.TimeToReachRPM - tp.RotationStartTime) / dt);
    const float tpass = dt * step;
    if ((tpass < tp.RotationStartTime) || (tp.AngleOfRotationInDegree == 0)) ang = 0.0f;
    else if ((tpass >= tp.RotationStartTime) && (tpass < tp.TimeToReachRPM))
        ang = (tp.AngleOfRotationInDegree / (req + 1)) * (step - (tp.RotationStartTime / dt));
    else ang = tp.AngleOfRotationInDegree;
    if (ang == 0) return;
    for (int q = 0; q < 3; ++q) {
        const float m = ref_dist(tp.SecondPointOfRotation, tp.CenterOfRotation);
        Scalar3 nv = s3(0, 0, 0);
        if (m > 0)
            nv = s3((tp.SecondPointOfRotation.x - tp.CenterOfRotation.x) / m,
                    (tp.SecondPointOfRotation.y - tp.CenterOfRotation.y) / m,
                    (tp.SecondPointOfRotation.z - tp.CenterOfRotation.z) / m);
        const float th = (float)((ang * 3.141592653589793238) / 180.0);
        const float a = tp.CenterOfRotation.x, bb = tp.CenterOfRotation.y, c = tp.CenterOfRotation.z;
        const float u = nv.x, v = nv.y, w = nv.z;
        const float x = T.Vertex[q].x, y = T.Vertex[q].y, z = T.Vertex[q].z;
        const float ct = cosf(th), st = sinf(th);
        T.Vertex[q].x = (a * (v * v + w * w) - (u * (bb * v + c * w - u * x - v * y - w * z))) * (1 - ct) + (x * ct) +
                        (((-c * v) + bb * w - w * y + v * z) * st);
        T.Vertex[q].y = (bb * (u * u + w * w) - (v * (a * u + c * w - u * x - v * y - w * z))) * (1 - ct) + (y * ct) +
                        (((c * u) - a * w + w * x - u * z) * st);
        T.Vertex[q].z = (c * (u * u + v * v) - (w * (a * u + bb * v - u * x - v * y - w * z))) * (1 - ct) + (z * ct) +
                        (((-bb * u) + a * v - v * x + u * y) * st);
    }
}

// ResetWallPosition_Kernel (DeviceProcess_Kernel.h:690-704)
__global__ void k_tri_reset_wall(int t, int step, const CTriangle* __restrict__ orig, const __grid_constant__ RefBind b) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= t) return;
    const CTriangleParameters& tp = b.tri_params[b.triangles[id].ModelIDNumber];
    if (tp.LinearMovableOrNot && tp.LinearResetInterval != 0 && 0 == ((step + 1) % tp.LinearResetInterval))
        b.triangles[id] = orig[id];
}

// Nearest triangle over the 27 cells, (k, j, i) order, first minimum wins.
__device__ void ref_nearest(const RefBind& b, const Scalar3& p, bool drag_only, CDistance& nd, int& nid) {
    int cx, cy, cz;
    const int cid = ref_cell(b.box, p, cx, cy, cz);
    if (!(cid >= 0 && cid < b.cell_num)) return;
    for (int k = -1; k <= 1; ++k)
        for (int j = -1; j <= 1; ++j)
            for (int i = -1; i <= 1; ++i) {
                const int m = cell_key(b.box.m_GridSize, cx + i, cy + j, cz + k);
                if (m < 0 || m >= b.cell_num) continue;
                const unsigned tn = b.cells[m].m_TriangleNum;
                for (unsigned l = 0; l < tn && l < CELLMAXTRIANGLENUM; ++l) {
                    const int t = b.cells[m].m_TriangleID[l];
                    if (t < 0 || t >= b.triangle_num) continue;
                    if (drag_only && !b.tri_params[b.triangles[t].ModelIDNumber].isDrag) continue;
                    if (t != nid) {
                        CDistance d;
                        d.Magnitude = ref_tri_distance(b.triangles[t], p, d.Direction);
                        if (d.Magnitude < nd.Magnitude) {
                            nd = d;
                            nid = t;
                        }
                    }
                }
            }
}

// CalcSTLDistance_Kernel (DeviceProcess_Kernel.h:853-919)
__global__ void k_ref_stl_distance(int n, const __grid_constant__ RefBind b) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    CDistance nd;
    nd.Magnitude = 1e8f;
    nd.Direction = s3(0, 0, 0);
    int nid = -1;
    ref_nearest(b, b.pos[id], false, nd, nid);
    b.stl_distance[id] = nd;
    b.stl_id[id] = nid;
}

// CalcDragEffect_Kernel and mode helpers (DeviceProcess_Kernel.h:125-389), with the
// reference's index use and brace placement (mode 'F' acts outside the region).
__global__ void k_ref_drag(int n, const __grid_constant__ RefBind b) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const CParameter& P = b.param;
    if (b.magnifier_count[id] > 0) b.magnifier_count[id]++;
    if (b.magnifier_count[id] == 10) b.magnifier_count[id] = 0;
    CDistance nd;
    nd.Magnitude = 1e8f;
    nd.Direction = s3(0, 0, 0);
    int nid = -1;
    if (b.out_id[id] < -1) {
        b.stl_distance[id] = nd;
        b.stl_id[id] = nid;
    } else {
        ref_nearest(b, b.pos[id], true, nd, nid);
    }
    b.drag_acc[id] = s3(0, 0, 0);
    b.drag_temperature[id] = 0;
    b.out_type[id] = TYPE_HEAVY_WEIGHT;
    if (!(nid != -1 && nd.Magnitude != 1e8f)) return;
    const DragParameter dp = b.drag_params[b.tri_params[b.triangles[nid].ModelIDNumber].DragTriangleID];
    if (nd.Magnitude <= dp.CoefficientofInflueneRegion * P.InitialParticleDistance) {
        b.out_type[id] = TYPE_LIGHT_WEIGHT;
        if (dp.DragToken == 'E') {
            if (dp.InputVelocityToken1 == 'V' || dp.InputVelocityToken1 == 'B') {
                float pr = 0.0f;
                const float sv = ref_mag(b.vel[id]);
                pr += dp.VelocityIndex * powf(sv, dp.VelocityExponential);
                const Scalar3 nrm = b.triangles[nid].Normal;
                if (dp.VelocityDragPermiabilityConstant != 0)
                    b.drag_acc[id] = s3((pr * (nrm.x) / dp.VelocityDragPermiabilityConstant),
                                        (pr * (nrm.y) / dp.VelocityDragPermiabilityConstant),
                                        (pr * (nrm.z) / dp.VelocityDragPermiabilityConstant));
            } else if (dp.InputVelocityToken1 == 'T') {
                const float sv = ref_mag(b.vel[id]);
                const float enth = dp.TempIndex * powf(sv, dp.TempExponential);
                const float den = ref_mag(b.vel[id]) * P.Density * P.FruidSpecificHeat;
                if (den != 0)
                    b.drag_temperature[id] = (enth * dp.TempDragPermiabilityConstant * P.Dt * P.ThermalStep) / (den);
                b.out_solid_rate[id] = b.drag_temperature[id];
            }
        } else if (dp.DragToken == 'C') {
            if (dp.InputVelocityToken1 == 'V' || dp.InputVelocityToken1 == 'v') {
                b.out_vel[id] = s3(dp.ConstantVx, dp.ConstantVy, dp.ConstantVz);
                b.vel[id] = s3(dp.ConstantVx, dp.ConstantVy, dp.ConstantVz);
            }
        }
    } else if (dp.DragToken == 'F') {
        if ((dp.InputVelocityToken1 == 'V' || dp.InputVelocityToken1 == 'v') && b.magnifier_count[id] < 1) {
            const float f = dp.VelocityMagnitueFactor;
            b.vel[id].x *= f; b.vel[id].y *= f; b.vel[id].z *= f;
            b.out_vel[id].x *= f; b.out_vel[id].y *= f; b.out_vel[id].z *= f;
        }
    }
}

// ---------------------------------------------------------------------------
// particle operators (explicit schedule)
// ---------------------------------------------------------------------------
// 27-cell traversal in the reference order: k outer, j, i inner; particles of a
// cell in sorted order; neighbours whose out_id (indexed by sorted position, as in
// the reference) is negative are skipped.
// LE: neighbours at distance <= re (the temperature operator), else < re.
// Screen: ref_sqrt never returns less than sqrt(x) (1 - 3e-7) (its Newton step from
// below gives y <= 1/sqrt(x), the float roundings cost a few ulps), so a finite squared
// distance >= re^2 (1 + 1e-5) is rejected by the reference's own test and is skipped
// before the square root; the others take the reference's arithmetic unchanged
// (+inf is not screened: the reference's sqrt of it is -0, which it accepts).
__device__ __forceinline__ float ref_screen2(float re) { return re * re * 1.00001f; }
template <bool LE, class F>
__device__ __forceinline__ void ref_candidate(int x, const Scalar3& tp, const Scalar3& q, float re, float re2x, float mind,
                                              F& f) {
    const float dx = tp.x - q.x, dy = tp.y - q.y, dz = tp.z - q.z;
    const float d2 = dx * dx + dy * dy + dz * dz;   // ref_dist's sum (no contraction in this file)
    if (d2 >= re2x && d2 <= 3.402823466e38f) return;
    float d = ref_sqrt(d2);
    if (!(LE ? d <= re : d < re)) return;
    if (d < mind) d = mind;
    f(x, d, q);
}
template <bool LE = false, class F>
__device__ __forceinline__ void ref_neighbours(const RefBind& b, int id, const Scalar3& tp, int cx, int cy, int cz,
                                               float re, F&& f) {
    const float mind = (float)(re * 1e-3);
    const float re2x = ref_screen2(re);
    for (int k = -1; k <= 1; ++k)
        for (int j = -1; j <= 1; ++j)
            for (int i = -1; i <= 1; ++i) {
                const int m = cell_key(b.box.m_GridSize, cx + i, cy + j, cz + k);
                if (m < 0 || m >= b.cell_num) continue;
                const int s = b.cell_start[m];
                if (s == -1) continue;
                const int e = b.cell_end[m];
                for (int x = s; x < e; ++x) {
                    if (b.out_id[x] < 0) continue;
                    if (x == id) continue;
                    ref_candidate<LE>(x, tp, b.pos[x], re, re2x, mind, f);
                }
            }
}

// CalcExplicitly_Kernel (DeviceProcess_Kernel.h:390-582) for target id; nb(tp, cx, cy,
// cz, re, f) runs the neighbour traversal
template <class Nb>
__device__ __forceinline__ void ref_explicitly_body(const RefBind& b, int id, Nb&& nb) {
    const CParameter& P = b.param;
    const int orig = b.id[id];
    const Scalar3 tp = b.pos[id];
    if (!in_zone<float>(b.box, tp.x, tp.y, tp.z, P.Tolerance)) {
        b.out_id[orig] = -1;
        b.out_solid_rate[orig] = 9999;
        return;
    }
    int cx, cy, cz;
    const int cid = ref_cell(b.box, tp, cx, cy, cz);
    Scalar3 lap = s3(0, 0, 0), art = s3(0, 0, 0), col = s3(0, 0, 0);
    Scalar3 v0 = b.vel[id];
    Scalar3 tke = s3(0, 0, 0);
    const float re = P.LaplacianInfluenceRadiusCoefficient * P.InitialParticleDistance;
    const float rc = P.r_coeff * P.InitialParticleDistance;
    const float reg = P.GradientInfluenceRadiusCoefficient * P.InitialParticleDistance;
    const bool ep = P.bExplicitPressure;
    const bool turb = P.bTurbulance;
    if (cid >= 0 && cid < b.cell_num) {
        nb(tp, cx, cy, cz, re, [&](int x, float d, const Scalar3& q) {
            const float w = weight(re, d);
            const Scalar3 v1 = b.vel[x];
            lap.x += (v1.x - v0.x) * w;
            lap.y += (v1.y - v0.y) * w;
            lap.z += (v1.z - v0.z) * w;
            // turbulent kinetic energy gradient (:477-485)
            if (turb && d < reg) {
                const float w1 = weight(reg, d);
                const float sc = (b.strain[x] - b.strain[id]) * w1 / (d * d);
                tke = s3add(tke, s3mul(s3sub(q, tp), sc));
            }
            if (ep && d < rc) {
                const float a = P.ArtificialPressure * w / (d * d);
                art = s3add(art, s3mul(s3sub(q, tp), a));
                const float c = (rc - d) / d;
                col = s3add(col, s3mul(s3sub(q, tp), c));
            }
        });
    }
    const float wd = b.stl_distance[id].Magnitude;
    const int tri = b.stl_id[id];
    if (tri >= 0 && tri < b.triangle_num && wd > 0 && wd < re) {
        const float ww = ref_zlap(P.Dimension, wd, P.InitialParticleDistance);
        const Scalar3 v1 = b.tri_params[b.triangles[tri].ModelIDNumber].Velocity;
        lap.x += P.WallFrictionCoeffieicnt * (v1.x - v0.x) * ww;
        lap.y += P.WallFrictionCoeffieicnt * (v1.y - v0.y) * ww;
        lap.z += P.WallFrictionCoeffieicnt * (v1.z - v0.z) * ww;
    }
    const float coef = (float)((2.0 * P.Dimension) / (double)(P.LambdaValue * P.ConstantParticleDensity));
    lap.x *= coef; lap.y *= coef; lap.z *= coef;
    Scalar3 dragv = s3(0, 0, 0);
    Scalar3 acc = s3add(s3(0, 0, 0), P.GravityConstant);
    if (b.drag_num > 0) dragv = b.drag_acc[id];
    // laminar + turbulent viscosity (:545-552)
    lap = s3mul(lap, turb ? b.kin_visc[id] + b.turb_visc[id] : b.kin_visc[id]);
    acc = s3add(acc, lap);
    v0 = s3sub(s3add(v0, s3mul(acc, P.Dt)), dragv);
    if (turb) {
        // (2/3) is the integer quotient 0 in the reference (:560): the term vanishes
        tke = s3mul(tke, (float)(2 / 3));
        v0 = s3sub(v0, s3mul(tke, P.Dt));
    }
    if (ep) {
        const float c = (float)(-P.Dimension) / (P.ConstantParticleDensity * P.Density);
        acc = s3add(s3mul(art, c), s3mul(col, (float)0.01));
        v0 = s3add(v0, s3mul(acc, P.Dt));
    }
    if (isfinite(v0.x) && isfinite(v0.y) && isfinite(v0.z)) {
        b.out_pos[orig] = s3(tp.x + P.Dt * v0.x, tp.y + P.Dt * v0.y, tp.z + P.Dt * v0.z);
        b.out_vel[orig] = v0;
    }
}

// CalcTemperatureFactor_Kernel (DeviceProcess_Kernel.h:705-852): conduction over the
// neighbours within the temperature radius (distance <= re), the nearest wall through
// its gradient Z function, the drag heating; each sum counted only above FLT_EPSILON
// in magnitude; clamped; viscosity linear in the temperature (original index)
__global__ void k_ref_temperature(int n, const __grid_constant__ RefBind b) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const CParameter& P = b.param;
    const float rho = P.Density;
    const float ecoef = P.Dt * 2 * P.Dimension / (P.ConstantParticleDensity * rho * P.FruidSpecificHeat);
    float hf = 0.0f, hw = 0.0f;
    const float ret = P.TemperatureInfluenceRadiusCoefficient * P.InitialParticleDistance;
    const Scalar3 tp = b.pos[id];
    float tt = b.temperature[id];
    const int orig = b.id[id];
    if (!in_zone<float>(b.box, tp.x, tp.y, tp.z, P.Tolerance)) {
        b.out_id[orig] = -1;
        return;
    }
    int cx, cy, cz;
    const int cid = ref_cell(b.box, tp, cx, cy, cz);
    if (cid < 0 || cid >= b.cell_num) return;
    ref_neighbours<true>(b, id, tp, cx, cy, cz, ret, [&](int x, float d, const Scalar3&) {
        const float num = (b.temperature[x] - tt) * weight(ret, d);
        const float den = d * d * (1 / P.FruidThermalConductivity + P.FruidThermalResistance / d);
        hf += num / den;
    });
    const float wd = b.stl_distance[id].Magnitude;
    const int tri = b.stl_id[id];
    if (tri >= 0 && tri < b.triangle_num && wd > 0 && wd < ret) {
        const CTriangleParameters& tq = b.tri_params[b.triangles[tri].ModelIDNumber];
        const float res = tq.WallThermalResistivity;
        const float cond = (2 * P.FruidThermalConductivity * tq.WallThermalConductivity) /
                           (P.FruidThermalConductivity + tq.WallThermalConductivity);
        const float ww = ref_zgrad(P.Dimension, wd, P.InitialParticleDistance);
        const float num = (tq.Temperature - tt) * ww;
        const float den = wd * wd * (1 / cond + res / wd);
        hw = num / den;
    }
    if (b.drag_num > 0) tt += b.drag_temperature[id];
    float comb = 0.0f;
    if (fabsf(hf) > FLT_EPSILON) comb += hf;
    if (fabsf(hw) > FLT_EPSILON) comb += hw;
    tt += (ecoef * (comb));
    if (tt > P.MaxWallTemperature) tt = P.MaxWallTemperature;
    if (tt < P.MinWallTemperature) tt = P.MinWallTemperature;
    b.out_temperature[orig] = tt;
    b.out_kin_visc[orig] = P.ViscosityUpdateParameterA * tt + P.ViscosityUpdateParameterB;
}

// CalcTurbulenceViscosity_Kernel (DeviceProcess_Kernel.h:1273-1476): velocity gradient
// tensor within the gradient radius, strain-rate product, wall-damped Smagorinsky
// viscosity (capped) and turbulent kinetic energy (capped), sorted order.  The
// kernel's vorticity and PND are never read and are left out.
__global__ void k_ref_turbulence(int n, const __grid_constant__ RefBind b) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const CParameter& P = b.param;
    const int orig = b.id[id];
    const Scalar3 tp = b.pos[id];
    const Scalar3 v0 = b.vel[id];
    if (!in_zone<float>(b.box, tp.x, tp.y, tp.z, P.Tolerance)) {
        b.turb_visc[id] = 0.0f;
        b.out_id[orig] = -1;
        return;
    }
    Scalar3 X = s3(0, 0, 0), Y = s3(0, 0, 0), Z = s3(0, 0, 0), D = s3(0, 0, 0);
    int cx, cy, cz;
    const int cid = ref_cell(b.box, tp, cx, cy, cz);
    if (cid < 0 || cid >= b.cell_num) {
        b.pressure[id] = 0.0f;
        return;
    }
    const float re = P.GradientInfluenceRadiusCoefficient * P.InitialParticleDistance;
    ref_neighbours(b, id, tp, cx, cy, cz, re, [&](int x, float d, const Scalar3& q) {
        const float w = weight(re, d);
        const Scalar3 v1 = b.vel[x];
        X.x += ((v1.x - v0.x) * (q.x - tp.x) * w) / (d * d);
        X.y += ((v1.x - v0.x) * (q.y - tp.y) * w) / (d * d);
        X.z += ((v1.x - v0.x) * (q.z - tp.z) * w) / (d * d);
        Y.x += ((v1.y - v0.y) * (q.x - tp.x) * w) / (d * d);
        Y.y += ((v1.y - v0.y) * (q.y - tp.y) * w) / (d * d);
        Y.z += ((v1.y - v0.y) * (q.z - tp.z) * w) / (d * d);
        Z.x += ((v1.z - v0.z) * (q.x - tp.x) * w) / (d * d);
        Z.y += ((v1.z - v0.z) * (q.y - tp.y) * w) / (d * d);
        Z.z += ((v1.z - v0.z) * (q.z - tp.z) * w) / (d * d);
    });
    const float g = P.Dimension / P.ConstantParticleDensity;
    X.x = g * X.x; X.y = g * X.y; X.z = g * X.z;
    Y.x = g * Y.x; Y.y = g * Y.y; Y.z = g * Y.z;
    Z.x = g * Z.x; Z.y = g * Z.y; Z.z = g * Z.z;
    D.x = (float)(0.5 * (X.y + Y.x));
    D.y = (float)(0.5 * (X.z + Z.x));
    D.z = (float)(0.5 * (Y.z + Z.y));
    const float strain = X.x * X.x + Y.y * Y.y + Z.z * Z.z + 2 * D.x * D.x + 2 * D.y * D.y + 2 * D.z * D.z;
    const float riw = b.stl_distance[id].Magnitude;
    const float ratio = -(riw / re);
    const float damp = 1 - expf(ratio);
    const float smag = P.SmagorinskyConstant * damp;
    const float coef = (smag * P.FilterWidth) * (smag * P.FilterWidth);
    float tv = 0;
    if (strain > 0) tv = coef * sqrtf(2 * strain);
    if (tv > P.TurbulanViscosityRatio) tv = P.TurbulanViscosityRatio;
    b.turb_visc[id] = tv;
    const float tkc = 2 * P.Cnue * P.InitialParticleDistance * P.InitialParticleDistance / P.Cepsilon;
    float tke = strain * tkc;
    if (tke > P.TurbulanceIntensity) tke = P.TurbulanceIntensity;
    b.strain[id] = tke;
}

// CalcExplicitPressure_Kernel (DeviceProcess_Kernel.h:921-1054)
template <class Nb>
__device__ __forceinline__ void ref_pressure_body(const RefBind& b, int id, Nb&& nb) {
    const CParameter& P = b.param;
    const int orig = b.id[id];
    const Scalar3 tp = b.pos[id];
    if (!in_zone<float>(b.box, tp.x, tp.y, tp.z, P.Tolerance)) {
        b.out_id[orig] = -1;
        b.pressure[id] = 0.0f;
        return;
    }
    int cx, cy, cz;
    const int cid = ref_cell(b.box, tp, cx, cy, cz);
    if (cid < 0 || cid >= b.cell_num) {
        b.pressure[id] = 0.0f;
        return;
    }
    const float re = P.GradientInfluenceRadiusCoefficient * P.InitialParticleDistance;
    const float coef = P.SonicVelocity * P.SonicVelocity * P.Density / P.ConstantParticleDensity;
    float dens = 0.0f;
    nb(tp, cx, cy, cz, re, [&](int, float d, const Scalar3&) { dens += weight(re, d); });
    const float riw = b.stl_distance[id].Magnitude;
    float ww = 0.0f;
    if (b.stl_id[id] >= 0 && b.stl_id[id] < b.triangle_num && riw >= 0 && riw <= re)
        ww = ref_zgrad(P.Dimension, riw, P.InitialParticleDistance);
    dens += ww;
    if (isfinite(dens)) b.out_density[orig] = dens;
    float pr = 0.0f;
    if (dens > P.ConstantParticleDensity * P.FreeSurfaceThreshold) pr = coef * (dens - P.ConstantParticleDensity);
    if (isfinite(pr)) {
        b.out_pressure[orig] = pr;
        b.pressure[id] = pr;
    }
}

// CalcExplicitPressureGradient_Kernel (DeviceProcess_Kernel.h:1056-1271), without
// the negative-pressure branch.
template <class Nb>
__device__ __forceinline__ void ref_gradient_body(const RefBind& b, int id, Nb&& nb) {
    const CParameter& P = b.param;
    const int orig = b.id[id];
    const Scalar3 tp = b.pos[id];
    if (!in_zone<float>(b.box, tp.x, tp.y, tp.z, P.Tolerance)) {
        b.out_id[orig] = -1;
        return;
    }
    int cx, cy, cz;
    const int cid = ref_cell(b.box, tp, cx, cy, cz);
    if (cid < 0 || cid >= b.cell_num) return;
    const float re = P.GradientInfluenceRadiusCoefficient * P.InitialParticleDistance;
    Scalar3 gf = s3(0, 0, 0), gw = s3(0, 0, 0);
    const float tpress = b.pressure[id];
    nb(tp, cx, cy, cz, re, [&](int x, float d, const Scalar3& q) {
        const float pc = (float)(0.5 * (double)(b.pressure[x] + tpress) * (double)weight(re, d));
        gf.x += pc * (q.x - tp.x) / (d * d);
        gf.y += pc * (q.y - tp.y) / (d * d);
        gf.z += pc * (q.z - tp.z) / (d * d);
    });
    const float c1 = 2 * P.Dimension / (P.ConstantParticleDensity);
    const float c2 = P.Density / (P.Dt * P.Dt);
    const float c3 = -P.Dt / P.Density;
    gf.x *= c1; gf.y *= c1; gf.z *= c1;
    const CDistance riw = b.stl_distance[id];
    if (b.stl_id[id] >= 0 && b.stl_id[id] < b.triangle_num) {
        if (riw.Magnitude > 0 && riw.Magnitude <= re) {
            const float ww = ref_z(c_zgrad3, 21, riw.Magnitude, P.InitialParticleDistance);
            const float wc = (float)((((0.5 * (double)c1) * (double)ww) * (double)tpress) /
                                     (double)(riw.Magnitude * riw.Magnitude));
            gw = s3(wc * (-riw.Direction.x), wc * (-riw.Direction.y), wc * (-riw.Direction.z));
        }
        if (riw.Magnitude > 0 && riw.Magnitude <= P.InitialParticleDistance * P.OffSet) {
            const float dr = (P.InitialParticleDistance * P.OffSet - riw.Magnitude);
            const float mc = c2 * dr / riw.Magnitude;
            gw.x += mc * (-riw.Direction.x);
            gw.y += mc * (-riw.Direction.y);
            gw.z += mc * (-riw.Direction.z);
        }
    }
    const Scalar3 g = s3add(s3add(gf, gw), s3(0, 0, 0));
    Scalar3 iv = s3(c3 * g.x, c3 * g.y, c3 * g.z);
    if (isfinite(iv.x) && isfinite(iv.y) && isfinite(iv.z)) {
        const Scalar3 v = b.vel[id];
        Scalar3 ov = s3(v.x + iv.x, v.y + iv.y, v.z + iv.z);
        // CorrectVelocity (Utility_Inline.h:2369-2396)
        const float cmax = P.InitialParticleDistance * P.CourantNumber / P.Dt;
        const float a = ref_sqrt(ov.x * ov.x + ov.y * ov.y + ov.z * ov.z);
        if (a > cmax) ov = s3(cmax * ov.x / a, cmax * ov.y / a, cmax * ov.z / a);
        b.out_vel[orig] = ov;
        iv = s3(ov.x - v.x, ov.y - v.y, ov.z - v.z);
        b.out_pos[orig] = s3(tp.x + iv.x * P.Dt, tp.y + iv.y * P.Dt, tp.z + iv.z * P.Dt);
    }
}

enum { REF_EXPLICITLY = 0, REF_PRESSURE = 1, REF_GRADIENT = 2 };
template <int KIND, class Nb>
__device__ __forceinline__ void ref_op_body(const RefBind& b, int id, Nb&& nb) {
    if constexpr (KIND == REF_EXPLICITLY) ref_explicitly_body(b, id, nb);
    else if constexpr (KIND == REF_PRESSURE) ref_pressure_body(b, id, nb);
    else ref_gradient_body(b, id, nb);
}
// one thread per target, the traversal over global memory (the targets of a warp are
// consecutive in the sorted order: mostly one cell, whose candidates they load together)
template <int KIND>
__global__ void k_ref_op(int n, const __grid_constant__ RefBind b) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    ref_op_body<KIND>(b, id, [&](const Scalar3& tp, int cx, int cy, int cz, float re, auto&& f) {
        ref_neighbours(b, id, tp, cx, cy, cz, re, f);
    });
}

inline int grid_of(int n) { return div_up(n, kBlock); }

// the operator over targets 0 .. n-1
template <int KIND>
cudaError_t ref_op_launch(cudaStream_t st, int n) {
    MPS_COUNT_LAUNCH k_ref_op<KIND><<<grid_of(n), kBlock, 0, st>>>(n, g_bind);
    return cudaGetLastError();
}

CCTStatusType launch_status() { return cuda_status(cudaGetLastError()); }

}  // namespace mps

using namespace mps;

// ===========================================================================
// Reference-named C-ABI (DeviceProcess.h:78-120)
// ===========================================================================
extern "C" {

CCTStatusType InitializeDeviceMemConst(CParameter Parameter, Integer ParticleNum, CTriangle* Triangles,
                                       Integer TriangleNum, CTriangleParameters* TriangleParameters,
                                       Integer MaxParticleNum, CDistance* STLDistance, Integer* StlID, CCell* Cell,
                                       Integer CellNum, Integer* CellStart, Integer* CellEnd,
                                       Integer* GridParticleIndex, CGridBox BoundingBox) {
    g_bind.param = Parameter;
    g_bind.particle_num = ParticleNum;
    g_bind.triangles = Triangles;
    g_bind.triangle_num = TriangleNum;
    g_bind.tri_params = TriangleParameters;
    g_bind.max_particle_num = MaxParticleNum;
    g_bind.stl_distance = STLDistance;
    g_bind.stl_id = StlID;
    g_bind.cells = Cell;
    g_bind.cell_num = CellNum;
    g_bind.cell_start = CellStart;
    g_bind.cell_end = CellEnd;
    g_bind.grid_index = GridParticleIndex;
    g_bind.box = BoundingBox;
    return CCT_NOERR;
}

CCTStatusType InitializeDeviceConstOutPutParticles(Integer* OutputParticleID, Scalar3* OutputParticlePosition,
                                                   Scalar3* OutputParticleVelocity, Scalar* OutputParticlePressure,
                                                   Scalar* OutputParticleDensity, Scalar* OutputParticleTemperature,
                                                   Scalar* OutputParticleKineticViscosity,
                                                   Scalar* OutputParticleSolidPhaseRate,
                                                   ParticleType* OutputParticleType) {
    g_bind.out_id = OutputParticleID;
    g_bind.out_pos = OutputParticlePosition;
    g_bind.out_vel = OutputParticleVelocity;
    g_bind.out_pressure = OutputParticlePressure;
    g_bind.out_density = OutputParticleDensity;
    g_bind.out_temperature = OutputParticleTemperature;
    g_bind.out_kin_visc = OutputParticleKineticViscosity;
    g_bind.out_solid_rate = OutputParticleSolidPhaseRate;
    g_bind.out_type = (int*)OutputParticleType;
    return CCT_NOERR;
}

CCTStatusType InitializeDeviceConstInputParticles(Integer* InputParticleID, Scalar3* InputParticlePosition,
                                                  Scalar3* InputParticleVelocity, Scalar* InputParticlePressure,
                                                  Scalar* InputParticleDensity, Scalar* InputParticleTemperature,
                                                  Scalar* InputParticleKineticViscosity,
                                                  Scalar* InputParticleSolidPhaseRate, ParticleType* InputParticleType,
                                                  Scalar* ParticleTurbulaceViscosity,
                                                  Scalar* ParticleStrainTensorProduct) {
    g_bind.turb_visc = ParticleTurbulaceViscosity;
    g_bind.strain = ParticleStrainTensorProduct;
    g_bind.id = InputParticleID;
    g_bind.pos = InputParticlePosition;
    g_bind.vel = InputParticleVelocity;
    g_bind.pressure = InputParticlePressure;
    g_bind.density = InputParticleDensity;
    g_bind.temperature = InputParticleTemperature;
    g_bind.kin_visc = InputParticleKineticViscosity;
    g_bind.solid_rate = InputParticleSolidPhaseRate;
    g_bind.type = (int*)InputParticleType;
    return CCT_NOERR;
}

CCTStatusType ParticleNumberToConst(Integer ParticleNum) {
    g_bind.particle_num = ParticleNum;
    return CCT_NOERR;
}

CCTStatusType DragParametersToConst(DragParameter* InputDragParameter, Scalar3* InputDragAcc,
                                    Scalar* InputDragTemperature, Integer DragTriangleNum, Integer* MagnifierCount,
                                    CDragTriangle* DragTriangles) {
    g_bind.drag_params = InputDragParameter;
    g_bind.drag_acc = InputDragAcc;
    g_bind.drag_temperature = InputDragTemperature;
    g_bind.drag_num = DragTriangleNum;
    g_bind.magnifier_count = MagnifierCount;
    g_bind.drag_triangles = DragTriangles;
    return CCT_NOERR;
}

CCTStatusType CaculateCellIDandInitializeHash(cudaStream_t& Stream, Integer ParticleNum, Integer CellNum,
                                              int* dGridParticleHash, int* dGridParticleIndex,
                                              Scalar3* particlePosition) {
    (void)CellNum;
    if (ParticleNum <= 0) return CCT_NOERR;
    MPS_COUNT_LAUNCH k_ref_hash<<<grid_of(ParticleNum), kBlock, 0, Stream>>>(ParticleNum, g_bind.box, particlePosition,
                                                             dGridParticleHash, dGridParticleIndex);
    return launch_status();
}

CCTStatusType reorderDataAndFindCellStart(cudaStream_t& Stream, Integer numParticles, Integer numCells,
                                          int* gridParticleHash, int* gridParticleIndex, int* cellStart,
                                          int* cellEnd) {
    if (numParticles <= 0) return CCT_NOERR;
    MPS_CUDA_TRY(cudaMemsetAsync(cellStart, 0xff, sizeof(int) * (size_t)numCells, Stream));
    MPS_CUDA_TRY(cudaMemsetAsync(cellEnd, 0xff, sizeof(int) * (size_t)numCells, Stream));
    MPS_COUNT_LAUNCH k_ref_reorder<<<grid_of(numParticles), kBlock, 0, Stream>>>(numParticles, numCells, gridParticleHash,
                                                                 gridParticleIndex, cellStart, cellEnd, g_bind);
    return launch_status();
}

// tile sums of the multi-CTA scan (NULL when the slot cannot be had: one-CTA scan)
static unsigned* scan_sums() { return (unsigned*)scratch_get(8, sizeof(unsigned) * scan_tile_sums_capacity()); }

// thrust::sort_by_key replacement: stable LSD radix sort on the legacy default
// stream, keys of any int range (one min/max pass picks the digits to sort).
CCTStatusType SortUsingThrust(Integer MaxParticleNum, Integer* daNumberHash, Integer* daNumberIndex) {
    const int n = MaxParticleNum;
    if (n <= 1) return CCT_NOERR;
    cudaStream_t st = 0;
    int* mm = (int*)scratch_get(0, 2 * sizeof(int));
    if (!mm) return CCT_MEMERR;
    void* scr = scratch_get(1, radix_scratch_bytes(n));
    if (!scr) return CCT_MEMERR;
    // the key range stays on the device: the passes it does not need return at once
    MPS_CUDA_TRY(key_minmax(n, daNumberHash, mm, st));
    MPS_CUDA_TRY(radix_sort_pairs_range(n, daNumberHash, daNumberIndex, mm, scr, st));
    // thrust::sort_by_key with the default policy returns after the sort completed;
    // callers rely on that (they launch the reorder on their own stream next).
    MPS_CUDA_TRY(cudaStreamSynchronize(st));
    return launch_status();
}

CCTStatusType StableSortUsingThrust(Integer MaxParticleNum, Integer* daNumberHash, Integer* daNumberIndex) {
    return SortUsingThrust(MaxParticleNum, daNumberHash, daNumberIndex);
}

CCTStatusType CheckParticleOutsideComputeZone(cudaStream_t& Stream, Integer* ParticleNum) {
    const int n = *ParticleNum;
    if (n <= 0) return CCT_NOERR;
    unsigned* flag = (unsigned*)scratch_get(2, sizeof(unsigned) * ((size_t)n + 4));
    unsigned* rank = (unsigned*)scratch_get(3, sizeof(unsigned) * ((size_t)n + 4));
    if (!flag || !rank) return CCT_MEMERR;
    int* removed = (int*)(rank + n);
    MPS_CUDA_TRY(cudaMemsetAsync(removed, 0, sizeof(int), Stream));
    MPS_COUNT_LAUNCH k_ref_outside_flags<<<grid_of(n), kBlock, 0, Stream>>>(n, g_bind, flag);
    MPS_CUDA_TRY(cudaMemcpyAsync(rank, flag, sizeof(unsigned) * (size_t)n, cudaMemcpyDeviceToDevice, Stream));
    MPS_CUDA_TRY(scan_exclusive(rank, n, nullptr, Stream, scan_sums()));
    MPS_COUNT_LAUNCH k_ref_compact<<<grid_of(n), kBlock, 0, Stream>>>(n, g_bind, flag, rank, removed);
    int r = 0;
    MPS_CUDA_TRY(cudaMemcpyAsync(&r, removed, sizeof(int), cudaMemcpyDeviceToHost, Stream));
    MPS_CUDA_TRY(cudaStreamSynchronize(Stream));
    *ParticleNum = n - r;
    g_bind.particle_num = n - r;
    return launch_status();
}

CCTStatusType ResetTriangleTopology(cudaStream_t& Stream, Integer CellNum, CCell* aCell) {
    if (CellNum <= 0) return CCT_NOERR;
    MPS_COUNT_LAUNCH k_tri_reset<<<grid_of(CellNum), kBlock, 0, Stream>>>(CellNum, aCell);
    return launch_status();
}

CCTStatusType RegisterTriangleTopology(cudaStream_t& Stream, CTriangle* daTriangle, Integer TriangleNum, CCell* daCell,
                                       Integer CellNum) {
    const int t = TriangleNum;
    if (t <= 0 || CellNum <= 0) return CCT_NOERR;
    unsigned* off = (unsigned*)scratch_get(4, sizeof(unsigned) * ((size_t)t + 4));
    if (!off) return CCT_MEMERR;
    unsigned* total_dev = off + t;
    MPS_COUNT_LAUNCH k_tri_count<<<grid_of(t), kBlock, 0, Stream>>>(t, daTriangle, g_bind.box, CellNum, off);
    MPS_CUDA_TRY(scan_exclusive(off, t, total_dev, Stream, scan_sums()));
    unsigned nv = 0;
    MPS_CUDA_TRY(cudaMemcpyAsync(&nv, total_dev, sizeof(unsigned), cudaMemcpyDeviceToHost, Stream));
    MPS_CUDA_TRY(cudaStreamSynchronize(Stream));
    if (nv == 0) return launch_status();
    int* vcell = (int*)scratch_get(5, sizeof(int) * (size_t)nv * 2);
    int* vrange = (int*)scratch_get(6, sizeof(int) * (size_t)CellNum * 2);
    void* sscr = scratch_get(7, radix_scratch_bytes((int)nv));
    if (!vcell || !vrange || !sscr) return CCT_MEMERR;
    int* vtri = vcell + nv;
    MPS_COUNT_LAUNCH k_tri_fill<<<grid_of(t), kBlock, 0, Stream>>>(t, daTriangle, g_bind.box, CellNum, off, vcell, vtri);
    MPS_CUDA_TRY(radix_sort_pairs((int)nv, vcell, vtri, 0, radix_passes((unsigned)CellNum), sscr, Stream));
    MPS_CUDA_TRY(cudaMemsetAsync(vrange, 0xff, sizeof(int) * (size_t)CellNum * 2, Stream));
    MPS_COUNT_LAUNCH k_tri_bounds<<<grid_of((int)nv), kBlock, 0, Stream>>>((int)nv, vcell, vrange, vrange + CellNum);
    MPS_COUNT_LAUNCH k_tri_cells<<<grid_of(CellNum), kBlock, 0, Stream>>>(CellNum, vrange, vrange + CellNum, vtri, daCell);
    return launch_status();
}

CCTStatusType UpdateTrianglePosition(cudaStream_t& Stream, const Integer TriangleNum, CTriangle* daTriangles) {
    if (TriangleNum <= 0) return CCT_NOERR;
    MPS_COUNT_LAUNCH k_tri_translate<<<grid_of(TriangleNum), kBlock, 0, Stream>>>(TriangleNum, daTriangles, g_bind);
    return launch_status();
}

CCTStatusType RotateTrianglePosition(cudaStream_t& Stream, const Integer TriangleNum, CTriangle* daTriangles,
                                     const Integer analysisStep) {
    if (TriangleNum <= 0) return CCT_NOERR;
    MPS_COUNT_LAUNCH k_tri_rotate<<<grid_of(TriangleNum), kBlock, 0, Stream>>>(TriangleNum, daTriangles, analysisStep, g_bind);
    return launch_status();
}

CCTStatusType ResetWallPosition(cudaStream_t& Stream, const Integer TriangleNum, const Integer AnalysisStep,
                                const CTriangle* daTriangles) {
    if (TriangleNum <= 0) return CCT_NOERR;
    MPS_COUNT_LAUNCH k_tri_reset_wall<<<grid_of(TriangleNum), kBlock, 0, Stream>>>(TriangleNum, AnalysisStep, daTriangles, g_bind);
    return launch_status();
}

CCTStatusType CalcSTLDistance(cudaStream_t& Stream, Integer ComputeParticleNum) {
    if (ComputeParticleNum <= 0) return CCT_NOERR;
    MPS_CUDA_TRY(cudaMemsetAsync(g_bind.stl_id, 0xff, sizeof(int) * (size_t)ComputeParticleNum, Stream));
    MPS_COUNT_LAUNCH k_ref_stl_distance<<<grid_of(ComputeParticleNum), kBlock, 0, Stream>>>(ComputeParticleNum, g_bind);
    return launch_status();
}

CCTStatusType CalcDragEffect(cudaStream_t& Stream, Integer ComputeParticleNum) {
    if (ComputeParticleNum <= 0) return CCT_NOERR;
    MPS_COUNT_LAUNCH k_ref_drag<<<grid_of(ComputeParticleNum), kBlock, 0, Stream>>>(ComputeParticleNum, g_bind);
    return launch_status();
}

CCTStatusType CalcExplicitly(cudaStream_t& Stream, Integer ParticleNum) {
    if (ParticleNum <= 0) return CCT_NOERR;
    if (g_bind.param.bTurbulance && (!g_bind.turb_visc || !g_bind.strain)) return CCT_PARAMERR;
    MPS_CUDA_TRY(ref_op_launch<REF_EXPLICITLY>(Stream, ParticleNum));
    return launch_status();
}

CCTStatusType CalcExplicitPressure(cudaStream_t& Stream, Integer ComputeParticleNum) {
    if (ComputeParticleNum <= 0) return CCT_NOERR;
    MPS_CUDA_TRY(ref_op_launch<REF_PRESSURE>(Stream, ComputeParticleNum));
    return launch_status();
}

CCTStatusType CalcExplicitPressureGradient(cudaStream_t& Stream, Integer ComputeParticleNum) {
    if (ComputeParticleNum <= 0) return CCT_NOERR;
    if (g_bind.param.bNegativePressure) return CCT_PARAMERR;
    MPS_CUDA_TRY(ref_op_launch<REF_GRADIENT>(Stream, ComputeParticleNum));
    return launch_status();
}

CCTStatusType CalcTemperatureFactor(cudaStream_t& Stream, Integer ComputeParticleNum) {
    if (ComputeParticleNum <= 0) return CCT_NOERR;
    if (!g_bind.temperature || !g_bind.out_temperature || !g_bind.out_kin_visc) return CCT_PARAMERR;
    MPS_COUNT_LAUNCH k_ref_temperature<<<grid_of(ComputeParticleNum), kBlock, 0, Stream>>>(ComputeParticleNum, g_bind);
    return launch_status();
}

CCTStatusType CalcTurbulenceViscosity(cudaStream_t& Stream, Integer ComputeParticleNum) {
    if (ComputeParticleNum <= 0) return CCT_NOERR;
    if (!g_bind.turb_visc || !g_bind.strain) return CCT_PARAMERR;
    MPS_COUNT_LAUNCH k_ref_turbulence<<<grid_of(ComputeParticleNum), kBlock, 0, Stream>>>(ComputeParticleNum, g_bind);
    return launch_status();
}

}  // extern "C"
