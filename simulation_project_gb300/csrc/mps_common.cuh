// mps_common.cuh - device-side helpers shared by the GB300 MPS kernels.
//
// Two families of arithmetic live here:
//  * "ref" functions reproduce the reference solver's float arithmetic operation by
//    operation (radix/SPVSOLVER/MultiGPUSolver/Utility_Inline.h, DataType.h).  They
//    are compiled in translation units built with -fmad=false so no multiply-add is
//    contracted, which makes them round exactly like the reference's source text.
//  * "exact" templates (float or double) use true square roots and the exact
//    point-triangle distance; they serve the semi-implicit solver.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mps_types.h"

namespace mps {

constexpr int kBlock = 256;

// 32-byte aligned double4 (one 256-bit access) for the FP64 particle state
typedef double4_32a dbl4;
__host__ __device__ __forceinline__ dbl4 make_dbl4(double x, double y, double z, double w) {
    dbl4 t;
    t.x = x; t.y = y; t.z = z; t.w = w;
    return t;
}

__host__ __device__ inline int div_up(long long a, int b) { return (int)((a + b - 1) / b); }

// ---------------------------------------------------------------------------
// float3-like helpers on the boundary type Scalar3
// ---------------------------------------------------------------------------
__device__ __forceinline__ Scalar3 s3(float x, float y, float z) { Scalar3 t; t.x = x; t.y = y; t.z = z; return t; }
__device__ __forceinline__ Scalar3 s3sub(const Scalar3& a, const Scalar3& b) { return s3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ Scalar3 s3add(const Scalar3& a, const Scalar3& b) { return s3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ Scalar3 s3mul(const Scalar3& a, float s) { return s3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ Scalar3 ld3(const Scalar3* p) { return *p; }

// float -> int with truncation, saturation and NaN -> 0 (cvt.rzi.s32.f32)
__device__ __forceinline__ int f2i(float v) { return __float2int_rz(v); }
__device__ __forceinline__ int f2i(double v) { return __double2int_rz(v); }

// Cell key with 32-bit wrap-around: (Gy*Gz)*i + Gz*j + k  (GetCellID, Utility_Inline.h:1729-1733)
__device__ __forceinline__ int cell_key(const Integer3& g, int i, int j, int k) {
    uint32_t gyz = (uint32_t)g.y * (uint32_t)g.z;
    return (int)(gyz * (uint32_t)i + (uint32_t)g.z * (uint32_t)j + (uint32_t)k);
}

// ---------------------------------------------------------------------------
// reference float arithmetic (use only in -fmad=false translation units)
// ---------------------------------------------------------------------------
// sqrt_utility (Utility_Inline.h:19-26): inverse-sqrt estimate from the 0x5f3759df
// bit trick, one Newton step, reciprocal.
__device__ __forceinline__ float ref_sqrt(float x) {
    float xhalf = 0.5f * x;
    int i = __float_as_int(x);
    i = 0x5f3759df - (i >> 1);
    float y = __int_as_float(i);
    y = y * (1.5f - xhalf * y * y);
    return 1.0f / y;
}
__device__ __forceinline__ float ref_dist(const Scalar3& a, const Scalar3& b) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return ref_sqrt(dx * dx + dy * dy + dz * dz);
}
__device__ __forceinline__ float ref_mag(const Scalar3& v) { return ref_sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
__device__ __forceinline__ float ref_dot(const Scalar3& a, const Scalar3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// GetWeight (Utility_Inline.h:233-245)
template <class T>
__device__ __forceinline__ T weight(T re, T r) {
    if (r > re) return T(0);
    if (r > T(0)) return re / r - T(1);
    return T(1e6);
}

// GetCellID (Utility_Inline.h:1697-1728), float
__device__ __forceinline__ int ref_cell(const CGridBox& B, const Scalar3& p, int& i, int& j, int& k) {
    float rx = p.x - B.m_BufferedZone.m_MinBound.x;
    float ry = p.y - B.m_BufferedZone.m_MinBound.y;
    float rz = p.z - B.m_BufferedZone.m_MinBound.z;
    rx /= B.m_CellSize;
    ry /= B.m_CellSize;
    rz /= B.m_CellSize;
    i = f2i(rx);
    j = f2i(ry);
    k = f2i(rz);
    return cell_key(B.m_GridSize, i, j, k);
}

// IsInclude (Utility_Inline.h:2036-2077)
template <class T>
__device__ __forceinline__ bool in_zone(const CGridBox& B, T x, T y, T z, T tol) {
    const CBox& Z = B.m_ComputeZone;
    if (x < (T(Z.m_MinBound.x) - tol)) return false;
    if (y < (T(Z.m_MinBound.y) - tol)) return false;
    if (z < (T(Z.m_MinBound.z) - tol)) return false;
    if (x > (T(Z.m_MaxBound.x) + tol)) return false;
    if (y > (T(Z.m_MaxBound.y) + tol)) return false;
    if (z > (T(Z.m_MaxBound.z) + tol)) return false;
    return true;
}

// Piecewise-linear wall weights of the reference (Z functions, Utility_Inline.h:
// 261-398 gradient 3D, 399-571 gradient 2D, 575-747 Laplacian 3D, 749-897 Laplacian
// 2D). Row = (upper bound of r/l0, slope, value at the bound).
struct ZRow { double bound, a, c; };
static __constant__ ZRow c_zgrad3[21] = {
    {0.1, -5.0474610E+03, 2.9725900E+01}, {0.2, -1.1272200E+02, 1.8453700E+01},
    {0.3, -4.3342000E+01, 1.4119500E+01}, {0.4, -2.6328000E+01, 1.1486700E+01},
    {0.5, -1.9648400E+01, 9.5218600E+00}, {0.6, -1.5636200E+01, 7.9582400E+00},
    {0.7, -1.2591500E+01, 6.6990900E+00}, {0.8, -1.0988800E+01, 5.6002100E+00},
    {0.9, -9.0692000E+00, 4.6932900E+00}, {1.0, -7.5385000E+00, 3.9394400E+00},
    {1.1, -6.9148000E+00, 3.2479600E+00}, {1.2, -5.9144000E+00, 2.6565200E+00},
    {1.3, -5.4670000E+00, 2.1098200E+00}, {1.4, -5.0626000E+00, 1.6035600E+00},
    {1.5, -4.6948000E+00, 1.1340800E+00}, {1.6, -3.6959000E+00, 7.6449000E-01},
    {1.7, -2.7022800E+00, 4.9426200E-01}, {1.8, -2.4819500E+00, 2.4606700E-01},
    {1.9, -1.4080400E+00, 1.0526300E-01}, {2.0, -5.5263200E-01, 4.9999800E-02},
    {2.1, -4.9999800E-01, 0.0}};
static __constant__ ZRow c_zgrad2[23] = {
    {0.01, -9.996E+05, 3.837E+02}, {0.05, -3.027E+02, 8.101E+01}, {0.1, 3.812E+01, 4.289E+01},
    {0.2, -1.950E+01, 2.339E+01},  {0.3, -6.917E+00, 1.647E+01},  {0.4, -3.779E+00, 1.269E+01},
    {0.5, -2.523E+00, 1.017E+01},  {0.6, -1.889E+00, 8.282E+00},  {0.7, -1.484E+00, 6.798E+00},
    {0.8, -1.214E+00, 5.584E+00},  {0.9, -9.752E-01, 4.609E+00},  {1.0, -7.931E-01, 3.816E+00},
    {1.1, -6.940E-01, 3.122E+00},  {1.2, -5.320E-01, 2.590E+00},  {1.3, -4.727E-01, 2.117E+00},
    {1.4, -4.229E-01, 1.694E+00},  {1.5, -3.806E-01, 1.314E+00},  {1.6, -3.442E-01, 9.693E-01},
    {1.7, -3.127E-01, 6.566E-01},  {1.8, -2.851E-01, 3.715E-01},  {1.9, -1.820E-01, 1.895E-01},
    {2.0, -9.947E-02, 9.000E-02},  {2.1, -9.000E-02, 0.0}};
static __constant__ ZRow c_zlap3[25] = {
    {0.1, -9.6379E+03, 1.1497E+02}, {0.2, -2.3979E+02, 9.0990E+01}, {0.3, -1.0777E+02, 8.0213E+01},
    {0.4, -7.4088E+01, 7.2804E+01}, {0.5, -6.0259E+01, 6.6778E+01}, {0.6, -5.2803E+01, 6.1498E+01},
    {0.7, -4.8681E+01, 5.6630E+01}, {0.8, -4.4630E+01, 5.2167E+01}, {0.9, -4.1171E+01, 4.8050E+01},
    {1.0, -3.8583E+01, 4.4191E+01}, {1.1, -3.6846E+01, 4.0507E+01}, {1.2, -3.5476E+01, 3.6959E+01},
    {1.3, -3.4183E+01, 3.3541E+01}, {1.4, -3.1589E+01, 3.0382E+01}, {1.5, -2.9258E+01, 2.7456E+01},
    {1.6, -2.7047E+01, 2.4751E+01}, {1.7, -2.5690E+01, 2.2182E+01}, {1.8, -2.3305E+01, 1.9852E+01},
    {1.9, -2.0982E+01, 1.7754E+01}, {2.0, -1.9268E+01, 1.5827E+01}, {2.4, -1.6887E+01, 9.0719E+00},
    {2.8, -1.1091E+01, 4.6355E+00}, {3.2, -6.5068E+00, 2.0327E+00}, {3.6, -3.7565E+00, 5.3011E-01},
    {4.0, -1.3253E+00, 0.0}};
static __constant__ ZRow c_zlap2[23] = {
    {0.01, -9.992E+05, 7.507E+02}, {0.05, -5.766E+02, 1.741E+02}, {0.1, -7.280E+01, 1.013E+02},
    {0.2, -3.761E+01, 6.368E+01},  {0.4, -2.128E+01, 4.240E+01},  {0.6, -9.280E+00, 3.312E+01},
    {0.8, -6.104E+00, 2.701E+01},  {1.0, -4.682E+00, 2.233E+01},  {1.2, -3.842E+00, 1.849E+01},
    {1.4, -3.260E+00, 1.523E+01},  {1.6, -2.763E+00, 1.247E+01},  {1.8, -2.048E+00, 1.042E+01},
    {2.0, -2.034E+00, 8.385E+00},  {2.2, -1.726E+00, 6.659E+00},  {2.4, -1.543E+00, 5.116E+00},
    {2.6, -1.306E+00, 3.810E+00},  {2.8, -1.051E+00, 2.759E+00},  {3.0, -8.115E-01, 1.948E+00},
    {3.2, -5.864E-01, 1.361E+00},  {3.4, -5.298E-01, 8.314E-01},  {3.6, -3.773E-01, 4.541E-01},
    {3.8, -2.946E-01, 1.594E-01},  {4.0, -1.594E-01, 0.0}};

__device__ __forceinline__ float ref_z(const ZRow* t, int n, float r, float l0) {
    const float x = r / l0;
    for (int i = 0; i < n; ++i) {
        if ((double)x <= t[i].bound) {
            const float a = (float)t[i].a, b = (float)t[i].bound, c = (float)t[i].c;
            return a * (x - b) + c;
        }
    }
    return 0.0f;
}
template <class T>
__device__ __forceinline__ T exact_z(const ZRow* t, int n, T r, T l0) {
    const T x = r / l0;
    for (int i = 0; i < n; ++i)
        if ((double)x <= t[i].bound) return T(t[i].a) * (x - T(t[i].bound)) + T(t[i].c);
    return T(0);
}
__device__ __forceinline__ float ref_zgrad(int dim, float r, float l0) {
    return dim == 2 ? ref_z(c_zgrad2, 23, r, l0) : ref_z(c_zgrad3, 21, r, l0);
}
__device__ __forceinline__ float ref_zlap(int dim, float r, float l0) {
    return dim == 2 ? ref_z(c_zlap2, 23, r, l0) : ref_z(c_zlap3, 25, r, l0);
}

}  // namespace mps

// Error flag bits written by kernels into a device word (MPS_ERR_*, public in
// include/mps_solver.h, read by the host after a step).
#include "../../include/mps_solver.h"
