/*
 * mps_oracle.cpp - CPU oracle (checker) for the GB300 MPS hot path.
 *
 * TEST INFRASTRUCTURE ONLY: this file is the restatement of the reference
 * solver's algorithm that the CUDA kernels are checked against.  It is built into
 * oracle/liborc.so and loaded only by tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py.  Nothing in the product library links or calls it.
 *
 * Parity is pinned: oracle/ref_harness.cpp compiles the reference's own kernel
 * header (radix/SPVSOLVER/MultiGPUSolver/DeviceProcess_Kernel.h and the headers it
 * includes) for the CPU into oracle/_ref/libref.so, and tests/test_oracle_pin.py
 * runs both on the same inputs and requires bit-identical outputs.  Golden
 * outputs of that harness are committed under tests/golden/ so the pin also runs
 * where the reference sources are absent.
 *
 * Part 1 ("ref" functions, float, exact reference arithmetic): each function
 * follows the reference line by line in its floating-point operation order,
 * including the reference's quirks (fast inverse square root, SegmentRatio
 * precedence, swapped segment end cases, neighbour filter indexed by sorted
 * position).  Build with -ffp-contract=off so that no FMA contraction changes a
 * rounding.
 *
 * Part 2 (OrcSim, double): the semi-implicit step with a pressure Poisson
 * equation and Jacobi-preconditioned CG.  Its source term carries a relaxation
 * coefficient gamma (quasi-compressible MPS, Tanaka & Masunaga, J. Comput. Phys.
 * 229 (2010) 4279-4290): b = gamma rho/dt^2 (n* - n0)/n0, and drag models act on
 * the fluid only through the drag term (they are not walls here; the reference's
 * wall-distance kernel has that filter commented out, DeviceProcess_Kernel.h:897-900).  The reference declares but never
 * defines a PPE solver (S/CGPUCellSet.h:218-240 declarations only), so this part
 * is the specification the GPU FP64 path is checked against; it has no
 * reference counterpart to pin to.
 */
#include "mps_oracle.h"

#include <algorithm>
#include <climits>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef Scalar3 S3;

/* ------------------------------------------------------------------------ */
/* reference float math                                                     */
/* ------------------------------------------------------------------------ */

/* sqrt_utility, Utility_Inline.h:19-26: one Newton step of the 0x5f3759df
 * inverse-square-root estimate, then a reciprocal. */
inline float sqrt_q(float x) {
    float xhalf = 0.5f * x;
    int32_t i;
    std::memcpy(&i, &x, 4);
    i = 0x5f3759df - (i >> 1);
    float y;
    std::memcpy(&y, &i, 4);
    y = y * (1.5f - xhalf * y * y);
    return 1.0f / y;
}

inline S3 mk(float x, float y, float z) { S3 t; t.x = x; t.y = y; t.z = z; return t; }
inline S3 sub(const S3& a, const S3& b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline S3 add(const S3& a, const S3& b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline S3 mul(const S3& a, float s) { return mk(a.x * s, a.y * s, a.z * s); }

/* CalcDistance(point, point), Utility_Inline.h:28-31 */
inline float dist_q(const S3& a, const S3& b) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return sqrt_q(dx * dx + dy * dy + dz * dz);
}

/* Magnitude, Utility_Inline.h:37-41 */
inline float mag_q(const S3& v) { return sqrt_q(v.x * v.x + v.y * v.y + v.z * v.z); }
inline float dot_q(const S3& a, const S3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

/* GetWeight, Utility_Inline.h:233-245: w = re/r - 1 inside, 1e6 at r = 0 */
inline float weight_q(float re, float r) {
    if (r > re) return 0.0f;
    if (r > 0.0f) return re / r - 1.0f;
    return 1e6f;
}

/* Piecewise-linear wall-weight tables.  Row = (upper bound of r/l0, slope a,
 * value c at the bound); value = a*(r/l0 - bound) + c, evaluated in float with
 * the bound compared in double.  Coefficients are those of the reference's
 * Z functions (Utility_Inline.h:261-398, 399-571, 575-747, 749-897). */
struct ZRow { double bound, a, c; };

const ZRow kZGrad3[] = {
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
const ZRow kZGrad2[] = {
    {0.01, -9.996E+05, 3.837E+02}, {0.05, -3.027E+02, 8.101E+01}, {0.1, 3.812E+01, 4.289E+01},
    {0.2, -1.950E+01, 2.339E+01},  {0.3, -6.917E+00, 1.647E+01},  {0.4, -3.779E+00, 1.269E+01},
    {0.5, -2.523E+00, 1.017E+01},  {0.6, -1.889E+00, 8.282E+00},  {0.7, -1.484E+00, 6.798E+00},
    {0.8, -1.214E+00, 5.584E+00},  {0.9, -9.752E-01, 4.609E+00},  {1.0, -7.931E-01, 3.816E+00},
    {1.1, -6.940E-01, 3.122E+00},  {1.2, -5.320E-01, 2.590E+00},  {1.3, -4.727E-01, 2.117E+00},
    {1.4, -4.229E-01, 1.694E+00},  {1.5, -3.806E-01, 1.314E+00},  {1.6, -3.442E-01, 9.693E-01},
    {1.7, -3.127E-01, 6.566E-01},  {1.8, -2.851E-01, 3.715E-01},  {1.9, -1.820E-01, 1.895E-01},
    {2.0, -9.947E-02, 9.000E-02},  {2.1, -9.000E-02, 0.0}};
const ZRow kZLap3[] = {
    {0.1, -9.6379E+03, 1.1497E+02}, {0.2, -2.3979E+02, 9.0990E+01}, {0.3, -1.0777E+02, 8.0213E+01},
    {0.4, -7.4088E+01, 7.2804E+01}, {0.5, -6.0259E+01, 6.6778E+01}, {0.6, -5.2803E+01, 6.1498E+01},
    {0.7, -4.8681E+01, 5.6630E+01}, {0.8, -4.4630E+01, 5.2167E+01}, {0.9, -4.1171E+01, 4.8050E+01},
    {1.0, -3.8583E+01, 4.4191E+01}, {1.1, -3.6846E+01, 4.0507E+01}, {1.2, -3.5476E+01, 3.6959E+01},
    {1.3, -3.4183E+01, 3.3541E+01}, {1.4, -3.1589E+01, 3.0382E+01}, {1.5, -2.9258E+01, 2.7456E+01},
    {1.6, -2.7047E+01, 2.4751E+01}, {1.7, -2.5690E+01, 2.2182E+01}, {1.8, -2.3305E+01, 1.9852E+01},
    {1.9, -2.0982E+01, 1.7754E+01}, {2.0, -1.9268E+01, 1.5827E+01}, {2.4, -1.6887E+01, 9.0719E+00},
    {2.8, -1.1091E+01, 4.6355E+00}, {3.2, -6.5068E+00, 2.0327E+00}, {3.6, -3.7565E+00, 5.3011E-01},
    {4.0, -1.3253E+00, 0.0}};
const ZRow kZLap2[] = {
    {0.01, -9.992E+05, 7.507E+02}, {0.05, -5.766E+02, 1.741E+02}, {0.1, -7.280E+01, 1.013E+02},
    {0.2, -3.761E+01, 6.368E+01},  {0.4, -2.128E+01, 4.240E+01},  {0.6, -9.280E+00, 3.312E+01},
    {0.8, -6.104E+00, 2.701E+01},  {1.0, -4.682E+00, 2.233E+01},  {1.2, -3.842E+00, 1.849E+01},
    {1.4, -3.260E+00, 1.523E+01},  {1.6, -2.763E+00, 1.247E+01},  {1.8, -2.048E+00, 1.042E+01},
    {2.0, -2.034E+00, 8.385E+00},  {2.2, -1.726E+00, 6.659E+00},  {2.4, -1.543E+00, 5.116E+00},
    {2.6, -1.306E+00, 3.810E+00},  {2.8, -1.051E+00, 2.759E+00},  {3.0, -8.115E-01, 1.948E+00},
    {3.2, -5.864E-01, 1.361E+00},  {3.4, -5.298E-01, 8.314E-01},  {3.6, -3.773E-01, 4.541E-01},
    {3.8, -2.946E-01, 1.594E-01},  {4.0, -1.594E-01, 0.0}};

template <size_t N>
inline float zeval_q(const ZRow (&t)[N], float r, float l0) {
    const float x = r / l0;
    for (size_t i = 0; i < N; ++i) {
        if ((double)x <= t[i].bound) {
            const float a = (float)t[i].a, b = (float)t[i].bound, c = (float)t[i].c;
            return a * (x - b) + c;
        }
    }
    return 0.0f;
}
template <size_t N>
inline double zeval_d(const ZRow (&t)[N], double r, double l0) {
    const double x = r / l0;
    for (size_t i = 0; i < N; ++i)
        if (x <= t[i].bound) return t[i].a * (x - t[i].bound) + t[i].c;
    return 0.0;
}

/* float -> int conversion with CUDA cvt.rzi.s32.f32 semantics (truncate,
 * saturate, NaN -> 0) so host and device agree on every input. */
inline int f2i_sat(float v) {
    if (v != v) return 0;
    if (v >= 2147483647.0f) return INT_MAX;
    if (v <= -2147483648.0f) return INT_MIN;
    return (int)v;
}
inline int f2i_sat(double v) {
    if (v != v) return 0;
    if (v >= 2147483647.0) return INT_MAX;
    if (v <= -2147483648.0) return INT_MIN;
    return (int)v;
}
/* key = (Gy*Gz)*i + Gz*j + k with 32-bit wrap-around (as on the device) */
inline int key_of(const CGridBox& B, int i, int j, int k) {
    uint32_t gyz = (uint32_t)B.m_GridSize.y * (uint32_t)B.m_GridSize.z;
    uint32_t v = gyz * (uint32_t)i + (uint32_t)B.m_GridSize.z * (uint32_t)j + (uint32_t)k;
    return (int)v;
}

/* GetCellID, Utility_Inline.h:1697-1733 */
inline int cell_q(const CGridBox& B, const S3& p, int& i, int& j, int& k) {
    float rx = p.x - B.m_BufferedZone.m_MinBound.x;
    float ry = p.y - B.m_BufferedZone.m_MinBound.y;
    float rz = p.z - B.m_BufferedZone.m_MinBound.z;
    rx /= B.m_CellSize;
    ry /= B.m_CellSize;
    rz /= B.m_CellSize;
    i = f2i_sat(rx);
    j = f2i_sat(ry);
    k = f2i_sat(rz);
    return key_of(B, i, j, k);
}

/* IsInclude, Utility_Inline.h:2036-2077 */
inline bool include_q(const CGridBox& B, const S3& p, float tol) {
    const CBox& Z = B.m_ComputeZone;
    if (p.x < (Z.m_MinBound.x - tol)) return false;
    if (p.y < (Z.m_MinBound.y - tol)) return false;
    if (p.z < (Z.m_MinBound.z - tol)) return false;
    if (p.x > (Z.m_MaxBound.x + tol)) return false;
    if (p.y > (Z.m_MaxBound.y + tol)) return false;
    if (p.z > (Z.m_MaxBound.z + tol)) return false;
    return true;
}

/* CorrectVelocity, Utility_Inline.h:2369-2396: Courant clamp |v| <= l0*Cr/dt */
inline void correct_velocity_q(const CParameter& P, S3& v) {
    const float c = P.InitialParticleDistance * P.CourantNumber / P.Dt;
    float a = sqrt_q(v.x * v.x + v.y * v.y + v.z * v.z);
    if (a > c) {
        v.x = c * v.x / a;
        v.y = c * v.y / a;
        v.z = c * v.z / a;
    }
}

/* SegmentRatio, Utility_Inline.h:56-75 (only the z term is divided) */
inline float segment_ratio_q(const S3& p1, const S3& p2, const S3& p3) {
    S3 d = sub(p2, p1);
    float den = d.x * d.x + d.y * d.y + d.z * d.z;
    if (den == 0.0f) den = (float)1e-5;
    return (p3.x - p1.x) * (p2.x - p1.x) + (p3.y - p1.y) * (p2.y - p1.y) +
           (p3.z - p1.z) * (p2.z - p1.z) / den;
}

/* CalcDistanceVectorLine, Utility_Inline.h:91-113 (end cases return L1-p, L0-p) */
inline S3 line_q(const S3& l0, const S3& l1, const S3& p) {
    float u = segment_ratio_q(l0, l1, p);
    S3 dv = mk(0, 0, 0);
    if (u >= 0 && u <= 1) {
        S3 v = sub(l1, l0);
        S3 q = mk(l0.x + u * v.x, l0.y + u * v.y, l0.z + u * v.z);
        dv = sub(p, q);
    }
    if (u < 0) dv = sub(l1, p);
    if (u > 1) dv = sub(l0, p);
    return dv;
}

/* CalcNormalDistance, Utility_Inline.h:124-191 */
inline S3 normal_distance_q(const CTriangle& T, const S3& p) {
    const S3 n = T.Normal;
    S3 c;
    c.x = (float)((double)(T.Vertex[0].x + T.Vertex[1].x + T.Vertex[2].x) / 3.0);
    c.y = (float)((double)(T.Vertex[0].y + T.Vertex[1].y + T.Vertex[2].y) / 3.0);
    c.z = (float)((double)(T.Vertex[0].z + T.Vertex[1].z + T.Vertex[2].z) / 3.0);
    const float sd = sqrt_q(n.x * n.x + n.y * n.y + n.z * n.z);
    S3 dv = mk(0, 0, 0);
    if (sd == 0.0f) return dv;
    const float coef = ((n.x * p.x + n.y * p.y + n.z * p.z) - (n.x * c.x + n.y * c.y + n.z * c.z)) / sd;
    dv.x = coef / sd * n.x;
    dv.y = coef / sd * n.y;
    dv.z = coef / sd * n.z;
    return dv;
}

/* CalcDistance(triangle), Utility_Inline.h:193-232: distance magnitude, and in
 * *dir the vector from the wall point to the particle. */
inline float tri_distance_q(const CTriangle& T, const S3& p, S3* dir) {
    S3 dv = normal_distance_q(T, p);
    S3 P = mk(p.x - dv.x, p.y - dv.y, p.z - dv.z);
    S3 v0 = sub(T.Vertex[2], T.Vertex[0]);
    S3 v1 = sub(T.Vertex[1], T.Vertex[0]);
    S3 v2 = sub(P, T.Vertex[0]);
    float d00 = dot_q(v0, v0), d01 = dot_q(v0, v1), d02 = dot_q(v0, v2);
    float d11 = dot_q(v1, v1), d12 = dot_q(v1, v2);
    float inv = 1.0f / (d00 * d11 - d01 * d01);
    float u = (d11 * d02 - d01 * d12) * inv;
    float v = (d00 * d12 - d01 * d02) * inv;
    if (u >= 0 && v >= 0 && u + v > 1) dv = line_q(T.Vertex[1], T.Vertex[2], p);
    if (u < 0) dv = line_q(T.Vertex[0], T.Vertex[1], p);
    if (v < 0) dv = line_q(T.Vertex[0], T.Vertex[2], p);
    if (dir) *dir = dv;
    return mag_q(dv);
}

/* Triangle binning of one triangle, RegisterTriangle / RegisterLine,
 * Utility_Inline.h:1745-1855.  Cells receive the triangle id once (set
 * semantics, capacity CELLMAXTRIANGLENUM). The ring loop is capped at 100000
 * iterations (the reference has no cap). */
inline void cell_add(CCell* cells, int cid, int tid) {
    CCell& c = cells[cid];
    for (unsigned l = 0; l < c.m_TriangleNum; ++l)
        if (c.m_TriangleID[l] == tid) return;
    if (c.m_TriangleNum < CELLMAXTRIANGLENUM) c.m_TriangleID[c.m_TriangleNum++] = tid;
}
void register_line_q(const CGridBox& B, S3 v, S3 d, float m, int tid, CCell* cells, int ncell) {
    float tab = 0.0f;
    int guard = 0;
    do {
        S3 t = mk(v.x + tab * d.x, v.y + tab * d.y, v.z + tab * d.z);
        int i, j, k;
        int cid = cell_q(B, t, i, j, k);
        if (cid >= 0 && cid < ncell) cell_add(cells, cid, tid);
        tab += B.m_CellSize;
    } while (tab <= m && ++guard < 100000);
}
void register_triangle_q(const CGridBox& B, const CTriangle& T, int tid, CCell* cells, int ncell) {
    S3 A = T.Vertex[0], Bv = T.Vertex[1], C = T.Vertex[2];
    const float cs = B.m_CellSize;
    float mbc, mab, mca;
    int guard = 0;
    do {
        S3 ab = sub(Bv, A), ba = sub(A, Bv), bc = sub(C, Bv), cb = sub(Bv, C), ca = sub(A, C), ac = sub(C, A);
        mbc = mag_q(bc);
        mab = mag_q(ab);
        mca = mag_q(ca);
        if (mab > 0.0f) register_line_q(B, A, mk(ab.x / mab, ab.y / mab, ab.z / mab), mab, tid, cells, ncell);
        if (mbc > 0.0f) register_line_q(B, Bv, mk(bc.x / mbc, bc.y / mbc, bc.z / mbc), mbc, tid, cells, ncell);
        if (mca > 0.0f) register_line_q(B, C, mk(ca.x / mca, ca.y / mca, ca.z / mca), mca, tid, cells, ncell);
        S3 am = add(ab, ac), bm = add(ba, bc), cm = add(ca, cb);
        float mam = mag_q(am), mbm = mag_q(bm), mcm = mag_q(cm);
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

/* Nearest triangle over the 27 cells around p in (k, j, i) order, first minimum
 * wins; drag_only restricts to triangles of drag models (CalcNearestDistance,
 * DeviceProcess_Kernel.h:125-180; CalcSTLDistance_Kernel :853-919). */
void nearest_triangle_q(const OrcBindings* b, const S3& p, bool drag_only, CDistance& nd, int& nid) {
    int cx, cy, cz;
    int cid = cell_q(b->box, p, cx, cy, cz);
    if (!(cid >= 0 && cid < b->cell_num)) return;
    for (int k = -1; k <= 1; ++k)
        for (int j = -1; j <= 1; ++j)
            for (int i = -1; i <= 1; ++i) {
                int m = key_of(b->box, cx + i, cy + j, cz + k);
                if (m < 0 || m >= b->cell_num) continue;
                unsigned tn = b->cells[m].m_TriangleNum;
                for (unsigned l = 0; l < tn; ++l) {
                    int t = b->cells[m].m_TriangleID[l];
                    if (drag_only) {
                        if (t < 0 || t >= b->triangle_num) continue;
                        if (!b->tri_params[b->triangles[t].ModelIDNumber].isDrag) continue;
                    }
                    if (t >= 0 && t < b->triangle_num && t != nid) {
                        CDistance d;
                        d.Magnitude = tri_distance_q(b->triangles[t], p, &d.Direction);
                        if (d.Magnitude < nd.Magnitude) {
                            nd = d;
                            nid = t;
                        }
                    }
                }
            }
}

}  // namespace

/* ======================================================================== */
/* C interface, part 1                                                      */
/* ======================================================================== */
extern "C" {

float orc_sqrt_utility(float x) { return sqrt_q(x); }
float orc_calc_distance(const Scalar3* a, const Scalar3* b) { return dist_q(*a, *b); }
float orc_get_weight(float re, float r) { return weight_q(re, r); }
float orc_zgrad(float r, float l0) { return zeval_q(kZGrad3, r, l0); }
float orc_zlap(float r, float l0) { return zeval_q(kZLap3, r, l0); }
float orc_zgrad2d(float r, float l0) { return zeval_q(kZGrad2, r, l0); }
float orc_zlap2d(float r, float l0) { return zeval_q(kZLap2, r, l0); }
float orc_triangle_distance(const CTriangle* t, const Scalar3* p, Scalar3* dir) { return tri_distance_q(*t, *p, dir); }
int orc_cell_id(const CGridBox* box, const Scalar3* p, int* i, int* j, int* k) { return cell_q(*box, *p, *i, *j, *k); }
int orc_is_include(const CGridBox* box, const Scalar3* p, float tol) { return include_q(*box, *p, tol) ? 1 : 0; }
void orc_correct_velocity(const CParameter* param, Scalar3* v) { correct_velocity_q(*param, *v); }

/* CalculateLambdaValueLocal, MultiGPUHandler.cpp:757-921.  Each branch test is
 * written "lo < l0 <= hi", which C evaluates as (lo < l0) <= hi: a bool compared
 * with hi.  The branch taken is therefore the first row whose lower bound is not
 * below l0 (l0 promoted to double), or the first row with hi >= 1. */
float orc_lambda_table(float l0) {
    struct Row { double lo, hi, a, b; };
    static const Row rows[] = {
        {0, 0.0001, 5.02608E-06, 3.82946E-10},     {0.0001, 0.0005, 0.000124918, 1.81984E-08},
        {0.0005, 0.001, 0.0017886, -4.84707E-07},  {0.001, 0.002, 0.00373277, -2.15486E-06},
        {0.002, 0.003, 0.0066746, -6.72384E-06},   {0.003, 0.004, 0.0107452, -1.76386E-05},
        {0.004, 0.005, 0.0141993, -3.08052E-05},   {0.005, 0.006, 0.0164975, -4.14937E-05},
        {0.006, 0.007, 0.0181782, -4.95251E-05},   {0.007, 0.008, 0.0205885, -6.28759E-05},
        {0.008, 0.009, 0.0222761, -7.17244E-05},   {0.009, 0.01, 0.0231972, -7.34117E-05},
        {0.01, 0.02, 0.0369119, -0.000210081},     {0.02, 0.03, 0.0667457, -0.000672376},
        {0.03, 0.04, 0.106105, -0.00171939},       {0.04, 0.05, 0.141998, -0.00308074},
        {0.05, 0.06, 0.164981, -0.00414971},       {0.05, 0.06, 0.164981, -0.00414971},
        {0.06, 0.07, 0.178483, -0.00474469},       {0.07, 0.08, 0.197539, -0.00567825},
        {0.08, 0.09, 0.208407, -0.00598107},       {0.09, 0.1, 0.211437, -0.00543137},
        {0.01, 0.5, 0.369118, -0.021008},          {0.5, 1, 1.78861, -0.48471},
        {1, 10, 0.423015, 4.1213},                 {10, 1000, 0.0138964, 745.762}};
    float a = 0.0f, b = 0.0f;
    for (const Row& r : rows) {
        const int lt = (r.lo < (double)l0) ? 1 : 0;
        if ((double)lt <= r.hi) {
            a = (float)r.a;
            b = (float)r.b;
            break;
        }
    }
    return a * l0 + b;
}

/* calcHashD, DeviceProcess_Kernel.h:39-50 */
int orc_calc_hash(const OrcBindings* b, int n, int* hash, int* index, const Scalar3* pos) {
    for (int i = 0; i < n; ++i) {
        int cx, cy, cz;
        hash[i] = cell_q(b->box, pos[i], cx, cy, cz);
        index[i] = i;
    }
    return CCT_NOERR;
}

/* SortUsingThrust, DeviceProcess.cu:207-220: sort of (key, index) by key.  The
 * radix sort Thrust dispatches to for int keys is stable, so the result is the
 * stable order. */
int orc_sort(int n, int* hash, int* index) {
    if (n <= 0) return CCT_NOERR;
    std::vector<int> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int c) { return hash[a] < hash[c]; });
    std::vector<int> h(n), v(n);
    for (int i = 0; i < n; ++i) {
        h[i] = hash[perm[i]];
        v[i] = index[perm[i]];
    }
    std::memcpy(hash, h.data(), sizeof(int) * n);
    std::memcpy(index, v.data(), sizeof(int) * n);
    return CCT_NOERR;
}

/* reorderDataAndFindCellStartD + the two memsets, DeviceProcess_Kernel.h:54-124,
 * DeviceProcess.cu:191-206.  Keys outside [0, cells) are not recorded (the
 * reference writes out of bounds there). */
int orc_reorder_find_cell_start(OrcBindings* b, int n, int cells, const int* hash,
                                const int* index, int* cs, int* ce) {
    if (n <= 0) return CCT_NOERR;
    for (int c = 0; c < cells; ++c) { cs[c] = -1; ce[c] = -1; }
    for (int i = 0; i < n; ++i) {
        const int h = hash[i];
        const bool ok = h >= 0 && h < cells;
        if (i == 0 || h != hash[i - 1]) {
            if (ok) cs[h] = i;
            if (i > 0 && hash[i - 1] >= 0 && hash[i - 1] < cells) ce[hash[i - 1]] = i;
        }
        if (i == n - 1 && ok) ce[h] = i + 1;
        const int s = index[i];
        b->pos[i] = b->out_pos[s];
        b->vel[i] = b->out_vel[s];
        b->pressure[i] = b->out_pressure[s];
        b->density[i] = b->out_density[s];
        b->temperature[i] = b->out_temperature[s];
        b->kin_visc[i] = b->out_kin_visc[s];
        b->solid_rate[i] = b->out_solid_rate[s];
        b->type[i] = b->out_type[s];
        b->id[i] = s;
    }
    return CCT_NOERR;
}

/* CCellSet::CheckParticleOutsideComputeZone, CGPUCellSet.cpp:1160-1202: host
 * compaction of the original-order arrays; a deleted slot takes the current last
 * particle, which is not re-checked. */
int orc_check_outside_compute_zone(OrcBindings* b, int* n) {
    int N = *n;
    for (int i = 0; i < N; ++i) {
        if (!include_q(b->box, b->out_pos[i], b->param.Tolerance)) {
            const int l = N - 1;
            b->out_pos[i] = b->out_pos[l];
            b->out_vel[i] = b->out_vel[l];
            b->out_pressure[i] = b->out_pressure[l];
            b->out_density[i] = b->out_density[l];
            b->out_temperature[i] = b->out_temperature[l];
            b->out_kin_visc[i] = b->out_kin_visc[l];
            b->out_solid_rate[i] = b->out_solid_rate[l];
            b->out_type[i] = b->out_type[l];
            b->out_id[i] = b->out_id[l];
            --N;
        }
    }
    *n = N;
    return CCT_NOERR;
}

/* ResetTriangleTopology_Kernel, DeviceProcess_Kernel.h:594-602 */
int orc_reset_triangle_topology(int cells, CCell* cell) {
    for (int c = 0; c < cells; ++c) cell[c].m_TriangleNum = 0;
    return CCT_NOERR;
}

/* RegisterTriangleTopology_Kernel, DeviceProcess_Kernel.h:584-593.  Triangles
 * are processed in id order, so each cell lists its triangles in ascending id. */
int orc_register_triangle_topology(OrcBindings* b, const CTriangle* tri, int t, CCell* cell, int cells) {
    for (int i = 0; i < t; ++i) register_triangle_q(b->box, tri[i], i, cell, cells);
    return CCT_NOERR;
}

/* UpdateTrianglePosition_Kernel, DeviceProcess_Kernel.h:603-621 */
int orc_update_triangle_position(OrcBindings* b, int t) {
    for (int i = 0; i < t; ++i) {
        S3 v = b->tri_params[b->triangles[i].ModelIDNumber].Velocity;
        const float dt = b->param.Dt;
        v.x = v.x * dt; v.y = v.y * dt; v.z = v.z * dt;
        for (int q = 0; q < 3; ++q) b->triangles[i].Vertex[q] = add(b->triangles[i].Vertex[q], v);
    }
    return CCT_NOERR;
}

/* ResetWallPosition_Kernel, DeviceProcess_Kernel.h:690-704: a triangle of a linearly
 * moving model (LinearMovableOrNot) is copied back whole from the original triangles
 * every LinearResetInterval steps, at the steps with (step + 1) % interval == 0.  The
 * reference's modulo is undefined for an interval of 0; here such a model is never
 * reset (the library does the same). */
int orc_reset_wall_position(OrcBindings* b, int t, int step, const CTriangle* orig) {
    for (int id = 0; id < t; ++id) {
        const CTriangleParameters& tp = b->tri_params[b->triangles[id].ModelIDNumber];
        if (!tp.LinearMovableOrNot) continue;
        if (tp.LinearResetInterval == 0) continue;
        if ((step + 1) % tp.LinearResetInterval == 0) std::memcpy(&b->triangles[id], &orig[id], sizeof(CTriangle));
    }
    return CCT_NOERR;
}

/* RotateTrianglePosition_Kernel, DeviceProcess_Kernel.h:622-689: incremental
 * rotation by the per-step angle about the axis CenterOfRotation ->
 * SecondPointOfRotation, ramped linearly between RotationStartTime and
 * TimeToReachRPM. */
int orc_rotate_triangle_position(OrcBindings* b, int t, int step) {
    const float dt = b->param.Dt;
    for (int id = 0; id < t; ++id) {
        CTriangle& T = b->triangles[id];
        const CTriangleParameters tp = b->tri_params[T.ModelIDNumber];
        if (!tp.RotatingOrNot) continue;
        if ((step * dt) < tp.RotationStartTime) continue;
        float ang = 0.0f;
        const int req = (int)((tp.TimeToReachRPM - tp.RotationStartTime) / dt);
        const float tpass = dt * step;
        if ((tpass < tp.RotationStartTime) || (tp.AngleOfRotationInDegree == 0)) ang = 0.0f;
        else if ((tpass >= tp.RotationStartTime) && (tpass < tp.TimeToReachRPM))
            ang = (tp.AngleOfRotationInDegree / (req + 1)) * (step - (tp.RotationStartTime / dt));
        else ang = tp.AngleOfRotationInDegree;
        if (ang == 0) continue;
        for (int q = 0; q < 3; ++q) {
            /* CalcNormal, Utility_Inline.h:114-123 */
            float m = dist_q(tp.SecondPointOfRotation, tp.CenterOfRotation);
            S3 nv = mk(0, 0, 0);
            if (m > 0) nv = mk((tp.SecondPointOfRotation.x - tp.CenterOfRotation.x) / m,
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
    return CCT_NOERR;
}

/* CalcSTLDistance_Kernel, DeviceProcess_Kernel.h:853-919 (with the STLID memset
 * of CCellSet::CalculateSTLDistance, CGPUCellSet.cpp:1057). */
int orc_calc_stl_distance(OrcBindings* b, int n) {
    for (int id = 0; id < n; ++id) {
        CDistance nd;
        nd.Magnitude = 1e8f;
        nd.Direction = mk(0, 0, 0);
        int nid = -1;
        nearest_triangle_q(b, b->pos[id], false, nd, nid);
        b->stl_distance[id] = nd;
        b->stl_id[id] = nid;
    }
    return CCT_NOERR;
}

/* CalcDragEffect_Kernel and its mode helpers, DeviceProcess_Kernel.h:182-389.
 * The reference indexes some original-order arrays with the sorted index and
 * applies mode 'F' outside the influence region (brace placement, :375-388);
 * both are reproduced. */
int orc_calc_drag_effect(OrcBindings* b, int n) {
    const CParameter& P = b->param;
    for (int id = 0; id < n; ++id) {
        if (b->magnifier_count[id] > 0) b->magnifier_count[id]++;
        if (b->magnifier_count[id] == 10) b->magnifier_count[id] = 0;
        CDistance nd;
        nd.Magnitude = 1e8f;
        nd.Direction = mk(0, 0, 0);
        int nid = -1;
        if (b->out_id[id] < -1) {
            b->stl_distance[id] = nd;
            b->stl_id[id] = nid;
        } else {
            nearest_triangle_q(b, b->pos[id], true, nd, nid);
        }
        b->drag_acc[id] = mk(0, 0, 0);
        b->drag_temperature[id] = 0;
        b->out_type[id] = TYPE_HEAVY_WEIGHT;
        if (!(nid != -1 && nd.Magnitude != 1e8f)) continue;
        const DragParameter dp = b->drag_params[b->tri_params[b->triangles[nid].ModelIDNumber].DragTriangleID];
        if (nd.Magnitude <= dp.CoefficientofInflueneRegion * P.InitialParticleDistance) {
            b->out_type[id] = TYPE_LIGHT_WEIGHT;
            if (dp.DragToken == 'E') {
                if (dp.InputVelocityToken1 == 'V' || dp.InputVelocityToken1 == 'B') {
                    float pr = 0.0f;
                    const float sv = mag_q(b->vel[id]);
                    pr += dp.VelocityIndex * powf(sv, dp.VelocityExponential);
                    const S3 nrm = b->triangles[nid].Normal;
                    if (dp.VelocityDragPermiabilityConstant != 0) {
                        b->drag_acc[id].x = (pr * (nrm.x) / dp.VelocityDragPermiabilityConstant);
                        b->drag_acc[id].y = (pr * (nrm.y) / dp.VelocityDragPermiabilityConstant);
                        b->drag_acc[id].z = (pr * (nrm.z) / dp.VelocityDragPermiabilityConstant);
                    }
                } else if (dp.InputVelocityToken1 == 'T') {
                    const float sv = mag_q(b->vel[id]);
                    const float enth = dp.TempIndex * powf(sv, dp.TempExponential);
                    const float den = mag_q(b->vel[id]) * P.Density * P.FruidSpecificHeat;
                    if (den != 0)
                        b->drag_temperature[id] =
                            (enth * dp.TempDragPermiabilityConstant * P.Dt * P.ThermalStep) / (den);
                    b->out_solid_rate[id] = b->drag_temperature[id];
                }
            } else if (dp.DragToken == 'C') {
                if (dp.InputVelocityToken1 == 'V' || dp.InputVelocityToken1 == 'v') {
                    b->out_vel[id] = mk(dp.ConstantVx, dp.ConstantVy, dp.ConstantVz);
                    b->vel[id] = mk(dp.ConstantVx, dp.ConstantVy, dp.ConstantVz);
                }
            }
        } else if (dp.DragToken == 'F') {
            if (dp.InputVelocityToken1 == 'V' || dp.InputVelocityToken1 == 'v') {
                if (b->magnifier_count[id] < 1) {
                    const float f = dp.VelocityMagnitueFactor;
                    b->vel[id].x *= f; b->vel[id].y *= f; b->vel[id].z *= f;
                    b->out_vel[id].x *= f; b->out_vel[id].y *= f; b->out_vel[id].z *= f;
                }
            }
        }
    }
    return CCT_NOERR;
}

/* CalcExplicitly_Kernel, DeviceProcess_Kernel.h:390-582 (viscosity + gravity
 * predictor; artificial-pressure and collision terms when bExplicitPressure; with
 * bTurbulance the laminar plus turbulent viscosity scales the Laplacian (:545-552) and
 * the gradient of the strain product is accumulated (:477-485) but multiplied by the
 * integer quotient 2/3 = 0 before it reaches the velocity (:558-562)). */
int orc_calc_explicitly(OrcBindings* b, int n) {
    const CParameter& P = b->param;
    for (int id = 0; id < n; ++id) {
        const int orig = b->id[id];
        const float rho = P.Density;
        const S3 tp = b->pos[id];
        if (!include_q(b->box, tp, P.Tolerance)) {
            b->out_id[orig] = -1;
            b->out_solid_rate[orig] = 9999;
            continue;
        }
        int cx, cy, cz;
        const int cid = cell_q(b->box, tp, cx, cy, cz);
        S3 lap = mk(0, 0, 0), art = mk(0, 0, 0), col = mk(0, 0, 0);
        S3 v0 = b->vel[id];
        S3 tke = mk(0, 0, 0);
        const float re = P.LaplacianInfluenceRadiusCoefficient * P.InitialParticleDistance;
        const float rc = P.r_coeff * P.InitialParticleDistance;
        const float reg = P.GradientInfluenceRadiusCoefficient * P.InitialParticleDistance;
        if (cid >= 0 && cid < b->cell_num) {
            const float mind = (float)(re * 1e-3);
            for (int k = -1; k <= 1; ++k)
                for (int j = -1; j <= 1; ++j)
                    for (int i = -1; i <= 1; ++i) {
                        const int m = key_of(b->box, cx + i, cy + j, cz + k);
                        if (m < 0 || m >= b->cell_num) continue;
                        const int s = b->cell_start[m];
                        if ((unsigned)s == 0xffffffffu) continue;
                        const int e = b->cell_end[m];
                        for (int x = s; x < e; ++x) {
                            if (b->out_id[x] < 0) continue;
                            if (x == id) continue;
                            float d = dist_q(tp, b->pos[x]);
                            if (!(d < re)) continue;
                            if (d < mind) d = mind;
                            const float w = weight_q(re, d);
                            const S3 v1 = b->vel[x];
                            lap.x += (v1.x - v0.x) * w;
                            lap.y += (v1.y - v0.y) * w;
                            lap.z += (v1.z - v0.z) * w;
                            if (P.bTurbulance && d < reg) {
                                const float w1 = weight_q(reg, d);
                                const float sc = (b->strain[x] - b->strain[id]) * w1 / (d * d);
                                tke = add(tke, mul(sub(b->pos[x], tp), sc));
                            }
                            if (P.bExplicitPressure && d < rc) {
                                const float a = P.ArtificialPressure * w / (d * d);
                                art = add(art, mul(sub(b->pos[x], tp), a));
                                const float c = (rc - d) / d;
                                col = add(col, mul(sub(b->pos[x], tp), c));
                            }
                        }
                    }
        }
        const float wd = b->stl_distance[id].Magnitude;
        const int tri = b->stl_id[id];
        if (tri >= 0 && tri < b->triangle_num && wd > 0 && wd < re) {
            const float ww = (2 == P.Dimension) ? zeval_q(kZLap2, wd, P.InitialParticleDistance)
                                                : zeval_q(kZLap3, wd, P.InitialParticleDistance);
            const S3 v1 = b->tri_params[b->triangles[tri].ModelIDNumber].Velocity;
            lap.x += P.WallFrictionCoeffieicnt * (v1.x - v0.x) * ww;
            lap.y += P.WallFrictionCoeffieicnt * (v1.y - v0.y) * ww;
            lap.z += P.WallFrictionCoeffieicnt * (v1.z - v0.z) * ww;
        }
        const float coef = (float)((2.0 * P.Dimension) / (double)(P.LambdaValue * P.ConstantParticleDensity));
        lap.x *= coef; lap.y *= coef; lap.z *= coef;
        S3 dragv = mk(0, 0, 0);
        S3 acc = add(mk(0, 0, 0), P.GravityConstant);
        if (b->drag_num > 0) dragv = b->drag_acc[id];
        if (P.bTurbulance) lap = mul(lap, b->kin_visc[id] + b->turb_visc[id]);
        else lap = mul(lap, b->kin_visc[id]);
        acc = add(acc, lap);
        v0 = sub(add(v0, mul(acc, P.Dt)), dragv);
        if (P.bTurbulance) {
            tke = mul(tke, (float)(2 / 3));
            v0 = sub(v0, mul(tke, P.Dt));
        }
        if (P.bExplicitPressure) {
            const float c = (float)(-P.Dimension) / (P.ConstantParticleDensity * rho);
            acc = add(mul(art, c), mul(col, (float)0.01));
            v0 = add(v0, mul(acc, P.Dt));
        }
        if (std::isfinite(v0.x) && std::isfinite(v0.y) && std::isfinite(v0.z)) {
            b->out_pos[orig].x = tp.x + P.Dt * v0.x;
            b->out_pos[orig].y = tp.y + P.Dt * v0.y;
            b->out_pos[orig].z = tp.z + P.Dt * v0.z;
            b->out_vel[orig] = v0;
        }
    }
    return CCT_NOERR;
}

/* CalcTemperatureFactor_Kernel, DeviceProcess_Kernel.h:705-852: heat conduction
 * over the neighbours within the temperature radius (distance <= re, clamped below at
 * 1e-3 re; conductance 1 / (1/k + R/r) over r^2), the nearest wall through its
 * gradient Z function with the harmonic mean of the fluid and wall conductivities, the
 * drag heating; both sums enter only when larger than FLT_EPSILON in magnitude; the
 * result clamped to [MinWallTemperature, MaxWallTemperature] and the viscosity updated
 * linearly in it (output arrays at the original index). */
int orc_calc_temperature_factor(OrcBindings* b, int n) {
    const CParameter& P = b->param;
    for (int id = 0; id < n; ++id) {
        const float rho = P.Density;
        const float ecoef = P.Dt * 2 * P.Dimension / (P.ConstantParticleDensity * rho * P.FruidSpecificHeat);
        float hf = 0.0f, hw = 0.0f;
        const float ret = P.TemperatureInfluenceRadiusCoefficient * P.InitialParticleDistance;
        float num = 0, den = 0;
        const S3 tp = b->pos[id];
        float tt = b->temperature[id];
        const int orig = b->id[id];
        if (!include_q(b->box, tp, P.Tolerance)) {
            b->out_id[orig] = -1;
            continue;
        }
        int cx, cy, cz;
        const int cid = cell_q(b->box, tp, cx, cy, cz);
        if (cid < 0 || cid >= b->cell_num) continue;
        const float mind = (float)(ret * 1e-3);
        for (int k = -1; k <= 1; ++k)
            for (int j = -1; j <= 1; ++j)
                for (int i = -1; i <= 1; ++i) {
                    const int m = key_of(b->box, cx + i, cy + j, cz + k);
                    if (m < 0 || m >= b->cell_num) continue;
                    const int s = b->cell_start[m];
                    if ((unsigned)s == 0xffffffffu) continue;
                    const int e = b->cell_end[m];
                    for (int x = s; x < e; ++x) {
                        if (b->out_id[x] < 0) continue;
                        if (x == id) continue;
                        float d = dist_q(tp, b->pos[x]);
                        if (!(d <= ret)) continue;
                        if (d < mind) d = mind;
                        num = (b->temperature[x] - tt) * weight_q(ret, d);
                        den = d * d * (1 / P.FruidThermalConductivity + P.FruidThermalResistance / d);
                        hf += num / den;
                    }
                }
        const float wd = b->stl_distance[id].Magnitude;
        const int tri = b->stl_id[id];
        if (tri >= 0 && tri < b->triangle_num && wd > 0 && wd < ret) {
            const CTriangleParameters& tq = b->tri_params[b->triangles[tri].ModelIDNumber];
            const float res = tq.WallThermalResistivity;
            const float cond = (2 * P.FruidThermalConductivity * tq.WallThermalConductivity) /
                               (P.FruidThermalConductivity + tq.WallThermalConductivity);
            const float ww = (2 == P.Dimension) ? zeval_q(kZGrad2, wd, P.InitialParticleDistance)
                                                : zeval_q(kZGrad3, wd, P.InitialParticleDistance);
            num = (tq.Temperature - tt) * ww;
            den = wd * wd * (1 / cond + res / wd);
            hw = num / den;
        }
        if (b->drag_num > 0) tt += b->drag_temperature[id];
        float comb = 0.0f;
        if (std::fabs(hf) > FLT_EPSILON) comb += hf;
        if (std::fabs(hw) > FLT_EPSILON) comb += hw;
        tt += (ecoef * (comb));
        if (tt > P.MaxWallTemperature) tt = P.MaxWallTemperature;
        if (tt < P.MinWallTemperature) tt = P.MinWallTemperature;
        b->out_temperature[orig] = tt;
        b->out_kin_visc[orig] = P.ViscosityUpdateParameterA * tt + P.ViscosityUpdateParameterB;
    }
    return CCT_NOERR;
}

/* CalcTurbulenceViscosity_Kernel, DeviceProcess_Kernel.h:1273-1476: the velocity
 * gradient tensor over the neighbours within the gradient radius (scaled by d / n0),
 * the strain-rate product S = A^2 + B^2 + C^2 + 2 (D^2 + E^2 + F^2) of its diagonal and
 * symmetrised off-diagonal parts, a Smagorinsky viscosity with the wall damping
 * 1 - exp(-r_w / re) capped at TurbulanViscosityRatio, and the turbulent kinetic
 * energy S 2 Cnue l0^2 / Cepsilon capped at TurbulanceIntensity (sorted-order arrays).
 * The kernel's vorticity and neighbour PND are never read (its vorticity uses a
 * distance vector that stays zero) and are left out. */
int orc_calc_turbulence_viscosity(OrcBindings* b, int n) {
    const CParameter& P = b->param;
    for (int id = 0; id < n; ++id) {
        const int orig = b->id[id];
        const S3 tp = b->pos[id];
        const S3 v0 = b->vel[id];
        if (!include_q(b->box, tp, P.Tolerance)) {
            b->turb_visc[id] = 0.0f;
            b->out_id[orig] = -1;
            continue;
        }
        S3 X = mk(0, 0, 0), Y = mk(0, 0, 0), Z = mk(0, 0, 0), D = mk(0, 0, 0);
        float strain = 0.0f, coef = 0.0f;
        int cx, cy, cz;
        const int cid = cell_q(b->box, tp, cx, cy, cz);
        if (cid < 0 || cid >= b->cell_num) {
            b->pressure[id] = 0.0f;
            continue;
        }
        const float re = P.GradientInfluenceRadiusCoefficient * P.InitialParticleDistance;
        const float mind = (float)(re * 1e-3);
        for (int k = -1; k <= 1; ++k)
            for (int j = -1; j <= 1; ++j)
                for (int i = -1; i <= 1; ++i) {
                    const int m = key_of(b->box, cx + i, cy + j, cz + k);
                    if (m < 0 || m >= b->cell_num) continue;
                    const int s = b->cell_start[m];
                    if ((unsigned)s == 0xffffffffu) continue;
                    const int e = b->cell_end[m];
                    for (int x = s; x < e; ++x) {
                        if (b->out_id[x] < 0) continue;
                        if (x == id) continue;
                        float d = dist_q(tp, b->pos[x]);
                        if (!(d < re)) continue;
                        if (d < mind) d = mind;
                        const float w = weight_q(re, d);
                        const S3 v1 = b->vel[x];
                        const S3 q = b->pos[x];
                        X.x += ((v1.x - v0.x) * (q.x - tp.x) * w) / (d * d);
                        X.y += ((v1.x - v0.x) * (q.y - tp.y) * w) / (d * d);
                        X.z += ((v1.x - v0.x) * (q.z - tp.z) * w) / (d * d);
                        Y.x += ((v1.y - v0.y) * (q.x - tp.x) * w) / (d * d);
                        Y.y += ((v1.y - v0.y) * (q.y - tp.y) * w) / (d * d);
                        Y.z += ((v1.y - v0.y) * (q.z - tp.z) * w) / (d * d);
                        Z.x += ((v1.z - v0.z) * (q.x - tp.x) * w) / (d * d);
                        Z.y += ((v1.z - v0.z) * (q.y - tp.y) * w) / (d * d);
                        Z.z += ((v1.z - v0.z) * (q.z - tp.z) * w) / (d * d);
                    }
                }
        const float g = P.Dimension / P.ConstantParticleDensity;
        X.x = g * X.x; X.y = g * X.y; X.z = g * X.z;
        Y.x = g * Y.x; Y.y = g * Y.y; Y.z = g * Y.z;
        Z.x = g * Z.x; Z.y = g * Z.y; Z.z = g * Z.z;
        D.x = (float)(0.5 * (X.y + Y.x));
        D.y = (float)(0.5 * (X.z + Z.x));
        D.z = (float)(0.5 * (Y.z + Z.y));
        strain = X.x * X.x + Y.y * Y.y + Z.z * Z.z + 2 * D.x * D.x + 2 * D.y * D.y + 2 * D.z * D.z;
        const float riw = b->stl_distance[id].Magnitude;
        const float ratio = -(riw / re);
        const float damp = 1 - std::exp(ratio);
        const float smag = P.SmagorinskyConstant * damp;
        coef = (smag * P.FilterWidth) * (smag * P.FilterWidth);
        float tv = 0;
        if (strain > 0) tv = coef * std::sqrt(2 * strain);
        if (tv > P.TurbulanViscosityRatio) tv = P.TurbulanViscosityRatio;
        b->turb_visc[id] = tv;
        const float tkc = 2 * P.Cnue * P.InitialParticleDistance * P.InitialParticleDistance / P.Cepsilon;
        float tke = strain * tkc;
        if (tke > P.TurbulanceIntensity) tke = P.TurbulanceIntensity;
        b->strain[id] = tke;
    }
    return CCT_NOERR;
}

/* CalcExplicitPressure_Kernel, DeviceProcess_Kernel.h:921-1054: PND with the
 * gradient radius plus the wall weight, then P = c^2 rho / n0 (n - n0) where
 * n > beta n0. */
int orc_calc_explicit_pressure(OrcBindings* b, int n) {
    const CParameter& P = b->param;
    for (int id = 0; id < n; ++id) {
        const int orig = b->id[id];
        const S3 tp = b->pos[id];
        if (!include_q(b->box, tp, P.Tolerance)) {
            b->out_id[orig] = -1;
            b->pressure[id] = 0.0f;
            continue;
        }
        const float rho = P.Density;
        int cx, cy, cz;
        const int cid = cell_q(b->box, tp, cx, cy, cz);
        if (cid < 0 || cid >= b->cell_num) {
            b->pressure[id] = 0.0f;
            continue;
        }
        const float re = P.GradientInfluenceRadiusCoefficient * P.InitialParticleDistance;
        const float mind = (float)(re * 1e-3);
        const float coef = P.SonicVelocity * P.SonicVelocity * rho / P.ConstantParticleDensity;
        float dens = 0.0f;
        for (int k = -1; k <= 1; ++k)
            for (int j = -1; j <= 1; ++j)
                for (int i = -1; i <= 1; ++i) {
                    const int m = key_of(b->box, cx + i, cy + j, cz + k);
                    if (m < 0 || m >= b->cell_num) continue;
                    const int s = b->cell_start[m];
                    if ((unsigned)s == 0xffffffffu) continue;
                    const int e = b->cell_end[m];
                    for (int x = s; x < e; ++x) {
                        if (b->out_id[x] < 0) continue;
                        if (x == id) continue;
                        float d = dist_q(tp, b->pos[x]);
                        if (!(d < re)) continue;
                        if (d < mind) d = mind;
                        dens += weight_q(re, d);
                    }
                }
        const float riw = b->stl_distance[id].Magnitude;
        float ww = 0.0f;
        if (b->stl_id[id] >= 0 && b->stl_id[id] < b->triangle_num && riw >= 0 && riw <= re)
            ww = (2 == P.Dimension) ? zeval_q(kZGrad2, riw, P.InitialParticleDistance)
                                    : zeval_q(kZGrad3, riw, P.InitialParticleDistance);
        dens += ww;
        if (std::isfinite(dens)) b->out_density[orig] = dens;
        float pr = 0.0f;
        if (dens > P.ConstantParticleDensity * P.FreeSurfaceThreshold) pr = coef * (dens - P.ConstantParticleDensity);
        if (std::isfinite(pr)) {
            b->out_pressure[orig] = pr;
            b->pressure[id] = pr;
        }
    }
    return CCT_NOERR;
}

/* CalcExplicitPressureGradient_Kernel, DeviceProcess_Kernel.h:1056-1271: pressure
 * gradient (fluid term, Yamada wall term, Harada penalty), velocity and position
 * correction, Courant clamp.  The negative-pressure branch is not supported. */
int orc_calc_explicit_pressure_gradient(OrcBindings* b, int n) {
    const CParameter& P = b->param;
    if (P.bNegativePressure) return CCT_PARAMERR;
    for (int id = 0; id < n; ++id) {
        const int orig = b->id[id];
        const float rho = P.Density;
        const S3 tp = b->pos[id];
        if (!include_q(b->box, tp, P.Tolerance)) {
            b->out_id[orig] = -1;
            continue;
        }
        int cx, cy, cz;
        const int cid = cell_q(b->box, tp, cx, cy, cz);
        if (cid < 0 || cid >= b->cell_num) continue;
        const float re = P.GradientInfluenceRadiusCoefficient * P.InitialParticleDistance;
        S3 gf = mk(0, 0, 0), gw = mk(0, 0, 0);
        const float tpress = b->pressure[id];
        const float mind = (float)(re * 1e-3);
        for (int k = -1; k <= 1; ++k)
            for (int j = -1; j <= 1; ++j)
                for (int i = -1; i <= 1; ++i) {
                    const int m = key_of(b->box, cx + i, cy + j, cz + k);
                    if (m < 0 || m >= b->cell_num) continue;
                    const int s = b->cell_start[m];
                    if ((unsigned)s == 0xffffffffu) continue;
                    const int e = b->cell_end[m];
                    for (int x = s; x < e; ++x) {
                        if (b->out_id[x] < 0) continue;
                        if (x == id) continue;
                        float d = dist_q(tp, b->pos[x]);
                        if (!(d < re)) continue;
                        if (d < mind) d = mind;
                        const float pc = (float)(0.5 * (double)(b->pressure[x] + tpress) * (double)weight_q(re, d));
                        gf.x += pc * (b->pos[x].x - tp.x) / (d * d);
                        gf.y += pc * (b->pos[x].y - tp.y) / (d * d);
                        gf.z += pc * (b->pos[x].z - tp.z) / (d * d);
                    }
                }
        const float c1 = 2 * P.Dimension / (P.ConstantParticleDensity);
        const float c2 = rho / (P.Dt * P.Dt);
        const float c3 = -P.Dt / rho;
        gf.x *= c1; gf.y *= c1; gf.z *= c1;
        const CDistance riw = b->stl_distance[id];
        if (b->stl_id[id] >= 0 && b->stl_id[id] < b->triangle_num) {
            if (riw.Magnitude > 0 && riw.Magnitude <= re) {
                const float ww = zeval_q(kZGrad3, riw.Magnitude, P.InitialParticleDistance);
                const float wc = (float)((((0.5 * (double)c1) * (double)ww) * (double)tpress) /
                                         (double)(riw.Magnitude * riw.Magnitude));
                gw.x = wc * (-riw.Direction.x);
                gw.y = wc * (-riw.Direction.y);
                gw.z = wc * (-riw.Direction.z);
            }
            if (riw.Magnitude > 0 && riw.Magnitude <= P.InitialParticleDistance * P.OffSet) {
                const float dr = (P.InitialParticleDistance * P.OffSet - riw.Magnitude);
                const float mc = c2 * dr / riw.Magnitude;
                gw.x += mc * (-riw.Direction.x);
                gw.y += mc * (-riw.Direction.y);
                gw.z += mc * (-riw.Direction.z);
            }
        }
        const S3 g = add(add(gf, gw), mk(0, 0, 0));
        S3 iv = mk(c3 * g.x, c3 * g.y, c3 * g.z);
        if (std::isfinite(iv.x) && std::isfinite(iv.y) && std::isfinite(iv.z)) {
            S3 ov = mk(b->vel[id].x + iv.x, b->vel[id].y + iv.y, b->vel[id].z + iv.z);
            correct_velocity_q(P, ov);
            b->out_vel[orig] = ov;
            iv = mk(ov.x - b->vel[id].x, ov.y - b->vel[id].y, ov.z - b->vel[id].z);
            b->out_pos[orig].x = tp.x + iv.x * P.Dt;
            b->out_pos[orig].y = tp.y + iv.y * P.Dt;
            b->out_pos[orig].z = tp.z + iv.z * P.Dt;
        }
    }
    return CCT_NOERR;
}

}  // extern "C"

/* ======================================================================== */
/* Part 2: FP64 semi-implicit solver                                        */
/* ======================================================================== */
namespace {

struct D3 { double x, y, z; };
inline D3 d3(double x, double y, double z) { D3 t; t.x = x; t.y = y; t.z = z; return t; }
inline D3 dsub(const D3& a, const D3& b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline D3 dadd(const D3& a, const D3& b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline D3 dmul(const D3& a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
inline double ddot(const D3& a, const D3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double dlen(const D3& a) { return std::sqrt(ddot(a, a)); }

/* Closest point on triangle (a, b, c) to p, by Voronoi-region classification
 * (Ericson, Real-Time Collision Detection, section 5.1.5). */
D3 closest_on_triangle(const D3& p, const D3& a, const D3& b, const D3& c) {
    const D3 ab = dsub(b, a), ac = dsub(c, a), ap = dsub(p, a);
    const double d1 = ddot(ab, ap), d2 = ddot(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) return a;
    const D3 bp = dsub(p, b);
    const double d3v = ddot(ab, bp), d4 = ddot(ac, bp);
    if (d3v >= 0.0 && d4 <= d3v) return b;
    const double vc = d1 * d4 - d3v * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3v <= 0.0) return dadd(a, dmul(ab, d1 / (d1 - d3v)));
    const D3 cp = dsub(p, c);
    const double d5 = ddot(ab, cp), d6 = ddot(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) return c;
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) return dadd(a, dmul(ac, d2 / (d2 - d6)));
    const double va = d3v * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3v) >= 0.0 && (d5 - d6) >= 0.0)
        return dadd(b, dmul(dsub(c, b), (d4 - d3v) / ((d4 - d3v) + (d5 - d6))));
    const double den = 1.0 / (va + vb + vc);
    return dadd(a, dadd(dmul(ab, vb * den), dmul(ac, vc * den)));
}

inline double weight_d(double re, double r) {
    if (r > re) return 0.0;
    if (r > 0.0) return re / r - 1.0;
    return 1e6;
}

/* Deterministic sum: fixed 4096-element blocks, block partials added in order,
 * independent of the thread count. */
double det_sum(const std::vector<double>& v, int n) {
    const int B = 4096;
    const int nb = (n + B - 1) / B;
    std::vector<double> part(nb > 0 ? nb : 1, 0.0);
#pragma omp parallel for schedule(static)
    for (int q = 0; q < nb; ++q) {
        double s = 0.0;
        const int e = std::min(n, (q + 1) * B);
        for (int i = q * B; i < e; ++i) s += v[i];
        part[q] = s;
    }
    double s = 0.0;
    for (int q = 0; q < nb; ++q) s += part[q];
    return s;
}

struct SimTri { D3 v[3]; D3 nrm; int model; };

}  // namespace

struct OrcSim {
    OrcSimConfig cfg;
    int maxn = 0;
    int n = 0;
    /* original-order state */
    std::vector<D3> pos, vel;
    std::vector<double> press, pnd, visc;
    std::vector<int> type, id;
    /* walls */
    std::vector<SimTri> tris;
    std::vector<CTriangleParameters> tparams;
    std::vector<DragParameter> drag;
    std::vector<int> tcell_start, tcell_ids;
    /* grid */
    int cells = 0;
    std::vector<int> cstart, cend;
    std::vector<int> sid;
    std::vector<D3> spos, svel;
    std::vector<double> spress, svisc;
    std::vector<int> stype;
    std::vector<double> wdist;
    std::vector<D3> wdir;
    std::vector<int> wid;
    std::vector<D3> dragv;
    /* last PPE (sorted order) */
    std::vector<double> l_pnd, l_diag, l_rhs, l_sol, l_idsum;
    std::vector<int> l_rowptr, l_col;
    std::vector<double> l_val;
    std::vector<int> l_sid, l_cnt, l_id;

    double l0() const { return cfg.param.InitialParticleDistance; }
    double re_lap() const { return (double)cfg.param.LaplacianInfluenceRadiusCoefficient * l0(); }
    double re_grad() const { return (double)cfg.param.GradientInfluenceRadiusCoefficient * l0(); }

    bool include(const D3& p) const {
        const CBox& Z = cfg.box.m_ComputeZone;
        const double t = cfg.param.Tolerance;
        if (p.x < ((double)Z.m_MinBound.x - t)) return false;
        if (p.y < ((double)Z.m_MinBound.y - t)) return false;
        if (p.z < ((double)Z.m_MinBound.z - t)) return false;
        if (p.x > ((double)Z.m_MaxBound.x + t)) return false;
        if (p.y > ((double)Z.m_MaxBound.y + t)) return false;
        if (p.z > ((double)Z.m_MaxBound.z + t)) return false;
        return true;
    }
    int cell_of(const D3& p, int& i, int& j, int& k) const {
        const CGridBox& B = cfg.box;
        const double cs = B.m_CellSize;
        i = f2i_sat((p.x - (double)B.m_BufferedZone.m_MinBound.x) / cs);
        j = f2i_sat((p.y - (double)B.m_BufferedZone.m_MinBound.y) / cs);
        k = f2i_sat((p.z - (double)B.m_BufferedZone.m_MinBound.z) / cs);
        return key_of(B, i, j, k);
    }

    /* reference compaction order (CGPUCellSet.cpp:1160-1202) on the FP64 state */
    void compact() {
        int N = n;
        for (int i = 0; i < N; ++i) {
            if (!include(pos[i])) {
                const int l = N - 1;
                pos[i] = pos[l]; vel[i] = vel[l]; press[i] = press[l]; pnd[i] = pnd[l];
                visc[i] = visc[l]; type[i] = type[l]; id[i] = id[l];
                --N;
            }
        }
        n = N;
    }

    void build_grid() {
        std::vector<int> key(n), perm(n);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            int a, b, c;
            key[i] = cell_of(pos[i], a, b, c);
        }
        std::iota(perm.begin(), perm.end(), 0);
        std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return key[a] < key[b]; });
        cstart.assign(cells, -1);
        cend.assign(cells, -1);
        sid.resize(n); spos.resize(n); svel.resize(n); spress.resize(n); svisc.resize(n); stype.resize(n);
        for (int s = 0; s < n; ++s) {
            const int o = perm[s];
            const int h = key[o];
            const bool ok = h >= 0 && h < cells;
            if (s == 0 || h != key[perm[s - 1]]) {
                if (ok) cstart[h] = s;
                if (s > 0) {
                    const int hp = key[perm[s - 1]];
                    if (hp >= 0 && hp < cells) cend[hp] = s;
                }
            }
            if (s == n - 1 && ok) cend[h] = s + 1;
            sid[s] = o; spos[s] = pos[o]; svel[s] = vel[o]; spress[s] = press[o];
            svisc[s] = visc[o]; stype[s] = type[o];
        }
    }

    /* Triangle -> cell lists: every cell the triangle's bounding box overlaps,
     * ascending triangle id within a cell.  A superset of the cells the triangle
     * touches, so the nearest triangle within one cell size is always found. */
    void bin_triangles() {
        const CGridBox& B = cfg.box;
        const double cs = B.m_CellSize;
        std::vector<std::vector<int>> lists(cells);
        for (int t = 0; t < (int)tris.size(); ++t) {
            D3 lo = tris[t].v[0], hi = tris[t].v[0];
            for (int q = 1; q < 3; ++q) {
                lo.x = std::min(lo.x, tris[t].v[q].x); hi.x = std::max(hi.x, tris[t].v[q].x);
                lo.y = std::min(lo.y, tris[t].v[q].y); hi.y = std::max(hi.y, tris[t].v[q].y);
                lo.z = std::min(lo.z, tris[t].v[q].z); hi.z = std::max(hi.z, tris[t].v[q].z);
            }
            int i0 = f2i_sat((lo.x - (double)B.m_BufferedZone.m_MinBound.x) / cs);
            int j0 = f2i_sat((lo.y - (double)B.m_BufferedZone.m_MinBound.y) / cs);
            int k0 = f2i_sat((lo.z - (double)B.m_BufferedZone.m_MinBound.z) / cs);
            int i1 = f2i_sat((hi.x - (double)B.m_BufferedZone.m_MinBound.x) / cs);
            int j1 = f2i_sat((hi.y - (double)B.m_BufferedZone.m_MinBound.y) / cs);
            int k1 = f2i_sat((hi.z - (double)B.m_BufferedZone.m_MinBound.z) / cs);
            i0 = std::max(i0, 0); j0 = std::max(j0, 0); k0 = std::max(k0, 0);
            i1 = std::min(i1, B.m_GridSize.x - 1); j1 = std::min(j1, B.m_GridSize.y - 1);
            k1 = std::min(k1, B.m_GridSize.z - 1);
            for (int i = i0; i <= i1; ++i)
                for (int j = j0; j <= j1; ++j)
                    for (int k = k0; k <= k1; ++k) {
                        const int c = key_of(B, i, j, k);
                        if (c >= 0 && c < cells) lists[c].push_back(t);
                    }
        }
        tcell_start.assign(cells + 1, 0);
        for (int c = 0; c < cells; ++c) tcell_start[c + 1] = tcell_start[c] + (int)lists[c].size();
        tcell_ids.resize(tcell_start[cells]);
        for (int c = 0; c < cells; ++c)
            std::copy(lists[c].begin(), lists[c].end(), tcell_ids.begin() + tcell_start[c]);
    }

    /* Nearest triangle of the 27 cells around p: the candidates (each triangle once)
     * in increasing id, a candidate replacing the current nearest only when closer by
     * more than 1e-12 l0, so that triangles at the same distance (closest point on a
     * shared edge or vertex) resolve to the lowest id rather than to rounding. */
    void nearest(const D3& p, bool drag_only, double& md, D3& mdir, int& mid) const {
        md = 1e8; mdir = d3(0, 0, 0); mid = -1;
        int cx, cy, cz;
        const int cid = cell_of(p, cx, cy, cz);
        if (!(cid >= 0 && cid < cells)) return;
        std::vector<int> cand;
        for (int k = -1; k <= 1; ++k)
            for (int j = -1; j <= 1; ++j)
                for (int i = -1; i <= 1; ++i) {
                    const int m = key_of(cfg.box, cx + i, cy + j, cz + k);
                    if (m < 0 || m >= cells) continue;
                    for (int l = tcell_start[m]; l < tcell_start[m + 1]; ++l) {
                        const int t = tcell_ids[l];
                        if (drag_only == (bool)tparams[tris[t].model].isDrag) cand.push_back(t);
                    }
                }
        std::sort(cand.begin(), cand.end());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
        const double tol = 1e-12 * l0();
        for (const int t : cand) {
            const D3 q = closest_on_triangle(p, tris[t].v[0], tris[t].v[1], tris[t].v[2]);
            const D3 dv = dsub(p, q);
            const double d = dlen(dv);
            if (d < md - tol) { md = d; mdir = dv; mid = t; }
        }
    }

    void wall_distance() {
        wdist.resize(n); wdir.resize(n); wid.resize(n);
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < n; ++s) nearest(spos[s], false, wdist[s], wdir[s], wid[s]);
    }

    /* Drag (per-body model of DeviceProcess_Kernel.h:309-389 without the
     * sorted/original index mix-up): the nearest drag-model triangle within the
     * influence radius acts on the particle. */
    void apply_drag() {
        dragv.assign(n, d3(0, 0, 0));
        if (drag.empty()) return;
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < n; ++s) {
            double md; D3 mdir; int mid;
            nearest(spos[s], true, md, mdir, mid);
            if (mid < 0) continue;
            const DragParameter& dp = drag[tparams[tris[mid].model].DragTriangleID];
            if (!(md <= (double)dp.CoefficientofInflueneRegion * l0())) continue;
            if (dp.DragToken == 'E' && (dp.InputVelocityToken1 == 'V' || dp.InputVelocityToken1 == 'B')) {
                const double sv = dlen(svel[s]);
                const double pr = (double)dp.VelocityIndex * std::pow(sv, (double)dp.VelocityExponential);
                if (dp.VelocityDragPermiabilityConstant != 0)
                    dragv[s] = dmul(tris[mid].nrm, pr / (double)dp.VelocityDragPermiabilityConstant);
            } else if (dp.DragToken == 'C' && (dp.InputVelocityToken1 == 'V' || dp.InputVelocityToken1 == 'v')) {
                svel[s] = d3(dp.ConstantVx, dp.ConstantVy, dp.ConstantVz);
            } else if (dp.DragToken == 'F' && (dp.InputVelocityToken1 == 'V' || dp.InputVelocityToken1 == 'v')) {
                svel[s] = dmul(svel[s], (double)dp.VelocityMagnitueFactor);
            }
        }
    }

    template <class F>
    void for_neighbours(int s, double re, F&& f) const {
        const D3 p = spos[s];
        int cx, cy, cz;
        const int cid = cell_of(p, cx, cy, cz);
        if (!(cid >= 0 && cid < cells)) return;
        for (int k = -1; k <= 1; ++k)
            for (int j = -1; j <= 1; ++j)
                for (int i = -1; i <= 1; ++i) {
                    const int m = key_of(cfg.box, cx + i, cy + j, cz + k);
                    if (m < 0 || m >= cells) continue;
                    const int st = cstart[m];
                    if (st < 0) continue;
                    const int en = cend[m];
                    for (int x = st; x < en; ++x) {
                        if (x == s) continue;
                        const D3 dv = dsub(spos[x], p);
                        const double r = dlen(dv);
                        if (!(r < re)) continue;
                        f(x, r, dv);
                    }
                }
    }

    /* Viscosity/gravity predictor (CalcExplicitly_Kernel semantics, FP64). */
    void predictor() {
        const CParameter& P = cfg.param;
        const double re = re_lap(), mind = re * 1e-3;
        const double coef = 2.0 * P.Dimension / (cfg.lambda * cfg.n0_lap);
        const double dt = P.Dt;
        std::vector<D3> npos(n), nvel(n);
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < n; ++s) {
            const D3 v0 = svel[s];
            D3 lap = d3(0, 0, 0);
            for_neighbours(s, re, [&](int x, double r, const D3&) {
                const double w = weight_d(re, std::max(r, mind));
                lap = dadd(lap, dmul(dsub(svel[x], v0), w));
            });
            if (wid[s] >= 0 && wdist[s] > 0 && wdist[s] < re) {
                const double ww = (2 == P.Dimension) ? zeval_d(kZLap2, wdist[s], l0()) : zeval_d(kZLap3, wdist[s], l0());
                const CTriangleParameters& tp = tparams[tris[wid[s]].model];
                const D3 vw = d3(tp.Velocity.x, tp.Velocity.y, tp.Velocity.z);
                lap = dadd(lap, dmul(dsub(vw, v0), (double)P.WallFrictionCoeffieicnt * ww));
            }
            lap = dmul(lap, coef * svisc[s]);
            const D3 g = d3(P.GravityConstant.x, P.GravityConstant.y, P.GravityConstant.z);
            D3 v = dsub(dadd(v0, dmul(dadd(g, lap), dt)), dragv[s]);
            npos[s] = dadd(spos[s], dmul(v, dt));
            nvel[s] = v;
        }
        for (int s = 0; s < n; ++s) { pos[sid[s]] = npos[s]; vel[sid[s]] = nvel[s]; }
    }

    int solve_ppe(OrcStepStats* st) {
        const CParameter& P = cfg.param;
        const double rel = re_lap(), mindl = rel * 1e-3;
        const double reg = re_grad(), mindg = reg * 1e-3;
        const double dt = P.Dt, rho = P.Density;
        const double c = 2.0 * P.Dimension / (cfg.lambda * cfg.n0_lap);
        const double kappa = cfg.compressibility * rho / (dt * dt);
        /* neighbour lists (Laplacian radius) and PND (gradient radius) */
        std::vector<int> cnt(n);
        std::vector<std::vector<std::pair<int, double>>> nb(n);
        std::vector<double> npnd(n);
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < n; ++s) {
            double dens = 0.0;
            for_neighbours(s, rel, [&](int x, double r, const D3&) {
                nb[s].push_back(std::make_pair(x, weight_d(rel, std::max(r, mindl))));
                if (r < reg) dens += weight_d(reg, std::max(r, mindg));
            });
            if (wid[s] >= 0 && wdist[s] >= 0 && wdist[s] <= reg)
                dens += (2 == P.Dimension) ? zeval_d(kZGrad2, wdist[s], l0()) : zeval_d(kZGrad3, wdist[s], l0());
            npnd[s] = dens;
        }
        std::vector<char> inner(n);
        std::vector<double> diag(n, 1.0), rhs(n, 0.0), x(n, 0.0);
        int ninner = 0;
        for (int s = 0; s < n; ++s) {
            inner[s] = npnd[s] > (double)P.FreeSurfaceThreshold * cfg.n0_pnd;
            ninner += inner[s];
        }
#pragma omp parallel for schedule(static)
        for (int s = 0; s < n; ++s) {
            if (!inner[s]) continue;
            double sw = 0.0;
            for (auto& e : nb[s]) sw += e.second;
            diag[s] = c * sw + kappa;
            rhs[s] = cfg.source_relaxation * rho / (dt * dt) * (npnd[s] - cfg.n0_pnd) / cfg.n0_pnd;
            x[s] = spress[s];
        }
        auto spmv = [&](const std::vector<double>& in, std::vector<double>& out) {
#pragma omp parallel for schedule(static)
            for (int s = 0; s < n; ++s) {
                if (!inner[s]) { out[s] = 0.0; continue; }
                double acc = diag[s] * in[s];
                for (auto& e : nb[s])
                    if (inner[e.first]) acc -= c * e.second * in[e.first];
                out[s] = acc;
            }
        };
        std::vector<double> r(n), z(n), p(n), q(n), tmp(n);
        spmv(x, q);
        for (int s = 0; s < n; ++s) r[s] = inner[s] ? rhs[s] - q[s] : 0.0;
        for (int s = 0; s < n; ++s) tmp[s] = rhs[s] * rhs[s];
        const double bnorm = std::sqrt(det_sum(tmp, n));
        const double tol = cfg.cg_rtol * bnorm;
        for (int s = 0; s < n; ++s) tmp[s] = r[s] * r[s];
        double rnorm = std::sqrt(det_sum(tmp, n));
        int it = 0;
        if (bnorm == 0.0) {
            std::fill(x.begin(), x.end(), 0.0);
            rnorm = 0.0;
        } else {
            for (int s = 0; s < n; ++s) { z[s] = r[s] / diag[s]; p[s] = z[s]; tmp[s] = r[s] * z[s]; }
            double rz = det_sum(tmp, n);
            while (rnorm > tol && it < cfg.cg_max_iter) {
                spmv(p, q);
                for (int s = 0; s < n; ++s) tmp[s] = p[s] * q[s];
                const double alpha = rz / det_sum(tmp, n);
                for (int s = 0; s < n; ++s) { x[s] += alpha * p[s]; r[s] -= alpha * q[s]; }
                ++it;
                for (int s = 0; s < n; ++s) tmp[s] = r[s] * r[s];
                rnorm = std::sqrt(det_sum(tmp, n));
                if (rnorm <= tol) break;
                for (int s = 0; s < n; ++s) { z[s] = r[s] / diag[s]; tmp[s] = r[s] * z[s]; }
                const double rzn = det_sum(tmp, n);
                const double beta = rzn / rz;
                rz = rzn;
                for (int s = 0; s < n; ++s) p[s] = z[s] + beta * p[s];
            }
        }
        for (int s = 0; s < n; ++s) spress[s] = inner[s] ? x[s] : 0.0;
        for (int s = 0; s < n; ++s) { press[sid[s]] = spress[s]; pnd[sid[s]] = npnd[s]; }
        l_pnd = npnd; l_diag = diag; l_rhs = rhs; l_sol = spress; l_sid = sid;
        /* the PPE operator of this solve as CSR rows in the solver order: interior rows
         * hold their diagonal and -c w_ij of every interior neighbour; other rows the
         * identity (P = 0) */
        l_rowptr.assign(n + 1, 0);
        l_col.clear();
        l_val.clear();
        for (int s = 0; s < n; ++s) {
            l_col.push_back(s);
            l_val.push_back(inner[s] ? diag[s] : 1.0);
            if (inner[s])
                for (auto& e : nb[s])
                    if (inner[e.first]) {
                        l_col.push_back(e.first);
                        l_val.push_back(-c * e.second);
                    }
            l_rowptr[s + 1] = (int)l_col.size();
        }
        l_cnt.resize(n); l_idsum.resize(n); l_id.resize(n);
        for (int s = 0; s < n; ++s) {
            double acc = 0.0;
            for (auto& e : nb[s]) acc += (double)id[sid[e.first]];
            l_cnt[s] = (int)nb[s].size();
            l_idsum[s] = acc;
            l_id[s] = id[sid[s]];
        }
        if (st) {
            st->cg_iterations = it;
            st->cg_relres = bnorm > 0 ? rnorm / bnorm : 0.0;
            st->b_norm = bnorm;
            st->interior = ninner;
            st->particles = n;
        }
        return (rnorm <= tol || bnorm == 0.0) ? CCT_NOERR : CCT_CALCERR;
    }

    /* Pressure-gradient correction (CalcExplicitPressureGradient_Kernel
     * semantics, FP64, exact square roots). */
    void correct() {
        const CParameter& P = cfg.param;
        const double re = re_grad(), mind = re * 1e-3;
        const double dt = P.Dt, rho = P.Density;
        const double c1 = 2.0 * P.Dimension / cfg.n0_pnd, c2 = rho / (dt * dt), c3 = -dt / rho;
        const double vmax = (double)P.InitialParticleDistance * P.CourantNumber / dt;
        std::vector<D3> npos(n), nvel(n);
#pragma omp parallel for schedule(dynamic, 256)
        for (int s = 0; s < n; ++s) {
            const double pi = spress[s];
            D3 gf = d3(0, 0, 0), gw = d3(0, 0, 0);
            for_neighbours(s, re, [&](int x, double r, const D3& dv) {
                const double rr = std::max(r, mind);
                const double pc = 0.5 * (spress[x] + pi) * weight_d(re, rr);
                gf = dadd(gf, dmul(dv, pc / (rr * rr)));
            });
            gf = dmul(gf, c1);
            if (wid[s] >= 0) {
                const double m = wdist[s];
                if (m > 0 && m <= re) {
                    const double ww = zeval_d(kZGrad3, m, l0());
                    gw = dmul(wdir[s], -(0.5 * c1 * ww * pi / (m * m)));
                }
                const double off = (double)P.InitialParticleDistance * P.OffSet;
                if (m > 0 && m <= off) gw = dadd(gw, dmul(wdir[s], -(c2 * (off - m) / m)));
            }
            const D3 g = dadd(gf, gw);
            D3 v = dadd(svel[s], dmul(g, c3));
            const double a = dlen(v);
            if (a > vmax) v = dmul(v, vmax / a);
            nvel[s] = v;
            npos[s] = dadd(spos[s], dmul(dsub(v, svel[s]), dt));
        }
        for (int s = 0; s < n; ++s) { pos[sid[s]] = npos[s]; vel[sid[s]] = nvel[s]; }
    }

    /* Wall motion: translation (UpdateTrianglePosition_Kernel) and incremental
     * rotation with a linear ramp (RotateTrianglePosition_Kernel), FP64 with an
     * exactly normalised axis. */
    void move_walls(int step) {
        const double dt = cfg.param.Dt;
        for (auto& T : tris) {
            const CTriangleParameters& tp = tparams[T.model];
            for (int q = 0; q < 3; ++q)
                T.v[q] = dadd(T.v[q], d3(tp.Velocity.x * dt, tp.Velocity.y * dt, tp.Velocity.z * dt));
            if (!tp.RotatingOrNot) continue;
            const double tpass = dt * step;
            if (tpass < tp.RotationStartTime || tp.AngleOfRotationInDegree == 0) continue;
            double ang;
            if (tpass < tp.TimeToReachRPM) {
                const int req = (int)((tp.TimeToReachRPM - tp.RotationStartTime) / dt);
                ang = (tp.AngleOfRotationInDegree / (double)(req + 1)) * (step - tp.RotationStartTime / dt);
            } else {
                ang = tp.AngleOfRotationInDegree;
            }
            if (ang == 0) continue;
            const D3 c = d3(tp.CenterOfRotation.x, tp.CenterOfRotation.y, tp.CenterOfRotation.z);
            D3 ax = dsub(d3(tp.SecondPointOfRotation.x, tp.SecondPointOfRotation.y, tp.SecondPointOfRotation.z), c);
            const double al = dlen(ax);
            if (!(al > 0)) continue;
            ax = dmul(ax, 1.0 / al);
            const double th = ang * 3.14159265358979323846 / 180.0;
            const double ct = std::cos(th), st = std::sin(th);
            for (int q = 0; q < 3; ++q) {
                /* Rodrigues: v' = v cos + (k x v) sin + k (k.v)(1 - cos), about c */
                const D3 v = dsub(T.v[q], c);
                const D3 kxv = d3(ax.y * v.z - ax.z * v.y, ax.z * v.x - ax.x * v.z, ax.x * v.y - ax.y * v.x);
                const double kv = ddot(ax, v);
                T.v[q] = dadd(c, dadd(dadd(dmul(v, ct), dmul(kxv, st)), dmul(ax, kv * (1.0 - ct))));
            }
            const D3 e1 = dsub(T.v[1], T.v[0]), e2 = dsub(T.v[2], T.v[0]);
            D3 nn = d3(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x);
            const double nl = dlen(nn);
            if (nl > 0) T.nrm = dmul(nn, 1.0 / nl);
        }
    }
};

extern "C" {

OrcSim* orc_sim_create(const OrcSimConfig* cfg, int max_particles) {
    OrcSim* s = new OrcSim();
    s->cfg = *cfg;
    s->maxn = max_particles;
    s->cells = cfg->box.m_GridSize.x * cfg->box.m_GridSize.y * cfg->box.m_GridSize.z;
#ifdef _OPENMP
    if (cfg->threads > 0) omp_set_num_threads(cfg->threads);
#endif
    return s;
}

void orc_sim_destroy(OrcSim* s) { delete s; }

int orc_sim_set_particles(OrcSim* s, int n, const double* pos, const double* vel, const double* pressure,
                          const double* kin_visc, const int* type) {
    if (n < 0 || n > s->maxn) return CCT_PARAMERR;
    s->n = n;
    s->pos.resize(s->maxn); s->vel.resize(s->maxn); s->press.assign(s->maxn, 0.0); s->pnd.assign(s->maxn, 0.0);
    s->visc.resize(s->maxn); s->type.resize(s->maxn); s->id.resize(s->maxn);
    for (int i = 0; i < n; ++i) {
        s->pos[i] = d3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        s->vel[i] = d3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        s->press[i] = pressure ? pressure[i] : 0.0;
        s->visc[i] = kin_visc[i];
        s->type[i] = type ? type[i] : 0;
        s->id[i] = i;
    }
    return CCT_NOERR;
}

int orc_sim_set_triangles(OrcSim* s, int t, const double* v, const int* model, int models,
                          const CTriangleParameters* params) {
    s->tris.resize(t);
    for (int i = 0; i < t; ++i) {
        SimTri& T = s->tris[i];
        for (int q = 0; q < 3; ++q) T.v[q] = d3(v[9 * i + 3 * q], v[9 * i + 3 * q + 1], v[9 * i + 3 * q + 2]);
        T.model = model[i];
        const D3 e1 = dsub(T.v[1], T.v[0]), e2 = dsub(T.v[2], T.v[0]);
        D3 nn = d3(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x);
        const double nl = dlen(nn);
        T.nrm = nl > 0 ? dmul(nn, 1.0 / nl) : d3(0, 0, 0);
    }
    s->tparams.assign(params, params + models);
    return CCT_NOERR;
}

int orc_sim_set_drag(OrcSim* s, int count, const DragParameter* params) {
    s->drag.assign(params, params + count);
    return CCT_NOERR;
}

/* One semi-implicit step in the reference's schedule
 * (MultiGPUHandler.cpp:1389-1559 with the explicit pressure replaced by the PPE):
 * compact, grid, walls, drag, predictor, compact, grid, walls, PND + PPE + CG,
 * pressure-gradient correction, wall motion. */
int orc_sim_step(OrcSim* s, int step, OrcStepStats* st) {
    s->compact();
    s->build_grid();
    s->bin_triangles();
    s->wall_distance();
    s->apply_drag();
    s->predictor();
    s->compact();
    s->build_grid();
    s->wall_distance();
    int rc = s->solve_ppe(st);
    s->correct();
    s->move_walls(step);
    return rc;
}

int orc_sim_get(OrcSim* s, int* n, double* pos, double* vel, double* pressure, double* pnd) {
    *n = s->n;
    for (int i = 0; i < s->n; ++i) {
        if (pos) { pos[3 * i] = s->pos[i].x; pos[3 * i + 1] = s->pos[i].y; pos[3 * i + 2] = s->pos[i].z; }
        if (vel) { vel[3 * i] = s->vel[i].x; vel[3 * i + 1] = s->vel[i].y; vel[3 * i + 2] = s->vel[i].z; }
        if (pressure) pressure[i] = s->press[i];
        if (pnd) pnd[i] = s->pnd[i];
    }
    return CCT_NOERR;
}

int orc_sim_get_triangles(OrcSim* s, double* v) {
    for (size_t i = 0; i < s->tris.size(); ++i)
        for (int q = 0; q < 3; ++q) {
            v[9 * i + 3 * q] = s->tris[i].v[q].x;
            v[9 * i + 3 * q + 1] = s->tris[i].v[q].y;
            v[9 * i + 3 * q + 2] = s->tris[i].v[q].z;
        }
    return CCT_NOERR;
}

int orc_sim_get_ids(OrcSim* s, int* ids) {
    for (int i = 0; i < s->n; ++i) ids[i] = s->id[i];
    return s->n;
}

/* Laplacian neighbour count and sum of neighbour particle ids of the last PPE, and
 * the particle id, per sorted position. */
int orc_sim_last_nbr(OrcSim* s, int* cnt, double* idsum, int* pid) {
    const size_t n = s->l_cnt.size();
    for (size_t i = 0; i < n; ++i) {
        cnt[i] = s->l_cnt[i];
        idsum[i] = s->l_idsum[i];
        pid[i] = s->l_id[i];
    }
    return (int)n;
}

/* The last solve's PPE operator (CSR, solver order; rows of particles outside the PPE
 * are identity rows): returns the entry count; arrays may be NULL. */
long long orc_sim_last_matrix(OrcSim* s, int* rowptr, int* col, double* val) {
    if (rowptr) std::copy(s->l_rowptr.begin(), s->l_rowptr.end(), rowptr);
    if (col) std::copy(s->l_col.begin(), s->l_col.end(), col);
    if (val) std::copy(s->l_val.begin(), s->l_val.end(), val);
    return (long long)s->l_col.size();
}

int orc_sim_last_ppe(OrcSim* s, double* pnd, double* diag, double* rhs, double* sol, int* sorted_id) {
    const size_t n = s->l_sid.size();
    for (size_t i = 0; i < n; ++i) {
        if (pnd) pnd[i] = s->l_pnd[i];
        if (diag) diag[i] = s->l_diag[i];
        if (rhs) rhs[i] = s->l_rhs[i];
        if (sol) sol[i] = s->l_sol[i];
        if (sorted_id) sorted_id[i] = s->l_sid[i];
    }
    return (int)n;
}

}  // extern "C"
