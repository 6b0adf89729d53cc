// io.cpp - the reference's input formats (include/mps_io.h), host C++ without Boost.
#include <algorithm>
#include <cfloat>
#include <charconv>
#include <cstdio>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mps_io.h"

namespace {

struct Tokens {
    std::vector<std::string> t;
    size_t i = 0;
    bool more() const { return i < t.size(); }
    template <class T>
    bool get(T& v) {
        if (i >= t.size()) return false;
        std::istringstream ss(t[i++]);
        ss >> v;
        return !ss.fail();
    }
    bool on() { return i < t.size() && t[i++] == "ON"; }
};

// float helper: fast inverse square root of the reference (sqrt_stl, STLSerializer.h:23-29)
float sqrt_stl(float x) {
    float xhalf = 0.5f * x;
    int32_t i;
    std::memcpy(&i, &x, 4);
    i = 0x5f3759df - (i >> 1);
    std::memcpy(&x, &i, 4);
    x = x * (1.5f - xhalf * x * x);
    return 1.0f / x;
}

// CalcTriangleNormal (IO.cpp:449-467): the normal keeps its file value when the
// cross product vanishes
void triangle_normal(CTriangle& T) {
    const Scalar3 a = {T.Vertex[1].x - T.Vertex[0].x, T.Vertex[1].y - T.Vertex[0].y, T.Vertex[1].z - T.Vertex[0].z};
    const Scalar3 b = {T.Vertex[2].x - T.Vertex[0].x, T.Vertex[2].y - T.Vertex[0].y, T.Vertex[2].z - T.Vertex[0].z};
    Scalar3 n;
    n.x = a.y * b.z - b.y * a.z;
    n.y = a.z * b.x - b.z * a.x;
    n.z = a.x * b.y - b.x * a.y;
    const float ab = sqrt_stl(n.x * n.x + n.y * n.y + n.z * n.z);
    if (ab != 0.0f) {
        T.Normal.x = n.x / ab;
        T.Normal.y = n.y / ab;
        T.Normal.z = n.z / ab;
    }
}

}  // namespace

extern "C" {

CCTStatusType mps_read_parameter_file(const char* path, CParameter* P) {
    if (!path || !P) return CCT_PARAMERR;
    std::ifstream f(path);
    if (!f.is_open()) return CCT_FILEERR;
    Tokens tk;
    std::string w;
    while (f >> w) tk.t.push_back(w);
    std::memset(P, 0, sizeof(*P));
    bool ok = true;
    ok &= tk.get(P->Dimension);
    ok &= tk.get(P->GravityConstant.x) && tk.get(P->GravityConstant.y) && tk.get(P->GravityConstant.z);
    ok &= tk.get(P->Density) && tk.get(P->ConstantParticleDensity) && tk.get(P->SurfaceTensionCoefficient);
    ok &= tk.get(P->InitialParticleDistance) && tk.get(P->FreeSurfaceThreshold);
    ok &= tk.get(P->GradientInfluenceRadiusCoefficient) && tk.get(P->LaplacianInfluenceRadiusCoefficient);
    ok &= tk.get(P->TemperatureInfluenceRadiusCoefficient);
    ok &= tk.get(P->FruidInitializeialTemperature) && tk.get(P->WallInitializeialTemperature);
    ok &= tk.get(P->FruidThermalResistance) && tk.get(P->WallThermalResistance);
    ok &= tk.get(P->FruidThermalConductivity) && tk.get(P->WallThermalConductivity);
    ok &= tk.get(P->FruidSpecificHeat) && tk.get(P->FruidDensity);
    ok &= tk.get(P->Dt) && tk.get(P->AnalysisStep) && tk.get(P->ThermalStep);
    ok &= tk.get(P->NegativeCalculationStep) && tk.get(P->OutputStep) && tk.get(P->LambdaID);
    ok &= tk.get(P->SORJacobianRelaxationCoefficient) && tk.get(P->SORLoopMax) && tk.get(P->SORConvergenceConstant);
    if (!ok) return CCT_FILEERR;
    P->bUpdateTemperature = tk.on();
    if (tk.more()) {
        tk.get(P->ViscosityUpdateParameterA);
        tk.get(P->ViscosityUpdateParameterB);
        tk.get(P->MaxWallTemperature);
        tk.get(P->MinWallTemperature);
    }
    if (tk.more()) tk.get(P->CourantNumber);
    if (tk.more()) {
        tk.get(P->InitialTimeForZeroAngle);
        tk.get(P->FinalTimeToReachAngle);
        tk.get(P->CellSize.z);
    }
    if (tk.more()) {
        tk.get(P->MvVelocity.x);
        tk.get(P->MvVelocity.y);
        tk.get(P->MvVelocity.z);
    }
    if (tk.more()) tk.get(P->OffSet);
    if (tk.more()) {
        tk.get(P->ParticleGenerationStep);
        tk.get(P->TotalGenerationStep);
    }
    if (tk.more()) tk.get(P->Alpha);
    if (tk.more()) tk.get(P->AlphaLightWeight);
    if (tk.more()) {
        P->bExplicitCollisonCheck = tk.on();
        P->bExplicitCollisionOut = tk.on();
        P->bImplicitCollisonCheck = tk.on();
    }
    if (tk.more()) {
        tk.get(P->CollisionCheckCoefficient);
        tk.get(P->MinDistanceCoefficient);
    }
    P->Time1 = P->Dt;
    if (tk.more()) {
        P->bFreeSurfacePressureUpdate = tk.on();
        tk.get(P->BasePressure);
        tk.get(P->MaxPressure);
        tk.get(P->Time1);
        tk.get(P->TriggerStep);
        tk.get(P->EndStep);
        tk.get(P->AnalysisArea);
    }
    if (tk.more()) P->bExplicitOut = tk.on();
    if (tk.more()) tk.get(P->WallFrictionCoeffieicnt);
    if (tk.more()) tk.get(P->DragCoefficient);
    if (tk.more()) P->bTwoPhase = tk.on();
    P->StopWallStep = INT_MAX;
    if (tk.more()) tk.get(P->StopWallStep);
    if (tk.more()) tk.get(P->Tolerance);
    if (tk.more()) tk.get(P->ImplicitSurfaceThreshold);
    if (tk.more()) P->bCGSolver = tk.on();
    if (tk.more()) P->bUpdateInnerPressure = tk.on();
    if (tk.more()) tk.get(P->SurfaceInfluenceRadiusCoefficient);
    if (tk.more()) tk.get(P->SurfaceThreshold);
    if (tk.more()) tk.get(P->GradientForce);
    if (tk.more()) tk.get(P->StartStep);
    if (tk.more()) tk.get(P->InitialForce);
    if (tk.more()) tk.get(P->VelocityThreshold);
    if (tk.more()) P->bExplicitPressure = tk.on();
    if (tk.more()) tk.get(P->SonicVelocity);
    if (tk.more()) tk.get(P->ArtificialPressure);
    if (tk.more()) tk.get(P->r_coeff);
    if (tk.more()) P->bImplicitVelocity = tk.on();
    if (tk.more()) P->bNJPCGSolver = tk.on();
    P->PressureMax = FLT_MAX;
    if (tk.more()) tk.get(P->PressureMax);
    P->RLimitCoefficient = FLT_MAX;
    if (tk.more()) tk.get(P->RLimitCoefficient);
    P->SmagorinskyConstant = 0.1f;
    P->FilterWidth = P->InitialParticleDistance;
    if (tk.more()) {
        P->bTurbulance = tk.on();
        tk.get(P->SmagorinskyConstant);
        tk.get(P->FilterWidth);
        tk.get(P->TurbulanViscosityRatio);
        tk.get(P->Cnue);
        tk.get(P->Cepsilon);
        tk.get(P->TurbulanceIntensity);
    }
    P->ConstantCheckStep = -1;
    if (tk.more()) P->bNegativePressure = tk.on();
    if (tk.more()) tk.get(P->ConstantCheckStep);
    P->MaxNeighborhoodNum = P->Dimension == 2 ? 81 : 729;
    P->LambdaValue = mps_lambda_table(P->InitialParticleDistance);
    return CCT_NOERR;
}

CCTStatusType mps_read_particle_file(const char* path, int* count, CParticle* out, int capacity) {
    if (!path || !count) return CCT_PARAMERR;
    std::ifstream f(path);
    if (!f.is_open()) return CCT_FILEERR;
    int n = 0;
    for (;;) {
        CParticle p;
        std::memset(&p, 0, sizeof(p));
        int type = 0;
        f >> p.Position.x >> p.Position.y >> p.Position.z >> p.Velocity.x >> p.Velocity.y >> p.Velocity.z >>
            p.Pressure >> p.Density >> p.Temperature >> p.KineticViscosity >> p.SolidPhaseRate >> type;
        if (f.fail()) break;
        p.Type = type == 1 ? TYPE_HEAVY_WEIGHT_FREE_SURFACE : (type == 2 ? TYPE_LIGHT_WEIGHT : TYPE_HEAVY_WEIGHT);
        p.ID = n;
        if (out) {
            if (n >= capacity) return CCT_PARAMERR;
            out[n] = p;
        }
        ++n;
    }
    *count = n;
    return CCT_NOERR;
}

}  // extern "C"

namespace mps_io {
// The triangles of one STL file with the file's normals (CSTLSerializer::Load,
// STLSerializer.cpp:225-357): ASCII when the first token is "solid", else binary.
CCTStatusType stl_load_raw(const char* path, std::vector<CTriangle>& tris) {
    std::ifstream probe(path);
    if (!probe.is_open()) return CCT_FILEERR;
    std::string first;
    probe >> first;
    probe.close();
    if (first == "solid") {
        std::ifstream f(path);
        std::string w;
        CTriangle T;
        std::memset(&T, 0, sizeof(T));
        int v = 0;
        bool in_facet = false;
        while (f >> w) {
            if (w == "facet") {
                std::memset(&T, 0, sizeof(T));
                std::string nrm;
                f >> nrm >> T.Normal.x >> T.Normal.y >> T.Normal.z;
                v = 0;
                in_facet = true;
            } else if (w == "vertex" && in_facet) {
                if (v < 3) f >> T.Vertex[v].x >> T.Vertex[v].y >> T.Vertex[v].z;
                ++v;
            } else if (w == "endfacet" && in_facet) {
                if (v != 3) return CCT_FILEERR;
                tris.push_back(T);
                in_facet = false;
            }
            if (f.fail()) return CCT_FILEERR;
        }
    } else {
        std::ifstream f(path, std::ios::binary);
        char header[80];
        f.read(header, 80);
        uint32_t nt = 0;
        f.read((char*)&nt, 4);
        if (!f) return CCT_FILEERR;
        for (uint32_t i = 0; i < nt; ++i) {
            float rec[12];
            char attr[2];
            f.read((char*)rec, sizeof(rec));
            f.read(attr, 2);
            if (!f) return CCT_FILEERR;
            CTriangle T;
            T.Normal = {rec[0], rec[1], rec[2]};
            for (int q = 0; q < 3; ++q) T.Vertex[q] = {rec[3 + 3 * q], rec[4 + 3 * q], rec[5 + 3 * q]};
            tris.push_back(T);
        }
    }
    return CCT_NOERR;
}
}  // namespace mps_io

extern "C" {

CCTStatusType mps_read_stl(const char* path, int model_id, const Scalar3* offset, int* count, CTriangle* out,
                           int capacity) {
    if (!path || !count) return CCT_PARAMERR;
    std::vector<CTriangle> tris;
    const CCTStatusType rc = mps_io::stl_load_raw(path, tris);
    if (rc != CCT_NOERR) return rc;
    for (auto& T : tris) {
        T.ModelIDNumber = model_id;
        if (offset)
            for (int q = 0; q < 3; ++q) {
                T.Vertex[q].x += offset->x;
                T.Vertex[q].y += offset->y;
                T.Vertex[q].z += offset->z;
            }
        triangle_normal(T);
    }
    *count = (int)tris.size();
    if (out) {
        if ((int)tris.size() > capacity) return CCT_PARAMERR;
        std::memcpy(out, tris.data(), sizeof(CTriangle) * tris.size());
    }
    return CCT_NOERR;
}

// CalculateLambdaValueLocal (MultiGPUHandler.cpp:757-921): "lo < l0 <= hi" evaluates
// as (lo < l0) <= hi, so the first row whose lower bound is not below l0 (l0 promoted
// to double), or whose upper bound is >= 1, is taken; lambda = a*l0 + b in float.
float mps_lambda_table(float l0) {
    struct Row { double lo, hi, a, b; };
    static const Row rows[] = {
        {0, 0.0001, 5.02608E-06, 3.82946E-10},   {0.0001, 0.0005, 0.000124918, 1.81984E-08},
        {0.0005, 0.001, 0.0017886, -4.84707E-07}, {0.001, 0.002, 0.00373277, -2.15486E-06},
        {0.002, 0.003, 0.0066746, -6.72384E-06},  {0.003, 0.004, 0.0107452, -1.76386E-05},
        {0.004, 0.005, 0.0141993, -3.08052E-05},  {0.005, 0.006, 0.0164975, -4.14937E-05},
        {0.006, 0.007, 0.0181782, -4.95251E-05},  {0.007, 0.008, 0.0205885, -6.28759E-05},
        {0.008, 0.009, 0.0222761, -7.17244E-05},  {0.009, 0.01, 0.0231972, -7.34117E-05},
        {0.01, 0.02, 0.0369119, -0.000210081},    {0.02, 0.03, 0.0667457, -0.000672376},
        {0.03, 0.04, 0.106105, -0.00171939},      {0.04, 0.05, 0.141998, -0.00308074},
        {0.05, 0.06, 0.164981, -0.00414971},      {0.05, 0.06, 0.164981, -0.00414971},
        {0.06, 0.07, 0.178483, -0.00474469},      {0.07, 0.08, 0.197539, -0.00567825},
        {0.08, 0.09, 0.208407, -0.00598107},      {0.09, 0.1, 0.211437, -0.00543137},
        {0.01, 0.5, 0.369118, -0.021008},         {0.5, 1, 1.78861, -0.48471},
        {1, 10, 0.423015, 4.1213},                {10, 1000, 0.0138964, 745.762}};
    float a = 0.0f, b = 0.0f;
    for (const Row& r : rows) {
        const double lt = (r.lo < (double)l0) ? 1.0 : 0.0;
        if (lt <= r.hi) {
            a = (float)r.a;
            b = (float)r.b;
            break;
        }
    }
    return a * l0 + b;
}

CCTStatusType mps_grid_box(const CBox* zone, const CParameter* P, CGridBox* B) {
    if (!zone || !P || !B) return CCT_PARAMERR;
    std::memset(B, 0, sizeof(*B));
    const float mx = std::max(P->LaplacianInfluenceRadiusCoefficient, P->GradientInfluenceRadiusCoefficient);
    const float r = P->InitialParticleDistance * mx;
    if (!(r > 0.0f)) return CCT_PARAMERR;
    const Scalar3 lo = zone->m_MinBound, hi = zone->m_MaxBound;
    B->m_ComputeZone = *zone;
    B->m_ParentZone = *zone;
    B->m_PressureZone.m_MinBound = {lo.x - r, lo.y - r, lo.z - r};
    B->m_PressureZone.m_MaxBound = {hi.x + r, hi.y + r, hi.z + r};
    B->m_BufferedZone.m_MinBound = {lo.x - 2 * r, lo.y - 2 * r, lo.z - 2 * r};
    B->m_BufferedZone.m_MaxBound = {hi.x + 2 * r, hi.y + 2 * r, hi.z + 2 * r};
    B->m_CellSize = r;
    B->m_GridSize.x = (int)std::ceil((hi.x - lo.x) / r + 4);
    B->m_GridSize.y = (int)std::ceil((hi.y - lo.y) / r + 4);
    B->m_GridSize.z = (int)std::ceil((hi.z - lo.z) / r + 4);
    return CCT_NOERR;
}

CCTStatusType mps_lattice_constants(double re, double l0, int dim, double* n0, double* lambda) {
    if (!(re > 0) || !(l0 > 0) || (dim != 2 && dim != 3) || !n0 || !lambda) return CCT_PARAMERR;
    const int m = (int)std::ceil(re) + 1;
    double sw = 0.0, sr2w = 0.0;
    for (int i = -m; i <= m; ++i)
        for (int j = -m; j <= m; ++j)
            for (int k = (dim == 3 ? -m : 0); k <= (dim == 3 ? m : 0); ++k) {
                const double r = std::sqrt((double)(i * i + j * j + k * k));
                if (r > 0 && r < re) {
                    const double w = re / r - 1.0;
                    sw += w;
                    sr2w += r * r * w;
                }
            }
    *n0 = sw;
    *lambda = sr2w / sw * l0 * l0;
    return CCT_NOERR;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Output frames: IO::Save / SaveAscii / SaveBinary, radix/SPVSOLVER/MultiGPUSolver/
// IO.cpp:649-756.  ASCII: the count, one line per particle "x y z vx vy vz P n T nu
// solidRate type" (std::ostream defaults: %g with 6 significant digits, the type as an
// integer), the time, the model count and "x\ty\tz\tangle" per model.  Binary: int32
// count, per particle 3 + 3 + 5 floats and an int32 type (48 bytes), the float time,
// int32 model count and 3 + 1 floats per model.  Built in one host buffer, one write.
// ---------------------------------------------------------------------------
static_assert(sizeof(ParticleType) == 4 && sizeof(Scalar3) == 12, "ParticleType is an int32, Scalar3 3 floats");

namespace {

// %g with 6 significant digits, as std::ostream's defaults and printf("%g") print a
// float; std::to_chars in chars_format::general with a precision is specified to give
// printf's %.*g text and is much faster than snprintf
void put_g(std::string& b, double v) {
    char t[32];
    const std::to_chars_result r = std::to_chars(t, t + sizeof t, v, std::chars_format::general, 6);
    b.append(t, (size_t)(r.ptr - t));
}
void put_i(std::string& b, long long v) {
    char t[24];
    const int k = std::snprintf(t, sizeof t, "%lld", v);
    b.append(t, (size_t)(k > 0 ? k : 0));
}

}  // namespace

namespace {

struct FrameRecord {   // one binary record of IO::SaveBinary (IO.cpp:729-739)
    Scalar3 pos, vel;
    Scalar pressure, density, temperature, viscosity, solid;
    Integer type;
};
static_assert(sizeof(FrameRecord) == 48, "binary frame records are 48 bytes");

// the ASCII lines of particles [a, b)
void ascii_lines(std::string& b, int a, int e, const Scalar3* pos, const Scalar3* vel, const Scalar* pressure,
                 const Scalar* density, const Scalar* temperature, const Scalar* viscosity, const Scalar* solid_rate,
                 const ParticleType* type) {
    b.reserve((size_t)(e - a) * 96);
    for (int i = a; i < e; ++i) {
        put_g(b, pos[i].x); b += ' ';
        put_g(b, pos[i].y); b += ' ';
        put_g(b, pos[i].z); b += ' ';
        put_g(b, vel[i].x); b += ' ';
        put_g(b, vel[i].y); b += ' ';
        put_g(b, vel[i].z); b += ' ';
        put_g(b, pressure[i]); b += ' ';
        put_g(b, density[i]); b += ' ';
        put_g(b, temperature ? temperature[i] : 0.0f); b += ' ';
        put_g(b, viscosity[i]); b += ' ';
        put_g(b, solid_rate ? solid_rate[i] : 0.0f); b += ' ';
        put_i(b, (long long)type[i]);
        b += '\n';
    }
}

}  // namespace

extern "C" CCTStatusType mps_write_frame(const char* path, int ascii, int n, const Scalar3* pos, const Scalar3* vel,
                                         const Scalar* pressure, const Scalar* density, const Scalar* temperature,
                                         const Scalar* viscosity, const Scalar* solid_rate, const ParticleType* type,
                                         Scalar time, int models, const Scalar3* model_pos,
                                         const Scalar* model_angle) {
    if (!path || n < 0 || models < 0) return CCT_PARAMERR;
    if (n > 0 && (!pos || !vel || !pressure || !density || !viscosity || !type)) return CCT_PARAMERR;
    if (models > 0 && (!model_pos || !model_angle)) return CCT_PARAMERR;
    FILE* f = std::fopen(path, ascii ? "w" : "wb");
    if (!f) return CCT_FILEERR;
    bool ok = true;
    auto put = [&](const void* p, size_t bytes) { ok = ok && std::fwrite(p, 1, bytes, f) == bytes; };
    if (ascii) {
        std::string head;
        put_i(head, n);
        head += '\n';
        put(head.data(), head.size());
        // particle lines formatted by up to 16 host threads in contiguous chunks, written
        // in order (the bytes do not depend on the split)
        const int nt = n < 4096 ? 1 : (int)std::min<unsigned>(16u, std::max(1u, std::thread::hardware_concurrency()));
        std::vector<std::string> part((size_t)nt);
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t) {
            const int a = (int)((long long)n * t / nt), e = (int)((long long)n * (t + 1) / nt);
            auto job = [&, t, a, e]() {
                ascii_lines(part[(size_t)t], a, e, pos, vel, pressure, density, temperature, viscosity, solid_rate,
                            type);
            };
            if (t + 1 < nt) th.emplace_back(job);
            else job();
        }
        for (std::thread& x : th) x.join();
        for (const std::string& p : part) put(p.data(), p.size());
        std::string tail;
        put_g(tail, time);
        tail += '\n';
        put_i(tail, models);
        tail += '\n';
        for (int m = 0; m < models; ++m) {
            put_g(tail, model_pos[m].x); tail += '\t';
            put_g(tail, model_pos[m].y); tail += '\t';
            put_g(tail, model_pos[m].z); tail += '\t';
            put_g(tail, model_angle[m]);
            tail += '\n';
        }
        put(tail.data(), tail.size());
    } else {
        const Integer cnt = n;
        put(&cnt, sizeof cnt);
        constexpr int kChunk = 16384;   // records per write (768 KB)
        std::vector<FrameRecord> rec((size_t)std::min(n, kChunk));
        for (int a = 0; a < n && ok; a += kChunk) {
            const int e = std::min(n, a + kChunk);
            for (int i = a; i < e; ++i) {
                FrameRecord& r = rec[(size_t)(i - a)];
                r.pos = pos[i];
                r.vel = vel[i];
                r.pressure = pressure[i];
                r.density = density[i];
                r.temperature = temperature ? temperature[i] : 0.0f;
                r.viscosity = viscosity[i];
                r.solid = solid_rate ? solid_rate[i] : 0.0f;
                r.type = (Integer)type[i];
            }
            put(rec.data(), sizeof(FrameRecord) * (size_t)(e - a));
        }
        put(&time, sizeof time);
        const Integer mc = models;
        put(&mc, sizeof mc);
        for (int m = 0; m < models; ++m) {
            put(&model_pos[m], sizeof(Scalar3));
            put(&model_angle[m], sizeof(Scalar));
        }
    }
    const int c = std::fclose(f);
    return (ok && c == 0) ? CCT_NOERR : CCT_FILEERR;
}

// ---------------------------------------------------------------------------
// dt schedule: DtFrame::Load (DtFrame.cpp:11-35) and CheckAndUpdateDt
// (MultiGPUHandler.cpp:1256-1275)
// ---------------------------------------------------------------------------
extern "C" CCTStatusType mps_read_dt_file(const char* path, int* count, MpsDtRow* rows, int capacity) {
    if (!path || !count) return CCT_PARAMERR;
    std::ifstream f(path);
    if (!f.is_open()) return CCT_FILEERR;
    int k = 0;
    while (f.is_open() && f.good()) {
        Integer step = 0;
        Scalar dt = 0, cr = 0, inflow = 0, out = 0;
        f >> step;
        f >> dt;
        f >> cr;
        f >> inflow;
        f >> out;
        if (f.good()) {
            if (rows) {
                if (k >= capacity) return CCT_PARAMERR;
                rows[k] = MpsDtRow{step, dt, cr, inflow, out};
            }
            ++k;
        }
    }
    *count = k;
    return CCT_NOERR;
}

extern "C" CCTStatusType mps_dt_schedule_next(const MpsDtRow* rows, int count, int* next, int current_step,
                                              CParameter* param, int* applied) {
    if (!next || !param || (count > 0 && !rows)) return CCT_PARAMERR;
    if (applied) *applied = 0;
    const int k = *next;
    if (k >= 0 && k < count && current_step >= rows[k].step) {
        param->Dt = rows[k].dt;
        param->CourantNumber = rows[k].courant;
        param->ParticleGenerationStep = rows[k].inflow_step;
        param->OutputStep = static_cast<Integer>(rows[k].output_step);
        *next = k + 1;
        if (applied) *applied = 1;
    }
    return CCT_NOERR;
}
