// config_io.cpp - the reference's run configuration file and drag file (include/mps_io.h),
// host C++ without Boost.
//
// CConfiguration::ReadConfigurationFileWithDrag (Configuration.cpp:21-452) reads the file
// line by line and each line's fields with a std::stringstream; the same stream rules
// hold here (std::istringstream), so fields parse, fail and keep their defaults as
// they do there.  IO::Load(drag file) (IO.cpp:524-648) reads a whitespace token stream.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mps_io.h"

namespace mps_io {
CCTStatusType stl_load_raw(const char* path, std::vector<CTriangle>& tris);
}

namespace {

// one line as std::getline gives it in text mode on Windows: the LF removed, and the CR
// of a CRLF pair with it
bool get_line(std::istream& in, std::string& line) {
    if (!std::getline(in, line)) {
        line.clear();
        return false;
    }
    if (!line.empty() && line.back() == '\r') line.pop_back();
    return true;
}

std::string upper(std::string s) {
    for (char& c : s) c = (char)std::toupper((unsigned char)c);
    return s;
}

bool copy_str(char* dst, const std::string& s) {
    if (s.size() >= MPS_PATH_MAX) return false;
    std::memcpy(dst, s.c_str(), s.size() + 1);
    return true;
}

// boost::lexical_cast<float>: the whole token must be a number
bool whole_float(const std::string& tok, float& v) {
    if (tok.empty() || std::isspace((unsigned char)tok[0])) return false;
    errno = 0;
    char* end = nullptr;
    const float f = std::strtof(tok.c_str(), &end);
    if (end != tok.c_str() + tok.size() || errno == ERANGE) return false;
    v = f;
    return true;
}

// a bool field read as an integer (noboolalpha): 0 / 1, anything else fails
void rd_bool(std::istringstream& s, int& v) {
    bool b = v != 0;
    s >> b;
    v = b ? 1 : 0;
}
void rd3(std::istringstream& s, Scalar3& v) {
    s >> v.x;
    s >> v.y;
    s >> v.z;
}

// the default model record of a wall line (fields a short line lacks keep these)
MpsConfigModel wall_defaults() {
    MpsConfigModel m;
    std::memset(&m, 0, sizeof(m));
    m.drag_id = -1;
    return m;
}

// a drag line (Configuration.cpp:86-274); `s` is past the mode token
void drag_line(std::istringstream& s, const std::string& mode, int drag_id, MpsConfigModel& m) {
    std::memset(&m.drag, 0, sizeof(m.drag));
    DragParameter& d = m.drag;
    m.is_drag = 1;
    m.drag_id = drag_id;
    d.DragID = drag_id;
    std::string in_tok, out_tok;
    s >> in_tok;
    s >> out_tok;
    in_tok = upper(in_tok);
    out_tok = upper(out_tok);
    s >> d.CoefficientofInflueneRegion;
    if (mode == "D" || mode == "DE") {
        d.DragToken = 'E';
        if (in_tok == "V") {
            d.InputVelocityToken1 = d.OutputVelocityToken2 = 'V';
            s >> d.VelocityIndex;
            s >> d.VelocityExponential;
            s >> d.VelocityDragPermiabilityConstant;
        } else if (in_tok == "T") {
            d.InputVelocityToken1 = d.OutputVelocityToken2 = 'T';
            s >> d.TempIndex;
            s >> d.TempExponential;
            s >> d.TempDragPermiabilityConstant;
        } else {
            // the reference's `inputToken == "VT" || "TV"` is always true: any other
            // token takes the velocity-and-temperature branch
            d.InputVelocityToken1 = d.OutputVelocityToken2 = 'B';
            s >> d.VelocityIndex;
            s >> d.VelocityExponential;
            s >> d.VelocityDragPermiabilityConstant;
            s >> d.TempIndex;
            s >> d.TempExponential;
            s >> d.TempDragPermiabilityConstant;
        }
    }
    if (mode == "DF") {
        d.DragToken = 'F';
        if (in_tok == "V") {
            d.InputVelocityToken1 = d.OutputVelocityToken2 = 'V';
            s >> d.VelocityMagnitueFactor;
        }
    } else if (mode == "DC") {
        d.InputVelocityToken1 = d.OutputVelocityToken2 = 'V';
        d.DragToken = 'C';
        s >> d.ConstantVx;
        s >> d.ConstantVy;
        s >> d.ConstantVz;
    }
    // the per-model values of a drag model (Configuration.cpp:219-271)
    m.temperature = 533.0f;
}

// a wall line after its file name; `first` is the velocity x token
bool wall_line(std::istringstream& s, const std::string& first, MpsConfigModel& m) {
    if (!whole_float(first, m.velocity.x)) return false;
    s >> m.velocity.y;
    s >> m.velocity.z;
    s >> m.temperature;
    rd3(s, m.position);
    rd_bool(s, m.linear_movable);
    s >> m.reset_interval;
    rd_bool(s, m.rotating);
    s >> m.rpm;
    s >> m.rotation_start;
    s >> m.time_to_reach_rpm;
    rd3(s, m.center_of_rotation);
    rd3(s, m.second_point_of_rotation);
    s >> m.wall_friction;
    s >> m.wall_thermal_resistivity;
    s >> m.wall_thermal_conductivity;
    rd_bool(s, m.negative_pressure_check);
    s >> m.influence_region;
    rd3(s, m.direction);
    s >> m.pressure_gas;
    return true;
}

std::string join_path(const std::string& dir, const std::string& name) {
    if (dir.empty()) return name;
    std::string p = dir;
    const char last = p.back();
    if (last != '/' && last != '\\') p.push_back('\\');
    return p + name;
}

}  // namespace

extern "C" {

CCTStatusType mps_read_configuration(const char* path, MpsConfiguration* cfg, MpsConfigBucket* buckets,
                                     int bucket_capacity, MpsConfigModel* models, int model_capacity) {
    if (!path || !cfg) return CCT_PARAMERR;
    std::ifstream f(path, std::ios::binary);
    if (!f.is_open()) return CCT_FILEERR;
    MpsConfiguration c;
    std::memset(&c, 0, sizeof(c));
    c.output_ascii = 1;
    std::string line;
    get_line(f, line);
    if (!copy_str(c.input_path, line)) return CCT_FILEERR;
    get_line(f, line);
    if (!copy_str(c.parameter_file, line)) return CCT_FILEERR;
    get_line(f, line);
    if (!copy_str(c.particle_file, line)) return CCT_FILEERR;

    // inflow buckets until an empty line
    std::vector<MpsConfigBucket> bk;
    get_line(f, line);
    while (!line.empty()) {
        std::istringstream s(line);
        MpsConfigBucket b;
        std::memset(&b, 0, sizeof(b));
        std::string name;
        s >> name;
        s >> b.interval;
        s >> b.total_steps;
        if (!copy_str(b.file, name)) return CCT_FILEERR;
        bk.push_back(b);
        get_line(f, line);
    }
    // STL models until an empty line
    std::vector<MpsConfigModel> md;
    int drags = 0;
    get_line(f, line);
    while (!line.empty()) {
        std::istringstream s(line);
        std::string name, tok;
        s >> name;
        s >> tok;
        MpsConfigModel m = wall_defaults();
        if (!copy_str(m.file, name)) return CCT_FILEERR;
        const std::string mode = upper(tok);
        if (mode == "D" || mode == "DE" || mode == "DC" || mode == "DF") {
            drag_line(s, mode, drags, m);
            ++drags;
        } else if (!wall_line(s, mode, m)) {
            return CCT_FILEERR;
        }
        md.push_back(m);
        get_line(f, line);
    }
    get_line(f, line);
    if (!copy_str(c.output_path, line)) return CCT_FILEERR;
    get_line(f, line);
    if (!copy_str(c.output_name, line)) return CCT_FILEERR;
    get_line(f, line);
    {
        std::istringstream s(line);
        s >> c.output_interval;
    }
    // compute zone: all extents nonzero, else automatic
    get_line(f, line);
    {
        std::istringstream s(line);
        CBox z;
        std::memset(&z, 0, sizeof(z));
        s >> z.m_MinBound.x;
        s >> z.m_MinBound.y;
        s >> z.m_MinBound.z;
        s >> z.m_MaxBound.x;
        s >> z.m_MaxBound.y;
        s >> z.m_MaxBound.z;
        const bool pass = std::fabs(z.m_MaxBound.x - z.m_MinBound.x) != 0.0f &&
                          std::fabs(z.m_MaxBound.y - z.m_MinBound.y) != 0.0f &&
                          std::fabs(z.m_MaxBound.z - z.m_MinBound.z) != 0.0f;
        c.has_compute_zone = pass ? 1 : 0;
        if (pass) c.compute_zone = z;
    }
    get_line(f, line);
    {
        std::istringstream s(line);
        s >> c.section.x;
        s >> c.section.y;
        s >> c.section.z;
    }
    get_line(f, line);
    {
        std::istringstream s(line);
        s >> c.start_step;
    }
    get_line(f, line);
    {
        std::istringstream s(line);
        std::string a;
        s >> a;
        c.output_ascii = upper(a) == "BINARY" ? 0 : 1;
    }
    c.bucket_count = (int)bk.size();
    c.model_count = (int)md.size();
    c.drag_count = drags;
    if (buckets) {
        if (bucket_capacity < c.bucket_count) return CCT_PARAMERR;
        std::copy(bk.begin(), bk.end(), buckets);
    }
    if (models) {
        if (model_capacity < c.model_count) return CCT_PARAMERR;
        std::copy(md.begin(), md.end(), models);
    }
    *cfg = c;
    return CCT_NOERR;
}

CCTStatusType mps_configuration_path(const char* dir, const char* name, char* out, int capacity) {
    if (!dir || !name || !out || capacity <= 0) return CCT_PARAMERR;
    const std::string p = join_path(dir, name);
    if ((int)p.size() >= capacity) return CCT_PARAMERR;
    std::memcpy(out, p.c_str(), p.size() + 1);
    return CCT_NOERR;
}

CCTStatusType mps_configuration_triangle_parameters(const MpsConfigModel* models, int count, const CParameter* param,
                                                    CTriangleParameters* out) {
    if (count < 0 || (count > 0 && (!models || !out)) || !param) return CCT_PARAMERR;
    for (int i = 0; i < count; ++i) {
        const MpsConfigModel& m = models[i];
        CTriangleParameters t;
        std::memset(&t, 0, sizeof(t));
        t.Velocity = m.velocity;
        t.Temperature = m.temperature;
        t.LinearMovableOrNot = m.linear_movable != 0;
        t.LinearResetInterval = m.reset_interval;
        t.RotatingOrNot = m.rotating != 0;
        t.RotationStartTime = m.rotation_start;
        t.TimeToReachRPM = m.time_to_reach_rpm;
        t.CenterOfRotation = m.center_of_rotation;
        t.SecondPointOfRotation = m.second_point_of_rotation;
        t.InfluenceRegion = m.influence_region;
        t.DirectionVector = m.direction;
        t.PressureGas = m.pressure_gas;
        // Scalar RotationInDegree = RotationInRPM * Dt * 6 (Integer * float * int, in float)
        const Scalar rpm_dt = (Scalar)m.rpm * param->Dt;
        t.AngleOfRotationInDegree = rpm_dt * (Scalar)6;
        t.RotationInRPM = (Scalar)m.rpm;
        t.NegativePressureCheck = m.negative_pressure_check != 0;
        t.WallFrictionCoefficient = m.wall_friction;
        t.WallThermalResistivity = m.wall_thermal_resistivity;
        t.WallThermalConductivity = m.wall_thermal_conductivity;
        t.isDrag = m.is_drag != 0;
        t.DragTriangleID = m.drag_id;
        out[i] = t;
    }
    return CCT_NOERR;
}

CCTStatusType mps_read_drag_file(const char* path, int* count, CDragTriangle* out, int capacity,
                                 char* inner_pressure_file, int name_capacity) {
    if (!path || !count) return CCT_PARAMERR;
    std::ifstream f(path);
    if (!f.is_open()) return CCT_FILEERR;
    std::string root, inner;
    f >> root;
    if (root.empty()) return CCT_FILEERR;
    f >> inner;
    struct Rec {
        std::string file;
        CDragTriangle p;
    };
    std::vector<Rec> recs;
    while (!f.eof()) {
        Rec r;
        std::memset(&r.p, 0, sizeof(r.p));
        f >> r.file;
        f >> r.p.DragLength;
        f >> r.p.StartStep01;
        f >> r.p.StartStep02;
        f >> r.p.EndStep;
        f >> r.p.InitialAcc.x;
        f >> r.p.InitialAcc.y;
        f >> r.p.InitialAcc.z;
        f >> r.p.GradAcc.x;
        f >> r.p.GradAcc.y;
        f >> r.p.GradAcc.z;
        if (f.good()) recs.push_back(r);
        else if (f.fail()) break;   // the reference's loop never ends on a field that does not parse
    }
    if (inner_pressure_file) {
        const std::string ip = join_path(root, inner);
        if ((int)ip.size() >= name_capacity) return CCT_PARAMERR;
        std::memcpy(inner_pressure_file, ip.c_str(), ip.size() + 1);
    }
    // each record's model, loaded in order; a model that does not open is skipped, and
    // the drag values then follow the loaded models' order (vDragParameters[i] of the
    // i-th loaded model, IO.cpp:616-634)
    std::vector<CTriangle> tris;
    std::vector<size_t> per_model;
    for (const Rec& r : recs) {
        const std::string name = join_path(root, r.file);
        std::ifstream probe(name.c_str());
        if (!probe.is_open()) continue;
        probe.close();
        const size_t before = tris.size();
        if (mps_io::stl_load_raw(name.c_str(), tris) != CCT_NOERR) return CCT_FILEERR;
        per_model.push_back(tris.size() - before);
    }
    const int total = (int)tris.size();
    *count = total;
    if (total == 0) return CCT_ETCERR;
    if (!out) return CCT_NOERR;
    if (capacity < total) return CCT_PARAMERR;
    int tid = 0;
    for (size_t i = 0; i < per_model.size(); ++i) {
        for (size_t j = 0; j < per_model[i]; ++j, ++tid) {
            CDragTriangle d = recs[i].p;
            d.Normal = tris[tid].Normal;
            for (int k = 0; k < 3; ++k) d.Vertex[k] = tris[tid].Vertex[k];
            d.ID = tid;
            out[tid] = d;
        }
    }
    return CCT_NOERR;
}

}  // extern "C"
