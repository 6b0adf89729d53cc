/*
 * mps_io.h - the reference solver's input formats and setup helpers (host code).
 *
 *   mps_read_parameter_file  IO::Load(parameter file), radix/SPVSOLVER/MultiGPUSolver/IO.cpp:65-446
 *                            positional whitespace-separated fields; every optional
 *                            trailing group is read only while input remains, and
 *                            missing groups take the reference's defaults.
 *   mps_read_particle_file   IO::Load(particle file), IO.cpp:6-63: rows of
 *                            "x y z vx vy vz P n T nu solidRate type(0|1|2)", no
 *                            header, IDs 0..N-1 in file order; call with out = NULL to
 *                            count, then with a buffer of that capacity.
 *   mps_read_stl             IO::Load(model list) + CSTLSerializer::Load, IO.cpp:470-523,
 *                            STLSerializer.cpp:225-357: ASCII when the first token is
 *                            "solid", else binary (80-byte header, uint32 count, 50-byte
 *                            records); normals recomputed from the vertices with the
 *                            reference's float arithmetic (CalcTriangleNormal,
 *                            IO.cpp:449-467); the model offset is added to every vertex
 *                            (MultiGPUHandler.cpp:713-735).  out = NULL counts.
 *   mps_lambda_table         CalculateLambdaValueLocal, MultiGPUHandler.cpp:757-921,
 *                            including its chained-comparison branch selection.
 *   mps_grid_box             CCellSet::SetComputeZone, CGPUCellSet.cpp:109-152.
 *   mps_lattice_constants    n0 and lambda of the cubic lattice for a radius (FP64);
 *                            no reference counterpart (it reads n0 from the file).
 *   mps_read_dt_file         DtFrame::Load, DtFrame.cpp:11-35: the dt schedule.
 *   mps_dt_schedule_next     CMultiGPUHandler::CheckAndUpdateDt, MultiGPUHandler.cpp:
 *                            1256-1275: applies the next due schedule row to a CParameter.
 *   mps_write_frame          IO::Save / SaveAscii / SaveBinary, IO.cpp:649-756: an output
 *                            frame.  ASCII: count; "x y z vx vy vz P n T nu solidRate
 *                            type" per particle (%g, 6 significant digits, as the
 *                            reference's std::ostream); time; model count; "x\ty\tz\t
 *                            angle" per model.  Binary: int32 count, 48-byte records
 *                            (3+3+5 floats, int32 type), float time, int32 model count,
 *                            4 floats per model.  temperature / solid_rate may be NULL
 *                            (written as 0).
 *   mps_read_configuration   CConfiguration::ReadConfigurationFileWithDrag,
 *                            Configuration.cpp:21-452: the run's configuration file
 *                            (paths, inflow buckets, STL model lines in both dialects,
 *                            drag model lines D|DE|DC|DF, output settings).
 *   mps_configuration_path   CConfiguration::GetParameterFile and siblings,
 *                            Configuration.cpp:646-825: a file name joined to a path.
 *   mps_configuration_triangle_parameters
 *                            the per-model CTriangleParameters that CMultiGPUHandler
 *                            builds from the configuration, MultiGPUHandler.cpp:466-555.
 *   mps_read_drag_file       IO::Load(drag file, CDragTriangle*&), IO.cpp:524-648: drag
 *                            triangle models with their drag schedule.
 * All return CCT_NOERR, CCT_FILEERR (cannot open / malformed) or CCT_PARAMERR.
 */
#ifndef MPS_IO_H
#define MPS_IO_H

#include "mps_types.h"

#ifdef __cplusplus
extern "C" {
#endif

CCTStatusType mps_read_parameter_file(const char* path, CParameter* out);
CCTStatusType mps_read_particle_file(const char* path, int* count, CParticle* out, int capacity);
CCTStatusType mps_read_stl(const char* path, int model_id, const Scalar3* offset, int* count, CTriangle* out,
                           int capacity);
float mps_lambda_table(float l0);
CCTStatusType mps_grid_box(const CBox* compute_zone, const CParameter* param, CGridBox* out);
CCTStatusType mps_lattice_constants(double re_coefficient, double l0, int dimension, double* n0, double* lambda);
/* One row of the dt schedule file (DtFrame::Load, radix/SPVSOLVER/MultiGPUSolver/
 * DtFrame.cpp:11-35; DeltaTime, DataType.h:565-571): from `step` on, Dt, CourantNumber,
 * ParticleGenerationStep (inflow_step) and OutputStep take these values. */
typedef struct MpsDtRow {
    Integer step;
    Scalar dt;
    Scalar courant;
    Scalar inflow_step;
    Scalar output_step;
} MpsDtRow;
/* Reads the rows "Step Dt CourantNumber InflowStep OutputStep" with the reference's
 * stream semantics: reading stops at the first field that does not parse or at the end
 * of the file, and a row counts only if the stream is still good after its fifth field
 * (a last row not followed by whitespace is dropped, as DtFrame::Load drops it).
 * rows = NULL counts. */
CCTStatusType mps_read_dt_file(const char* path, int* count, MpsDtRow* rows, int capacity);
/* CMultiGPUHandler::CheckAndUpdateDt (MultiGPUHandler.cpp:1256-1275): if row *next is
 * due (current_step >= its step), copies it into param (Dt, CourantNumber,
 * ParticleGenerationStep, OutputStep as an integer) and advances *next; one row per
 * call.  *applied = 1 when a row was applied. */
CCTStatusType mps_dt_schedule_next(const MpsDtRow* rows, int count, int* next, int current_step, CParameter* param,
                                   int* applied);
#define MPS_PATH_MAX 512
/* Inflow bucket line "file interval totalSteps" (until an empty line). */
typedef struct MpsConfigBucket {
    char file[MPS_PATH_MAX];
    Integer interval;         /* steps between insertions */
    Integer total_steps;      /* last step of insertions */
} MpsConfigBucket;
/* One STL model line.  Wall line (both dialects; fields missing at the end of a line
 * keep the defaults below): file vx vy vz T ox oy oz linearMovable(0|1) resetInterval
 * rotating(0|1) rpm tStart tReachRPM cx cy cz px py pz wallFriction wallThermalR
 * wallThermalK negativePressure(0|1) influence dx dy dz pressureGas.  Drag line: file
 * D|DE|DC|DF inToken outToken influence <mode parameters> (drag models: velocity 0,
 * temperature 533, nothing moves, drag_id counts the drag lines from 0). */
typedef struct MpsConfigModel {
    char file[MPS_PATH_MAX];
    int is_drag;
    Integer drag_id;          /* -1 for a wall model */
    Scalar3 velocity;
    Scalar temperature;
    Scalar3 position;         /* offset added to the model's vertices */
    int linear_movable;
    Integer reset_interval;
    int rotating;
    Integer rpm;
    Scalar rotation_start;
    Scalar time_to_reach_rpm;
    Scalar3 center_of_rotation;
    Scalar3 second_point_of_rotation;
    Scalar wall_friction;
    Scalar wall_thermal_resistivity;
    Scalar wall_thermal_conductivity;
    int negative_pressure_check;
    Scalar influence_region;
    Scalar3 direction;
    Scalar pressure_gas;
    DragParameter drag;       /* drag lines only (zero for walls) */
} MpsConfigModel;
typedef struct MpsConfiguration {
    char input_path[MPS_PATH_MAX];
    char parameter_file[MPS_PATH_MAX];
    char particle_file[MPS_PATH_MAX];
    char output_path[MPS_PATH_MAX];
    char output_name[MPS_PATH_MAX];
    int bucket_count;
    int model_count;
    int drag_count;
    Integer output_interval;
    int has_compute_zone;     /* 0: every extent of the zone line is 0 (automatic zone) */
    CBox compute_zone;
    Integer3 section;
    Integer start_step;
    int output_ascii;         /* 0 when the last line says BINARY (any case) */
} MpsConfiguration;
/* Reads a configuration file with the reference's line and stream rules: lines end at
 * LF, a CR before it is dropped (the reference reads in text mode on Windows); the
 * bucket and model lists end at an empty line; model and drag tokens are compared in
 * upper case; a drag line's input token other than V or T selects both ('B'), as the
 * reference's always-true test does; fields a line lacks keep their defaults; the lines
 * after the model list may be missing (zone automatic, sections 0, start 0, ASCII).
 * buckets / models = NULL: only cfg (with the counts) is filled; else the arrays must
 * hold the counts (CCT_PARAMERR otherwise).  A wall line whose velocity token is not a
 * number is CCT_FILEERR (the reference's boost::lexical_cast throws there). */
CCTStatusType mps_read_configuration(const char* path, MpsConfiguration* cfg, MpsConfigBucket* buckets,
                                     int bucket_capacity, MpsConfigModel* models, int model_capacity);
/* `dir` + "\\" + `name` (no separator added when dir ends with '/' or '\\'), or `name`
 * alone for an empty dir, as the reference's Get*File methods join the configuration's
 * input and output paths. */
CCTStatusType mps_configuration_path(const char* dir, const char* name, char* out, int capacity);
/* The CTriangleParameters of each model (MultiGPUHandler.cpp:466-555):
 * AngleOfRotationInDegree = rpm * Dt * 6 in float, RotationInRPM = rpm, isDrag /
 * DragTriangleID from the drag line, the rest field by field. */
CCTStatusType mps_configuration_triangle_parameters(const MpsConfigModel* models, int count, const CParameter* param,
                                                    CTriangleParameters* out);
/* Drag file (IO::Load, IO.cpp:524-648): a root path, the inner-pressure parameter file
 * name, then records "stlFile dragLength startStep01 startStep02 endStep ax ay az gx gy
 * gz" (a record counts only if the stream is still good after its last field; reading
 * stops at the first field that does not parse, where the reference would loop
 * forever).  Each record's STL model (root + file, joined as mps_configuration_path
 * does) is loaded; a model that cannot be opened is skipped and, as in the reference,
 * the records' drag values then go to the loaded models in order.  Triangles keep the
 * STL file's normals; ID = index.  inner_pressure_file receives root + inner-pressure
 * name (may be NULL).  out = NULL counts.  No triangle at all: CCT_ETCERR. */
CCTStatusType mps_read_drag_file(const char* path, int* count, CDragTriangle* out, int capacity,
                                 char* inner_pressure_file, int name_capacity);
CCTStatusType mps_write_frame(const char* path, int ascii, int n, const Scalar3* pos, const Scalar3* vel,
                              const Scalar* pressure, const Scalar* density, const Scalar* temperature,
                              const Scalar* viscosity, const Scalar* solid_rate, const ParticleType* type,
                              Scalar time, int models, const Scalar3* model_pos, const Scalar* model_angle);

#ifdef __cplusplus
}
#endif

#endif
