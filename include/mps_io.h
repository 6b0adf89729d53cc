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
CCTStatusType mps_write_frame(const char* path, int ascii, int n, const Scalar3* pos, const Scalar3* vel,
                              const Scalar* pressure, const Scalar* density, const Scalar* temperature,
                              const Scalar* viscosity, const Scalar* solid_rate, const ParticleType* type,
                              Scalar time, int models, const Scalar3* model_pos, const Scalar* model_angle);

#ifdef __cplusplus
}
#endif

#endif
