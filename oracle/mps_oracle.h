/*
 * mps_oracle.h - C interface of the CPU oracle for the MPS hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is the checker for the CUDA kernels of
 * simulation_project_gb300; it is never linked into, called by, or shipped with
 * the product library.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load it.
 *
 * Two implementations export this interface:
 *   oracle/liborc.so        - the restatement in oracle/mps_oracle.cpp
 *   oracle/_ref/libref.so   - the reference's own kernel header compiled for the
 *                             CPU by oracle/ref_harness.cpp (built only where the
 *                             reference sources are available)
 * so a test can run the same call on both and compare the outputs bit for bit.
 *
 * OrcBindings mirrors the reference's constant-memory bindings
 * (radix/SPVSOLVER/MultiGPUSolver/Constant.h:4-76): the "sorted" arrays are the
 * c_daParticle* set, the "out" arrays the c_daOutputParticle* set (original order).
 */
#ifndef MPS_ORACLE_H
#define MPS_ORACLE_H

#include "../include/mps_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OrcBindings {
    CParameter param;
    CGridBox box;
    int particle_num;
    int max_particle_num;
    /* sorted-order particle arrays (c_daParticle*) */
    int* id;
    Scalar3* pos;
    Scalar3* vel;
    float* pressure;
    float* density;
    float* temperature;
    float* kin_visc;
    float* solid_rate;
    int* type;
    /* original-order particle arrays (c_daOutputParticle*) */
    int* out_id;
    Scalar3* out_pos;
    Scalar3* out_vel;
    float* out_pressure;
    float* out_density;
    float* out_temperature;
    float* out_kin_visc;
    float* out_solid_rate;
    int* out_type;
    /* walls */
    CTriangle* triangles;
    int triangle_num;
    CTriangleParameters* tri_params;
    CDistance* stl_distance;
    int* stl_id;
    CCell* cells;
    int cell_num;
    int* cell_start;
    int* cell_end;
    /* drag */
    DragParameter* drag_params;
    int drag_num;
    Scalar3* drag_acc;
    float* drag_temperature;
    int* magnifier_count;
    /* turbulence (c_daParticleTurbulaceViscosity, c_daParticleStrainTensorProduct) */
    float* turb_visc;
    float* strain;
} OrcBindings;

/* ---- math helpers (reference float arithmetic) ---- */
float orc_sqrt_utility(float x);
float orc_calc_distance(const Scalar3* a, const Scalar3* b);
float orc_get_weight(float re, float r);
float orc_zgrad(float r, float l0);
float orc_zlap(float r, float l0);
float orc_zgrad2d(float r, float l0);
float orc_zlap2d(float r, float l0);
float orc_triangle_distance(const CTriangle* tri, const Scalar3* p, Scalar3* dir);
int orc_cell_id(const CGridBox* box, const Scalar3* p, int* i, int* j, int* k);
int orc_is_include(const CGridBox* box, const Scalar3* p, float tol);
void orc_correct_velocity(const CParameter* param, Scalar3* v);
float orc_lambda_table(float l0);

/* ---- grid ---- */
int orc_calc_hash(const OrcBindings* b, int n, int* hash, int* index, const Scalar3* pos);
int orc_sort(int n, int* hash, int* index);
int orc_reorder_find_cell_start(OrcBindings* b, int n, int cells, const int* hash,
                                const int* index, int* cell_start, int* cell_end);
int orc_check_outside_compute_zone(OrcBindings* b, int* n);

/* ---- walls ---- */
int orc_reset_triangle_topology(int cells, CCell* cell);
int orc_register_triangle_topology(OrcBindings* b, const CTriangle* tri, int t, CCell* cell, int cells);
int orc_update_triangle_position(OrcBindings* b, int t);
int orc_rotate_triangle_position(OrcBindings* b, int t, int step);
int orc_reset_wall_position(OrcBindings* b, int t, int step, const CTriangle* orig);
int orc_calc_stl_distance(OrcBindings* b, int n);
int orc_calc_drag_effect(OrcBindings* b, int n);

/* ---- particle operators (explicit schedule) ---- */
int orc_calc_explicitly(OrcBindings* b, int n);
int orc_calc_temperature_factor(OrcBindings* b, int n);
int orc_calc_turbulence_viscosity(OrcBindings* b, int n);
int orc_calc_explicit_pressure(OrcBindings* b, int n);
int orc_calc_explicit_pressure_gradient(OrcBindings* b, int n);

/* ---- FP64 semi-implicit solver (PPE + Jacobi-PCG); no reference counterpart ---- */
typedef struct OrcSimConfig {
    CParameter param;
    CGridBox box;
    int quirks;          /* 0 = exact arithmetic; the sim is always FP64 */
    double n0_pnd;       /* reference density for PND / source / gradient */
    double n0_lap;       /* reference density for the Laplacian coefficient */
    double lambda;       /* Laplacian lambda */
    double compressibility;  /* artificial compressibility alpha [1/Pa] */
    double cg_rtol;
    int cg_max_iter;
    int threads;         /* OpenMP threads (0 = library default) */
    double source_relaxation;  /* gamma of the PND source term */
} OrcSimConfig;

typedef struct OrcStepStats {
    int cg_iterations;
    double cg_relres;
    double b_norm;
    int interior;
    int particles;
} OrcStepStats;

typedef struct OrcSim OrcSim;
OrcSim* orc_sim_create(const OrcSimConfig* cfg, int max_particles);
void orc_sim_destroy(OrcSim* s);
int orc_sim_set_particles(OrcSim* s, int n, const double* pos, const double* vel,
                          const double* pressure, const double* kin_visc, const int* type);
int orc_sim_set_triangles(OrcSim* s, int t, const double* vertices /* t*9 */,
                          const int* model, int models, const CTriangleParameters* params);
int orc_sim_set_drag(OrcSim* s, int count, const DragParameter* params);
int orc_sim_step(OrcSim* s, int step, OrcStepStats* stats);
int orc_sim_get(OrcSim* s, int* n, double* pos, double* vel, double* pressure, double* pnd);
int orc_sim_get_triangles(OrcSim* s, double* vertices);
int orc_sim_get_ids(OrcSim* s, int* ids);
int orc_sim_last_nbr(OrcSim* s, int* cnt, double* idsum, int* pid);
/* One PPE solve on the current state's sorted arrays (for operator tests):
 * writes the per-particle PND, diagonal, rhs and solution in sorted order. */
int orc_sim_last_ppe(OrcSim* s, double* pnd, double* diag, double* rhs, double* sol, int* sorted_id);
/* The last solve's PPE operator as CSR rows in the solver order (identity rows for
 * particles outside the PPE); returns the entry count, arrays may be NULL. */
long long orc_sim_last_matrix(OrcSim* s, int* rowptr, int* col, double* val);

#ifdef __cplusplus
}
#endif

#endif
