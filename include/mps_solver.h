/*
 * mps_solver.h - the GB300-native semi-implicit MPS step (one GPU, library-owned memory).
 *
 * No single reference function corresponds to this API: it runs the reference's
 * per-step schedule (CMultiGPUHandler::Calculate, MultiGPUHandler.cpp:1389-1559:
 * topology, walls, drag, predictor, topology, walls, pressure, pressure-gradient
 * correction, wall motion) with the pressure obtained from a pressure Poisson
 * equation solved by Jacobi-preconditioned CG.  The reference parses the switches for
 * that solver (bCGSolver / bNJPCGSolver, IO.cpp:273-283, 364-373) and declares, but
 * never defines, CalculatePressureCG / CalculatePressureNJPCG
 * (solver/MPS_SOLVER_WITH_ROTATION/PMMultiGPU/Source/CGPUCellSet.h:218-240).
 *
 * Inputs use the reference's parameter and wall types (mps_types.h).  Particle state
 * is kept in FP64 on the device, permanently in cell-sorted order; particle identity
 * travels in an id array.  Precision modes:
 *   MPS_PREC_FP64     every operator, the PPE and CG in FP64 (the "plain FP64
 *                     Jacobi-CG" path);
 *   MPS_PREC_FP32_IR  particle operators and CG in FP32, inside an FP64 iterative
 *                     refinement of the PPE (FP64 dot products, residual norms,
 *                     refinement residual, n0 and position/velocity accumulation).
 * A learned initial guess and diagonal scaling (mps_solver_set_learned) drive a
 * flexible CG; plain Jacobi-CG is the fallback whenever it does not converge.
 * Every call returns a CCTStatusType.
 */
#ifndef MPS_SOLVER_H
#define MPS_SOLVER_H

#include <stddef.h>

#include "mps_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct MpsSolver MpsSolver;

enum { MPS_PREC_FP64 = 0, MPS_PREC_FP32_IR = 1 };
enum { MPS_PRESSURE_PPE = 0, MPS_PRESSURE_EXPLICIT = 1 };
/* preconditioner of the FP32 inner CG (the FP64 solver is always Jacobi):
 *   MPS_PRECOND_JACOBI      diagonal
 *   MPS_PRECOND_MULTILEVEL  diagonal + cell-aggregate coarse correction: level-1 unknowns
 *                           are the non-empty neighbour-search cells, coarser levels
 *                           aggregate 2x2x2 cells down to <= 128 unknowns (explicit
 *                           inverse there), one weighted-Jacobi V-cycle per application */
enum { MPS_PRECOND_JACOBI = 0, MPS_PRECOND_MULTILEVEL = 1 };

typedef struct MpsSolverOptions {
    int precision;          /* MPS_PREC_* */
    int pressure_mode;      /* MPS_PRESSURE_PPE, or the reference's equation of state */
    int learned;            /* bit 0: learned initial guess (A-norm line search along the
                               predicted increment); bit 1: learned diagonal scaling */
    double n0_pnd;          /* reference PND at the gradient radius (<= 0: CParameter n0) */
    double n0_lap;          /* reference PND at the Laplacian radius (<= 0: CParameter n0) */
    double lambda;          /* Laplacian lambda (<= 0: CParameter LambdaValue) */
    double compressibility; /* artificial compressibility alpha [1/Pa] (Ikeda et al.) */
    double cg_rtol;         /* PPE relative residual target (||b - A p|| / ||b||) */
    int cg_max_iter;        /* CG iteration cap (per solve) */
    double ir_inner_rtol;   /* floor of the FP32 inner CG tolerance relative to the refinement
                               residual; <= 0: automatic (7e-4 for the FP16-weight operator
                               under the multilevel preconditioner, about the contraction a
                               refinement pass can reach with that operator; else 2e-6) */
    int ir_max_outer;       /* refinement pass cap */
    int max_neighbours;     /* capacity of a Laplacian neighbour row */
    int check_every;        /* CG convergence is read back every this many iterations */
    double source_relaxation; /* gamma in b = gamma rho/dt^2 (n* - n0)/n0 (Tanaka & Masunaga 2010) */
    int profile;            /* 1: time every phase with CUDA events on the solver stream */
    int preconditioner;     /* MPS_PRECOND_* (FP32_IR) */
    double mg_omega;        /* Jacobi weight of the multilevel smoothing sweeps (default 1.3;
                               the V-cycle stops being a positive definite preconditioner
                               above about 1.6 on the MPS Laplacians measured) */
    int compress_rows;      /* 1: 16-bit column offsets for the FP32 SpMV where a 32-row
                               slice spans <= 65535 columns (same results, fewer bytes) */
    int mg_sweeps;          /* weighted-Jacobi sweeps on level 1 before the restriction and
                               after the prolongation (coarser levels: 1) */
    int matrix_free;        /* FP32 inner SpMV: 0 streams the stored FP32 weights; 4 or 8
                               recompute each weight from the FP32 positions the neighbour
                               pass used (same bits), 4 or 8 entries per unrolled group,
                               streaming only the columns */
    int spmv_stream;        /* SpMV over 16-bit slices: 0 register walk; 1 rows streamed
                               through shared memory by bulk copies (a ring of 2 stages of
                               8 entries per warp); same row values.  Both solvers: the
                               FP32 inner CG, and the FP64 solver's CG products and
                               residuals over its FP64 weights; also the multilevel
                               preconditioner's level-1 assembly (same sums) */
    int inner_weights;      /* 16 (default): the inner CG uses FP16 copies of the FP32 weights
                               with the diagonal recomputed from the rounded weights (a
                               consistent Laplacian within ~5e-4 of the FP32 one; the
                               refinement still drives the FP32-weight residual to cg_rtol);
                               needs spmv_stream = 1 and matrix_free = 0.  32: the inner CG
                               uses the FP32 weights (the refinement's operator) */
    int spmv_wide;          /* streamed SpMV columns: 0 automatic (32-bit columns of every
                               slice when most entries of the last step needed them, else the
                               16-bit slices), 1 always 32-bit, -1 never; same row values */
    int warm_start;         /* start of the PPE solve from each particle's pressure history
                               (interior rows): 0 the previous pressure P_{n-1}; 1 linear in
                               time, 2 P_{n-1} - P_{n-2}; 2 quadratic, 3 P_{n-1} - 3 P_{n-2} +
                               P_{n-3}; -1 (default) 2 in FP32_IR, 0 in FP64.  Limited to the
                               history held (reset by mps_solver_set_particles and
                               mps_solver_set_time_step) */
    int flexible;           /* inner CG: 1 flexible CG (Notay, one direction kept: beta =
                               -(z.q) / (p.q), q = A p of the last direction), -1 plain PCG,
                               0 (default) flexible while the preconditioner is not a fixed
                               symmetric one (fine_smoother 1, or the learned diagonal
                               scaling, learned bit 1), else plain */
    int learned_gate;       /* 1 (default): the learned initial guess runs only while it
                               pays: after each learned step the solver compares the CG
                               iterations it saved (the residual reduction it gave, at the
                               step's own contraction per iteration) with its cost: the
                               CUDA-event time from the rows' assembly to the solve (a
                               span that holds the first refinement residual in every
                               step, with or without the guess) minus the same span of the
                               last step without the guess, in iterations of the same
                               step; when it costs more,
                               it is skipped for 2, 8, 32, 64 steps before the next trial,
                               longer (doubling up to the ratio of its cost to its saving,
                               at most 64) the further it falls short.
                               The first step with the guess is followed by one without it
                               (the span it is compared with).  0: it runs every step */
    int fine_smoother;      /* fine level of the multilevel preconditioner: 0 (default)
                               additive Jacobi (z = m r + P e1); 1 post-smoothing of the coarse
                               correction through the short-range couplings (the neighbours
                               within the gradient radius): z = P e1 + w m (r - A_s P e1),
                               a diagonal-plus-neighbour fine operator, not symmetric, so
                               the inner solve runs as flexible CG */
    double smoother_weight; /* w of fine_smoother 1 (default 0.8) */
    int rows_sell;          /* transpose of the list pass's row-major FP32 rows into SELL-32:
                               0 (default) 16-byte asynchronous copies into swizzled,
                               double-buffered shared-memory tiles; 1 register-staged tiles;
                               same rows either way */
} MpsSolverOptions;

/* error_flags bits of MpsStepStats (set by kernels, read after the step) */
#define MPS_ERR_KEY_RANGE 1u       /* a hash key fell outside [0, cells) */
#define MPS_ERR_NEIGHBOUR_CAP 2u   /* a neighbour list overflowed its capacity */
#define MPS_ERR_NONFINITE 4u       /* a non-finite value was produced */
#define MPS_ERR_TRI_CAP 8u         /* a cell exceeded its triangle capacity */
#define MPS_ERR_CG 16u             /* the CG solve did not converge */
#define MPS_ERR_STAGE_TIMEOUT 32u  /* a bulk copy into shared memory did not complete in time
                                      (the kernel fell back to global loads) */

typedef struct MpsStepStats {
    int particles;
    int interior;           /* particles in the PPE (not free surface) */
    int cg_iterations;      /* total CG iterations of the step (inner ones in FP32_IR) */
    int ir_passes;          /* refinement passes (FP32_IR) */
    int fallback;           /* 1 if the learned solve fell back to plain Jacobi-CG */
    int max_row;            /* longest neighbour row */
    double cg_relres;       /* final FP64 relative residual */
    double b_norm;
    unsigned error_flags;   /* MPS_ERR_* bits seen during the step */
    long long nnz;          /* Laplacian neighbour entries of interior rows (PPE matrix) */
    long long pairs;        /* Laplacian neighbour entries of all rows */
    /* phase times [ms] and launch counts (profile = 1 only) */
    float ms_grid, ms_walls, ms_predictor, ms_list, ms_ppe_setup, ms_spmv, ms_cg_vec, ms_correct, ms_learned;
    int spmv_launches;
    float ms_precond;       /* multilevel setup and V-cycles */
    int mg_levels;          /* coarse levels of the multilevel preconditioner (0: Jacobi) */
    int mg_level1;          /* level-1 aggregates */
    double r0_relres;       /* ||b - A p0|| / ||b|| of the start (warm start or learned guess) */
    long long nnz_wide;     /* interior entries stored with 32-bit columns (the rest: 16-bit) */
    int rows16;             /* 1 if the FP32 SpMV used compressed columns this step */
    int inner16;            /* 1 if the inner CG ran on the FP16-weight operator this step */
    int warm_start;         /* extrapolation order of this step's warm start (0: P_{n-1}) */
    int learned_applied;    /* 1 if the learned initial guess ran this step */
    float learned_saved_its;/* CG iterations it saved (estimate, see learned_gate) */
    float learned_cost_its; /* its cost in CG iterations of this step (CUDA events) */
    int flexible;           /* 1 if the inner CG ran as flexible CG */
} MpsStepStats;

void mps_solver_default_options(MpsSolverOptions* opt);
CCTStatusType mps_solver_create(const CParameter* param, const CGridBox* box, int max_particles,
                                const MpsSolverOptions* opt, MpsSolver** out);
void mps_solver_destroy(MpsSolver* s);
/* host arrays: pos/vel n*3, press/visc n (press may be NULL), type n (may be NULL) */
CCTStatusType mps_solver_set_particles(MpsSolver* s, int n, const double* pos, const double* vel,
                                       const double* press, const double* visc, const int* type);
/* vertices t*9 (three vertices per triangle), model t, params per model */
CCTStatusType mps_solver_set_triangles(MpsSolver* s, int t, const double* vertices, const int* model, int models,
                                       const CTriangleParameters* params);
CCTStatusType mps_solver_set_drag(MpsSolver* s, int count, const DragParameter* params);
CCTStatusType mps_solver_step(MpsSolver* s, int step, MpsStepStats* stats);
/* current particle state in the solver's (cell-sorted) order, with particle ids;
 * any pointer may be NULL */
CCTStatusType mps_solver_get_particles(MpsSolver* s, int* n, double* pos, double* vel, double* press, double* pnd,
                                       int* id);
CCTStatusType mps_solver_get_triangles(MpsSolver* s, double* vertices);
/* PPE data of the last step in sorted order: PND, diagonal, right-hand side,
 * solution, particle id, Laplacian neighbour count, sum of neighbour ids */
CCTStatusType mps_solver_debug_ppe(MpsSolver* s, double* pnd, double* diag, double* rhs, double* sol, int* id,
                                   int* nbr_count, double* nbr_idsum);
/* Pressure history of the warm start (solver order, n entries each): the particles'
 * last two increments P_n - P_{n-1} and P_{n-1} - P_{n-2} (0 where a particle was not
 * interior), the interior flags of the last solve, the ids, and how many increments
 * are held (0..2). */
CCTStatusType mps_solver_debug_history(MpsSolver* s, float* dph1, float* dph2, unsigned char* inner, int* id,
                                       int* held);
/* Wall bins of the current triangles (binned first if they moved or changed): for every
 * list key c = 2 * cell + kind (kind 0 walls, 1 drag bodies) bounds[c] / bounds[2 cells + c]
 * are the start and end of its entries (-1 / -1: empty), tids the triangle of each entry
 * (cap entries at most; NULL: not copied), *entries how many there are.  A cell's list
 * holds the triangles whose cell box, grown by one cell, holds the cell, in increasing
 * triangle order (the 27-cell candidate set of the cell; CCell lists of
 * RegisterTriangleTopology, Utility_Inline.h:1745-1855, in the reference). */
CCTStatusType mps_solver_debug_wall_bins(MpsSolver* s, int* bounds, int* tids, int cap, int* entries);
/* refinement residual r = b - A p of the current state (FP32_IR solvers; host
 * array of n doubles, may be NULL) and ||r|| / ||b||: variant 0 with FP64
 * products and sums, variant 1 with the double-float kernel the solver uses (rows
 * streamed through shared memory when spmv_stream is on), variant 2 the double-float
 * register walk, variant 3 the double-float kernel streaming 32-bit columns */
CCTStatusType mps_solver_debug_residual(MpsSolver* s, int variant, double* r, double* relres);
/* One FP32 inner SpMV y = A x over the current rows (FP32_IR solvers; host arrays of
 * n floats in the solver's order): kernel 0 register walk, 1 rows streamed through
 * shared memory (16-bit columns; needs the 16-bit slices), 3 streamed with the 32-bit
 * columns, 4 / 8 matrix-free: all give the same bits; 2 / 6 the streamed FP16-weight
 * operator (inner_weights = 16) with 16-bit / 32-bit columns, the same bits as each
 * other. */
CCTStatusType mps_solver_debug_spmv(MpsSolver* s, int kernel, const float* x, float* y);
/* Level-1 Galerkin stencil of the multilevel preconditioner, reassembled from the
 * current rows (FP32_IR after a step with the multilevel preconditioner): variant 0 the
 * register walk over the SELL-32 rows, 1 the rows streamed through shared memory by
 * bulk copies (spmv_stream = 1); both give the same bits.  *n1 = level-1 unknowns; with
 * a non-null a (room for cap >= 27 n1 floats) the stencil is copied out, 27 slots per
 * unknown, slot (dx+1)*9 + (dy+1)*3 + (dz+1) of the neighbouring cell. */
CCTStatusType mps_solver_debug_level1(MpsSolver* s, int variant, float* a, int cap, int* n1);
/* Time step from the next step on (a dt schedule row, mps_dt_schedule_next in
 * mps_io.h): Dt, and CourantNumber when courant > 0; the constants that depend on them
 * are recomputed as at creation, so the solver continues exactly as one created with
 * these values. */
CCTStatusType mps_solver_set_time_step(MpsSolver* s, double dt, double courant);
/* Particle inflow (CMultiGPUHandler::AddBucketParticles / InsertBucket,
 * radix/SPVSOLVER/MultiGPUSolver/MultiGPUHandler.cpp:1156-1210) on the device state:
 * the bucket's particles (reference CParticle records; ID, Density, Temperature and
 * SolidPhaseRate are not used) take the IDs below the ID extent that no particle
 * carries (removed by the compute-zone compaction), in increasing order; the rest are
 * appended at the extent when all of them fit under max_particles, else dropped, as
 * the reference does.  *added = particles inserted.  The next step sorts them in. */
CCTStatusType mps_solver_add_particles(MpsSolver* s, int count, const CParticle* bucket, int* added);
/* Output frame of the current state in the reference's format (IO::Save,
 * radix/SPVSOLVER/MultiGPUSolver/IO.cpp:649-756; see mps_write_frame in mps_io.h):
 * particles in ID order with position, velocity, pressure, PND as the density,
 * viscosity and type (temperature and solid rate, not modelled here, are written as 0),
 * the time and `models` model positions / rotation angles.  The state is packed on the
 * solver stream at this point of the step sequence and copied to pinned host memory on
 * a stream of its own; a host thread writes the file while later steps run (two frames
 * in flight).  mps_solver_wait_frames waits for them and returns the first write error. */
CCTStatusType mps_solver_save_frame(MpsSolver* s, const char* path, int ascii, double time, int models,
                                    const Scalar3* model_pos, const Scalar* model_angle);
CCTStatusType mps_solver_wait_frames(MpsSolver* s);
/* Device pointer of the pressure array (FP64, sorted order) and particle count. */
CCTStatusType mps_solver_device_pressure(MpsSolver* s, const double** press, int* n);
/* Pressure read back to a host buffer, in the solver's order (e2e output). */
CCTStatusType mps_solver_copy_pressure(MpsSolver* s, double* host_press);
/* Replace the particle state (n entries, in the solver's current order, e.g. as
 * returned by mps_solver_download_state) from host arrays: pos/vel n*3, press n.
 * Pinned host memory makes the copies asynchronous DMA. */
CCTStatusType mps_solver_upload_state(MpsSolver* s, const double* pos, const double* vel, const double* press);
CCTStatusType mps_solver_download_state(MpsSolver* s, double* pos, double* vel, double* press);
/* Stream the solver launches on (cudaStream_t), for event timing by the caller. */
CCTStatusType mps_solver_stream(MpsSolver* s, void** stream);

/* ---- learned initial guess / preconditioner (BF16 tensor-core MLP) ---- */
/* MLP 12 -> 128 -> 128 -> 128 -> 2 (SiLU); FP32 master parameters, layout:
 * W1[12][128] b1[128] W2[128][128] b2[128] W3[128][128] b3[128] W4[128][2] b4[2]
 * (row-major, input-major) = 34,946 floats. */
#define MPS_MLP_PARAMS 34946
#define MPS_MLP_FEATURES 12
CCTStatusType mps_solver_set_learned(MpsSolver* s, const float* params, int count);
/* Features (n*12, FP32) and training targets (n*2: normalised pressure increment,
 * log of the ideal diagonal scale) of the last PPE solve, sorted order. */
CCTStatusType mps_solver_learned_samples(MpsSolver* s, float* features, float* targets, int* n);
/* 1: compute features and targets at every PPE solve (for mps_solver_learned_samples) */
CCTStatusType mps_solver_collect(MpsSolver* s, int on);

/* ---- reserved names of the reference and the precision / learned-part controls ----
 *
 * The reference declares CCellSet::CalculatePressureCG and CalculatePressureNJPCG
 * (solver/MPS_SOLVER_WITH_ROTATION/PMMultiGPU/Source/CGPUCellSet.h:224-225) but never
 * defines them.  Here they solve the pressure Poisson equation for the solver's current
 * particle state: topology, wall distance, PND and PPE assembly at the current positions,
 * then the solve from the previous pressure to cg_rtol (positions and velocities are
 * unchanged, the state is re-sorted).  CG: Jacobi preconditioner, no network.  NJPCG:
 * the multilevel preconditioner (FP32_IR) and the learned initial guess when one is
 * installed. */
CCTStatusType CalculatePressureCG(MpsSolver* s, MpsStepStats* stats);
CCTStatusType CalculatePressureNJPCG(MpsSolver* s, MpsStepStats* stats);
/* CalcPoisson: the reserved prototype of the same tree's DeviceProcess.h:50-53
 * (CalcPoisson(cudaStream_t&, ParticleNum, CParticle*, Scalar* distance, Integer* ID,
 * TriangleNum, CTriangle*, CDistance*, Scalar* dA, Scalar* dB, Scalar* dX, Scalar* dX0),
 * declared there but never defined), as a context-handle variant: the particles, walls,
 * drag bodies and their distances are the solver's, in place of the AoS particle and
 * wall arguments; the solver's buffers carry the old variant's per-particle A_ii, B, X
 * and X0 (CGPUCellSet.h:69-81 of that tree).  It solves the PPE of the solver's current
 * state as CalculatePressureCG does (topology, wall distance, PND and assembly at the
 * current positions, Jacobi-PCG to cg_rtol at the solver's precision) and writes device
 * arrays of ParticleNum Scalars indexed by particle ID:
 *   dA  the PPE diagonal A_ii (0 for particles outside the PPE: free surface, P = 0),
 *   dB  the right-hand side (0 outside the PPE),
 *   dX  the solved pressure;
 * dX0 (may be NULL: the solver's pressure history) is the start of the solve, read by
 * ID; any of dA, dB, dX may be NULL.  Entries of IDs no particle carries are left as
 * they are.  Stream (a cudaStream_t, may be NULL): the solve starts after the work
 * already queued there (which may write dX0); the outputs are complete on return.
 * CCT_PARAMERR for a particle ID >= ParticleNum, CCT_CALCERR when CG misses cg_rtol
 * (stats, may be NULL, has the details). */
CCTStatusType CalcPoisson(void* Stream, MpsSolver* s, Integer ParticleNum, Scalar* dA, Scalar* dB, Scalar* dX,
                          const Scalar* dX0, MpsStepStats* stats);
/* switches between MPS_PREC_FP64 and MPS_PREC_FP32_IR for the following steps */
CCTStatusType mps_set_precision(MpsSolver* s, int precision);

typedef struct MpsLearnedInfo {
    int samples;            /* (state, converged pressure) pairs kept */
    int val_samples;        /* of which held out for validation (10 %) */
    int adam_steps;
    int batch;
    float val_loss_before;  /* validation loss of the initial network */
    float val_loss_after;
    double collect_ms, train_ms;
} MpsLearnedInfo;
/* Runs `steps` steps of the solver itself (step indices first_step ...; the simulation
 * advances as usual and the PPE is solved without the network), keeps up to
 * max_samples (<= 0: 400,000) randomly chosen (features, converged pressure) pairs of
 * interior particles, trains the network on the GPU (Adam, `epochs` passes of `batch`
 * rows, learning rate halved per pass, 10 % validation) and installs it with the
 * learned initial guess enabled (options.learned |= 1). */
CCTStatusType mps_learned_train(MpsSolver* s, int first_step, int steps, int max_samples, int epochs, int batch,
                                float lr, unsigned long long seed, MpsLearnedInfo* info);
/* Network outputs (pressure increment in units of the step's pressure scale, log
 * diagonal scale; host array of 2 n floats, may be NULL) for the features of the last
 * step; requires an installed network and a last step that computed features. */
CCTStatusType mps_learned_infer(MpsSolver* s, float* out, int* n);

#ifdef __cplusplus
}
#endif

#endif
