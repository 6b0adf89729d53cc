// native.cuh - data layout and kernel declarations of the GB300-native solver.
//
// Layout in HBM (all arrays indexed by the current cell-sorted particle order):
//   pos, vel        dbl4  (x, y, z, unused)   FP64 master state, 32 B each
//   opos, ovel      float4                        FP32 operator copies; opos.w holds the
//                                                 particle's global z bin (cell z * 64 + bin)
//   press           double                        pressure (PPE solution)
//   visc            float, type int, id int       carried per particle
//   key, idx        int                           hash keys / sort permutation
//   cstart, cend    int[cells]                    cell ranges (-1 = empty)
//   nbr, nbrw       int / T [ceil(n/32)*32 * K]  Laplacian neighbour rows in SELL-32
//                                                 layout: entry k of row i at
//                                                 ((i/32)*K + k)*32 + i%32; nbr_cnt[i] entries
//   nbr16, sbase    u16 [same] / int [slices]    the interior rows' columns as 16-bit
//                                                 offsets from the slice's smallest column
//                                                 (sbase -1: the slice spans > 65535)
//   gnbr, gnbrr     int / T [n * KG]              gradient-radius rows (index, r)
//   tri             double[9*T], tnrm double[3*T] walls; tcs[4*cells]/tids: per cell key
//                   2*cell + (drag), the triangles whose cell box (grown by one cell) holds it
// Kernels take the whole record as one __grid_constant__ parameter.
#pragma once

#include <cuda_fp16.h>

#include "mps_common.cuh"
#include "mps_internal.h"
#include "../../include/mps_solver.h"

namespace mps {

struct Consts {
    double l0, re_lap, re_grad, mind_lap, mind_grad;
    double coef_lap;      // 2d / (lambda n0_lap)
    double n0_pnd, n0_lap, beta, rho, dt, kappa;
    double c1;            // 2d / n0_pnd
    double c2;            // rho / dt^2
    double vmax;          // l0 * Courant / dt
    double wall_fric, offset_l0, tol, sonic2, gamma;
    double g[3];
    int dim;
    int explicit_pressure;
};

struct Dev {
    int n, cells, K, KG, tri_n, drag_n;
    CGridBox box;
    Consts c;
    dbl4 *pos, *vel;
    double* press;
    float* visc;
    int *type, *id;
    dbl4 *pos2, *vel2;
    double* press2;
    float* visc2;
    int *type2, *id2;
    float4 *opos, *ovel;
    int *key, *idx;
    int* skey;                 // sort key: cell << zbits | z bin of the particle inside its cell
    int zbits;                 // z-bin bits of the sort key (6; 0 for grids too large for them)
    int *cstart, *cend;
    int* cell_list;
    int* cell_count;
    // walls
    double* tri;
    float* tri32;              // FP32 copy of tri (FP32 wall distance and drag)
    unsigned char* tdrag;      // 1 for triangles of drag models
    double* tnrm;
    int* tmodel;
    CTriangleParameters* tparams;
    DragParameter* drag;
    int *tcs, *tids;
    double* wdist;
    double* wdir;
    int* wid;
    double* dragv;
    // neighbour rows: the list pass writes each row contiguously (row i at i*K: rnbr, rw);
    // k_rows_sell turns the interior rows into SELL-32 (nbr, nbrw, nbr16, w16)
    int* rnbr;
    void* rw;
    int* nbr;                  // SELL-32 32-bit columns: slices with sbase = -1, or every slice when rows_c32
    void* nbrw;
    unsigned short* nbr16;     // SELL-32 column offsets from the slice base (interior rows)
    int* sbase;                // [slices] smallest column index of the slice, -1: 32-bit slice
    int* skmax;                // [slices] longest interior row of a 16-bit slice, -1: 32-bit slice
    int rows16;                // nbr16 / sbase are valid for the current rows
    int rows_c32;              // nbr holds the 32-bit columns of every slice
    __half* w16;               // FP16 copies of the FP32 weights (interior rows; inner CG operator)
    double* diag16;            // diagonal of the FP16-weight operator: coef * sum of FP16 weights + kappa
    int rows_w16;              // w16 / diag16 are valid for the current rows
    int* nbr_cnt;
    int* gnbr;
    void* gnbrr;
    int* gcnt;
    // PPE
    double *pnd, *diag, *rhs, *sumw;
    unsigned char* inner;
    double *r, *z, *p, *q;     // FP64 CG vectors
    float *r32, *z32, *p32, *q32, *d32, *m32;  // FP32 inner CG vectors, m32 = preconditioner
    double* minv;              // FP64 preconditioner (1/diag or learned)
    float2* xs;                // x = xs.x + xs.y (to ~2^-48): split pressure for the double-float
                               // residual, both words of a row in one 8-byte gather
    float* pf32;               // FP32 pressure (neighbour-pressure feature)
    double* red;               // block partial sums
    double* scal;              // device scalars
    unsigned* red_count;       // last-block counters
    unsigned* err;
    int* istat;                // [0] longest neighbour row
    double* pprev;             // the particle's pressure before this step's solve (P_{n-1})
    float *dph1, *dph2;        // the particle's last two pressure increments P_{n-1} - P_{n-2}
                               // and P_{n-2} - P_{n-3} (warm-start extrapolation)
    float *dph1b, *dph2b;      // their permutation buffers (sort, compaction)
    float* feat;               // [n][12] learned features
    float* mlp_out;            // [n][2] network outputs
    float* targets;            // [n][2] training targets
};

// device scalar slots
enum {
    S_RZ = 0, S_PQ, S_ALPHA, S_BETA, S_RR, S_BNORM, S_TOL, S_CONV, S_ITER, S_RZNEW, S_RNORM, S_R0NORM,
    S_IRTOL, S_TMP0, S_TMP1, S_PSCALE, S_MAXIT, S_NNZ0, S_NNZ1, S_LS0, S_LS1, S_NINT, S_COUNT
};

}  // namespace mps
