// solver.cu - host orchestration of the GB300-native semi-implicit MPS step and its
// C-ABI (include/mps_solver.h).
//
// One step follows the reference's schedule (CMultiGPUHandler::Calculate,
// MultiGPUHandler.cpp:1389-1559) with the explicit pressure replaced by a pressure
// Poisson equation:
//   compact -> hash / radix sort / gather -> wall bins + wall distance -> drag ->
//   viscosity/gravity predictor -> compact -> hash / sort / gather -> wall distance ->
//   neighbour rows + PND -> PPE (Jacobi-PCG, FP64 or FP32 inside FP64 refinement) ->
//   pressure-gradient correction -> wall motion.
// All state stays on the device in cell-sorted order; the host reads back only the
// particle count after each compaction and the CG convergence word every
// `check_every` iterations.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "../../include/mps_io.h"
#include "native_kernels.cuh"
#include "coarse.cuh"
#include "../../include/mps_learned.h"

namespace mps {
cudaError_t mlp_forward(MpsMlp* m, int M, const float* X, float* Y, cudaStream_t st, unsigned* err);

namespace {

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count) {
        n = count;
        return cudaMalloc((void**)&p, sizeof(T) * std::max<size_t>(count, 1));
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
    }
};

inline int blocks_for(int n, int threads = kBlock) { return std::max(1, div_up(n, threads)); }

enum Phase { PH_GRID = 0, PH_WALLS, PH_PRED, PH_LIST, PH_SETUP, PH_SPMV, PH_VEC, PH_CORRECT, PH_LEARNED, PH_PRECOND,
             PH_OTHER, PH_COUNT };

// CUDA events on the solver stream at phase boundaries; the interval between two
// consecutive marks is attributed to the first mark's phase.
struct PhaseTimer {
    std::vector<cudaEvent_t> pool;
    std::vector<int> cat;
    size_t used = 0;
    bool on = false;
    void mark(int c, cudaStream_t st) {
        if (!on) return;
        if (used == pool.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            pool.push_back(e);
            cat.push_back(0);
        }
        cat[used] = c;
        cudaEventRecord(pool[used], st);
        ++used;
    }
    void collect(float* ms) {
        for (size_t k = 0; k + 1 < used; ++k) {
            float t = 0.f;
            cudaEventElapsedTime(&t, pool[k], pool[k + 1]);
            ms[cat[k]] += t;
        }
        used = 0;
    }
    void release() {
        for (auto e : pool) cudaEventDestroy(e);
        pool.clear();
    }
};

}  // namespace

struct Solver {
    MpsSolverOptions opt;
    CParameter param;
    Dev d{};
    int nmax = 0;
    int bins_dirty = 1;
    int models = 0;
    int walls_move = 0;
    cudaStream_t st = nullptr;
    // second stream: the multilevel setup runs there beside the rows' transpose, the first
    // refinement residual and the learned guess
    cudaStream_t st2 = nullptr;
    cudaEvent_t ev_setup = nullptr, ev_rows = nullptr, ev_mg = nullptr, ev_walls = nullptr, ev_bins = nullptr;
    bool mg_setup_done = false;   // this step's hierarchy is already built
    std::vector<void*> allocs;
    void* sort_scratch = nullptr;
    size_t sort_scratch_bytes = 0;
    unsigned *keep = nullptr, *rank = nullptr;
    unsigned* scan_sums = nullptr;   // tile sums of the multi-CTA scans
    unsigned* scan_sums2 = nullptr;  // the same for the wall bins on the second stream
    double* h_scal = nullptr;   // pinned mirror of the device scalars
    int* h_int = nullptr;       // pinned small ints
    int* h_bins = nullptr;      // pinned small ints of the wall binning
    // wall-bin scratch
    unsigned* bin_off = nullptr;
    size_t bin_off_cap = 0;
    int bin_entries = 0;   // (cell, triangle) entries of the last binning
    int* bin_visit = nullptr;
    size_t bin_visit_cap = 0;
    void* bin_sort = nullptr;
    size_t bin_sort_bytes = 0;
    MpsStepStats last{};
    PhaseTimer timer;
    int spmv_launches = 0;
    double* stage = nullptr;   // host-exchange staging (7 n doubles)
    // learned parameters (optional)
    bool learned_ready = false;
    bool collect = false;
    bool feat_valid = false;   // d.feat holds the features of the last step
    bool residual_ready = false;   // d.r / S_RNORM / S_BNORM hold the start's residual
    MpsMlp* mlp = nullptr;
    // multilevel preconditioner
    Mg mg{};
    int mg_grid_levels = 0;    // levels with a grid (1 .. mg_grid_levels)
    bool mg_on = false;        // enabled and supported by the grid
    bool mg_ready = false;     // set up for the current step
    bool mg_init_done = false; // level buffers allocated
    unsigned* mg_flag = nullptr;
    unsigned* mg_counts = nullptr;
    unsigned* h_counts = nullptr;

    template <class T>
    cudaError_t mk(T** ptr, size_t count) {
        cudaError_t e = cudaMalloc((void**)ptr, sizeof(T) * std::max<size_t>(count, 1));
        if (e == cudaSuccess) allocs.push_back((void*)*ptr);
        return e;
    }

    bool fp64() const { return opt.precision == MPS_PREC_FP64; }

    // ---- gate of the learned initial guess (MpsSolverOptions::learned_gate) ----
    // events on the solver stream: [0] rows ready (the warm start, the first refinement
    // residual, the learned guess and the multilevel setup on the second stream follow),
    // [4, 5] the solve.  The span [0, 4] of a step without the guess (warm start, first
    // residual beside the multilevel setup) is kept as the baseline; the guess costs what
    // its step's span adds to it.
    cudaEvent_t gate_ev[6] = {};
    int gate_skip = 0, gate_period = 2;
    double gate_rb = 0.0, gate_ra = 0.0;
    double gate_span_off = -1.0;   // span of the last step without the guess [ms] (< 0: none yet)
    int gate_pending = 0;          // 1 / 2: this step's events (without / with the guess) await reading
    void gate_update(MpsStepStats& S, bool learned) {
        float t_span = 0.f, t_s = 0.f;
        cudaEventElapsedTime(&t_span, gate_ev[0], gate_ev[4]);
        cudaEventElapsedTime(&t_s, gate_ev[4], gate_ev[5]);
        if (!learned) {
            gate_span_off = t_span;
            return;
        }
        if (gate_span_off < 0.0) {   // no baseline yet: measure one step without the guess
            gate_skip = 1;
            return;
        }
        const int its = S.cg_iterations;
        if (its <= 0 || !(gate_rb > 0.0) || !(gate_ra > 0.0) || !(S.cg_relres > 0.0) || !(S.r0_relres > S.cg_relres))
            return;
        // contraction per iteration of this solve, and the iterations the guess's
        // residual reduction is worth at that rate
        const double per_it = std::log(S.r0_relres / S.cg_relres) / its;
        const double saved = std::log(gate_rb / gate_ra) / per_it;
        const double t_it = (double)t_s / its;
        const double cost = ((double)t_span - gate_span_off) / t_it;
        S.learned_saved_its = (float)saved;
        S.learned_cost_its = (float)cost;
        if (saved < cost) {
            // the further the guess falls short of paying for itself, the longer it sits
            // out: at least the current period, doubled up to the cost / saving ratio
            // (a guess that recovers a twentieth of its cost is tried again after 32
            // steps), at most 64
            const double ratio = saved > 0.0 ? cost / saved : 64.0;
            int skip = gate_period;
            while (skip < 64 && skip < ratio) skip *= 2;
            gate_skip = std::min(skip, 64);
            gate_period = std::min(4 * gate_skip, 64);
        } else {
            gate_period = 2;
        }
    }
    // inner CG iterations of each refinement pass in the last step (first batch sizes)
    static constexpr int kPassMemory = 4;
    int pass_its[kPassMemory] = {0, 0, 0, 0};
    // pressure increments recorded for the particles (0..2); reset with a new particle
    // set or time step
    int hist = 0;
    // warm-start extrapolation order of this step: the option, or automatically
    // quadratic in FP32_IR and the previous pressure in FP64; at most the history held
    int warm_order() const {
        const int w = opt.warm_start < 0 ? (fp64() ? 0 : 2) : opt.warm_start;
        return std::min(w, hist);
    }

    CCTStatusType init(const CParameter* prm, const CGridBox* box, int max_particles, const MpsSolverOptions* o) {
        opt = *o;
        param = *prm;
        nmax = max_particles;
        d.box = *box;
        d.cells = box->m_GridSize.x * box->m_GridSize.y * box->m_GridSize.z;
        if (d.cells <= 0 || nmax <= 0) return CCT_PARAMERR;
        // row capacity: a multiple of 128 (16-byte vector rows), at most 512
        d.K = opt.max_neighbours > 0 ? opt.max_neighbours : 384;
        d.K = std::min(512, std::max(128, (d.K + 127) / 128 * 128));
        d.KG = 64;
        Consts& c = d.c;
        const CParameter& P = param;
        c.l0 = P.InitialParticleDistance;
        c.re_lap = (double)P.LaplacianInfluenceRadiusCoefficient * c.l0;
        c.re_grad = (double)P.GradientInfluenceRadiusCoefficient * c.l0;
        c.mind_lap = c.re_lap * 1e-3;
        c.mind_grad = c.re_grad * 1e-3;
        c.n0_pnd = opt.n0_pnd > 0 ? opt.n0_pnd : (double)P.ConstantParticleDensity;
        c.n0_lap = opt.n0_lap > 0 ? opt.n0_lap : (double)P.ConstantParticleDensity;
        const double lam = opt.lambda > 0 ? opt.lambda : (double)P.LambdaValue;
        c.dim = P.Dimension;
        c.coef_lap = 2.0 * c.dim / (lam * c.n0_lap);
        c.beta = P.FreeSurfaceThreshold;
        c.rho = P.Density;
        c.dt = P.Dt;
        c.kappa = opt.compressibility * c.rho / (c.dt * c.dt);
        c.c1 = 2.0 * c.dim / c.n0_pnd;
        c.c2 = c.rho / (c.dt * c.dt);
        c.vmax = c.l0 * (double)P.CourantNumber / c.dt;
        c.wall_fric = P.WallFrictionCoeffieicnt;
        c.offset_l0 = c.l0 * (double)P.OffSet;
        c.tol = P.Tolerance;
        c.sonic2 = (double)P.SonicVelocity * (double)P.SonicVelocity;
        c.gamma = opt.source_relaxation > 0 ? opt.source_relaxation : 1.0;
        c.g[0] = P.GravityConstant.x;
        c.g[1] = P.GravityConstant.y;
        c.g[2] = P.GravityConstant.z;
        c.explicit_pressure = opt.pressure_mode == MPS_PRESSURE_EXPLICIT;
        timer.on = opt.profile != 0;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return CCT_CUDAERR;
        for (auto& e : gate_ev)
            if (cudaEventCreate(&e) != cudaSuccess) return CCT_CUDAERR;
        // the second stream at a higher priority: the work it takes (wall bins, multilevel
        // setup) is on the step's critical path, and the solver-stream kernels beside it
        // (compaction, grid, transpose, first residual) fill the SMs it leaves
        int prio_low = 0, prio_high = 0;
        cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
        if (cudaStreamCreateWithPriority(&st2, cudaStreamNonBlocking, prio_high) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev_setup, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev_rows, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev_mg, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev_walls, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev_bins, cudaEventDisableTiming) != cudaSuccess)
            return CCT_CUDAERR;
        const size_t N = nmax;
        const size_t wsz = sizeof(double);   // room for FP64 rows: the precision can be switched
        cudaError_t e = cudaSuccess;
        e = e ? e : mk(&d.pos, N); e = e ? e : mk(&d.vel, N); e = e ? e : mk(&d.pos2, N); e = e ? e : mk(&d.vel2, N);
        e = e ? e : mk(&d.press, N); e = e ? e : mk(&d.press2, N); e = e ? e : mk(&d.visc, N); e = e ? e : mk(&d.visc2, N);
        e = e ? e : mk(&d.dph1, N); e = e ? e : mk(&d.dph2, N); e = e ? e : mk(&d.dph1b, N); e = e ? e : mk(&d.dph2b, N);
        e = e ? e : mk(&d.type, N); e = e ? e : mk(&d.type2, N); e = e ? e : mk(&d.id, N); e = e ? e : mk(&d.id2, N);
        e = e ? e : mk(&d.opos, N); e = e ? e : mk(&d.ovel, N);
        e = e ? e : mk(&d.key, N); e = e ? e : mk(&d.idx, N); e = e ? e : mk(&d.skey, N);
        d.zbits = d.cells < (1 << 24) ? 6 : 0;   // the sort key stays below 2^30
        e = e ? e : mk(&d.cstart, (size_t)d.cells); e = e ? e : mk(&d.cend, (size_t)d.cells);
        e = e ? e : mk(&d.cell_list, (size_t)d.cells); e = e ? e : mk(&d.cell_count, 1);
        e = e ? e : mk(&d.wdist, N); e = e ? e : mk(&d.wdir, 3 * N); e = e ? e : mk(&d.wid, N);
        e = e ? e : mk(&d.dragv, 3 * N);
        e = e ? e : mk(&d.tcs, 4 * (size_t)d.cells);   // list bounds of the 2 cells keys (walls, drag)
        const size_t N32 = (N + 31) / 32 * 32;
        e = e ? e : mk(&d.rnbr, N32 * d.K); e = e ? e : mk((char**)&d.rw, N32 * d.K * wsz);
        e = e ? e : mk(&d.nbr, N32 * d.K); e = e ? e : mk((char**)&d.nbrw, N32 * d.K * wsz);
        e = e ? e : mk(&d.nbr16, N32 * d.K); e = e ? e : mk(&d.sbase, N32 / 32 + 1);
        e = e ? e : mk(&d.skmax, N32 / 32 + 1);
        if (opt.inner_weights == 16) {
            e = e ? e : mk(&d.w16, N32 * d.K);
            e = e ? e : mk(&d.diag16, N);
        }
        e = e ? e : mk(&d.nbr_cnt, N);
        e = e ? e : mk(&d.gnbr, N * d.KG); e = e ? e : mk((char**)&d.gnbrr, N * d.KG * wsz);
        e = e ? e : mk(&d.gcnt, N);
        e = e ? e : mk(&d.pnd, N); e = e ? e : mk(&d.diag, N); e = e ? e : mk(&d.rhs, N); e = e ? e : mk(&d.sumw, N);
        e = e ? e : mk(&d.inner, N);
        e = e ? e : mk(&d.r, N); e = e ? e : mk(&d.z, N); e = e ? e : mk(&d.p, N); e = e ? e : mk(&d.q, N);
        e = e ? e : mk(&d.minv, N);
        e = e ? e : mk(&d.r32, N); e = e ? e : mk(&d.z32, N); e = e ? e : mk(&d.pf32, N); e = e ? e : mk(&d.q32, N);
        e = e ? e : mk(&d.d32, N); e = e ? e : mk(&d.m32, N);
        e = e ? e : mk(&d.xs, N); e = e ? e : mk(&d.p32, N);
        e = e ? e : mk(&d.red, 4 * (size_t)kRedBlocks);
        e = e ? e : mk(&d.scal, (size_t)S_COUNT);
        e = e ? e : mk(&d.red_count, 16);
        e = e ? e : mk(&d.err, 1);
        e = e ? e : mk(&d.istat, 4);
        e = e ? e : mk(&stage, 7 * N);
        e = e ? e : mk(&d.pprev, N);
        e = e ? e : mk(&d.feat, 12 * N);
        e = e ? e : mk(&d.mlp_out, 2 * N);
        e = e ? e : mk(&d.targets, 2 * N);
        e = e ? e : mk(&scan_sums, scan_tile_sums_capacity());
        e = e ? e : mk(&scan_sums2, scan_tile_sums_capacity());
        e = e ? e : mk(&keep, N + 1);
        e = e ? e : mk(&rank, N + 1);
        if (e != cudaSuccess) return CCT_MEMERR;
        sort_scratch_bytes = radix_scratch_bytes(nmax);
        if (cudaMalloc(&sort_scratch, sort_scratch_bytes) != cudaSuccess) return CCT_MEMERR;
        allocs.push_back(sort_scratch);
        if (cudaMallocHost((void**)&h_scal, sizeof(double) * S_COUNT) != cudaSuccess) return CCT_MEMERR;
        if (cudaMallocHost((void**)&h_int, sizeof(int) * 8) != cudaSuccess) return CCT_MEMERR;
        if (cudaMallocHost((void**)&h_bins, sizeof(int) * 8) != cudaSuccess) return CCT_MEMERR;
        if (opt.preconditioner == MPS_PRECOND_MULTILEVEL && !fp64()) {
            const CCTStatusType rc = mg_init();
            if (rc != CCT_NOERR) return rc;
        }
        cudaMemset(d.red_count, 0, sizeof(unsigned) * 16);
        cudaMemset(d.scal, 0, sizeof(double) * S_COUNT);
        cudaMemset(d.err, 0, sizeof(unsigned));
        return cudaDeviceSynchronize() == cudaSuccess ? CCT_NOERR : CCT_CUDAERR;
    }

    void destroy() {
        frames_wait();
        for (FrameSlot& f : fslot) {
            if (f.h) cudaFreeHost(f.h);
            if (f.ht) cudaFreeHost(f.ht);
            if (f.copied) cudaEventDestroy(f.copied);
        }
        // d_frame, d_ftype, d_fflag and the inflow buffers come from mk(): freed with
        // `allocs` below; the bucket staging does not
        if (d_bucket) cudaFree(d_bucket);
        d_bucket = nullptr;
        if (ev_packed) cudaEventDestroy(ev_packed);
        if (st_io) cudaStreamDestroy(st_io);
        cudaDeviceSynchronize();
        for (void* p : allocs) cudaFree(p);
        allocs.clear();
        if (bin_off) cudaFree(bin_off);
        if (bin_visit) cudaFree(bin_visit);
        if (bin_sort) cudaFree(bin_sort);
        if (d.tri) cudaFree(d.tri);
        if (d.tnrm) cudaFree(d.tnrm);
        if (d.tmodel) cudaFree(d.tmodel);
        if (d.tparams) cudaFree(d.tparams);
        if (d.tri32) cudaFree(d.tri32);
        if (d.tdrag) cudaFree(d.tdrag);
        if (d.drag) cudaFree(d.drag);
        if (h_scal) cudaFreeHost(h_scal);
        if (h_int) cudaFreeHost(h_int);
        if (h_bins) cudaFreeHost(h_bins);
        if (h_counts) cudaFreeHost(h_counts);
        timer.release();
        if (mlp) mps_mlp_destroy(mlp);
        mlp = nullptr;
        if (st) cudaStreamDestroy(st);
        if (st2) cudaStreamDestroy(st2);
        if (ev_setup) cudaEventDestroy(ev_setup);
        if (ev_rows) cudaEventDestroy(ev_rows);
        if (ev_mg) cudaEventDestroy(ev_mg);
        if (ev_walls) cudaEventDestroy(ev_walls);
        if (ev_bins) cudaEventDestroy(ev_bins);
        for (auto& e : gate_ev)
            if (e) cudaEventDestroy(e);
    }

    void swap_state() {
        std::swap(d.pos, d.pos2);
        std::swap(d.vel, d.vel2);
        std::swap(d.press, d.press2);
        std::swap(d.visc, d.visc2);
        std::swap(d.type, d.type2);
        std::swap(d.id, d.id2);
        std::swap(d.dph1, d.dph1b);
        std::swap(d.dph2, d.dph2b);
    }

    CCTStatusType set_particles(int n, const double* pos, const double* vel, const double* press, const double* visc,
                                const int* type) {
        if (n < 0 || n > nmax) return CCT_PARAMERR;
        std::vector<dbl4> P(n), V(n);
        std::vector<double> pr(n, 0.0);
        std::vector<float> vi(n);
        std::vector<int> ty(n, 0), id(n);
        for (int i = 0; i < n; ++i) {
            P[i] = make_dbl4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 0.0);
            V[i] = make_dbl4(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2], 0.0);
            if (press) pr[i] = press[i];
            vi[i] = (float)visc[i];
            if (type) ty[i] = type[i];
            id[i] = i;
        }
        d.n = n;
        idext = n;
        cudaError_t e = cudaMemcpyAsync(d.pos, P.data(), sizeof(dbl4) * n, cudaMemcpyHostToDevice, st);
        if (!e) e = cudaMemcpyAsync(d.vel, V.data(), sizeof(dbl4) * n, cudaMemcpyHostToDevice, st);
        if (!e) e = cudaMemcpyAsync(d.press, pr.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st);
        if (!e) e = cudaMemcpyAsync(d.visc, vi.data(), sizeof(float) * n, cudaMemcpyHostToDevice, st);
        if (!e) e = cudaMemcpyAsync(d.type, ty.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
        if (!e) e = cudaMemcpyAsync(d.id, id.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
        if (!e) e = cudaMemsetAsync(d.dph1, 0, sizeof(float) * std::max(n, 1), st);
        if (!e) e = cudaMemsetAsync(d.dph2, 0, sizeof(float) * std::max(n, 1), st);
        if (!e) e = cudaStreamSynchronize(st);
        hist = 0;
        return cuda_status(e);
    }

    CCTStatusType set_triangles(int t, const double* v, const int* model, int nmodels, const CTriangleParameters* tp) {
        if (d.tri) { cudaFree(d.tri); cudaFree(d.tnrm); cudaFree(d.tmodel); cudaFree(d.tparams); cudaFree(d.tri32); cudaFree(d.tdrag); }
        d.tri = nullptr; d.tnrm = nullptr; d.tmodel = nullptr; d.tparams = nullptr; d.tri32 = nullptr; d.tdrag = nullptr;
        d.tri_n = t;
        models = nmodels;
        walls_move = 0;
        for (int m = 0; m < nmodels; ++m) {
            const Scalar3 vv = tp[m].Velocity;
            if (tp[m].RotatingOrNot || vv.x != 0 || vv.y != 0 || vv.z != 0) walls_move = 1;
        }
        if (t <= 0) return CCT_NOERR;
        std::vector<double> nrm(3 * (size_t)t);
        for (int i = 0; i < t; ++i) {
            const double* q = v + 9 * (size_t)i;
            const double e1[3] = {q[3] - q[0], q[4] - q[1], q[5] - q[2]}, e2[3] = {q[6] - q[0], q[7] - q[1], q[8] - q[2]};
            double n3[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            const double l = std::sqrt(n3[0] * n3[0] + n3[1] * n3[1] + n3[2] * n3[2]);
            for (int a = 0; a < 3; ++a) nrm[3 * (size_t)i + a] = l > 0 ? n3[a] / l : 0.0;
        }
        cudaError_t e = cudaMalloc(&d.tri, sizeof(double) * 9 * (size_t)t);
        if (!e) e = cudaMalloc(&d.tnrm, sizeof(double) * 3 * (size_t)t);
        if (!e) e = cudaMalloc(&d.tmodel, sizeof(int) * (size_t)t);
        if (!e) e = cudaMalloc(&d.tparams, sizeof(CTriangleParameters) * std::max(nmodels, 1));
        if (!e) e = cudaMalloc(&d.tri32, sizeof(float) * 9 * (size_t)t);
        if (!e) e = cudaMalloc(&d.tdrag, (size_t)t);
        if (e) return CCT_MEMERR;
        std::vector<float> v32(9 * (size_t)t);
        std::vector<unsigned char> fl((size_t)t);
        for (size_t k = 0; k < v32.size(); ++k) v32[k] = (float)v[k];
        for (int k = 0; k < t; ++k) fl[k] = (model[k] >= 0 && model[k] < nmodels && tp[model[k]].isDrag) ? 1 : 0;
        e = cudaMemcpy(d.tri, v, sizeof(double) * 9 * (size_t)t, cudaMemcpyHostToDevice);
        if (!e) e = cudaMemcpy(d.tnrm, nrm.data(), sizeof(double) * 3 * (size_t)t, cudaMemcpyHostToDevice);
        if (!e) e = cudaMemcpy(d.tmodel, model, sizeof(int) * (size_t)t, cudaMemcpyHostToDevice);
        if (!e) e = cudaMemcpy(d.tparams, tp, sizeof(CTriangleParameters) * nmodels, cudaMemcpyHostToDevice);
        if (!e) e = cudaMemcpy(d.tri32, v32.data(), sizeof(float) * v32.size(), cudaMemcpyHostToDevice);
        if (!e) e = cudaMemcpy(d.tdrag, fl.data(), (size_t)t, cudaMemcpyHostToDevice);
        bins_dirty = 1;
        return cuda_status(e);
    }

    CCTStatusType set_drag(int count, const DragParameter* dp) {
        if (d.drag) cudaFree(d.drag);
        d.drag = nullptr;
        d.drag_n = count;
        if (count <= 0) return CCT_NOERR;
        if (cudaMalloc(&d.drag, sizeof(DragParameter) * count)) return CCT_MEMERR;
        return cuda_status(cudaMemcpy(d.drag, dp, sizeof(DragParameter) * count, cudaMemcpyHostToDevice));
    }

    // ---- multilevel preconditioner ----
    // level grids halve (rounding up) until one cell; cell coordinates are packed
    // in 10 bits, so every grid dimension must be below 1024
    CCTStatusType mg_init() {
        if (mg_init_done) return CCT_NOERR;
        mg_init_done = true;
        const CGridBox& b = d.box;
        if (b.m_GridSize.x >= 1024 || b.m_GridSize.y >= 1024 || b.m_GridSize.z >= 1024) return CCT_NOERR;
        int gx = b.m_GridSize.x, gy = b.m_GridSize.y, gz = b.m_GridSize.z;
        cudaError_t e = cudaSuccess;
        int l = 1;
        for (; l <= kMgMaxLevels; ++l) {
            MgLevel& L = mg.L[l];
            L.gx = gx; L.gy = gy; L.gz = gz; L.n = 0;
            const size_t nc = (size_t)gx * gy * gz;
            e = e ? e : mk(&L.cmap, nc); e = e ? e : mk(&L.ccell, nc); e = e ? e : mk(&L.nb, 27 * nc);
            e = e ? e : mk(&L.par, nc); e = e ? e : mk(&L.a, 27 * nc); e = e ? e : mk(&L.dinv, nc);
            e = e ? e : mk(&L.r, nc); e = e ? e : mk(&L.e, nc); e = e ? e : mk(&L.e2, nc);
            e = e ? e : mk(&L.child, 8 * nc); e = e ? e : mk(&L.nbp, 27 * nc);
            if (nc == 1) break;
            gx = (gx + 1) / 2; gy = (gy + 1) / 2; gz = (gz + 1) / 2;
        }
        mg_grid_levels = std::min(l, kMgMaxLevels);
        e = e ? e : mk(&mg.ainv, (size_t)kMgMaxDense * kMgMaxDense);
        // [0]: k_mg_down's finished CTAs; [1], [2]: k_mg_coarse_cycle's grid barrier
        e = e ? e : mk(&mg.done, 3);
        if (!e) e = cudaMemset(mg.done, 0, 3 * sizeof(unsigned));
        e = e ? e : mk(&mg.agg1, (size_t)nmax); e = e ? e : mk(&mg.pcc, (size_t)nmax);
        e = e ? e : mk(&mg.part, 27 * (size_t)nmax); e = e ? e : mk(&mg.partd, (size_t)nmax);
        e = e ? e : mk(&mg.rb, (size_t)d.cells + 1);
        e = e ? e : mk(&mg_flag, (size_t)d.cells + 1); e = e ? e : mk(&mg_counts, (size_t)kMgMaxLevels + 1);
        if (opt.fine_smoother == 1) {
            e = e ? e : mk(&sm_R, 27 * (size_t)nmax);
            e = e ? e : mk(&sm_mask, (size_t)nmax);
        }
        if (e) return CCT_MEMERR;
        if (cudaMallocHost((void**)&h_counts, sizeof(unsigned) * (kMgMaxLevels + 1)) != cudaSuccess) return CCT_MEMERR;
        const int smem = (kMgMaxDense * kMgMaxDense + kMgMaxDense) * (int)sizeof(float);
        if (cudaFuncSetAttribute(k_mg_dense_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) return CCT_CUDAERR;
        mg.omega = opt.mg_omega > 0 ? (float)opt.mg_omega : 1.3f;
        mg_on = mg_grid_levels >= 1;
        return CCT_NOERR;
    }

    // level-1 Galerkin stencil of the current rows (mg.L[1].a, dinv): variant 1 streams
    // the 16-bit slices' rows through shared memory, 0 walks them from registers (same
    // sums), -1 follows spmv_stream
    int asm_grid = 0;
    CCTStatusType mg_assemble(cudaStream_t ss, int variant) {
        const bool stream = variant < 0 ? use_stream() : variant == 1;
        if (stream) {
            auto k = k_mg_assemble_stream<kSsEntries, kSsStages, kSsWarps, kSsMinBlocks>;
            const int g = stream_grid_for(k, kSsSmem, asm_grid);
            if (g < 0) return CCT_CUDAERR;
            MPS_COUNT_LAUNCH k<<<g, kSsWarps * 32, kSsSmem, ss>>>(d, mg, (const float*)d.nbrw);
        } else {
            MPS_COUNT_LAUNCH k_mg_assemble_rows<float><<<kRedBlocks, kMgAsmWarps * 32, 0, ss>>>(d, mg,
                                                                                           (const float*)d.nbrw);
        }
        MPS_COUNT_LAUNCH k_mg_assemble_cells<<<div_up(mg.L[1].n * 32, 256), 256, 0, ss>>>(d, mg);
        return cuda_status(cudaGetLastError());
    }

    // aggregates, links and operators of the current particle order (after the PPE
    // setup: needs interior flags, diagonals and the FP32 neighbour rows)
    // In two parts: the topology (aggregate flags and counts of every level) needs only
    // the cell grid and the interior flags, the rest waits for the level counts on the
    // host and, from the Galerkin assembly on, for the rows (rows_ready when given).
    bool mg_topo_pending = false;   // mg_setup_topology ran, mg_setup_finish has not
    CCTStatusType mg_setup(cudaStream_t ss) {
        const CCTStatusType rc = mg_setup_topology(ss);
        return rc != CCT_NOERR ? rc : mg_setup_finish(ss, nullptr);
    }
    CCTStatusType mg_setup_topology(cudaStream_t ss) {
        mg_ready = false;
        mg_topo_pending = false;
        if (opt.preconditioner != MPS_PRECOND_MULTILEVEL && !mg_init_done) return CCT_NOERR;
        if (opt.preconditioner == MPS_PRECOND_MULTILEVEL && !mg_init_done) {
            const CCTStatusType rc = mg_init();
            if (rc != CCT_NOERR) return rc;
        }
        if (!mg_on || opt.preconditioner != MPS_PRECOND_MULTILEVEL || d.n <= 0) return CCT_NOERR;
        MgLevel* L = mg.L;
        MPS_COUNT_LAUNCH k_mg_flags1<<<blocks_for(d.cells), kBlock, 0, ss>>>(d, mg_flag);
        for (int l = 1; l <= mg_grid_levels; ++l) {
            const int nc = L[l].gx * L[l].gy * L[l].gz;
            if (l > 1) MPS_COUNT_LAUNCH k_mg_flags_up<<<blocks_for(nc), kBlock, 0, ss>>>(L[l - 1], L[l], mg_flag);
            if (scan_exclusive(mg_flag, nc, mg_flag + nc, ss, scan_sums)) return CCT_CUDAERR;
            MPS_COUNT_LAUNCH k_mg_fill<<<blocks_for(nc), kBlock, 0, ss>>>(L[l], mg_flag);
            cudaMemcpyAsync(mg_counts + l, mg_flag + nc, sizeof(unsigned), cudaMemcpyDeviceToDevice, ss);
        }
        cudaMemcpyAsync(h_counts, mg_counts, sizeof(unsigned) * (kMgMaxLevels + 1), cudaMemcpyDeviceToHost, ss);
        mg_topo_pending = true;
        return cuda_status(cudaGetLastError());
    }
    CCTStatusType mg_setup_finish(cudaStream_t ss, cudaEvent_t rows_ready) {
        if (!mg_topo_pending) return CCT_NOERR;
        mg_topo_pending = false;
        MgLevel* L = mg.L;
        if (cudaStreamSynchronize(ss)) return CCT_CUDAERR;
        int levels = 0;
        for (int l = 1; l <= mg_grid_levels; ++l) {
            L[l].n = (int)h_counts[l];
            if (!levels && L[l].n <= kMgMaxDense) levels = l;
        }
        if (!levels || L[1].n <= 0) return CCT_NOERR;   // no small enough level: Jacobi this step
        mg.levels = levels;
        for (int l = 2; l <= levels; ++l) cudaMemsetAsync(L[l].child, 0xff, sizeof(int) * 8 * (size_t)L[l].n, ss);
        for (int l = 1; l <= levels; ++l)
            MPS_COUNT_LAUNCH k_mg_links<<<blocks_for(L[l].n), kBlock, 0, ss>>>(L[l], L[l < levels ? l + 1 : l], l < levels);
        for (int l = 1; l < levels; ++l)
            MPS_COUNT_LAUNCH k_mg_nbpar<<<blocks_for(27 * L[l].n), kBlock, 0, ss>>>(L[l]);
        MPS_COUNT_LAUNCH k_mg_particles<<<blocks_for(d.n), kBlock, 0, ss>>>(d, mg);
        MPS_COUNT_LAUNCH k_mg_rows<<<blocks_for(L[1].n), kBlock, 0, ss>>>(d, mg);
        if (rows_ready) cudaStreamWaitEvent(ss, rows_ready, 0);
        if (mg_assemble(ss, -1) != CCT_NOERR) return CCT_CUDAERR;
        for (int l = 1; l < levels; ++l)
            MPS_COUNT_LAUNCH k_mg_coarsen<<<div_up(L[l + 1].n, kMgCoarsenWarps), kMgCoarsenWarps * 32, 0, ss>>>(L[l], L[l + 1]);
        const int nd = L[levels].n;
        MPS_COUNT_LAUNCH k_mg_dense_inverse<<<1, 1024, (nd * nd + nd) * sizeof(float), ss>>>(L[levels], mg.ainv);
        if (fine_post())
            MPS_COUNT_LAUNCH k_mg_smoother_rows<<<blocks_for(d.n, kMgSmThreads), kMgSmThreads, 0, ss>>>(d, mg, sm_R,
                                                                                                       sm_mask);
        if (cudaGetLastError()) return CCT_CUDAERR;
        mg_ready = true;
        return CCT_NOERR;
    }

    // flexible CG for this step's inner solve (see MpsSolverOptions::flexible)
    bool flex_step = false;
    bool flexible_now() const {
        if (opt.flexible != 0) return opt.flexible > 0;
        return fine_post() || (learned_ready && (opt.learned & 2) != 0);
    }
    // post-smoothing fine level of the multilevel preconditioner (fine_smoother 1)
    float* sm_R = nullptr;       // [27 n] couplings lumped per neighbouring cell
    unsigned* sm_mask = nullptr; // [n] nonzero slots
    bool fine_post() const { return opt.fine_smoother == 1 && sm_R && mg_on && !fp64(); }
    // z = M^-1 r (interior rows), rz; mode 1 also sets p = z and S_RZ, mode 0 S_BETA.
    // restricted = true: level-1 r and the first sweep are already done (by
    // k_mg_update_restrict)
    // CTAs of the cooperative coarse V-cycle: all resident (SMs x the CTAs that fit),
    // no more than the level-2 aggregates need (a warp each); 0: not available
    int coop_resident = -1;
    unsigned* coop_bar = nullptr;
    int coarse_cycle_grid() {
        if (coop_resident < 0) {
            int dev = 0, sms = 0, per_sm = 0, coop = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
            if (!coop || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mg_coarse_cycle, 256, 0) != cudaSuccess)
                per_sm = 0;
            coop_resident = sms * per_sm;
            coop_bar = mg.done + 1;
        }
        if (coop_resident <= 0) return 0;
        return std::max(1, std::min(coop_resident, div_up(mg.L[2].n, 8)));
    }

    void mg_apply(const float* r, float* z, float* p, int mode, bool restricted = false) {
        MgLevel* L = mg.L;
        const int lv = mg.levels;
        const float om = mg.omega;
        if (!restricted)
            MPS_COUNT_LAUNCH k_mg_restrict_fine<float><<<div_up(L[1].n * 32, 256), 256, 0, st>>>(d, mg, r);
        // additional level-1 sweeps before the restriction and after the prolongation
        const int extra = lv > 1 ? std::max(0, opt.mg_sweeps - 1) : 0;
        for (int k = 0; k < extra; ++k) {
            MPS_COUNT_LAUNCH k_mg_smooth<<<div_up(L[1].n * 32, 256), 256, 0, st>>>(d.scal, L[1], L[1].e, L[1].e2, om);
            std::swap(L[1].e, L[1].e2);
        }
        // the level-2 -> level-1 up sweep carries the fine level when no extra level-1
        // sweeps follow it (and the reduction buffer holds its CTAs' partials)
        const int up1_blocks = div_up(L[1].n, kMgUpAgg * 8);   // 8 warps per CTA
        const bool post = fine_post();
        // the reduction buffer holds 2 partials per CTA of the fused kernel
        const bool fuse = !post && lv >= 2 && extra == 0 && up1_blocks <= 2 * kRedBlocks;
        const float* qf = (flex_step && mode == 0) ? d.q32 : nullptr;
        const int cg = fuse ? coarse_cycle_grid() : 0;
        if (cg > 0) {
            // levels 2 .. last in one cooperative launch (grid barriers between stages)
            void* args[] = {(void*)&d.scal, (void*)&mg, (void*)&coop_bar, (void*)&d.err};
            MPS_COUNT_LAUNCH cudaLaunchCooperativeKernel((const void*)k_mg_coarse_cycle, dim3(cg), dim3(256), args, 0,
                                                         st);
        } else {
            // the last restriction also solves the last level densely (its last CTA, of
            // 1024 threads like the stand-alone dense solve)
            for (int l = 1; l < lv; ++l) {
                const int tpb = l + 1 == lv ? 1024 : 256;
                MPS_COUNT_LAUNCH k_mg_down<<<div_up(L[l + 1].n * 32, tpb), tpb, 0, st>>>(
                    d.scal, L[l], L[l + 1], om, l + 1 == lv ? mg.ainv : nullptr, mg.done);
            }
            if (lv == 1) MPS_COUNT_LAUNCH k_mg_dense_solve<<<1, 1024, 0, st>>>(d.scal, L[lv], mg.ainv);
            for (int l = lv - 1; l >= (fuse ? 2 : 1); --l)
                MPS_COUNT_LAUNCH k_mg_up<<<div_up(L[l].n * 32, 256), 256, 0, st>>>(d.scal, L[l], L[l + 1], om);
        }
        if (fuse) {
            if (pdl) {
                if (MPS_COUNT_LAUNCH launch_pdl(k_mg_up_fine_z<float>, up1_blocks, 256, 0, st, d, mg, r, z, p,
                                                (const float*)d.m32, mode, 7, qf))
                    stream_failed = true;
            } else {
                MPS_COUNT_LAUNCH k_mg_up_fine_z<float><<<up1_blocks, 256, 0, st>>>(d, mg, r, z, p, d.m32, mode, 7, qf);
            }
            return;
        }
        for (int k = 0; k < extra; ++k) {
            MPS_COUNT_LAUNCH k_mg_smooth<<<div_up(L[1].n * 32, 256), 256, 0, st>>>(d.scal, L[1], L[1].e2, L[1].e, om);
            std::swap(L[1].e, L[1].e2);
        }
        if (post)
            MPS_COUNT_LAUNCH k_mg_fine_post<float><<<kRedBlocks, 256, 0, st>>>(d, mg, r, z, p, d.m32, mode, 7, qf, sm_R,
                                                                                sm_mask, (float)opt.smoother_weight);
        else
            MPS_COUNT_LAUNCH k_mg_fine_z<float><<<kRedBlocks, 256, 0, st>>>(d, mg, r, z, p, d.m32, mode, 7, qf);
    }

    // ---- phases ----
    CCTStatusType compact() {
        compact_launch();
        return compact_finish();
    }
    // the compaction's launches (no host wait) and, after them, the wait for the new count
    void compact_launch() {
        const int n = d.n;
        if (n <= 0) return;
        MPS_COUNT_LAUNCH k_zone_flags<<<blocks_for(n), kBlock, 0, st>>>(d, keep);
        cudaMemcpyAsync(rank, keep, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, st);
        scan_exclusive(rank, n, rank + n, st, scan_sums);
        MPS_COUNT_LAUNCH k_compact<<<blocks_for(n), kBlock, 0, st>>>(d, keep, rank);
        cudaMemcpyAsync(h_int, rank + n, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    }
    CCTStatusType compact_finish() {
        if (d.n <= 0) return CCT_NOERR;
        if (cudaStreamSynchronize(st) != cudaSuccess) return CCT_CUDAERR;
        swap_state();
        d.n = h_int[0];
        return CCT_NOERR;
    }

    CCTStatusType grid() {
        const int n = d.n;
        if (n <= 0) {   // no particles: empty cell tables (the neighbour passes find no cell)
            cudaMemsetAsync(d.cell_count, 0, sizeof(int), st);
            return cuda_status(cudaGetLastError());
        }
        MPS_COUNT_LAUNCH k_hash<<<blocks_for(n), kBlock, 0, st>>>(d);
        const unsigned krange = ((unsigned)d.cells << d.zbits) - 1u;
        if (radix_sort_pairs(n, d.skey, d.idx, 0, radix_passes(krange), sort_scratch, st)) return CCT_CUDAERR;
        cudaMemsetAsync(d.cstart, 0xff, sizeof(int) * d.cells, st);
        cudaMemsetAsync(d.cend, 0xff, sizeof(int) * d.cells, st);
        cudaMemsetAsync(d.cell_count, 0, sizeof(int), st);
        MPS_COUNT_LAUNCH k_gather<<<blocks_for(n), kBlock, 0, st>>>(d);
        swap_state();
        return cuda_status(cudaGetLastError());
    }

    // on stream ss with its own host buffer and scan scratch (the second stream, beside
    // the particles' compaction, in a step)
    CCTStatusType bin_walls(cudaStream_t ss, int* hb, unsigned* scr) {
        const int t = d.tri_n;
        if (t <= 0) return CCT_NOERR;
        // counts (t + 1 with the scan's total) and the 64-bit sum of the counts behind them
        if ((size_t)t > bin_off_cap) {   // sized for the largest wall set seen
            if (bin_off) cudaFree(bin_off);
            bin_off = nullptr;
            bin_off_cap = 0;
            if (cudaMalloc(&bin_off, sizeof(unsigned) * ((size_t)t + 2) + sizeof(unsigned long long) * 2))
                return CCT_MEMERR;
            bin_off_cap = (size_t)t;
        }
        unsigned long long* total = (unsigned long long*)(bin_off + ((size_t)t + 3) / 2 * 2);
        cudaMemsetAsync(total, 0, sizeof(unsigned long long), ss);
        MPS_COUNT_LAUNCH k_bin_count<<<blocks_for(t), kBlock, 0, ss>>>(d, bin_off, total);
        cudaMemcpyAsync(hb + 4, total, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ss);
        if (cudaStreamSynchronize(ss)) return CCT_CUDAERR;
        unsigned long long total_h = 0;
        std::memcpy(&total_h, hb + 4, sizeof(total_h));
        // every (cell, triangle) entry is indexed by an int in the sort and by the 32-bit
        // scan: a wall whose boxes hold more entries is refused, never truncated
        if (total_h > (unsigned long long)INT32_MAX) {
            note_message("wall bins: the triangles' cell boxes hold more than 2^31 - 1 (cell, triangle) entries");
            return CCT_MEMERR;
        }
        scan_exclusive(bin_off, t + 1, nullptr, ss, scr);
        cudaMemcpyAsync(hb, bin_off + t, sizeof(unsigned), cudaMemcpyDeviceToHost, ss);
        if (cudaStreamSynchronize(ss)) return CCT_CUDAERR;
        const unsigned nv = (unsigned)hb[0];
        bin_entries = (int)nv;
        if (nv == 0) {
            cudaMemsetAsync(d.tcs, 0xff, sizeof(int) * 4 * d.cells, ss);
            bins_dirty = 0;
            return CCT_NOERR;
        }
        if (nv > bin_visit_cap) {
            if (bin_visit) cudaFree(bin_visit);
            if (bin_sort) cudaFree(bin_sort);
            bin_visit_cap = std::min<size_t>((size_t)nv + nv / 2, (size_t)INT32_MAX);
            if (cudaMalloc(&bin_visit, sizeof(int) * 2 * bin_visit_cap)) return CCT_MEMERR;
            bin_sort_bytes = radix_scratch_bytes((int)bin_visit_cap);
            if (cudaMalloc(&bin_sort, bin_sort_bytes)) return CCT_MEMERR;
            d.tids = bin_visit + bin_visit_cap;
        }
        int* vcell = bin_visit;
        d.tids = bin_visit + bin_visit_cap;
        MPS_COUNT_LAUNCH k_bin_fill<<<div_up(t * 32, 256), 256, 0, ss>>>(d, bin_off, vcell, d.tids);
        if (radix_sort_pairs((int)nv, vcell, d.tids, 0, radix_passes((unsigned)(2 * d.cells - 1)), bin_sort, ss))
            return CCT_CUDAERR;
        cudaMemsetAsync(d.tcs, 0xff, sizeof(int) * 4 * d.cells, ss);
        MPS_COUNT_LAUNCH k_bin_bounds<<<blocks_for((int)nv), kBlock, 0, ss>>>((int)nv, vcell, d.tcs,
                                                                               d.tcs + 2 * d.cells);
        bins_dirty = 0;
        return cuda_status(cudaGetLastError());
    }

    // SELL-32 transpose of the current rows (k_rows_sell flags)
    void rows_sell(int flags) {
        const int slices = (d.n + 31) / 32;
        if (slices == 0) return;
        if (fp64())
            MPS_COUNT_LAUNCH k_rows_sell<double><<<div_up(slices, rows_sell_warps<double>()), rows_sell_warps<double>() * 32,
                                                   0, st>>>(d, flags);
        else if (opt.rows_sell == 1)
            MPS_COUNT_LAUNCH k_rows_sell<float><<<div_up(slices, rows_sell_warps<float>()), rows_sell_warps<float>() * 32,
                                                  0, st>>>(d, flags);
        else
            MPS_COUNT_LAUNCH k_rows_sell_async<<<div_up(slices, kRsWarps), kRsWarps * 32, 0, st>>>(d, flags);
    }
    // the 32-bit columns of every slice (debug entries that force the wide SpMV)
    void ensure_cols32() {
        if (d.rows_c32 || d.n <= 0) return;
        rows_sell(d.rows16 | (d.rows_w16 << 1) | 4 | 8);
        d.rows_c32 = 1;
    }

    template <class T>
    void walls_distance() {
        if (d.tri_n > 0) {
            MPS_COUNT_LAUNCH k_wall_distance<T><<<blocks_for(d.n), kBlock, 0, st>>>(d);
        } else {
            cudaMemsetAsync(d.wid, 0xff, sizeof(int) * d.n, st);
        }
    }

    template <class T>
    // One step; pressure_only: only topology, walls, PND and the PPE solve at the
    // current positions (no predictor, no correction, walls do not move).
    CCTStatusType run_step(int step, MpsStepStats* out, bool pressure_only = false) {
        MpsStepStats S{};
        spmv_launches = 0;
        feat_valid = false;
        prefer_wide = opt.spmv_wide == 1 || (opt.spmv_wide == 0 && last.nnz > 0 && 2 * last.nnz_wide > last.nnz);
        residual_ready = false;
        d.rows16 = 0;
        d.rows_w16 = 0;
        d.rows_c32 = 0;
        timer.mark(PH_GRID, st);
        cudaMemsetAsync(d.err, 0, sizeof(unsigned), st);
        cudaMemsetAsync(d.istat, 0, 2 * sizeof(int), st);
        CCTStatusType rc;
        if (!pressure_only) {
            // the wall bins (the triangles moved at the end of the last step) on the second
            // stream, their host waits and kernels beside the compaction and the grid
            const bool bins = d.tri_n > 0 && bins_dirty;
            if (bins) cudaEventRecord(ev_walls, st);
            compact_launch();
            if (bins) {
                cudaStreamWaitEvent(st2, ev_walls, 0);
                if ((rc = bin_walls(st2, h_bins, scan_sums2))) return rc;
                cudaEventRecord(ev_bins, st2);
            }
            if ((rc = compact_finish())) return rc;
            if ((rc = grid())) return rc;
            timer.mark(PH_WALLS, st);
            if (bins) cudaStreamWaitEvent(st, ev_bins, 0);
            walls_distance<T>();
            if (d.drag_n > 0 && d.tri_n > 0) MPS_COUNT_LAUNCH k_drag<T><<<blocks_for(d.n), kBlock, 0, st>>>(d);
            else cudaMemsetAsync(d.dragv, 0, sizeof(double) * 3 * d.n, st);
            timer.mark(PH_PRED, st);
            const int nb_grid = std::max(1, std::min(d.cells, d.n));
            MPS_COUNT_LAUNCH k_neighbours<T, NB_PREDICT><<<nb_grid, kNbThreads, 0, st>>>(d);
            std::swap(d.pos, d.pos2);
            std::swap(d.vel, d.vel2);
            timer.mark(PH_GRID, st);
        }
        if ((rc = compact())) return rc;
        if ((rc = grid())) return rc;
        timer.mark(PH_WALLS, st);
        if (pressure_only && d.tri_n > 0 && bins_dirty && (rc = bin_walls(st, h_int, scan_sums))) return rc;
        walls_distance<T>();
        timer.mark(PH_LIST, st);
        const int nb_cells = std::max(1, std::min(d.cells, d.n));
        MPS_COUNT_LAUNCH k_neighbours<T, NB_LIST><<<nb_cells, kNbThreads, 0, st>>>(d);
        timer.mark(PH_SETUP, st);
        if (opt.pressure_mode == MPS_PRESSURE_EXPLICIT) {
            MPS_COUNT_LAUNCH k_eos<<<blocks_for(d.n), kBlock, 0, st>>>(d);
        } else {
            MPS_COUNT_LAUNCH k_ppe_setup<<<blocks_for(d.n), kBlock, 0, st>>>(d);
            MPS_COUNT_LAUNCH k_count_nnz<<<kRedBlocks, 256, 0, st>>>(d, 4);
            // the multilevel setup runs on the second stream: its topology (grid and
            // interior flags only) beside the rows' transpose, its operators from the rows
            // on, beside the warm start, the first refinement residual and the learned guess
            const bool overlap_mg = !fp64() && opt.preconditioner == MPS_PRECOND_MULTILEVEL;
            mg_setup_done = false;
            if (overlap_mg) {
                cudaEventRecord(ev_setup, st);
                cudaStreamWaitEvent(st2, ev_setup, 0);
                if (mg_setup_topology(st2)) return CCT_CUDAERR;
            }
            // SELL-32 rows from the list pass's row-major rows: 16-bit column offsets for
            // the streamed SpMVs (the FP64 solver streams them with its FP64 weights), FP16
            // weight copies only for the FP32 inner CG, 32-bit columns where they are read
            {
                const int narrow = (opt.compress_rows && (!fp64() || opt.spmv_stream)) ? 1 : 0;
                const int w16 = (narrow && !fp64() && want_inner16() && d.w16) ? 1 : 0;
                // 32-bit columns: the wide streamed kernels, the register walks of uncompressed
                // rows, the non-streamed refinement residual (k_residual_df) and every FP64
                // register walk (the FP64 learned-guess SpMVs, the stream's timeout fallback)
                const int full32 = (!narrow || prefer_wide || !opt.spmv_stream || fp64()) ? 1 : 0;
                rows_sell(narrow | (w16 << 1) | (full32 << 2));
                d.rows16 = narrow;
                d.rows_w16 = w16;
                d.rows_c32 = full32;
            }
            bool use_learned = learned_ready && opt.learned && d.n > 0;
            // the gate: a learned guess that cost more than it saved sits out a few steps
            if (use_learned && opt.learned_gate && !fp64() && gate_skip > 0) {
                --gate_skip;
                use_learned = false;
            }
            // gated steps time the span from here to the solve (with and without the guess)
            const bool gated = learned_ready && opt.learned && opt.learned_gate && !fp64();
            if (gated) cudaEventRecord(gate_ev[0], st);
            S.learned_applied = use_learned ? 1 : 0;
            flex_step = flexible_now();
            S.flexible = flex_step ? 1 : 0;
            if (overlap_mg) cudaEventRecord(ev_rows, st);
            const int warm = warm_order();
            MPS_COUNT_LAUNCH k_warm_start<<<blocks_for(d.n), kBlock, 0, st>>>(d, warm);
            S.warm_start = warm;
            if (use_learned || collect) {
                timer.mark(PH_LEARNED, st);
                if (fp64())
                    MPS_COUNT_LAUNCH k_spmv<double, double, double, 1><<<kRedBlocks, 256, 0, st>>>(d, (const double*)d.nbrw, d.press,
                                                                                  d.r, d.rhs, 2);
                else
                    residual_df((const float*)d.nbrw);
                MPS_COUNT_LAUNCH k_pressure_scale<<<kRedBlocks, 256, 0, st>>>(d, 5);
                MPS_COUNT_LAUNCH k_to_float_p<<<blocks_for(d.n), kBlock, 0, st>>>(d.n, d.press, d.pf32);
                MPS_COUNT_LAUNCH k_features<T><<<blocks_for(d.n), kBlock, 0, st>>>(d);
                feat_valid = true;
                if (use_learned) {
                    if (mlp_forward(mlp, d.n, d.feat, d.mlp_out, st, d.err)) return CCT_CUDAERR;
                    MPS_COUNT_LAUNCH k_learned_apply<<<blocks_for(d.n), kBlock, 0, st>>>(d, (opt.learned & 2) ? 1 : 0);
                    if (fp64())
                        MPS_COUNT_LAUNCH k_spmv<double, double, double, 2><<<kRedBlocks, 256, 0, st>>>(d, (const double*)d.nbrw, d.z,
                                                                                      d.q, d.r, 6);
                    else   // FP32 products: the line search needs no more
                        spmv_ls((const float*)d.nbrw);
                    if (stream_failed) return CCT_CUDAERR;
                    if (fp64()) {
                        MPS_COUNT_LAUNCH k_learned_finish<<<blocks_for(d.n), kBlock, 0, st>>>(d);
                    } else {
                        MPS_COUNT_LAUNCH k_learned_finish_r<<<kRedBlocks, 256, 0, st>>>(d, 7);
                        residual_ready = true;
                    }
                }
                timer.mark(PH_SETUP, st);
            }
            if (!use_learned && !collect && !fp64()) {
                // the first refinement residual of the warm start, here so that the
                // multilevel setup runs beside it (and inside the span the gate compares)
                timer.mark(PH_VEC, st);
                residual_df((const float*)d.nbrw);
                if (stream_failed) return CCT_CUDAERR;
                residual_ready = true;
            }
            if (overlap_mg) {
                if (mg_setup_finish(st2, ev_rows)) return CCT_CUDAERR;
                cudaEventRecord(ev_mg, st2);
                timer.mark(PH_PRECOND, st);   // the solver stream waits for the rest of the setup
                cudaStreamWaitEvent(st, ev_mg, 0);
                timer.mark(PH_SETUP, st);
                mg_setup_done = true;
            }
            if (gated) cudaEventRecord(gate_ev[4], st);
            if ((rc = fp64() ? solve_fp64(S) : solve_ir(S))) return rc;
            if (gated) {
                cudaEventRecord(gate_ev[5], st);
                gate_pending = use_learned ? 2 : 1;   // read after the step's final synchronisation
            }
            if (use_learned && S.cg_relres > opt.cg_rtol) {
                // the learned solve did not reach the tolerance: plain Jacobi-CG from the warm start
                MPS_COUNT_LAUNCH k_restore_plain<<<blocks_for(d.n), kBlock, 0, st>>>(d);
                MpsStepStats S2{};
                if ((rc = fp64() ? solve_fp64(S2) : solve_ir(S2))) return rc;
                S.cg_iterations += S2.cg_iterations;
                S.ir_passes += S2.ir_passes;
                S.cg_relres = S2.cg_relres;
                S.error_flags = (S.error_flags & ~MPS_ERR_CG) | S2.error_flags;
                S.fallback = 1;
            }
            if (collect) MPS_COUNT_LAUNCH k_targets<<<blocks_for(d.n), kBlock, 0, st>>>(d, warm);
            MPS_COUNT_LAUNCH k_history<<<blocks_for(d.n), kBlock, 0, st>>>(d);
            hist = std::min(hist + 1, 2);
        }
        timer.mark(PH_CORRECT, st);
        if (!pressure_only) {
            if constexpr (sizeof(T) == 4)
                MPS_COUNT_LAUNCH k_correct_warp<<<blocks_for((d.n + 31) / 32, 8), 256, 0, st>>>(d);
            else
                MPS_COUNT_LAUNCH k_correct<T><<<blocks_for(d.n), kBlock, 0, st>>>(d);
            std::swap(d.pos, d.pos2);
            std::swap(d.vel, d.vel2);
        }
        timer.mark(PH_WALLS, st);
        if (!pressure_only && d.tri_n > 0 && walls_move) {
            MPS_COUNT_LAUNCH k_walls_move<<<blocks_for(d.tri_n), kBlock, 0, st>>>(d, step);
            MPS_COUNT_LAUNCH k_tri_to_float<<<blocks_for(9 * d.tri_n), kBlock, 0, st>>>(d);
            bins_dirty = 1;
        }
        timer.mark(PH_OTHER, st);
        cudaMemcpyAsync(h_int, d.err, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(h_int + 1, d.istat, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return CCT_CUDAERR;
        if (gate_pending) {
            gate_update(S, gate_pending == 2);
            gate_pending = 0;
        }
        S.error_flags |= (unsigned)h_int[0];
        S.max_row = h_int[1];
        S.nnz_wide = h_int[2];
        S.rows16 = d.rows16;
        S.inner16 = inner16() ? 1 : 0;
        S.particles = d.n;
        if (opt.pressure_mode != MPS_PRESSURE_EXPLICIT) {
            S.nnz = (long long)h_nnz[0];
            S.pairs = (long long)h_nnz[1];
            S.interior = (int)h_nnz[2];
        }
        if (timer.on) {
            float ms[PH_COUNT] = {0};
            timer.collect(ms);
            S.ms_grid = ms[PH_GRID]; S.ms_walls = ms[PH_WALLS]; S.ms_predictor = ms[PH_PRED];
            S.ms_list = ms[PH_LIST]; S.ms_ppe_setup = ms[PH_SETUP]; S.ms_spmv = ms[PH_SPMV];
            S.ms_cg_vec = ms[PH_VEC]; S.ms_correct = ms[PH_CORRECT]; S.ms_learned = ms[PH_LEARNED];
            S.ms_precond = ms[PH_PRECOND];
            S.spmv_launches = spmv_launches;
        }
        last = S;
        if (out) *out = S;
        return CCT_NOERR;
    }

    double h_nnz[3] = {0, 0, 0};
    // read the device scalars
    CCTStatusType pull_scal() {
        cudaMemcpyAsync(h_scal, d.scal, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return CCT_CUDAERR;
        return CCT_NOERR;
    }

    // streamed SpMV: ring of 2 stages of 8 entries per warp, CTAs of 8 warps, at least
    // 4 CTAs per SM (5 resident at 48 registers).  Measured on the 882k-particle
    // bucket against rings of 3-4 stages, 16 entries, and 6-8 or 16-32-warp CTAs:
    // more shared memory costs more in L1 hits of the x gathers than it gains in
    // copies in flight.  Dynamic shared memory opt-in and a persistent grid of
    // SMs x resident CTAs, set up on first use.
    static constexpr int kSsEntries = 8, kSsStages = 2, kSsWarps = 8, kSsMinBlocks = 4;
    static constexpr int kSsSmem = stream_smem_bytes<kSsEntries, kSsStages, kSsWarps>();
    int spmv_grid = 0, resid_grid = 0;
    bool stream_failed = false;
    // SMs x resident CTAs of a streamed kernel (after its shared-memory opt-in)
    template <class F>
    int persistent_grid(F kernel, int& cached, int smem = kSsSmem) {
        if (cached == 0) {
            int dev = 0, sms = 0, per_sm = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kSsWarps * 32, smem)) return -1;
            // the reduction buffer holds 2 partials per CTA for up to 2 x kRedBlocks CTAs
            cached = std::max(1, std::min(sms * std::max(per_sm, 1), 2 * kRedBlocks));
        }
        return cached;
    }
    int stream_blocks() {
        if (spmv_grid == 0) {
            auto k0 = k_spmv_stream<0, kSsEntries, kSsStages, kSsWarps, kSsMinBlocks>;
            auto k2 = k_spmv_stream<2, kSsEntries, kSsStages, kSsWarps, kSsMinBlocks>;
            if (cudaFuncSetAttribute(k0, cudaFuncAttributeMaxDynamicSharedMemorySize, kSsSmem) ||
                cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize, kSsSmem))
                return -1;
            return persistent_grid(k0, spmv_grid);
        }
        return spmv_grid;
    }
    int resid_blocks() {
        if (resid_grid == 0) {
            auto k = k_residual_stream<kSsEntries, kSsStages, kSsWarps, kSsMinBlocks>;
            if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kSsSmem)) return -1;
            return persistent_grid(k, resid_grid);
        }
        return resid_grid;
    }
    // a streamed kernel's persistent grid, after its shared-memory opt-in (cached)
    template <class K>
    int stream_grid_for(K kernel, int smem, int& cache) {
        if (cache == 0) {
            if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) return -1;
            int c = 0;
            if (persistent_grid(kernel, c, smem) < 0) return -1;
            cache = c;
        }
        return cache;
    }
    // most entries of the last step had 32-bit columns (a grid whose x planes span more
    // than the 16-bit offsets reach): stream the 32-bit columns of every slice instead
    bool prefer_wide = false;
    int spmv_wide_grid[2] = {0, 0}, spmv16_wide_grid = 0, resid_wide_grid = 0;
    template <int MODE>
    void spmv_stream(const float* w, const float* x, float* y, const double* b, int slot) {
        if (prefer_wide) {
            auto k = k_spmv_stream<MODE, kSsEntries, kSsStages, kSsWarps, kSsMinBlocks, float, true>;
            constexpr int smem = stream_smem_bytes<kSsEntries, kSsStages, kSsWarps, float, true>();
            const int g = stream_grid_for(k, smem, spmv_wide_grid[MODE == 0 ? 0 : 1]);
            if (g < 0) {
                stream_failed = true;
                return;
            }
            MPS_COUNT_LAUNCH k<<<g, kSsWarps * 32, smem, st>>>(d, w, x, y, b, slot);
            return;
        }
        const int g = stream_blocks();
        if (g < 0) {
            stream_failed = true;
            return;
        }
        MPS_COUNT_LAUNCH k_spmv_stream<MODE, kSsEntries, kSsStages, kSsWarps, kSsMinBlocks>
            <<<g, kSsWarps * 32, kSsSmem, st>>>(d, w, x, y, b, slot);
    }
    // the inner CG's SpMV over FP16 weights (w16, diag16): stages of 16 entries (2 KB,
    // the bytes in flight of the FP32 ring's 8), 2 stages, CTAs of 8 warps, at least 4
    // per SM (measured against 8 x 2-3, 24 x 2, 32 x 2 and 5 CTAs per SM)
    static constexpr int kS16Entries = 16;
    static constexpr int kS16Smem = stream_smem_bytes<kS16Entries, kSsStages, kSsWarps, __half>();
    int spmv16_grid = 0;
    void spmv_stream16(const float* x, float* y) {
        if (prefer_wide) {
            // 8 entries of 32-bit column + FP16 weight per stage: the FP32 ring's 1.5 KB
            auto kw = k_spmv_stream<0, kSsEntries, kSsStages, kSsWarps, kSsMinBlocks, __half, true>;
            constexpr int smem = stream_smem_bytes<kSsEntries, kSsStages, kSsWarps, __half, true>();
            const int g = stream_grid_for(kw, smem, spmv16_wide_grid);
            if (g < 0) {
                stream_failed = true;
                return;
            }
            MPS_COUNT_LAUNCH kw<<<g, kSsWarps * 32, smem, st>>>(d, d.w16, x, y, nullptr, 0);
            return;
        }
        auto k = k_spmv_stream<0, kS16Entries, kSsStages, kSsWarps, kSsMinBlocks, __half>;
        if (spmv16_grid == 0) {
            if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kS16Smem) ||
                persistent_grid(k, spmv16_grid, kS16Smem) < 0) {
                stream_failed = true;
                return;
            }
        }
        if (pdl) {
            if (MPS_COUNT_LAUNCH launch_pdl(k, spmv16_grid, kSsWarps * 32, kS16Smem, st, d, d.w16, x, y,
                                            (const double*)nullptr, 0))
                stream_failed = true;
        } else {
            MPS_COUNT_LAUNCH k<<<spmv16_grid, kSsWarps * 32, kS16Smem, st>>>(d, d.w16, x, y, nullptr, 0);
        }
    }
    // the CG iteration's kernels (SpMV, update and restriction, fine level of the
    // V-cycle, direction update) are launched with programmatic dependent launch
    bool pdl = true;
    // the streamed kernel needs the 16-bit slices of this step
    bool use_stream() const { return opt.spmv_stream != 0 && d.rows16; }
    // the inner CG runs on the FP16-weight operator (streamed, not matrix-free)
    bool want_inner16() const { return opt.inner_weights == 16 && opt.spmv_stream != 0 && opt.matrix_free == 0; }
    bool inner16() const { return want_inner16() && d.rows_w16 && use_stream(); }

    // FP64 rows streamed through shared memory (the plain FP64 solver): stages of 8
    // entries (512 B of 16-bit columns + 2 KB of FP64 weights), 2 stages, CTAs of 8
    // warps, at least 4 per SM
    static constexpr int kS64Entries = 8;
    int spmv64_grid[2] = {0, 0}, spmv64_wide_grid[2] = {0, 0};
    template <int MODE>
    void spmv_stream64(const double* w, const double* x, double* y, const double* b, int slot) {
        if (prefer_wide) {
            auto k = k_spmv_stream64<MODE, kS64Entries, kSsStages, kSsWarps, kSsMinBlocks, true>;
            constexpr int smem = stream_smem_bytes<kS64Entries, kSsStages, kSsWarps, double, true>();
            const int g = stream_grid_for(k, smem, spmv64_wide_grid[MODE]);
            if (g < 0) {
                stream_failed = true;
                return;
            }
            MPS_COUNT_LAUNCH k<<<g, kSsWarps * 32, smem, st>>>(d, w, x, y, b, slot);
            return;
        }
        auto k = k_spmv_stream64<MODE, kS64Entries, kSsStages, kSsWarps, kSsMinBlocks>;
        constexpr int smem = stream_smem_bytes<kS64Entries, kSsStages, kSsWarps, double>();
        const int g = stream_grid_for(k, smem, spmv64_grid[MODE]);
        if (g < 0) {
            stream_failed = true;
            return;
        }
        MPS_COUNT_LAUNCH k<<<g, kSsWarps * 32, smem, st>>>(d, w, x, y, b, slot);
    }
    // r = rhs - A press of the FP64 solver with its norms (streamed rows when available)
    void residual64(const double* w) {
        if (use_stream()) spmv_stream64<1>(w, d.press, d.r, d.rhs, 2);
        else MPS_COUNT_LAUNCH k_spmv<double, double, double, 1><<<kRedBlocks, 256, 0, st>>>(d, w, d.press, d.r, d.rhs, 2);
    }

    // q = A p of the inner CG (MODE 0): stored weights, or matrix-free FP32 rows
    template <class TW, class TV>
    void spmv_cg(const TW* w, const TV* p, TV* q) {
        if constexpr (std::is_same<TW, double>::value && std::is_same<TV, double>::value) {
            if (use_stream()) {
                spmv_stream64<0>(w, p, q, nullptr, 0);
                return;
            }
        }
        if constexpr (std::is_same<TW, float>::value && std::is_same<TV, float>::value) {
            if (opt.matrix_free == 0 && use_stream()) {
                if (inner16()) spmv_stream16(p, q);
                else spmv_stream<0>(w, p, q, nullptr, 0);
                return;
            }
            if (opt.matrix_free == 4) {
                MPS_COUNT_LAUNCH k_spmv<float, float, float, 0, 4><<<kRedBlocks, 256, 0, st>>>(d, w, p, q, nullptr, 0);
                return;
            }
            if (opt.matrix_free == 8) {
                MPS_COUNT_LAUNCH k_spmv<float, float, float, 0, 8><<<kRedBlocks, 256, 0, st>>>(d, w, p, q, nullptr, 0);
                return;
            }
        }
        MPS_COUNT_LAUNCH k_spmv<TW, TV, TV, 0><<<kRedBlocks, 256, 0, st>>>(d, w, p, q, nullptr, 0);
    }
    // q32 = A z32 with the line-search dots (MODE 2) of the learned guess, FP32
    void spmv_ls(const float* w) {
        if (opt.matrix_free == 0 && use_stream())
            spmv_stream<2>(w, d.z32, d.q32, d.r, 6);
        else if (opt.matrix_free == 4)
            MPS_COUNT_LAUNCH k_spmv<float, float, float, 2, 4><<<kRedBlocks, 256, 0, st>>>(d, w, d.z32, d.q32, d.r, 6);
        else if (opt.matrix_free == 8)
            MPS_COUNT_LAUNCH k_spmv<float, float, float, 2, 8><<<kRedBlocks, 256, 0, st>>>(d, w, d.z32, d.q32, d.r, 6);
        else
            MPS_COUNT_LAUNCH k_spmv<float, float, float, 2><<<kRedBlocks, 256, 0, st>>>(d, w, d.z32, d.q32, d.r, 6);
    }

    // CG iterations in batches with one convergence read-back after each (the kernels
    // of a batch return at once after convergence).  predict > 2 (the same pass's count
    // in the last step): a first batch of predict iterations, then batches of 2, so a
    // pass whose count repeats is read back once and few launches run past convergence;
    // else batches of check_every.
    template <class TW, class TV, class TXA>
    int cg_loop(TXA* x, TV* r, TV* z, TV* p, TV* q, const TW* w, const double* m64, const float* m32, int maxit,
                int predict = 0) {
        const int every = opt.check_every > 0 ? opt.check_every : 8;
        int batch = predict > 2 ? predict : every;
        int done = 0;
        while (done < maxit + every) {
            for (int k = 0; k < batch; ++k) {
                timer.mark(PH_SPMV, st);
                spmv_cg<TW, TV>(w, p, q);
                timer.mark(PH_VEC, st);
                const bool use_mg = std::is_same<TV, float>::value && mg_ready;
                if (!use_mg)
                    MPS_COUNT_LAUNCH k_cg_update<TV, TXA><<<kRedBlocks, 256, 0, st>>>(d, x, r, z, p, q, m64, m32, 1, 1,
                                                                                    flex_step ? 1 : 0);
                if constexpr (std::is_same<TV, float>::value) {
                    if (use_mg) {
                        // two level-1 aggregates per warp, within the reduction buffer's 2 x kRedBlocks CTAs
                        const int ur_blocks = std::max(1, std::min(div_up(mg.L[1].n, 16), 2 * kRedBlocks));
                        if (pdl) {
                            if (MPS_COUNT_LAUNCH launch_pdl(k_mg_update_restrict<TV, TXA>, ur_blocks, 256, 0, st, d, mg,
                                                            x, r, (const TV*)p, (const TV*)q, 1))
                                stream_failed = true;
                        } else {
                            MPS_COUNT_LAUNCH k_mg_update_restrict<TV, TXA><<<ur_blocks, 256, 0, st>>>(d, mg, x, r, p, q,
                                                                                                   1);
                        }
                        timer.mark(PH_PRECOND, st);
                        mg_apply(r, z, p, 0, true);
                        timer.mark(PH_VEC, st);
                    }
                }
                if (pdl && use_mg) {
                    if (MPS_COUNT_LAUNCH launch_pdl(k_cg_p<TV>, kRedBlocks, 256, 0, st, d, p, (const TV*)z))
                        stream_failed = true;
                } else {
                    MPS_COUNT_LAUNCH k_cg_p<TV><<<kRedBlocks, 256, 0, st>>>(d, p, z);
                }
                ++spmv_launches;
            }
            done += batch;
            if (stream_failed || pull_scal()) return -1;
            if (h_scal[S_CONV] != 0.0) break;
            batch = predict > 2 ? 2 : every;
        }
        return (int)h_scal[S_ITER];
    }

    // plain FP64 Jacobi-PCG from the warm start in press
    CCTStatusType solve_fp64(MpsStepStats& S) {
        const double* w = (const double*)d.nbrw;
        residual64(w);
        if (stream_failed || pull_scal()) return CCT_CUDAERR;
        h_nnz[0] = h_scal[S_NNZ0];
        h_nnz[1] = h_scal[S_NNZ1];
        h_nnz[2] = h_scal[S_NINT];
        const double bnorm = h_scal[S_BNORM];
        S.r0_relres = bnorm > 0 ? h_scal[S_RNORM] / bnorm : 0.0;
        const double tol = opt.cg_rtol * bnorm;
        MPS_COUNT_LAUNCH k_cg_start<double><<<kRedBlocks, 256, 0, st>>>(d, d.r, d.z, d.p, nullptr, 1.0, d.minv, nullptr, nullptr, 3, tol,
                                                       opt.cg_max_iter);
        const int it = cg_loop<double, double, double>(d.press, d.r, d.z, d.p, d.q, w, d.minv, nullptr, opt.cg_max_iter);
        if (it < 0) return CCT_CUDAERR;
        // true residual
        residual64(w);
        if (stream_failed || pull_scal()) return CCT_CUDAERR;
        S.cg_iterations += it;
        S.b_norm = bnorm;
        S.cg_relres = bnorm > 0 ? h_scal[S_RNORM] / bnorm : 0.0;
        if (bnorm > 0 && S.cg_relres > opt.cg_rtol) S.error_flags |= MPS_ERR_CG;
        return CCT_NOERR;
    }

    // r = rhs - A press (FP32 weights) in double-float arithmetic; norms to the scalars
    // (rows streamed through shared memory over the 16-bit slices, else the register walk)
    void residual_df(const float* w, bool stream = true) {
        MPS_COUNT_LAUNCH k_split_x<<<blocks_for(d.n), kBlock, 0, st>>>(d.n, d.press, d.xs);
        if (stream && use_stream() && prefer_wide) {
            auto k = k_residual_stream<kSsEntries, kSsStages, kSsWarps, kSsMinBlocks, true>;
            constexpr int smem = stream_smem_bytes<kSsEntries, kSsStages, kSsWarps, float, true>();
            const int g = stream_grid_for(k, smem, resid_wide_grid);
            if (g < 0) {
                stream_failed = true;
                return;
            }
            MPS_COUNT_LAUNCH k<<<g, kSsWarps * 32, smem, st>>>(d, w, d.press, d.r, d.rhs, 2);
        } else if (stream && use_stream()) {
            const int g = resid_blocks();
            if (g < 0) {
                stream_failed = true;
                return;
            }
            MPS_COUNT_LAUNCH k_residual_stream<kSsEntries, kSsStages, kSsWarps, kSsMinBlocks>
                <<<g, kSsWarps * 32, kSsSmem, st>>>(d, w, d.press, d.r, d.rhs, 2);
        } else {
            MPS_COUNT_LAUNCH k_residual_df<<<kRedBlocks, 256, 0, st>>>(d, w, d.press, d.r, d.rhs, 2);
        }
    }

    // the residual after a refinement pass from the pass's correction (streamed rows of
    // stored weights); else recomputed as b - A x
    bool residual_by_update() const { return use_stream() && opt.matrix_free == 0; }
    int upd_grid = 0, upd_wide_grid = 0;
    void residual_update(const float* w, double s) {
        if (prefer_wide) {
            auto k = k_residual_update_stream<kSsEntries, kSsStages, kSsWarps, kSsMinBlocks, true>;
            constexpr int smem = stream_smem_bytes<kSsEntries, kSsStages, kSsWarps, float, true>();
            const int g = stream_grid_for(k, smem, upd_wide_grid);
            if (g < 0) {
                stream_failed = true;
                return;
            }
            MPS_COUNT_LAUNCH k<<<g, kSsWarps * 32, smem, st>>>(d, w, d.d32, s, d.press, d.r, 2);
        } else {
            auto k = k_residual_update_stream<kSsEntries, kSsStages, kSsWarps, kSsMinBlocks>;
            const int g = stream_grid_for(k, kSsSmem, upd_grid);
            if (g < 0) {
                stream_failed = true;
                return;
            }
            MPS_COUNT_LAUNCH k<<<g, kSsWarps * 32, kSsSmem, st>>>(d, w, d.d32, s, d.press, d.r, 2);
        }
    }

    // inner-solve floor: the option, or automatically 7e-4 for the FP16-weight operator
    // under the multilevel preconditioner and 2e-6 otherwise.  With the FP16 weights a
    // refinement pass contracts the FP32-weight residual only down to about the weights'
    // relative rounding (2^-11 ~ 4.9e-4), so inner iterations past it are lost; measured
    // at 882k particles: 1e-4 -> 28.0, 7e-4 -> 27.0 CG iterations per step, 2 passes
    // either way (1e-3 and above add third passes)
    double ir_inner_rtol() const {
        if (opt.ir_inner_rtol > 0) return opt.ir_inner_rtol;
        return inner16() && mg_ready ? 7e-4 : 2e-6;
    }

    // FP32 Jacobi-PCG inside FP64 iterative refinement
    CCTStatusType solve_ir(MpsStepStats& S) {
        const float* w = (const float*)d.nbrw;
        MPS_COUNT_LAUNCH k_to_float<<<blocks_for(d.n), kBlock, 0, st>>>(d.n, d.minv, d.m32);
        timer.mark(PH_PRECOND, st);
        if (!mg_setup_done && mg_setup(st)) return CCT_CUDAERR;
        mg_setup_done = false;
        S.mg_levels = mg_ready ? mg.levels : 0;
        S.mg_level1 = mg_ready ? mg.L[1].n : 0;
        timer.mark(PH_VEC, st);
        double bnorm = 0.0;
        int outer = 0;
        for (;;) {
            // the residual is already there for the first pass when the step computed it
            // before the solve (or from the learned guess), and for the later passes when
            // the last pass updated it with its correction
            const bool have = residual_ready;
            if (!have) residual_df(w);
            if (stream_failed || pull_scal()) return CCT_CUDAERR;
            if (outer == 0) {
                h_nnz[0] = h_scal[S_NNZ0];
                h_nnz[1] = h_scal[S_NNZ1];
                h_nnz[2] = h_scal[S_NINT];
                S.r0_relres = h_scal[S_BNORM] > 0 ? h_scal[S_RNORM] / h_scal[S_BNORM] : 0.0;
                // the learned guess's residual norms before / after its update
                gate_rb = (have && S.learned_applied) ? h_scal[S_TMP1] : 0.0;
                gate_ra = h_scal[S_RNORM];
            }
            residual_ready = false;
            bnorm = h_scal[S_BNORM];
            const double rn = h_scal[S_RNORM];
            S.cg_relres = bnorm > 0 ? rn / bnorm : 0.0;
            if (bnorm == 0.0 || rn <= opt.cg_rtol * bnorm || outer >= opt.ir_max_outer) break;
            // inner FP32 solve of A d = r / ||r||: to the reduction still needed (with a
            // 0.3 margin), but not below what FP32 CG reliably reaches (ir_inner_rtol)
            const double need = 0.3 * opt.cg_rtol * bnorm / rn;
            const double inner_tol = std::max(need, ir_inner_rtol());
            MPS_COUNT_LAUNCH k_cg_start<float><<<kRedBlocks, 256, 0, st>>>(d, d.r32, d.z32, d.p32, d.r, 1.0 / rn, nullptr, d.m32, d.d32, 3,
                                                          inner_tol, opt.cg_max_iter);
            if (mg_ready) {
                timer.mark(PH_PRECOND, st);
                mg_apply(d.r32, d.z32, d.p32, 1);
                timer.mark(PH_VEC, st);
            }
            const int pi = outer < kPassMemory ? outer : kPassMemory - 1;
            const int it = cg_loop<float, float, float>(d.d32, d.r32, d.z32, d.p32, d.q32, w, nullptr, d.m32,
                                                        opt.cg_max_iter, pass_its[pi]);
            if (it < 0) return CCT_CUDAERR;
            pass_its[pi] = it;
            S.cg_iterations += it;
            if (residual_by_update()) {
                // x += rn d and the next pass's residual r -= rn A d, one pass over the rows
                residual_update(w, rn);
                if (stream_failed) return CCT_CUDAERR;
                residual_ready = true;
            } else {
                MPS_COUNT_LAUNCH k_axpy_ir<<<kRedBlocks, 256, 0, st>>>(d, d.press, d.d32, rn);
            }
            ++outer;
        }
        S.ir_passes = outer;
        S.b_norm = bnorm;
        if (bnorm > 0 && S.cg_relres > opt.cg_rtol) S.error_flags |= MPS_ERR_CG;
        return CCT_NOERR;
    }

    CCTStatusType upload(const double* p3, const double* v3, const double* pr) {
        const size_t n = d.n;
        cudaError_t e = cudaMemcpyAsync(stage, p3, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st);
        if (!e) e = cudaMemcpyAsync(stage + 3 * n, v3, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st);
        if (!e) e = cudaMemcpyAsync(stage + 6 * n, pr, sizeof(double) * n, cudaMemcpyHostToDevice, st);
        if (e) return CCT_CUDAERR;
        MPS_COUNT_LAUNCH k_pack_state<<<blocks_for(d.n), kBlock, 0, st>>>(d, stage, stage + 3 * n, stage + 6 * n);
        return cuda_status(cudaGetLastError());
    }
    CCTStatusType download(double* p3, double* v3, double* pr) {
        const size_t n = d.n;
        MPS_COUNT_LAUNCH k_unpack_state<<<blocks_for(d.n), kBlock, 0, st>>>(d, stage, stage + 3 * n, stage + 6 * n);
        cudaError_t e = cudaMemcpyAsync(p3, stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st);
        if (!e) e = cudaMemcpyAsync(v3, stage + 3 * n, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st);
        if (!e) e = cudaMemcpyAsync(pr, stage + 6 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        if (!e) e = cudaStreamSynchronize(st);
        return cuda_status(e);
    }

    // ---- time step (the dt schedule, CheckAndUpdateDt) ----
    // the constants that depend on dt, computed from the float Dt as at creation
    CCTStatusType set_time_step(double dt, double courant) {
        if (!(dt > 0.0) || !std::isfinite(dt)) return CCT_PARAMERR;
        param.Dt = (Scalar)dt;
        if (courant > 0.0) param.CourantNumber = (Scalar)courant;
        Consts& c = d.c;
        c.dt = param.Dt;
        c.kappa = opt.compressibility * c.rho / (c.dt * c.dt);
        c.c2 = c.rho / (c.dt * c.dt);
        c.vmax = c.l0 * (double)param.CourantNumber / c.dt;
        hist = 0;   // the increments were taken over the old step
        return CCT_NOERR;
    }

    // ---- particle inflow ----
    int idext = 0;                 // ID extent: IDs in use lie below it (holes: removed ones)
    unsigned *d_hole = nullptr, *d_hrank = nullptr;
    int* d_holes = nullptr;
    CParticle* d_bucket = nullptr;
    size_t bucket_cap = 0;
    // InsertBucket (MultiGPUHandler.cpp:1163-1210) on the device state: bucket particles
    // take the missing IDs below the extent in increasing order; the rest are appended at
    // the extent only if all of them fit under max_particles (else they are dropped)
    CCTStatusType add_particles(int count, const CParticle* bucket, int* added_out) {
        if (count < 0 || (count > 0 && !bucket)) return CCT_PARAMERR;
        if (added_out) *added_out = 0;
        if (count == 0) return CCT_NOERR;
        cudaError_t e = cudaSuccess;
        if (!d_hole) {
            e = e ? e : mk(&d_hole, (size_t)nmax + 1);
            e = e ? e : mk(&d_hrank, (size_t)nmax + 1);
            e = e ? e : mk(&d_holes, (size_t)nmax);
            if (e) return CCT_MEMERR;
        }
        if ((size_t)count > bucket_cap) {
            if (d_bucket) cudaFree(d_bucket);
            d_bucket = nullptr;
            if (cudaMalloc(&d_bucket, sizeof(CParticle) * (size_t)count)) {
                bucket_cap = 0;
                return CCT_MEMERR;
            }
            bucket_cap = (size_t)count;
        }
        int nholes = 0;
        if (idext > 0) {
            MPS_COUNT_LAUNCH k_fill_u32<<<blocks_for(idext), kBlock, 0, st>>>(d_hole, idext, 1u);
            if (d.n > 0) MPS_COUNT_LAUNCH k_clear_present<<<blocks_for(d.n), kBlock, 0, st>>>(d, d_hole, idext);
            cudaMemcpyAsync(d_hrank, d_hole, sizeof(unsigned) * (size_t)idext, cudaMemcpyDeviceToDevice, st);
            scan_exclusive(d_hrank, idext, d_hrank + idext, st, scan_sums);
            MPS_COUNT_LAUNCH k_hole_list<<<blocks_for(idext), kBlock, 0, st>>>(d_hole, d_hrank, idext, d_holes);
            cudaMemcpyAsync(h_int, d_hrank + idext, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) return CCT_CUDAERR;
            nholes = (int)h_int[0];
        }
        const int fill = std::min(count, nholes);
        const int rest = count - fill;
        const int app = ((long long)idext + rest <= (long long)nmax) ? rest : 0;
        const int added = fill + app;
        if (added > 0) {
            e = cudaMemcpyAsync(d_bucket, bucket, sizeof(CParticle) * (size_t)added, cudaMemcpyHostToDevice, st);
            if (e) return CCT_CUDAERR;
            MPS_COUNT_LAUNCH k_insert<<<blocks_for(added), kBlock, 0, st>>>(d, d_bucket, added, nholes, d_holes, idext);
            if (cudaStreamSynchronize(st) != cudaSuccess) return CCT_CUDAERR;
            d.n += added;
            idext += app;
        }
        if (added_out) *added_out = added;
        return cuda_status(cudaGetLastError());
    }

    // ---- output frames: packed on the solver stream, copied to pinned host memory on
    // a stream of their own, written to the file by a host thread (two slots) ----
    struct FrameSlot {
        float* h = nullptr;        // pinned: [pos 3n | vel 3n | press n | pnd n | visc n]
        int* ht = nullptr;         // pinned: type
        cudaEvent_t copied = nullptr;
        std::thread th;
        CCTStatusType rc = CCT_NOERR;
        std::vector<Scalar3> mpos;
        std::vector<Scalar> mang;
    };
    FrameSlot fslot[2];
    int fnext = 0;
    cudaStream_t st_io = nullptr;
    float* d_frame = nullptr;
    int* d_ftype = nullptr;
    unsigned* d_fflag = nullptr;
    CCTStatusType frame_rc = CCT_NOERR;   // first error of a finished write

    CCTStatusType frames_init() {
        if (d_frame) return CCT_NOERR;
        const size_t N = nmax;
        cudaError_t e = cudaStreamCreateWithFlags(&st_io, cudaStreamNonBlocking);
        e = e ? e : mk(&d_frame, 9 * N); e = e ? e : mk(&d_ftype, N); e = e ? e : mk(&d_fflag, N + 1);
        for (FrameSlot& f : fslot) {
            e = e ? e : cudaMallocHost((void**)&f.h, sizeof(float) * 9 * N);
            e = e ? e : cudaMallocHost((void**)&f.ht, sizeof(int) * N);
            e = e ? e : cudaEventCreateWithFlags(&f.copied, cudaEventDisableTiming);
        }
        return e ? CCT_MEMERR : CCT_NOERR;
    }
    void frame_join(FrameSlot& f) {
        if (f.th.joinable()) f.th.join();
        if (frame_rc == CCT_NOERR && f.rc != CCT_NOERR) frame_rc = f.rc;
        f.rc = CCT_NOERR;
    }
    CCTStatusType frames_wait() {
        for (FrameSlot& f : fslot) frame_join(f);
        const CCTStatusType rc = frame_rc;
        frame_rc = CCT_NOERR;
        return rc;
    }
    CCTStatusType save_frame(const char* path, int ascii, double time, int models, const Scalar3* mp, const Scalar* ma) {
        if (!path || models < 0 || (models > 0 && (!mp || !ma))) return CCT_PARAMERR;
        CCTStatusType rc = frames_init();
        if (rc != CCT_NOERR) return rc;
        FrameSlot& f = fslot[fnext];
        frame_join(f);                         // its previous write is done: reuse the buffers
        const int n = d.n;
        const int idcap = (int)nmax;
        // the previous frame's copy has left the device staging before it is repacked
        cudaStreamWaitEvent(st, fslot[fnext ^ 1].copied, 0);
        cudaMemsetAsync(d_fflag, 0, sizeof(unsigned) * ((size_t)idcap + 1), st);
        if (n > 0) {
            MPS_COUNT_LAUNCH k_frame_mark<<<blocks_for(n), kBlock, 0, st>>>(d, d_fflag, idcap);
            scan_exclusive(d_fflag, idcap, d_fflag + idcap, st, scan_sums);
            MPS_COUNT_LAUNCH k_frame_pack<<<blocks_for(n), kBlock, 0, st>>>(d, d_fflag, idcap, d_frame, d_ftype);
        }
        cudaEventRecord(ev_frame_packed(), st);
        cudaStreamWaitEvent(st_io, ev_frame_packed(), 0);
        cudaError_t e = cudaSuccess;
        if (n > 0) {
            e = cudaMemcpyAsync(f.h, d_frame, sizeof(float) * 9 * (size_t)n, cudaMemcpyDeviceToHost, st_io);
            if (!e) e = cudaMemcpyAsync(f.ht, d_ftype, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, st_io);
        }
        if (!e) e = cudaEventRecord(f.copied, st_io);
        if (e) return CCT_CUDAERR;
        f.mpos.assign(mp, mp + models);
        f.mang.assign(ma, ma + models);
        const std::string fpath(path);
        FrameSlot* fp = &f;
        fp->th = std::thread([fp, fpath, ascii, n, time, models]() {
            if (cudaEventSynchronize(fp->copied) != cudaSuccess) {
                fp->rc = CCT_CUDAERR;
                return;
            }
            const float* h = fp->h;
            const size_t m = (size_t)n;
            fp->rc = mps_write_frame(fpath.c_str(), ascii, n, (const Scalar3*)h, (const Scalar3*)(h + 3 * m), h + 6 * m,
                                     h + 7 * m, nullptr, h + 8 * m, nullptr, (const ParticleType*)fp->ht, (Scalar)time,
                                     models, fp->mpos.data(), fp->mang.data());
        });
        fnext ^= 1;
        return CCT_NOERR;
    }
    cudaEvent_t ev_packed = nullptr;
    cudaEvent_t ev_frame_packed() {
        if (!ev_packed) cudaEventCreateWithFlags(&ev_packed, cudaEventDisableTiming);
        return ev_packed;
    }

    CCTStatusType step(int stepi, MpsStepStats* out, bool pressure_only = false) {
        return fp64() ? run_step<double>(stepi, out, pressure_only) : run_step<float>(stepi, out, pressure_only);
    }
};

}  // namespace mps

using mps::Solver;

struct MpsSolver {
    Solver s;
};

extern "C" {

static_assert(sizeof(MpsSolverOptions) == 168 && sizeof(MpsStepStats) == 168,
              "the option and statistics records are part of the C ABI");

void mps_solver_default_options(MpsSolverOptions* o) {
    std::memset(o, 0, sizeof(*o));
    o->precision = MPS_PREC_FP32_IR;
    o->pressure_mode = MPS_PRESSURE_PPE;
    o->learned = 0;
    o->compressibility = 1e-9;
    o->cg_rtol = 1e-8;
    o->cg_max_iter = 5000;
    o->ir_inner_rtol = 0.0;
    o->ir_max_outer = 12;
    o->max_neighbours = 384;
    o->check_every = 8;
    o->source_relaxation = 0.05;
    o->preconditioner = MPS_PRECOND_MULTILEVEL;
    o->mg_omega = 1.3;   // over-relaxed: measured 27.2 -> 25.9 CG iterations at 882k; 1.7 diverges
    o->compress_rows = 1;
    o->mg_sweeps = 1;
    o->matrix_free = 0;
    o->spmv_stream = 1;
    o->inner_weights = 16;
    o->spmv_wide = 0;
    o->warm_start = -1;
    o->flexible = 0;
    o->learned_gate = 1;
    o->fine_smoother = 0;
    o->smoother_weight = 0.8;
    o->rows_sell = 0;
}

CCTStatusType mps_solver_create(const CParameter* param, const CGridBox* box, int max_particles,
                                const MpsSolverOptions* opt, MpsSolver** out) {
    if (!param || !box || !out) return CCT_PARAMERR;
    MpsSolverOptions o;
    if (opt) o = *opt; else mps_solver_default_options(&o);
    if (o.matrix_free != 0 && o.matrix_free != 4 && o.matrix_free != 8) return CCT_PARAMERR;
    if (o.spmv_stream != 0 && o.spmv_stream != 1) return CCT_PARAMERR;
    if (o.inner_weights != 32 && o.inner_weights != 16) return CCT_PARAMERR;
    if (o.spmv_wide < -1 || o.spmv_wide > 1) return CCT_PARAMERR;
    if (o.warm_start < -1 || o.warm_start > 2) return CCT_PARAMERR;
    if (o.flexible < -1 || o.flexible > 1 || o.learned_gate < 0 || o.learned_gate > 1) return CCT_PARAMERR;
    if (o.fine_smoother < 0 || o.fine_smoother > 1 || !(o.smoother_weight >= 0.0)) return CCT_PARAMERR;
    if (o.rows_sell < 0 || o.rows_sell > 1) return CCT_PARAMERR;
    MpsSolver* s = new MpsSolver();
    CCTStatusType rc = s->s.init(param, box, max_particles, &o);
    if (rc != CCT_NOERR) {
        s->s.destroy();
        delete s;
        return rc;
    }
    *out = s;
    return CCT_NOERR;
}

void mps_solver_destroy(MpsSolver* s) {
    if (!s) return;
    s->s.destroy();
    delete s;
}

CCTStatusType mps_solver_set_particles(MpsSolver* s, int n, const double* pos, const double* vel, const double* press,
                                       const double* visc, const int* type) {
    if (!s || !pos || !vel || !visc) return CCT_PARAMERR;
    return s->s.set_particles(n, pos, vel, press, visc, type);
}

CCTStatusType mps_solver_set_triangles(MpsSolver* s, int t, const double* v, const int* model, int models,
                                       const CTriangleParameters* params) {
    if (!s || (t > 0 && (!v || !model || !params))) return CCT_PARAMERR;
    return s->s.set_triangles(t, v, model, models, params);
}

CCTStatusType mps_solver_set_drag(MpsSolver* s, int count, const DragParameter* params) {
    if (!s) return CCT_PARAMERR;
    return s->s.set_drag(count, params);
}

CCTStatusType mps_solver_step(MpsSolver* s, int step, MpsStepStats* stats) {
    if (!s) return CCT_PARAMERR;
    return s->s.step(step, stats);
}

CCTStatusType mps_solver_get_particles(MpsSolver* s, int* n, double* pos, double* vel, double* press, double* pnd,
                                       int* id) {
    if (!s) return CCT_PARAMERR;
    mps::Dev& d = s->s.d;
    *n = d.n;
    std::vector<mps::dbl4> tmp(d.n);
    cudaError_t e = cudaStreamSynchronize(s->s.st);
    if (!e && pos) {
        e = cudaMemcpy(tmp.data(), d.pos, sizeof(mps::dbl4) * d.n, cudaMemcpyDeviceToHost);
        for (int i = 0; i < d.n; ++i) { pos[3 * i] = tmp[i].x; pos[3 * i + 1] = tmp[i].y; pos[3 * i + 2] = tmp[i].z; }
    }
    if (!e && vel) {
        e = cudaMemcpy(tmp.data(), d.vel, sizeof(mps::dbl4) * d.n, cudaMemcpyDeviceToHost);
        for (int i = 0; i < d.n; ++i) { vel[3 * i] = tmp[i].x; vel[3 * i + 1] = tmp[i].y; vel[3 * i + 2] = tmp[i].z; }
    }
    if (!e && press) e = cudaMemcpy(press, d.press, sizeof(double) * d.n, cudaMemcpyDeviceToHost);
    if (!e && pnd) e = cudaMemcpy(pnd, d.pnd, sizeof(double) * d.n, cudaMemcpyDeviceToHost);
    if (!e && id) e = cudaMemcpy(id, d.id, sizeof(int) * d.n, cudaMemcpyDeviceToHost);
    return mps::cuda_status(e);
}

CCTStatusType mps_solver_get_triangles(MpsSolver* s, double* v) {
    if (!s) return CCT_PARAMERR;
    if (s->s.d.tri_n <= 0) return CCT_NOERR;
    cudaStreamSynchronize(s->s.st);
    return mps::cuda_status(cudaMemcpy(v, s->s.d.tri, sizeof(double) * 9 * s->s.d.tri_n, cudaMemcpyDeviceToHost));
}

CCTStatusType mps_solver_debug_ppe(MpsSolver* s, double* pnd, double* diag, double* rhs, double* sol, int* id,
                                   int* nbr_count, double* nbr_idsum) {
    if (!s) return CCT_PARAMERR;
    mps::Dev& d = s->s.d;
    const int n = d.n;
    cudaError_t e = cudaStreamSynchronize(s->s.st);
    if (!e && pnd) e = cudaMemcpy(pnd, d.pnd, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (!e && diag) e = cudaMemcpy(diag, d.diag, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (!e && rhs) e = cudaMemcpy(rhs, d.rhs, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (!e && sol) e = cudaMemcpy(sol, d.press, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (!e && id) e = cudaMemcpy(id, d.id, sizeof(int) * n, cudaMemcpyDeviceToHost);
    if (!e && nbr_count) e = cudaMemcpy(nbr_count, d.nbr_cnt, sizeof(int) * n, cudaMemcpyDeviceToHost);
    if (!e && nbr_idsum && n > 0) {
        double* tmp = nullptr;
        e = cudaMalloc(&tmp, sizeof(double) * n);
        if (!e) {
            MPS_COUNT_LAUNCH mps::k_row_idsum<<<mps::blocks_for(n), mps::kBlock, 0, s->s.st>>>(d, tmp);
            e = cudaStreamSynchronize(s->s.st);
            if (!e) e = cudaMemcpy(nbr_idsum, tmp, sizeof(double) * n, cudaMemcpyDeviceToHost);
            cudaFree(tmp);
        }
    }
    return mps::cuda_status(e);
}

CCTStatusType mps_solver_debug_history(MpsSolver* s, float* dph1, float* dph2, unsigned char* inner, int* id,
                                       int* held) {
    if (!s || !dph1 || !dph2 || !inner || !id || !held) return CCT_PARAMERR;
    mps::Dev& d = s->s.d;
    const int n = d.n;
    cudaError_t e = cudaStreamSynchronize(s->s.st);
    if (!e && n > 0) e = cudaMemcpy(dph1, d.dph1, sizeof(float) * n, cudaMemcpyDeviceToHost);
    if (!e && n > 0) e = cudaMemcpy(dph2, d.dph2, sizeof(float) * n, cudaMemcpyDeviceToHost);
    if (!e && n > 0) e = cudaMemcpy(inner, d.inner, n, cudaMemcpyDeviceToHost);
    if (!e && n > 0) e = cudaMemcpy(id, d.id, sizeof(int) * n, cudaMemcpyDeviceToHost);
    *held = s->s.hist;
    return mps::cuda_status(e);
}

CCTStatusType mps_solver_debug_wall_bins(MpsSolver* s, int* bounds, int* tids, int cap, int* entries) {
    if (!s || !entries) return CCT_PARAMERR;
    mps::Solver& S = s->s;
    mps::Dev& d = S.d;
    *entries = 0;
    if (d.tri_n <= 0) return CCT_NOERR;
    if (S.bins_dirty) {
        const CCTStatusType rc = S.bin_walls(S.st, S.h_int, S.scan_sums);
        if (rc != CCT_NOERR) return rc;
    }
    if (cudaStreamSynchronize(S.st)) return CCT_CUDAERR;
    const int nv = S.bin_entries;
    *entries = nv;
    if (bounds) {
        const cudaError_t e = cudaMemcpy(bounds, d.tcs, sizeof(int) * 4 * (size_t)d.cells, cudaMemcpyDeviceToHost);
        if (e) return CCT_CUDAERR;
    }
    if (tids && nv > 0) {
        if (cap < nv) return CCT_PARAMERR;
        if (cudaMemcpy(tids, d.tids, sizeof(int) * (size_t)nv, cudaMemcpyDeviceToHost)) return CCT_CUDAERR;
    }
    return CCT_NOERR;
}

CCTStatusType mps_solver_debug_residual(MpsSolver* s, int variant, double* host_r, double* relres) {
    if (!s) return CCT_PARAMERR;
    mps::Solver& S = s->s;
    mps::Dev& d = S.d;
    if (S.fp64() || d.n <= 0 || variant < 0 || variant > 3) return CCT_PARAMERR;
    const float* w = (const float*)d.nbrw;
    if (variant == 0)
        MPS_COUNT_LAUNCH mps::k_spmv<float, double, double, 1><<<mps::kRedBlocks, 256, 0, S.st>>>(d, w, d.press, d.r,
                                                                                                  d.rhs, 2);
    else {
        const bool keep = S.prefer_wide;
        if (variant >= 2) S.ensure_cols32();   // k_residual_df and the wide stream read 32-bit columns
        if (variant == 3) S.prefer_wide = true;
        S.residual_df(w, variant == 1 || variant == 3);
        S.prefer_wide = keep;
    }
    if (S.stream_failed || S.pull_scal()) return CCT_CUDAERR;
    if (relres) *relres = S.h_scal[mps::S_BNORM] > 0 ? S.h_scal[mps::S_RNORM] / S.h_scal[mps::S_BNORM] : 0.0;
    if (host_r) return mps::cuda_status(cudaMemcpy(host_r, d.r, sizeof(double) * d.n, cudaMemcpyDeviceToHost));
    return CCT_NOERR;
}

CCTStatusType mps_solver_debug_level1(MpsSolver* s, int variant, float* host_a, int cap, int* n1) {
    if (!s || !n1 || variant < 0 || variant > 1) return CCT_PARAMERR;
    mps::Solver& S = s->s;
    if (S.fp64() || S.d.n <= 0 || !S.mg_ready) return CCT_PARAMERR;
    if (variant == 1 && !S.use_stream()) return CCT_PARAMERR;
    *n1 = S.mg.L[1].n;
    if (!host_a) return CCT_NOERR;
    if (cap < 27 * *n1) return CCT_PARAMERR;
    const CCTStatusType rc = S.mg_assemble(S.st, variant);
    if (rc != CCT_NOERR) return rc;
    cudaError_t e = cudaMemcpyAsync(host_a, S.mg.L[1].a, sizeof(float) * 27 * (size_t)*n1, cudaMemcpyDeviceToHost,
                                    S.st);
    if (!e) e = cudaStreamSynchronize(S.st);
    return mps::cuda_status(e);
}

CCTStatusType mps_solver_debug_spmv(MpsSolver* s, int kernel, const float* host_x, float* host_y) {
    if (!s || !host_x || !host_y) return CCT_PARAMERR;
    mps::Solver& S = s->s;
    mps::Dev& d = S.d;
    if (S.fp64() || d.n <= 0) return CCT_PARAMERR;
    if (kernel < 0 || kernel > 8 || kernel == 5 || kernel == 7) return CCT_PARAMERR;
    if ((kernel == 1 || kernel == 3) && !d.rows16) return CCT_PARAMERR;
    if ((kernel == 2 || kernel == 6) && !(d.rows16 && d.rows_w16)) return CCT_PARAMERR;
    const float* w = (const float*)d.nbrw;
    cudaError_t e = cudaMemcpyAsync(d.p32, host_x, sizeof(float) * d.n, cudaMemcpyHostToDevice, S.st);
    // MODE 0 returns at once after a converged solve: clear the flag (the next CG start sets it)
    if (!e) e = cudaMemsetAsync(d.scal + mps::S_CONV, 0, sizeof(double), S.st);
    if (e) return CCT_CUDAERR;
    if (kernel == 0)
        MPS_COUNT_LAUNCH mps::k_spmv<float, float, float, 0><<<mps::kRedBlocks, 256, 0, S.st>>>(d, w, d.p32, d.q32, nullptr, 0);
    else if (kernel == 1 || kernel == 2 || kernel == 3 || kernel == 6) {
        const bool keep = S.prefer_wide;
        S.prefer_wide = kernel == 3 || kernel == 6;
        if (S.prefer_wide) S.ensure_cols32();
        if (kernel == 1 || kernel == 3) S.spmv_stream<0>(w, d.p32, d.q32, nullptr, 0);
        else S.spmv_stream16(d.p32, d.q32);
        S.prefer_wide = keep;
    }
    else if (kernel == 4)
        MPS_COUNT_LAUNCH mps::k_spmv<float, float, float, 0, 4><<<mps::kRedBlocks, 256, 0, S.st>>>(d, w, d.p32, d.q32, nullptr, 0);
    else
        MPS_COUNT_LAUNCH mps::k_spmv<float, float, float, 0, 8><<<mps::kRedBlocks, 256, 0, S.st>>>(d, w, d.p32, d.q32, nullptr, 0);
    if (S.stream_failed) return CCT_CUDAERR;
    e = cudaMemcpyAsync(host_y, d.q32, sizeof(float) * d.n, cudaMemcpyDeviceToHost, S.st);
    if (!e) e = cudaStreamSynchronize(S.st);
    return mps::cuda_status(e);
}

CCTStatusType mps_solver_set_time_step(MpsSolver* s, double dt, double courant) {
    if (!s) return CCT_PARAMERR;
    return s->s.set_time_step(dt, courant);
}

CCTStatusType mps_solver_add_particles(MpsSolver* s, int count, const CParticle* bucket, int* added) {
    if (!s) return CCT_PARAMERR;
    return s->s.add_particles(count, bucket, added);
}

CCTStatusType mps_solver_save_frame(MpsSolver* s, const char* path, int ascii, double time, int models,
                                    const Scalar3* model_pos, const Scalar* model_angle) {
    if (!s) return CCT_PARAMERR;
    return s->s.save_frame(path, ascii, time, models, model_pos, model_angle);
}

CCTStatusType mps_solver_wait_frames(MpsSolver* s) {
    if (!s) return CCT_PARAMERR;
    return s->s.frames_wait();
}

CCTStatusType mps_solver_device_pressure(MpsSolver* s, const double** press, int* n) {
    if (!s) return CCT_PARAMERR;
    *press = s->s.d.press;
    *n = s->s.d.n;
    return CCT_NOERR;
}

CCTStatusType mps_solver_copy_pressure(MpsSolver* s, double* host_press) {
    if (!s) return CCT_PARAMERR;
    cudaError_t e = cudaMemcpyAsync(host_press, s->s.d.press, sizeof(double) * s->s.d.n, cudaMemcpyDeviceToHost, s->s.st);
    if (!e) e = cudaStreamSynchronize(s->s.st);
    return mps::cuda_status(e);
}

CCTStatusType mps_solver_upload_state(MpsSolver* s, const double* pos, const double* vel, const double* press) {
    if (!s || !pos || !vel || !press) return CCT_PARAMERR;
    return s->s.upload(pos, vel, press);
}

CCTStatusType mps_solver_download_state(MpsSolver* s, double* pos, double* vel, double* press) {
    if (!s || !pos || !vel || !press) return CCT_PARAMERR;
    return s->s.download(pos, vel, press);
}

CCTStatusType mps_solver_stream(MpsSolver* s, void** stream) {
    if (!s) return CCT_PARAMERR;
    *stream = (void*)s->s.st;
    return CCT_NOERR;
}

CCTStatusType mps_solver_set_learned(MpsSolver* s, const float* params, int count) {
    if (!s || !params || count != MPS_MLP_PARAMS) return CCT_PARAMERR;
    Solver& v = s->s;
    if (!v.mlp) {
        CCTStatusType rc = mps_mlp_create(std::min(v.nmax, 1 << 18), 1, &v.mlp);
        if (rc) return rc;
    }
    CCTStatusType rc = mps_mlp_set_params(v.mlp, params);
    if (rc) return rc;
    v.learned_ready = true;
    return CCT_NOERR;
}

CCTStatusType mps_solver_collect(MpsSolver* s, int on) {
    if (!s) return CCT_PARAMERR;
    s->s.collect = on != 0;
    return CCT_NOERR;
}

CCTStatusType mps_solver_learned_samples(MpsSolver* s, float* features, float* targets, int* n) {
    if (!s || !n) return CCT_PARAMERR;
    mps::Dev& d = s->s.d;
    *n = d.n;
    cudaError_t e = cudaStreamSynchronize(s->s.st);
    if (!e && features) e = cudaMemcpy(features, d.feat, sizeof(float) * 12 * d.n, cudaMemcpyDeviceToHost);
    if (!e && targets) e = cudaMemcpy(targets, d.targets, sizeof(float) * 2 * d.n, cudaMemcpyDeviceToHost);
    return mps::cuda_status(e);
}

// ---------------------------------------------------------------------------
// entry points under the reference's reserved names (S/CGPUCellSet.h:224-225)
// and the precision / learned-part controls
// ---------------------------------------------------------------------------
static CCTStatusType pressure_solve(MpsSolver* s, MpsStepStats* stats, int precond, int learned) {
    if (!s) return CCT_PARAMERR;
    Solver& v = s->s;
    if (v.opt.pressure_mode != MPS_PRESSURE_PPE) return CCT_PARAMERR;
    const int p0 = v.opt.preconditioner, l0 = v.opt.learned;
    v.opt.preconditioner = precond;
    v.opt.learned = learned;
    const CCTStatusType rc = v.step(0, stats, true);
    v.opt.preconditioner = p0;
    v.opt.learned = l0;
    return rc;
}

CCTStatusType CalculatePressureCG(MpsSolver* s, MpsStepStats* stats) {
    return pressure_solve(s, stats, MPS_PRECOND_JACOBI, 0);
}

CCTStatusType CalculatePressureNJPCG(MpsSolver* s, MpsStepStats* stats) {
    if (!s) return CCT_PARAMERR;
    const Solver& v = s->s;
    return pressure_solve(s, stats, MPS_PRECOND_MULTILEVEL, v.learned_ready ? (v.opt.learned ? v.opt.learned : 1) : 0);
}

CCTStatusType CalcPoisson(void* Stream, MpsSolver* s, Integer ParticleNum, Scalar* dA, Scalar* dB, Scalar* dX,
                          const Scalar* dX0, MpsStepStats* stats) {
    if (!s || ParticleNum < 0) return CCT_PARAMERR;
    Solver& v = s->s;
    if (v.opt.pressure_mode != MPS_PRESSURE_PPE) return CCT_PARAMERR;
    if (v.d.n > 0 && ParticleNum == 0) return CCT_PARAMERR;
    // the solve follows the caller's earlier work on Stream (it may have written dX0)
    if (Stream) {
        cudaEvent_t ev = nullptr;
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) return CCT_CUDAERR;
        cudaError_t e = cudaEventRecord(ev, (cudaStream_t)Stream);
        if (!e) e = cudaStreamWaitEvent(v.st, ev, 0);
        cudaEventDestroy(ev);
        if (e) return CCT_CUDAERR;
    }
    if (dX0 && v.d.n > 0) {
        MPS_COUNT_LAUNCH mps::k_poisson_start<<<mps::blocks_for(v.d.n), mps::kBlock, 0, v.st>>>(v.d, ParticleNum, dX0);
        v.hist = 0;   // the start replaces the pressure history
    }
    MpsStepStats st{};
    CCTStatusType rc = pressure_solve(s, &st, MPS_PRECOND_JACOBI, 0);
    if (rc != CCT_NOERR) return rc;
    if (dX0) v.hist = 0;
    if (v.d.n > 0) {
        cudaMemsetAsync(v.d.err, 0, sizeof(unsigned), v.st);
        MPS_COUNT_LAUNCH mps::k_poisson_out<<<mps::blocks_for(v.d.n), mps::kBlock, 0, v.st>>>(v.d, ParticleNum, dA, dB,
                                                                                              dX);
        cudaMemcpyAsync(v.h_int, v.d.err, sizeof(unsigned), cudaMemcpyDeviceToHost, v.st);
        if (cudaStreamSynchronize(v.st)) return CCT_CUDAERR;
        st.error_flags |= (unsigned)v.h_int[0];
    }
    if (stats) *stats = st;
    if (st.error_flags & MPS_ERR_KEY_RANGE) {
        mps::note_message("CalcPoisson: a particle ID lies at or above ParticleNum");
        return CCT_PARAMERR;
    }
    return (st.error_flags & MPS_ERR_CG) ? CCT_CALCERR : CCT_NOERR;
}

CCTStatusType mps_set_precision(MpsSolver* s, int precision) {
    if (!s || (precision != MPS_PREC_FP64 && precision != MPS_PREC_FP32_IR)) return CCT_PARAMERR;
    s->s.opt.precision = precision;
    return CCT_NOERR;
}

CCTStatusType mps_learned_train(MpsSolver* s, int first_step, int steps, int max_samples, int epochs, int batch,
                                float lr, unsigned long long seed, MpsLearnedInfo* info) {
    if (!s || steps <= 0 || epochs <= 0 || batch <= 0 || !(lr > 0.f)) return CCT_PARAMERR;
    Solver& v = s->s;
    if (v.opt.pressure_mode != MPS_PRESSURE_PPE) return CCT_PARAMERR;
    if (max_samples <= 0) max_samples = 400000;
    const auto t0 = std::chrono::steady_clock::now();
    std::mt19937_64 rng(seed);
    const int per_step = std::max(1, max_samples / steps);
    std::vector<float> F, T, f, t;
    std::vector<int> cand;
    const int learned0 = v.opt.learned;
    v.opt.learned = 0;
    v.collect = true;
    CCTStatusType rc = CCT_NOERR;
    for (int k = 0; k < steps && rc == CCT_NOERR; ++k) {
        MpsStepStats st;
        rc = v.step(first_step + k, &st);
        if (rc) break;
        const int n = v.d.n;
        f.resize(12 * (size_t)n);
        t.resize(2 * (size_t)n);
        cudaError_t e = cudaMemcpy(f.data(), v.d.feat, sizeof(float) * 12 * n, cudaMemcpyDeviceToHost);
        if (!e) e = cudaMemcpy(t.data(), v.d.targets, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost);
        if (e) { rc = mps::cuda_status(e); break; }
        cand.clear();
        for (int r = 0; r < n; ++r)
            if (std::isfinite(t[2 * (size_t)r]) && std::isfinite(t[2 * (size_t)r + 1])) cand.push_back(r);
        std::shuffle(cand.begin(), cand.end(), rng);
        if ((int)cand.size() > per_step) cand.resize(per_step);
        for (int r : cand) {
            F.insert(F.end(), f.begin() + 12 * (size_t)r, f.begin() + 12 * (size_t)r + 12);
            T.insert(T.end(), t.begin() + 2 * (size_t)r, t.begin() + 2 * (size_t)r + 2);
        }
    }
    v.collect = false;
    v.opt.learned = learned0;
    if (rc) return rc;
    const auto t1 = std::chrono::steady_clock::now();
    const int S = (int)(T.size() / 2);
    if (S < 2 * batch) return CCT_PARAMERR;
    std::vector<int> idx(S);
    for (int i = 0; i < S; ++i) idx[i] = i;
    std::shuffle(idx.begin(), idx.end(), rng);
    const int n_val = std::max(1, S / 10);
    std::vector<float> Xv(12 * (size_t)n_val), Tv(2 * (size_t)n_val), Xb(12 * (size_t)batch), Tb(2 * (size_t)batch);
    for (int i = 0; i < n_val; ++i) {
        std::copy_n(F.begin() + 12 * (size_t)idx[i], 12, Xv.begin() + 12 * (size_t)i);
        std::copy_n(T.begin() + 2 * (size_t)idx[i], 2, Tv.begin() + 2 * (size_t)i);
    }
    float *dXv = nullptr, *dTv = nullptr, *dXb = nullptr, *dTb = nullptr, *dg = nullptr;
    MpsMlp* m = nullptr;
    cudaError_t e = cudaMalloc(&dXv, sizeof(float) * Xv.size());
    if (!e) e = cudaMalloc(&dTv, sizeof(float) * Tv.size());
    if (!e) e = cudaMalloc(&dXb, sizeof(float) * Xb.size());
    if (!e) e = cudaMalloc(&dTb, sizeof(float) * Tb.size());
    if (!e) e = cudaMalloc(&dg, sizeof(float) * MPS_MLP_PARAMS);
    if (!e) e = cudaMemcpy(dXv, Xv.data(), sizeof(float) * Xv.size(), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(dTv, Tv.data(), sizeof(float) * Tv.size(), cudaMemcpyHostToDevice);
    if (e) rc = CCT_MEMERR;
    if (!rc) rc = mps_mlp_create(std::max(batch, n_val), seed, &m);
    float loss0 = 0.f, loss1 = 0.f;
    int adam = 0;
    if (!rc) rc = mps_mlp_loss_grad(m, n_val, dXv, dTv, 0.25f, dg, &loss0, nullptr);
    std::vector<int> tr(idx.begin() + n_val, idx.end());
    for (int ep = 0; ep < epochs && !rc; ++ep) {
        std::shuffle(tr.begin(), tr.end(), rng);
        const float lr_ep = lr * std::pow(0.5f, (float)ep);
        for (size_t b0 = 0; b0 + batch <= tr.size() && !rc; b0 += batch) {
            for (int i = 0; i < batch; ++i) {
                std::copy_n(F.begin() + 12 * (size_t)tr[b0 + i], 12, Xb.begin() + 12 * (size_t)i);
                std::copy_n(T.begin() + 2 * (size_t)tr[b0 + i], 2, Tb.begin() + 2 * (size_t)i);
            }
            e = cudaMemcpy(dXb, Xb.data(), sizeof(float) * Xb.size(), cudaMemcpyHostToDevice);
            if (!e) e = cudaMemcpy(dTb, Tb.data(), sizeof(float) * Tb.size(), cudaMemcpyHostToDevice);
            if (e) { rc = CCT_CUDAERR; break; }
            rc = mps_mlp_train_step(m, batch, dXb, dTb, 0.25f, lr_ep, nullptr, nullptr);
            ++adam;
        }
    }
    if (!rc) rc = mps_mlp_loss_grad(m, n_val, dXv, dTv, 0.25f, dg, &loss1, nullptr);
    std::vector<float> params(MPS_MLP_PARAMS);
    if (!rc) rc = mps_mlp_get_params(m, params.data());
    if (!rc) rc = mps_solver_set_learned(s, params.data(), MPS_MLP_PARAMS);
    if (!rc) v.opt.learned |= 1;
    if (m) mps_mlp_destroy(m);
    cudaFree(dXv); cudaFree(dTv); cudaFree(dXb); cudaFree(dTb); cudaFree(dg);
    if (info) {
        const auto t2 = std::chrono::steady_clock::now();
        info->samples = S;
        info->val_samples = n_val;
        info->adam_steps = adam;
        info->batch = batch;
        info->val_loss_before = loss0;
        info->val_loss_after = loss1;
        info->collect_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        info->train_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
    }
    return rc;
}

CCTStatusType mps_learned_infer(MpsSolver* s, float* host_out, int* n) {
    if (!s || !n) return CCT_PARAMERR;
    Solver& v = s->s;
    if (!v.learned_ready || !v.mlp || !v.feat_valid) return CCT_PARAMERR;
    *n = v.d.n;
    if (mps::mlp_forward(v.mlp, v.d.n, v.d.feat, v.d.mlp_out, v.st, v.d.err)) return CCT_CUDAERR;
    cudaError_t e = cudaStreamSynchronize(v.st);
    if (!e && host_out) e = cudaMemcpy(host_out, v.d.mlp_out, sizeof(float) * 2 * v.d.n, cudaMemcpyDeviceToHost);
    return mps::cuda_status(e);
}

}  // extern "C"
