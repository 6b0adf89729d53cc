// coarse.cuh - cell-aggregate multilevel preconditioner of the FP32 inner PPE solve.
//
// M^-1 r = D^-1 r + P1 V(P1^T r): the Jacobi part plus a coarse correction whose
// level-1 unknowns are the non-empty cells of the neighbour-search grid (one
// aggregate per cell, piecewise-constant prolongation P1 over its interior
// particles).  Level l+1 aggregates the 2x2x2 cells of level l, until at most
// kMgMaxDense aggregates remain; that level is solved with an explicit inverse.
// V is one V-cycle with weighted-Jacobi smoothing (one sweep down, one up), a
// symmetric operator, so plain PCG applies.  Coarse operators are Galerkin
// products A_{l+1} = P^T A_l P stored as 27-point stencils (cells interact only
// with their 26 neighbours because the Laplacian radius equals the cell size).
//
// Every sum has a fixed order (per-thread shared-memory columns, per-lane slot
// ownership, child cells in a fixed order), so the preconditioner is deterministic.
#pragma once

namespace mps {

constexpr int kMgMaxLevels = 10;
constexpr int kMgMaxDense = 128;

struct MgLevel {
    int n;             // aggregates
    int gx, gy, gz;    // grid of this level
    int* cmap;         // [cells] cell -> aggregate or -1
    int* ccell;        // [n] aggregate -> cell
    int* nb;           // [27 n] neighbour aggregates (-1: none), slot (dx+1)*9+(dy+1)*3+(dz+1)
    int* par;          // [n] aggregate of the next level containing it (-1 on the last level)
    int* nbp;          // [27 n] par of each stencil neighbour, loaded beside nb by the up sweeps
    int* child;        // [8 n] aggregates of the level below inside this one, octant order
                       //     ((x & 1) << 2 | (y & 1) << 1 | (z & 1)), -1: none (levels >= 2)
    float* a;          // [27 n] Galerkin stencil
    float* dinv;       // [n] 1 / diagonal (0 for an aggregate without interior particles)
    float* r;          // [n] restricted residual
    float* e;          // [n] correction after the down sweep
    float* e2;         // [n] correction after the up sweep (the level's result)
};

struct Mg {
    int levels;        // levels in use: 1 .. levels, the last one solved densely
    float omega;       // Jacobi weight of the smoothing sweeps
    MgLevel L[kMgMaxLevels + 1];   // L[0] unused
    float* ainv;       // [n_last^2] inverse of the last level's matrix
    unsigned* done;    // CTAs of the last restriction that finished (k_mg_down; reset to 0)
    int* agg1;         // [n] particle -> level-1 aggregate
    unsigned* pcc;     // [n] cell coordinates of the particle, 10 bits each (x<<20 | y<<10 | z),
                       //     bit 31 set for an interior particle
    float* part;       // [27 n] level-1 assembly: slot sums of a (slice, cell) row segment,
                       //     stored at the segment's first row
    double* partd;     // [n] diagonal sum of that segment
    int* rb;           // [n1 + 1] rows of level-1 aggregate I: [rb[I], rb[I + 1]) (aggregates are
                       //     numbered in cell order and the rows are sorted by cell)
};

__device__ __forceinline__ void mg_decode(int c, int gy, int gz, int& x, int& y, int& z) {
    x = c / (gy * gz);
    y = (c / gz) % gy;
    z = c % gz;
}
__device__ __forceinline__ int mg_slot_dx(int s) { return s / 9 - 1; }
__device__ __forceinline__ int mg_slot_dy(int s) { return (s / 3) % 3 - 1; }
__device__ __forceinline__ int mg_slot_dz(int s) { return s % 3 - 1; }

// ---------------------------------------------------------------------------
// setup: aggregates, links, operators (once per step)
// ---------------------------------------------------------------------------
// level-1 occupancy: a grid cell is an aggregate when it holds particles
__global__ void k_mg_flags1(const __grid_constant__ Dev d, unsigned* flag) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < d.cells) flag[c] = d.cstart[c] >= 0 ? 1u : 0u;
}

// level l occupancy from the 2x2x2 children at level l-1
__global__ void k_mg_flags_up(MgLevel lo, MgLevel hi, unsigned* flag) {
    const int C = blockIdx.x * blockDim.x + threadIdx.x;
    if (C >= hi.gx * hi.gy * hi.gz) return;
    int X, Y, Z;
    mg_decode(C, hi.gy, hi.gz, X, Y, Z);
    unsigned any = 0;
    for (int q = 0; q < 8; ++q) {
        const int x = 2 * X + (q >> 2), y = 2 * Y + ((q >> 1) & 1), z = 2 * Z + (q & 1);
        if (x < lo.gx && y < lo.gy && z < lo.gz && lo.cmap[(x * lo.gy + y) * lo.gz + z] >= 0) any = 1;
    }
    flag[C] = any;
}

// aggregate numbering from the exclusive scan of the occupancy (pre[cells] = total)
__global__ void k_mg_fill(MgLevel lv, const unsigned* pre) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= lv.gx * lv.gy * lv.gz) return;
    const unsigned f = pre[c + 1] - pre[c];
    lv.cmap[c] = f ? (int)pre[c] : -1;
    if (f) lv.ccell[pre[c]] = c;
}

// neighbour aggregates and parent of every aggregate of a level
__global__ void k_mg_links(MgLevel lv, MgLevel up, int has_up) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= lv.n) return;
    int x, y, z;
    mg_decode(lv.ccell[I], lv.gy, lv.gz, x, y, z);
    for (int s = 0; s < 27; ++s) {
        const int xx = x + mg_slot_dx(s), yy = y + mg_slot_dy(s), zz = z + mg_slot_dz(s);
        const bool in = xx >= 0 && yy >= 0 && zz >= 0 && xx < lv.gx && yy < lv.gy && zz < lv.gz;
        lv.nb[(size_t)I * 27 + s] = in ? lv.cmap[(xx * lv.gy + yy) * lv.gz + zz] : -1;
    }
    const int P = has_up ? up.cmap[((x >> 1) * up.gy + (y >> 1)) * up.gz + (z >> 1)] : -1;
    lv.par[I] = P;
    if (P >= 0) up.child[(size_t)P * 8 + (((x & 1) << 2) | ((y & 1) << 1) | (z & 1))] = I;
}

// row ranges of the level-1 aggregates
__global__ void k_mg_rows(const __grid_constant__ Dev d, const __grid_constant__ Mg mg) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const MgLevel& L1 = mg.L[1];
    if (I >= L1.n) return;
    const int c = L1.ccell[I];
    mg.rb[I] = d.cstart[c];
    if (I == L1.n - 1) mg.rb[L1.n] = d.cend[c];
}

// parent of every stencil neighbour (after the level's links)
__global__ void k_mg_nbpar(MgLevel lv) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 27 * lv.n) return;
    const int J = lv.nb[e];
    lv.nbp[e] = J >= 0 ? lv.par[J] : -1;
}

// per particle: level-1 aggregate and packed cell coordinates
__global__ void k_mg_particles(const __grid_constant__ Dev d, const __grid_constant__ Mg mg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const int c = d.key[i];
    if (c < 0 || c >= d.cells) {
        mg.agg1[i] = -1;
        mg.pcc[i] = 0x7fffffffu;   // not interior: never summed
        return;
    }
    int x, y, z;
    mg_decode(c, d.box.m_GridSize.y, d.box.m_GridSize.z, x, y, z);
    mg.pcc[i] = ((unsigned)x << 20) | ((unsigned)y << 10) | (unsigned)z | (d.inner[i] ? 0x80000000u : 0u);
    mg.agg1[i] = mg.L[1].cmap[c];
}

// Level-1 Galerkin stencil, pass 1 of 2: warp per 32-row slice, lane per row (the
// SELL walk: 8 entries' columns and weights in flight, 16-bit columns where the slice
// has them).  Each lane sums its row's interior-interior entries per stencil slot in
// its own shared-memory column; the slot follows from one subtraction of packed cell
// coordinates (each field offset by one, so a neighbour cell gives fields 0..2 and no
// borrow).  The lanes of each cell (contiguous rows) are then summed by a segmented
// shuffle tree, and the segment's first lane stores the 27 slot sums and the
// diagonal sum at its row.  Fixed orders: deterministic.
constexpr int kMgAsmWarps = 4;

// entries of one SELL-32 entry group into the lane's 27 slot sums A[.][lane]
__device__ __forceinline__ void mg_asm_add8(const Mg& mg, float (*A)[32], int lane, unsigned pi, const unsigned (&pq)[8],
                                            const float (&wv)[8]) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        if (!(pq[u] & 0x80000000u)) continue;   // not interior, or no entry
        const unsigned dd = (pq[u] & 0x3fffffffu) + 0x00100401u - pi;
        const unsigned fx = dd >> 20, fy = (dd >> 10) & 1023u, fz = dd & 1023u;
        if (fx <= 2u && fy <= 2u && fz <= 2u) A[fx * 9 + fy * 3 + fz][lane] += wv[u];
    }
}

// the register walk of one slice's rows (8 entries' columns and weights in flight)
template <class TW>
__device__ __forceinline__ void mg_asm_walk(const Dev& d, const Mg& mg, const TW* __restrict__ w, float (*A)[32],
                                            int lane, int sl, int cnt, unsigned pi) {
    const int kmax = __reduce_max_sync(0xffffffffu, cnt);
    const int sb = (sizeof(TW) == 4 && d.rows16) ? d.sbase[sl] : -1;
    const size_t base = (size_t)sl * d.K * 32 + lane;
    for (int k = 0; k < kmax; k += 8) {
        int jj[8];
        float wv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const size_t e = base + (size_t)min(k + u, kmax - 1) * 32;
            jj[u] = sb >= 0 ? sell_col<true>(d, e, sb) : sell_col<false>(d, e, sb);
            wv[u] = (float)__ldcs(w + e);
        }
        unsigned pq[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) pq[u] = k + u < cnt ? mg.pcc[jj[u]] : 0u;
        mg_asm_add8(mg, A, lane, pi, pq, wv);
    }
}

// segmented sums over the lanes of each cell (contiguous rows) into the segment's first
// lane, which stores the 27 slot sums and the diagonal sum at its row
__device__ __forceinline__ void mg_asm_finish(const Dev& d, const Mg& mg, float (*A)[32], int lane, int i, bool row,
                                              bool in, int seg) {
    __syncwarp();
    const int prev = __shfl_up_sync(0xffffffffu, seg, 1);
    const bool head = row && seg >= 0 && (lane == 0 || prev != seg);
    bool same[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        const int o = 1 << q;
        const int sn = __shfl_down_sync(0xffffffffu, seg, o);
        same[q] = lane + o < 32 && sn == seg;
    }
    double ds = in ? d.diag[i] : 0.0;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        const double t = __shfl_down_sync(0xffffffffu, ds, 1 << q);
        if (same[q]) ds += t;
    }
    if (head) mg.partd[i] = ds;
    for (int t = 0; t < 27; ++t) {
        float v = A[t][lane];
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            const float x = __shfl_down_sync(0xffffffffu, v, 1 << q);
            if (same[q]) v += x;
        }
        if (head) mg.part[(size_t)i * 27 + t] = v;
    }
    __syncwarp();
}

template <class TW>
__global__ void __launch_bounds__(kMgAsmWarps * 32) k_mg_assemble_rows(const __grid_constant__ Dev d,
                                                                       const __grid_constant__ Mg mg,
                                                                       const TW* __restrict__ w) {
    __shared__ float acc[kMgAsmWarps][27][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float (*A)[32] = acc[wib];
    const int gw = blockIdx.x * kMgAsmWarps + wib, nw = gridDim.x * kMgAsmWarps;
    const int nsl = (d.n + 31) >> 5;
    for (int sl = gw; sl < nsl; sl += nw) {
        const int i = sl * 32 + lane;
        const bool row = i < d.n;
        const bool in = row && d.inner[i];
        const int cnt = in ? d.nbr_cnt[i] : 0;
        const unsigned pi = (row ? mg.pcc[i] : 0u) & 0x3fffffffu;
        const int seg = row ? mg.agg1[i] : -1;
#pragma unroll
        for (int t = 0; t < 27; ++t) A[t][lane] = 0.f;
        __syncwarp();
        mg_asm_walk<TW>(d, mg, w, A, lane, sl, cnt, pi);
        mg_asm_finish(d, mg, A, lane, i, row, in, seg);
    }
}

// The same pass over streamed rows: the 16-bit slices' columns and FP32 weights move
// into a per-warp shared-memory ring by bulk copies (SliceRing, as the streamed SpMV),
// so only the pcc gathers wait on memory.  Each lane adds its row's entries in row
// order as the register walk does: the same sums, bit for bit.  32-bit slices, and
// every slice after a stage wait that timed out (which abandons the stream), take the
// register walk.
template <int SC, int SS, int W, int MINB>
__global__ void __launch_bounds__(W * 32, MINB) k_mg_assemble_stream(const __grid_constant__ Dev d,
                                                                     const __grid_constant__ Mg mg,
                                                                     const float* __restrict__ w) {
    static_assert(SC % 8 == 0, "stages hold whole groups of 8 entries");
    extern __shared__ __align__(128) unsigned char stream_smem[];
    __shared__ __align__(8) unsigned long long bars[W][SS];
    __shared__ float acc[W][27][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float (*A)[32] = acc[warp];
    const int gw = blockIdx.x * W + warp, nw = gridDim.x * W;
    SliceRing<SC, SS, float, false> R;
    R.init(d, w, stream_smem + warp * SS * SliceRing<SC, SS, float, false>::SB, bars[warp], gw, nw);
    for (int sl = gw; sl < R.nsl; sl += nw) {
        const int i = sl * 32 + lane;
        const bool row = i < d.n;
        const bool in = row && d.inner[i];
        const int cnt = in ? d.nbr_cnt[i] : 0;
        const unsigned pi = (row ? mg.pcc[i] : 0u) & 0x3fffffffu;
        const int seg = row ? mg.agg1[i] : -1;
        const int km = d.skmax[sl];
#pragma unroll
        for (int t = 0; t < 27; ++t) A[t][lane] = 0.f;
        __syncwarp();
        bool done = false;
        if (km >= 0 && R.streaming) {
            const int nc = (km + SC - 1) / SC;
            const int r0 = sl * 32;
            for (int c = 0; c < nc; ++c) {
                const unsigned char* cs;
                const float* ws;
                if (!R.acquire(cs, ws)) break;
                const int k0 = c * SC;
#pragma unroll
                for (int g = 0; g < SC; g += 8) {
                    int j[8];
                    float wv[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        j[u] = r0 + (int)(short)((const unsigned short*)cs)[(g + u) * 32 + lane];
                        wv[u] = ws[(g + u) * 32 + lane];
                    }
                    unsigned pq[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) pq[u] = k0 + g + u < cnt ? mg.pcc[j[u]] : 0u;
                    mg_asm_add8(mg, A, lane, pi, pq, wv);
                }
                R.release();
            }
            done = R.streaming;
        }
        if (!done) {
            // partial sums of an abandoned stream are dropped
            __syncwarp();
#pragma unroll
            for (int t = 0; t < 27; ++t) A[t][lane] = 0.f;
            __syncwarp();
            mg_asm_walk<float>(d, mg, w, A, lane, sl, cnt, pi);
        }
        mg_asm_finish(d, mg, A, lane, i, row, in, seg);
    }
}

// Level-1 Galerkin stencil, pass 2 of 2: warp per level-1 aggregate (cell) sums the
// segments of its rows in slice order (lane s: slot s, lane 27: the diagonals) and
// stores A1[I, .] = -coef * slot sums, with the diagonal sum added to the centre.
__global__ void k_mg_assemble_cells(const __grid_constant__ Dev d, const __grid_constant__ Mg mg) {
    const MgLevel& L1 = mg.L[1];
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (I >= L1.n) return;   // warp-uniform
    const int c = L1.ccell[I];
    const int b = d.cstart[c], e = d.cend[c];
    float v = 0.f;
    double ds = 0.0;
    if (e > b) {
        for (int sl = b >> 5; sl <= (e - 1) >> 5; ++sl) {
            const int h = sl == (b >> 5) ? b : sl * 32;
            if (lane < 27) v += mg.part[(size_t)h * 27 + lane];
            else if (lane == 27) ds += mg.partd[h];
        }
    }
    const float dsum = (float)__shfl_sync(0xffffffffu, ds, 27);
    const float centre = __shfl_sync(0xffffffffu, v, 13);
    if (lane < 27) {
        const float coef = (float)d.c.coef_lap;
        const float a = lane == 13 ? dsum - coef * centre : -coef * v;
        L1.a[(size_t)I * 27 + lane] = a;
        if (lane == 13) L1.dinv[I] = a > 0.f ? 1.f / a : 0.f;
    }
}

// Galerkin stencil of level hi from level lo: warp per hi aggregate.  The 8 x 28
// (child, slot) terms are spread over the lanes (7 each); each term's target slot
// and value go to shared memory, then lane s sums the values of slot s in term
// order (fixed order: deterministic).
constexpr int kMgCoarsenWarps = 8;
__global__ void __launch_bounds__(kMgCoarsenWarps * 32) k_mg_coarsen(MgLevel lo, MgLevel hi) {
    __shared__ float val[kMgCoarsenWarps][224];
    __shared__ signed char slot2[kMgCoarsenWarps][224];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int I2 = blockIdx.x * kMgCoarsenWarps + wib;
    if (I2 >= hi.n) return;   // warp-uniform
    int X, Y, Z;
    mg_decode(hi.ccell[I2], hi.gy, hi.gz, X, Y, Z);
    int child = -1;
    if (lane < 8) {
        const int x = 2 * X + (lane >> 2), y = 2 * Y + ((lane >> 1) & 1), z = 2 * Z + (lane & 1);
        if (x < lo.gx && y < lo.gy && z < lo.gz) child = lo.cmap[(x * lo.gy + y) * lo.gz + z];
    }
    for (int t = lane; t < 224; t += 32) {
        const int q = t / 28, s = t % 28;
        const int I = __shfl_sync(0xffffffffu, child, q);
        signed char tgt = -1;
        float v = 0.f;
        if (I >= 0 && s < 27 && lo.nb[(size_t)I * 27 + s] >= 0) {
            const int x = 2 * X + (q >> 2), y = 2 * Y + ((q >> 1) & 1), z = 2 * Z + (q & 1);
            const int px = ((x + mg_slot_dx(s)) >> 1) - X, py = ((y + mg_slot_dy(s)) >> 1) - Y,
                      pz = ((z + mg_slot_dz(s)) >> 1) - Z;
            tgt = (signed char)((px + 1) * 9 + (py + 1) * 3 + (pz + 1));
            v = lo.a[(size_t)I * 27 + s];
        }
        val[wib][t] = v;
        slot2[wib][t] = tgt;
    }
    __syncwarp();
    if (lane < 27) {
        float sum = 0.f;
        for (int t = 0; t < 224; ++t)
            if (slot2[wib][t] == lane) sum += val[wib][t];
        hi.a[(size_t)I2 * 27 + lane] = sum;
        if (lane == 13) hi.dinv[I2] = sum > 0.f ? 1.f / sum : 0.f;
    }
}

// explicit inverse of the last level (n <= kMgMaxDense) by Gauss-Jordan elimination
// in shared memory; the matrix is symmetric positive definite, so no pivoting.
// An aggregate without interior particles has an empty row: its diagonal is set
// to 1 (its residual is always 0).
__global__ void __launch_bounds__(1024) k_mg_dense_inverse(MgLevel lv, float* __restrict__ ainv) {
    extern __shared__ float sm[];
    const int n = lv.n;
    if (n <= 0 || n > kMgMaxDense) return;
    float* M = sm;           // [n][n], Gauss-Jordan in place: column k holds the inverse's after step k
    float* fk = sm + n * n;  // [n] the pivot column of the current step
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) M[t] = 0.f;
    __syncthreads();
    for (int t = threadIdx.x; t < n * 27; t += blockDim.x) {
        const int I = t / 27, s = t % 27;
        const int J = lv.nb[(size_t)I * 27 + s];
        if (J >= 0) M[I * n + J] = lv.a[(size_t)I * 27 + s];
    }
    __syncthreads();
    for (int I = threadIdx.x; I < n; I += blockDim.x)
        if (!(M[I * n + I] > 0.f)) M[I * n + I] = 1.f;
    __syncthreads();
    // each thread owns one column and the rows row0, row0 + rstep, ...  Step k reads the
    // pivot, the pivot row's entry of its column and (into fk) the pivot column, then,
    // after one barrier, writes: the pivot row divided by the pivot (1 / pivot in column
    // k), the other rows less their multiple of it (column k: minus the multiple of
    // 1 / pivot).  Per entry of the inverse these are the operations of elimination on
    // [A | I], in the same order.
    const int col = (int)threadIdx.x % n, row0 = (int)threadIdx.x / n, rstep = (int)blockDim.x / n;
    const bool owner = (int)threadIdx.x < rstep * n;
    for (int k = 0; k < n; ++k) {
        const float piv = M[k * n + k];
        const float mk = owner ? M[k * n + col] : 0.f;
        for (int i = threadIdx.x; i < n; i += blockDim.x) fk[i] = M[i * n + k];
        __syncthreads();
        if (owner) {
            const float mkn = col == k ? 1.f / piv : mk / piv;
            for (int i = row0; i < n; i += rstep) {
                if (i == k) M[i * n + col] = mkn;
                else if (col == k) M[i * n + col] = -(fk[i] * mkn);
                else M[i * n + col] = __fmaf_rn(-fk[i], mkn, M[i * n + col]);
            }
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) ainv[t] = M[t];
}

// ---------------------------------------------------------------------------
// application (every CG iteration); all return once the solve has converged
// ---------------------------------------------------------------------------
// level-1 residual: warp per aggregate sums its rows (non-interior rows hold r = 0);
// first down sweep from a zero start: e1 = omega D1^-1 r1
template <class TV>
__global__ void k_mg_restrict_fine(const __grid_constant__ Dev d, const __grid_constant__ Mg mg,
                                   const TV* __restrict__ r) {
    if (d.scal[S_CONV] != 0.0) return;
    const MgLevel& L1 = mg.L[1];
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (I >= L1.n) return;
    float s = 0.f;
    for (int i = mg.rb[I] + lane; i < mg.rb[I + 1]; i += 32) s += (float)r[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) {
        L1.r[I] = s;
        L1.e[I] = mg.omega * L1.dinv[I] * s;
    }
}

// Residual of the level-lo iterate summed over the children of level-hi aggregate I2,
// by one warp: the 8 x 28 (child, slot) terms, 7 per lane (t = lane + 32 q), then a
// fixed shuffle tree (every lane returns the sum).  Slot 27 is the child's own
// restricted residual.  The loads are issued in three waves (children; their stencil
// entries and residuals; the neighbours' corrections) instead of one dependent chain
// per term, and the terms are summed in the same order.
// lo.r and lo.e are read through L2 (CG) where other CTAs of the same launch wrote them
template <bool CG = false>
__device__ __forceinline__ float mg_child_residual_warp(const MgLevel& lo, const MgLevel& hi, int I2, int lane) {
    const int child = lane < 8 ? hi.child[(size_t)I2 * 8 + lane] : -1;
    int I[7], J[7];
    float a[7], x[7];
#pragma unroll
    for (int q = 0; q < 7; ++q) I[q] = __shfl_sync(0xffffffffu, child, (lane + 32 * q) / 28);
#pragma unroll
    for (int q = 0; q < 7; ++q) {
        const int s = (lane + 32 * q) % 28;
        J[q] = -1;
        a[q] = 0.f;
        x[q] = 0.f;
        if (I[q] >= 0) {
            if (s == 27) {
                x[q] = CG ? __ldcg(lo.r + I[q]) : lo.r[I[q]];
            } else {
                J[q] = lo.nb[(size_t)I[q] * 27 + s];
                a[q] = lo.a[(size_t)I[q] * 27 + s];
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 7; ++q)
        if (J[q] >= 0) x[q] = CG ? __ldcg(lo.e + J[q]) : lo.e[J[q]];
    float v = 0.f;
#pragma unroll
    for (int q = 0; q < 7; ++q) {
        if (I[q] < 0) continue;
        if ((lane + 32 * q) % 28 == 27) v += x[q];
        else if (J[q] >= 0) v -= a[q] * x[q];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// last level: e2 = A^-1 r with the explicit inverse, by one CTA (warp per row; r read
// through L2, it was written by other CTAs)
__device__ __forceinline__ void mg_dense_solve_cta(const MgLevel& lv, const float* __restrict__ ainv) {
    __shared__ float rs[kMgMaxDense];
    for (int I = threadIdx.x; I < lv.n; I += blockDim.x) rs[I] = __ldcg(lv.r + I);
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int I = w; I < lv.n; I += nw) {
        float v = 0.f;
        for (int J = lane; J < lv.n; J += 32) v += ainv[I * lv.n + J] * rs[J];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) lv.e2[I] = v;
    }
}

// restriction lo -> hi and the first down sweep on hi: warp per hi aggregate.  With
// ainv (hi is the last level) the CTA that finishes last (counted on `done`, reset by
// it) also solves hi with the explicit inverse, one launch less per V-cycle.
__global__ void k_mg_down(const double* __restrict__ scal, MgLevel lo, MgLevel hi, float omega,
                          const float* __restrict__ ainv, unsigned* __restrict__ done) {
    if (scal[S_CONV] != 0.0) return;   // the same for every CTA of the launch
    const int I2 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (I2 < hi.n) {   // warp-uniform
        const float s = mg_child_residual_warp(lo, hi, I2, lane);
        if (lane == 0) {
            hi.r[I2] = s;
            hi.e[I2] = omega * hi.dinv[I2] * s;
        }
    }
    if (!ainv) return;
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    mg_dense_solve_cta(hi, ainv);
    if (threadIdx.x == 0) *done = 0u;
}

// one more weighted-Jacobi sweep on a level: out = in + omega D^-1 (r - A in); warp per
// aggregate, lane per stencil slot (level 1 runs as many before the restriction as
// after the prolongation, so the V-cycle stays symmetric)
__global__ void k_mg_smooth(const double* __restrict__ scal, MgLevel lv, const float* __restrict__ in,
                            float* __restrict__ out, float omega) {
    if (scal[S_CONV] != 0.0) return;
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (I >= lv.n) return;   // warp-uniform
    float t = 0.f;
    if (lane < 27) {
        const int J = lv.nb[(size_t)I * 27 + lane];
        if (J >= 0) t = lv.a[(size_t)I * 27 + lane] * in[J];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) out[I] = in[I] + omega * lv.dinv[I] * (lv.r[I] - t);
}

// prolongation hi -> lo and the up sweep on lo: e' = e + P e_hi,
// e2 = e' + omega D^-1 (r - A e'); warp per lo aggregate, lane per stencil slot
__global__ void k_mg_up(const double* __restrict__ scal, MgLevel lo, MgLevel hi, float omega) {
    if (scal[S_CONV] != 0.0) return;
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (I >= lo.n) return;   // warp-uniform
    float t = 0.f;
    if (lane < 27) {
        const int J = lo.nb[(size_t)I * 27 + lane];
        if (J >= 0) t = lo.a[(size_t)I * 27 + lane] * (lo.e[J] + hi.e2[lo.nbp[(size_t)I * 27 + lane]]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) lo.e2[I] = lo.e[I] + hi.e2[lo.par[I]] + omega * lo.dinv[I] * (lo.r[I] - t);
}

// Bounded barrier of all CTAs of a cooperative launch (every CTA resident): arrive on
// bar[0], the last arrival resets it and advances the generation bar[1]; a wait that
// runs out sets MPS_ERR_STAGE_TIMEOUT and returns false (the CTA then stops, so the
// others run out too).
__device__ __forceinline__ bool coop_barrier(unsigned* bar, unsigned* err, long long spins) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = bar + 1;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(bar, 1u) == gridDim.x - 1) {
            bar[0] = 0u;
            __threadfence();
            atomicAdd(bar + 1, 1u);
            ok = 1;
        } else {
            long long k = 0;
            while (*gen == g && ++k < spins) {
            }
            ok = *gen != g;
            if (!ok) atomicOr(err, MPS_ERR_STAGE_TIMEOUT);
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// The coarse part of a V-cycle in one cooperative launch: the restrictions level 1 ->
// 2 -> ... -> last with their first down sweeps (as k_mg_down, a warp per aggregate of
// the coarser level), the dense solve of the last level (a warp per row),
// and the up sweeps of levels last-1 .. 2 (as k_mg_up), with a grid barrier between
// the stages; the level-2 -> 1 up sweep stays fused with the fine level
// (k_mg_up_fine_z).  Values other CTAs wrote in this launch are read through L2.
__global__ void __launch_bounds__(256) k_mg_coarse_cycle(const double* __restrict__ scal, Mg mg,
                                                         unsigned* __restrict__ bar, unsigned* __restrict__ err) {
    pdl_trigger();   // launched in stream order: only lets the next kernel's launch overlap
    if (scal[S_CONV] != 0.0) return;   // the same for every CTA of the launch
    const int lane = threadIdx.x & 31;
    const int w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int lv = mg.levels;
    const float omega = mg.omega;
    constexpr long long kSpins = 1ll << 20;
    for (int l = 1; l < lv; ++l) {
        const MgLevel& lo = mg.L[l];
        const MgLevel& hi = mg.L[l + 1];
        for (int I2 = w0; I2 < hi.n; I2 += nw) {   // warp-uniform
            const float s = l == 1 ? mg_child_residual_warp<false>(lo, hi, I2, lane)
                                   : mg_child_residual_warp<true>(lo, hi, I2, lane);
            if (lane == 0) {
                hi.r[I2] = s;
                hi.e[I2] = omega * hi.dinv[I2] * s;
            }
        }
        if (!coop_barrier(bar, err, kSpins)) return;
    }
    {   // the last level: e2 = A^-1 r with the explicit inverse, a warp per row
        const MgLevel& L = mg.L[lv];
        for (int I = w0; I < L.n; I += nw) {
            float v = 0.f;
            for (int J = lane; J < L.n; J += 32) v += mg.ainv[I * L.n + J] * __ldcg(L.r + J);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) L.e2[I] = v;
        }
    }
    if (lv <= 2) return;
    if (!coop_barrier(bar, err, kSpins)) return;
    for (int l = lv - 1; l >= 2; --l) {
        const MgLevel& lo = mg.L[l];
        const MgLevel& hi = mg.L[l + 1];
        for (int I = w0; I < lo.n; I += nw) {   // warp-uniform
            float t = 0.f;
            if (lane < 27) {
                const int J = lo.nb[(size_t)I * 27 + lane];
                if (J >= 0)
                    t = lo.a[(size_t)I * 27 + lane] * (__ldcg(lo.e + J) + __ldcg(hi.e2 + lo.nbp[(size_t)I * 27 + lane]));
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (lane == 0)
                lo.e2[I] = __ldcg(lo.e + I) + __ldcg(hi.e2 + lo.par[I]) + omega * lo.dinv[I] * (__ldcg(lo.r + I) - t);
        }
        if (l > 2 && !coop_barrier(bar, err, kSpins)) return;
    }
}

// the last prolongation and up sweep (level 2 -> level 1) fused with the fine level:
// warp per level-1 aggregate computes e1[I] as k_mg_up, then z = m r + e1[I] over the
// cell's rows (every row lies in one cell), p = z in mode 1, and r.z as k_mg_fine_z
// (S_RZ, or S_BETA and S_RZ); one pass over the rows instead of two launches
// With qf (flexible CG, mode 0): also z.q of the last direction's product q = A p, and
// S_BETA = -(z.q) / (p.q) (Notay's flexible CG keeping one direction) instead of the
// ratio of successive r.z.
// level-1 aggregates per warp in k_mg_up_fine_z (8 resident CTAs of 8 warps per SM at 32
// registers: the 16k aggregates of the 882k-particle bucket in one wave)
constexpr int kMgUpAgg = 2;
template <class TV>
__global__ void __launch_bounds__(256) k_mg_up_fine_z(const __grid_constant__ Dev d, const __grid_constant__ Mg mg,
                                                      const TV* __restrict__ r, TV* __restrict__ z,
                                                      TV* __restrict__ p, const float* __restrict__ m32, int mode,
                                                      int slot, const TV* __restrict__ qf = nullptr) {
    pdl_wait();
    pdl_trigger();
    if (d.scal[S_CONV] != 0.0) return;
    const MgLevel& lo = mg.L[1];
    const MgLevel& hi = mg.L[2];
    const float omega = mg.omega;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    TV prz = TV(0), pzq = TV(0);
    // kMgUpAgg adjacent aggregates per warp (one wave of warps for the level): every
    // aggregate's row range, first rows and stencil terms are loaded before any is
    // finished, so the warp has kMgUpAgg dependent-load chains in flight; the lane's first
    // row of each is loaded before the stencil gathers (it does not depend on them)
    constexpr int kPf = 1;
    int I[kMgUpAgg], rb0[kMgUpAgg], rb1[kMgUpAgg];
    TV pr[kMgUpAgg][kPf], pq[kMgUpAgg][kPf];
    float pm[kMgUpAgg][kPf], t[kMgUpAgg];
    bool pin[kMgUpAgg][kPf];
#pragma unroll
    for (int h = 0; h < kMgUpAgg; ++h) {
        I[h] = kMgUpAgg * wg + h;
        const bool on = I[h] < lo.n;   // warp-uniform
        rb0[h] = on ? mg.rb[I[h]] : 0;
        rb1[h] = on ? mg.rb[I[h] + 1] : 0;
    }
#pragma unroll
    for (int h = 0; h < kMgUpAgg; ++h) {
#pragma unroll
        for (int u = 0; u < kPf; ++u) {
            const int i = rb0[h] + lane + 32 * u;
            pin[h][u] = i < rb1[h] && d.inner[i];
            pr[h][u] = pin[h][u] ? r[i] : TV(0);
            pm[h][u] = pin[h][u] ? m32[i] : 0.f;
            pq[h][u] = (pin[h][u] && qf) ? qf[i] : TV(0);
        }
        t[h] = 0.f;
        if (I[h] < lo.n && lane < 27) {
            const int J = lo.nb[(size_t)I[h] * 27 + lane];
            if (J >= 0) t[h] = lo.a[(size_t)I[h] * 27 + lane] * (lo.e[J] + hi.e2[lo.nbp[(size_t)I[h] * 27 + lane]]);
        }
    }
#pragma unroll
    for (int h = 0; h < kMgUpAgg; ++h) {
        if (I[h] >= lo.n) break;   // warp-uniform; every thread reaches the grid reduction
        float th = t[h];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) th += __shfl_xor_sync(0xffffffffu, th, o);
        const int a = I[h];
        const float e1 = lo.e[a] + hi.e2[lo.par[a]] + omega * lo.dinv[a] * (lo.r[a] - th);
        if (lane == 0) lo.e2[a] = e1;
#pragma unroll
        for (int u = 0; u < kPf; ++u) {
            const int i = rb0[h] + lane + 32 * u;
            if (i >= rb1[h]) break;
            TV zi = TV(0);
            if (pin[h][u]) {
                zi = (TV)pm[h][u] * pr[h][u] + (TV)e1;
                prz += pr[h][u] * zi;
                if (qf) pzq += zi * pq[h][u];
            }
            z[i] = zi;
            if (mode == 1) p[i] = zi;
        }
        for (int i = rb0[h] + lane + 32 * kPf; i < rb1[h]; i += 32) {
            TV zi = TV(0);
            if (d.inner[i]) {
                zi = (TV)m32[i] * r[i] + (TV)e1;
                prz += r[i] * zi;
                if (qf) pzq += zi * qf[i];
            }
            z[i] = zi;
            if (mode == 1) p[i] = zi;
        }
    }
    double v[2] = {(double)prz, (double)pzq}, out[2];
    if (grid_reduce<2, TV>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        if (mode == 1) {
            d.scal[S_RZ] = out[0];
        } else if (qf) {
            const double pq = d.scal[S_PQ];
            d.scal[S_BETA] = pq != 0.0 ? -out[1] / pq : 0.0;
            d.scal[S_RZ] = out[0];
        } else {
            const double rz = d.scal[S_RZ];
            d.scal[S_BETA] = rz != 0.0 ? out[0] / rz : 0.0;
            d.scal[S_RZ] = out[0];
        }
    }
}

// CG update fused with the level-1 restriction (multilevel path): warp per level-1
// aggregate over its contiguous rows: x += alpha p, r -= alpha q on interior rows,
// r1[I] = sum of r over the cell, the first down sweep e1 = omega D1^-1 r1, and
// ||r||^2 with the convergence test (as k_cg_update with_z = 0).
template <class TV, class TXA>
__global__ void __launch_bounds__(256) k_mg_update_restrict(const __grid_constant__ Dev d, const __grid_constant__ Mg mg,
                                                            TXA* __restrict__ x, TV* __restrict__ r,
                                                            const TV* __restrict__ p, const TV* __restrict__ q, int slot) {
    pdl_wait();
    pdl_trigger();
    if (d.scal[S_CONV] != 0.0) return;
    const MgLevel& L1 = mg.L[1];
    const TV alpha = (TV)d.scal[S_ALPHA];
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    TV prr = TV(0);
    // two adjacent aggregates per warp and step of the grid-stride loop (the launch gives
    // about one pair per warp: one wave): both row ranges, then both first row chunks are
    // loaded before either is updated, so two dependent-load chains are in flight
    auto row = [&](int i, float& s) {
        if (!d.inner[i]) return;
        x[i] = x[i] + (TXA)alpha * (TXA)p[i];
        const TV ri = r[i] - alpha * q[i];
        r[i] = ri;
        prr += ri * ri;
        s += (float)ri;
    };
    for (int I = 2 * ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); I < L1.n; I += 2 * nw) {
        const bool two = I + 1 < L1.n;   // warp-uniform
        const int a0 = mg.rb[I], a1 = mg.rb[I + 1], b1 = two ? mg.rb[I + 2] : a1;
        float sa = 0.f, sb = 0.f;
        const int ia = a0 + lane, ib = a1 + lane;
        if (ia < a1) row(ia, sa);
        if (ib < b1) row(ib, sb);
        for (int i = ia + 32; i < a1; i += 32) row(i, sa);
        for (int i = ib + 32; i < b1; i += 32) row(i, sb);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sa += __shfl_down_sync(0xffffffffu, sa, o);
            sb += __shfl_down_sync(0xffffffffu, sb, o);
        }
        if (lane == 0) {
            L1.r[I] = sa;
            L1.e[I] = mg.omega * L1.dinv[I] * sa;
            if (two) {
                L1.r[I + 1] = sb;
                L1.e[I + 1] = mg.omega * L1.dinv[I + 1] * sb;
            }
        }
    }
    double v[1] = {(double)prr}, out[1];
    if (grid_reduce<1, TV>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        const double rn = sqrt(out[0]);
        d.scal[S_RNORM] = rn;
        const double it = d.scal[S_ITER] + 1.0;
        d.scal[S_ITER] = it;
        if (rn <= d.scal[S_TOL] || it >= d.scal[S_MAXIT] || !(rn == rn)) d.scal[S_CONV] = 1.0;
    }
}

// ---------------------------------------------------------------------------
// Post-smoothing of the coarse correction through the short-range couplings
// (MpsSolverOptions::fine_smoother = 1): z = P e1 + omega m (r - A_s P e1), where A_s
// is the PPE operator restricted to the neighbours within the gradient radius (its
// diagonal the full one) and m the fine diagonal preconditioner (1 / A_ii, or the
// learned scaling of it).  P e1 is constant per cell, so A_s P e1 at row i is a sum over
// the at most 27 neighbouring cells of the row's couplings lumped per cell: the rows
// R[slot][i] below, built once per step.  The preconditioner is not symmetric; the
// inner solve runs as flexible CG.
// ---------------------------------------------------------------------------
constexpr int kMgSmThreads = 128;
// R[s * n + i] = -(sum of c w_ij over interior j of the gradient row of i whose cell is
// at slot s of i's cell), plus A_ii at the centre slot 13; mask bit s for the nonzero
// slots.  Slot sums are kept in a per-thread shared-memory column.
__global__ void __launch_bounds__(kMgSmThreads) k_mg_smoother_rows(const __grid_constant__ Dev d,
                                                                   const __grid_constant__ Mg mg, float* R,
                                                                   unsigned* mask) {
    __shared__ float acc[27 * kMgSmThreads];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    if (!d.inner[i]) {
        mask[i] = 0u;
        return;
    }
    float* a = acc + threadIdx.x;
#pragma unroll
    for (int s = 0; s < 27; ++s) a[s * kMgSmThreads] = 0.f;
    const unsigned pi = mg.pcc[i];
    const float re = (float)d.c.re_lap, mind = (float)d.c.mind_lap, c = (float)d.c.coef_lap;
    const int cnt = min(d.gcnt[i], d.KG);
    const int* __restrict__ gj = d.gnbr + (size_t)i * d.KG;
    const float* __restrict__ gr = (const float*)d.gnbrr + (size_t)i * d.KG;
    for (int k = 0; k < cnt; ++k) {
        const int j = gj[k];
        if (!d.inner[j]) continue;
        const unsigned pj = mg.pcc[j];
        const int dx = (int)((pj >> 20) & 1023u) - (int)((pi >> 20) & 1023u);
        const int dy = (int)((pj >> 10) & 1023u) - (int)((pi >> 10) & 1023u);
        const int dz = (int)(pj & 1023u) - (int)(pi & 1023u);
        if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) continue;   // beyond one cell: none
        const int s = (dx + 1) * 9 + (dy + 1) * 3 + (dz + 1);
        a[s * kMgSmThreads] -= c * (re / fmaxf(gr[k], mind) - 1.f);
    }
    a[13 * kMgSmThreads] += (float)d.diag[i];
    unsigned m = 0u;
    const size_t n = (size_t)d.n;
#pragma unroll
    for (int s = 0; s < 27; ++s) {
        const float v = a[s * kMgSmThreads];
        R[s * n + i] = v;
        if (v != 0.f) m |= 1u << s;
    }
    mask[i] = m;
}

// fine level with post-smoothing: z = e1[a] + omega m32 (r - sum_s R[s][i] e1[nb(a, s)])
// on interior rows (0 elsewhere); r.z (and z.q with qf) as k_mg_fine_z
template <class TV>
__global__ void __launch_bounds__(256) k_mg_fine_post(const __grid_constant__ Dev d, const __grid_constant__ Mg mg,
                                                      const TV* __restrict__ r, TV* __restrict__ z, TV* __restrict__ p,
                                                      const float* __restrict__ m32, int mode, int slot,
                                                      const TV* __restrict__ qf, const float* __restrict__ R,
                                                      const unsigned* __restrict__ mask, float omega) {
    if (d.scal[S_CONV] != 0.0) return;
    const MgLevel& L1 = mg.L[1];
    const float* e1 = L1.e2;
    const size_t n = (size_t)d.n;
    TV prz = TV(0), pzq = TV(0);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x) {
        TV zi = TV(0);
        if (d.inner[i] && mg.agg1[i] < 0) {   // no aggregate: the diagonal term alone
            zi = (TV)m32[i] * r[i];
            prz += r[i] * zi;
            if (qf) pzq += zi * qf[i];
        } else if (d.inner[i]) {
            const int a = mg.agg1[i];
            float t = 0.f;
            unsigned msk = mask[i];
            while (msk) {
                const int s = __ffs(msk) - 1;
                msk &= msk - 1u;
                const int b = s == 13 ? a : L1.nb[(size_t)a * 27 + s];
                if (b >= 0) t = fmaf(R[s * n + i], e1[b], t);
            }
            zi = (TV)(e1[a] + omega * m32[i] * ((float)r[i] - t));
            prz += r[i] * zi;
            if (qf) pzq += zi * qf[i];
        }
        z[i] = zi;
        if (mode == 1) p[i] = zi;
    }
    double v[2] = {(double)prz, (double)pzq}, out[2];
    if (grid_reduce<2, TV>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        if (mode == 1) {
            d.scal[S_RZ] = out[0];
        } else if (qf) {
            const double pq = d.scal[S_PQ];
            d.scal[S_BETA] = pq != 0.0 ? -out[1] / pq : 0.0;
            d.scal[S_RZ] = out[0];
        } else {
            const double rz = d.scal[S_RZ];
            d.scal[S_BETA] = rz != 0.0 ? out[0] / rz : 0.0;
            d.scal[S_RZ] = out[0];
        }
    }
}

// last level: e2 = A^-1 r with the explicit inverse (one CTA, warp per row)
__global__ void __launch_bounds__(1024) k_mg_dense_solve(const double* __restrict__ scal, MgLevel lv,
                                                         const float* __restrict__ ainv) {
    if (scal[S_CONV] != 0.0) return;
    mg_dense_solve_cta(lv, ainv);
}

// fine level: z = m r + e1[aggregate] on interior rows (0 elsewhere), rz = r.z;
// mode 1 (start): S_RZ = rz and p = z; mode 0: S_BETA = rz / S_RZ, S_RZ = rz
template <class TV>
__global__ void __launch_bounds__(256) k_mg_fine_z(const __grid_constant__ Dev d, const __grid_constant__ Mg mg,
                                                   const TV* __restrict__ r, TV* __restrict__ z, TV* __restrict__ p,
                                                   const float* __restrict__ m32, int mode, int slot,
                                                   const TV* __restrict__ qf = nullptr) {
    if (d.scal[S_CONV] != 0.0) return;
    const float* e1 = mg.L[1].e2;
    TV prz = TV(0), pzq = TV(0);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x) {
        TV zi = TV(0);
        if (d.inner[i]) {
            const int a = mg.agg1[i];
            zi = (TV)m32[i] * r[i] + (a >= 0 ? (TV)e1[a] : TV(0));
            prz += r[i] * zi;
            if (qf) pzq += zi * qf[i];
        }
        z[i] = zi;
        if (mode == 1) p[i] = zi;
    }
    double v[2] = {(double)prz, (double)pzq}, out[2];
    if (grid_reduce<2, TV>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        if (mode == 1) {
            d.scal[S_RZ] = out[0];
        } else if (qf) {
            const double pq = d.scal[S_PQ];
            d.scal[S_BETA] = pq != 0.0 ? -out[1] / pq : 0.0;
            d.scal[S_RZ] = out[0];
        } else {
            const double rz = d.scal[S_RZ];
            d.scal[S_BETA] = rz != 0.0 ? out[0] / rz : 0.0;
            d.scal[S_RZ] = out[0];
        }
    }
}

}  // namespace mps
