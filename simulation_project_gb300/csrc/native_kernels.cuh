// native_kernels.cuh - kernels of the GB300-native semi-implicit step.
//
// Every particle kernel works in the cell-sorted order.  Neighbour passes run one CTA
// per non-empty cell: the CTA stages the nine z-runs of the 27 surrounding cells (each
// run is contiguous in sorted order) into shared memory as float4, then each warp takes
// one target particle at a time and its 32 lanes test 32 staged candidates per step;
// accepted neighbours are compacted with __ballot_sync/__popc so a warp writes each
// neighbour row as contiguous, coalesced segments.
#pragma once

#include <type_traits>

#include "native.cuh"

#include <utility>

namespace mps {

constexpr int kNbThreads = 256;
constexpr int kStageCap = 2048;
constexpr int kRedBlocks = 1216;   // 152 SMs x 8 resident CTAs of 256 threads
constexpr int kVecThreads = 256;

enum { NB_PREDICT = 0, NB_LIST = 1 };

template <class T> struct V3 { T x, y, z; };

// ---- programmatic dependent launch (the CG iteration's chain of kernels) ----
// A kernel launched by launch_pdl may be scheduled while the previous kernel of its
// stream still runs: it waits at pdl_wait() until that kernel has completed and its
// writes are visible, so only its launch overlaps the predecessor's tail.  Every kernel
// launched that way calls pdl_wait() before its first read of device data; pdl_trigger()
// lets the next kernel's CTAs be scheduled once every CTA of this one has started.
// Both are no-ops for an ordinary launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... KArgs, class... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), int grid, int block, size_t smem, cudaStream_t st, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// ---- bulk (TMA) copies global -> shared, completed on an mbarrier ----
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// one arrival that also announces `bytes` of transactions
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test_parity(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bytes (a multiple of 16) from a 16-byte-aligned global address to a 16-byte-aligned
// shared address; completion is counted on bar
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// L2 policy for streamed data read once: evict first (keeps the vectors that the
// next kernels reuse resident in L2)
__device__ __forceinline__ unsigned long long l2_evict_first_policy() {
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
// bulk copy as bulk_copy_g2s with an L2 cache policy
__device__ __forceinline__ void bulk_copy_g2s_hint(void* dst, const void* src, unsigned bytes, unsigned long long* bar,
                                                   unsigned long long pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}
// bounded wait on phase 0 of bar: false if it did not complete within `spins` polls
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, long long spins) {
    for (long long k = 0; k < spins; ++k)
        if (mbar_test_parity(bar, 0)) return true;
    return false;
}
// bounded wait for the completion of the phase with the given parity
__device__ __forceinline__ bool mbar_wait_parity_bounded(unsigned long long* bar, unsigned parity, long long spins) {
    for (long long k = 0; k < spins; ++k)
        if (mbar_test_parity(bar, parity)) return true;
    return false;
}
// orders this thread's earlier generic-proxy accesses to shared memory (after a warp
// barrier: the warp's reads of a stage) before later bulk copies into it
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// a / b: IEEE division in FP64; in FP32 the fast approximate form (<= 2 ulp), which
// the neighbour passes use for their weights (it is issued for every accepted pair)
template <class T>
__device__ __forceinline__ T wdiv(T a, T b) {
    if constexpr (sizeof(T) == 4) return __fdividef(a, b);
    return a / b;
}

// SELL-32 position of entry k of row i (row capacity K)
__device__ __forceinline__ size_t sell_index(int i, int k, int K) {
    return ((size_t)(i >> 5) * K + k) * 32 + (i & 31);
}
template <class T> __device__ __forceinline__ V3<T> v3(T x, T y, T z) { V3<T> r; r.x = x; r.y = y; r.z = z; return r; }

// ---------------------------------------------------------------------------
// deterministic block + grid reductions (last CTA finishes the sum)
// ---------------------------------------------------------------------------
// TS: type of the in-warp shuffle stage (float for the FP32 inner solve, whose
// per-thread partials are float anyway; the FP64 pipe is narrow on GB300); the
// cross-warp and cross-block stages are always FP64.
template <int NV, class TS = double>
__device__ __forceinline__ bool grid_reduce(double (&v)[NV], double* red, unsigned* counter, double (&out)[NV]) {
    __shared__ double sm[NV][32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        TS x = (TS)v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sm[k][w] = (double)x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = 0.0;
            for (int i = 0; i < nw; ++i) s += sm[k][i];
            red[(size_t)k * gridDim.x + blockIdx.x] = s;
        }
        __threadfence();
        const unsigned t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double s = 0.0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += ((volatile double*)red)[(size_t)k * gridDim.x + i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) sm[k][w] = s;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double s = 0.0;
        for (int i = 0; i < nw; ++i) s += sm[k][i];
        out[k] = s;
    }
    if (threadIdx.x == 0) *counter = 0;
    return true;
}

// ---------------------------------------------------------------------------
// grid build
// ---------------------------------------------------------------------------
__global__ void k_zone_flags(const __grid_constant__ Dev d, unsigned* keep) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const dbl4 p = d.pos[i];
    keep[i] = in_zone<double>(d.box, p.x, p.y, p.z, d.c.tol) ? 1u : 0u;
}

// stable compaction: survivors keep their relative order
__global__ void k_compact(const __grid_constant__ Dev d, const unsigned* keep, const unsigned* rank) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n || !keep[i]) return;
    const int o = (int)rank[i];
    d.pos2[o] = d.pos[i];
    d.vel2[o] = d.vel[i];
    d.press2[o] = d.press[i];
    d.visc2[o] = d.visc[i];
    d.type2[o] = d.type[i];
    d.id2[o] = d.id[i];
    d.dph1b[o] = d.dph1[i];
    d.dph2b[o] = d.dph2[i];
}

__global__ void k_hash(const __grid_constant__ Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const dbl4 p = d.pos[i];
    // cell coordinates from one reciprocal (FP64 divisions are slow on GB300's narrow
    // FP64 pipe); only a coordinate within an ulp of a cell face can land otherwise
    const double ics = 1.0 / (double)d.box.m_CellSize;
    const double fz = (p.z - (double)d.box.m_BufferedZone.m_MinBound.z) * ics;
    const int a = f2i((p.x - (double)d.box.m_BufferedZone.m_MinBound.x) * ics);
    const int b = f2i((p.y - (double)d.box.m_BufferedZone.m_MinBound.y) * ics);
    const int c = f2i(fz);
    int k = cell_key(d.box.m_GridSize, a, b, c);
    if (k < 0 || k >= d.cells) {
        atomicOr(d.err, MPS_ERR_KEY_RANGE);
        k = k < 0 ? 0 : d.cells - 1;
    }
    // particles of a cell are ordered by a z bin (1/64 of the cell): each 3-cell z-run
    // of the neighbour search is then sorted by z, so a target can clip it
    int zq = 0;
    if (d.zbits) {
        zq = f2i((fz - (double)c) * (double)(1 << d.zbits));
        zq = zq < 0 ? 0 : (zq > (1 << d.zbits) - 1 ? (1 << d.zbits) - 1 : zq);
    }
    d.skey[i] = (k << d.zbits) | zq;
    d.idx[i] = i;
}

// gather into sorted order + cell ranges + list of non-empty cells
__global__ void k_gather(const __grid_constant__ Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const int s = d.idx[i];
    const dbl4 p = d.pos[s], v = d.vel[s];
    d.pos2[i] = p;
    d.vel2[i] = v;
    d.press2[i] = d.press[s];
    d.visc2[i] = d.visc[s];
    d.type2[i] = d.type[s];
    d.id2[i] = d.id[s];
    d.dph1b[i] = d.dph1[s];
    d.dph2b[i] = d.dph2[s];
    const int sk = d.skey[i];
    const int h = sk >> d.zbits;
    // global z bin (cell z * 64 + bin inside the cell), exact in a float
    const float zbin = (float)((h % d.box.m_GridSize.z) * 64 + ((sk & ((1 << d.zbits) - 1)) << (6 - d.zbits)));
    d.opos[i] = make_float4((float)p.x, (float)p.y, (float)p.z, zbin);
    d.ovel[i] = make_float4((float)v.x, (float)v.y, (float)v.z, 0.f);
    d.key[i] = h;
    const int hp = i > 0 ? (d.skey[i - 1] >> d.zbits) : -1;
    if (i == 0 || h != hp) {
        d.cstart[h] = i;
        if (i > 0) d.cend[hp] = i;
        const int slot = atomicAdd(d.cell_count, 1);
        d.cell_list[slot] = h;
    }
    if (i == d.n - 1) d.cend[h] = i + 1;
}

// ---------------------------------------------------------------------------
// walls: bounding-box binning, exact distances, drag, motion
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tri_cell_box(const Dev& d, int t, int& i0, int& j0, int& k0, int& i1, int& j1, int& k1) {
    const double* v = d.tri + 9 * (size_t)t;
    double lo[3] = {v[0], v[1], v[2]}, hi[3] = {v[0], v[1], v[2]};
    for (int q = 1; q < 3; ++q)
        for (int a = 0; a < 3; ++a) {
            lo[a] = fmin(lo[a], v[3 * q + a]);
            hi[a] = fmax(hi[a], v[3 * q + a]);
        }
    const double cs = d.box.m_CellSize;
    const CBox& B = d.box.m_BufferedZone;
    i0 = max(f2i((lo[0] - (double)B.m_MinBound.x) / cs), 0);
    j0 = max(f2i((lo[1] - (double)B.m_MinBound.y) / cs), 0);
    k0 = max(f2i((lo[2] - (double)B.m_MinBound.z) / cs), 0);
    i1 = min(f2i((hi[0] - (double)B.m_MinBound.x) / cs), d.box.m_GridSize.x - 1);
    j1 = min(f2i((hi[1] - (double)B.m_MinBound.y) / cs), d.box.m_GridSize.y - 1);
    k1 = min(f2i((hi[2] - (double)B.m_MinBound.z) / cs), d.box.m_GridSize.z - 1);
    // halo: the cells whose 27-cell neighbourhood meets the triangle's cells (a cell's
    // list is then the union of its neighbours' box lists, each triangle once)
    if (i0 <= i1 && j0 <= j1 && k0 <= k1) {
        i0 = max(i0 - 1, 0); j0 = max(j0 - 1, 0); k0 = max(k0 - 1, 0);
        i1 = min(i1 + 1, d.box.m_GridSize.x - 1);
        j1 = min(j1 + 1, d.box.m_GridSize.y - 1);
        k1 = min(k1 + 1, d.box.m_GridSize.z - 1);
    }
}
// entries of each triangle's (grown) cell box; a box holds at most the grid's cells, so
// one count fits 32 bits, and the 64-bit total tells the host whether the 32-bit
// offsets of the scan (and the int entry indices of the sort) can hold them all
__global__ void k_bin_count(const __grid_constant__ Dev d, unsigned* cnt, unsigned long long* total) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.tri_n) return;
    int i0, j0, k0, i1, j1, k1;
    tri_cell_box(d, t, i0, j0, k0, i1, j1, k1);
    const long long c = (long long)max(i1 - i0 + 1, 0) * max(j1 - j0 + 1, 0) * max(k1 - k0 + 1, 0);
    cnt[t] = (unsigned)c;
    atomicAdd(total, (unsigned long long)c);
}
// warp per triangle: its lanes write the (cell key, triangle) entries of its cell box,
// entry q = ((i - i0) nj + (j - j0)) nk + (k - k0) at off[t] + q (at most the counted ones)
__global__ void k_bin_fill(const __grid_constant__ Dev d, const unsigned* off, int* vcell, int* vtri) {
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (t >= d.tri_n) return;   // warp-uniform
    int i0, j0, k0, i1, j1, k1;
    tri_cell_box(d, t, i0, j0, k0, i1, j1, k1);
    const unsigned o = off[t];
    const unsigned cnt = off[t + 1] - o;
    const int nj = j1 - j0 + 1, nk = k1 - k0 + 1;
    const int kind = d.tdrag[t] != 0 ? 1 : 0;   // wall and drag triangles in separate lists
    for (unsigned q = lane; q < cnt; q += 32) {
        const int k = k0 + (int)(q % (unsigned)nk);
        const int j = j0 + (int)((q / (unsigned)nk) % (unsigned)nj);
        const int i = i0 + (int)(q / ((unsigned)nk * (unsigned)nj));
        vcell[o + q] = 2 * cell_key(d.box.m_GridSize, i, j, k) + kind;
        vtri[o + q] = t;
    }
}
__global__ void k_bin_bounds(int nv, const int* vcell, int* ts, int* te) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int c = vcell[i];
    if (i == 0 || c != vcell[i - 1]) {
        ts[c] = i;
        if (i > 0) te[vcell[i - 1]] = i;
    }
    if (i == nv - 1) te[c] = i + 1;
}

// Closest point on triangle (a, b, c) to p by Voronoi-region classification
// (Ericson, Real-Time Collision Detection, 5.1.5).
template <class T>
__device__ V3<T> closest_on_tri(const V3<T>& p, const V3<T>& a, const V3<T>& b, const V3<T>& c) {
    const V3<T> ab = v3(b.x - a.x, b.y - a.y, b.z - a.z), ac = v3(c.x - a.x, c.y - a.y, c.z - a.z);
    const V3<T> ap = v3(p.x - a.x, p.y - a.y, p.z - a.z);
    const T d1 = ab.x * ap.x + ab.y * ap.y + ab.z * ap.z, d2 = ac.x * ap.x + ac.y * ap.y + ac.z * ap.z;
    if (d1 <= T(0) && d2 <= T(0)) return a;
    const V3<T> bp = v3(p.x - b.x, p.y - b.y, p.z - b.z);
    const T d3 = ab.x * bp.x + ab.y * bp.y + ab.z * bp.z, d4 = ac.x * bp.x + ac.y * bp.y + ac.z * bp.z;
    if (d3 >= T(0) && d4 <= d3) return b;
    const T vc = d1 * d4 - d3 * d2;
    if (vc <= T(0) && d1 >= T(0) && d3 <= T(0)) {
        const T s = d1 / (d1 - d3);
        return v3(a.x + s * ab.x, a.y + s * ab.y, a.z + s * ab.z);
    }
    const V3<T> cp = v3(p.x - c.x, p.y - c.y, p.z - c.z);
    const T d5 = ab.x * cp.x + ab.y * cp.y + ab.z * cp.z, d6 = ac.x * cp.x + ac.y * cp.y + ac.z * cp.z;
    if (d6 >= T(0) && d5 <= d6) return c;
    const T vb = d5 * d2 - d1 * d6;
    if (vb <= T(0) && d2 >= T(0) && d6 <= T(0)) {
        const T s = d2 / (d2 - d6);
        return v3(a.x + s * ac.x, a.y + s * ac.y, a.z + s * ac.z);
    }
    const T va = d3 * d6 - d5 * d4;
    if (va <= T(0) && (d4 - d3) >= T(0) && (d5 - d6) >= T(0)) {
        const T s = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        return v3(b.x + s * (c.x - b.x), b.y + s * (c.y - b.y), b.z + s * (c.z - b.z));
    }
    const T den = T(1) / (va + vb + vc);
    const T v = vb * den, w = vc * den;
    return v3(a.x + ab.x * v + ac.x * w, a.y + ab.y * v + ac.y * w, a.z + ab.z * v + ac.z * w);
}

// Nearest triangle of a particle.  Candidates are visited in increasing triangle id and
// one replaces the current nearest only when it is closer by more than a tolerance
// (1e-12 l0 in FP64, 1e-5 l0 in FP32): triangles at the same distance (a closest point
// on a shared edge or vertex, whose distances differ only by rounding) resolve to the
// lowest id instead of to the rounding of one implementation.  The choice matters for
// drag bodies, whose drag acts along the chosen triangle's normal.
template <class T>
__device__ void nearest_tri(const Dev& d, const V3<T>& p, bool drag_only, T& md, V3<T>& mdir, int& mid) {
    const T tol = sizeof(T) == 8 ? T(1e-12 * d.c.l0) : T(1e-5 * d.c.l0);
    md = T(1e8);
    mdir = v3(T(0), T(0), T(0));
    mid = -1;
    int cx, cy, cz;
    if constexpr (sizeof(T) == 4) {
        // FP32 path: cell of the candidate triangles in FP32 (the wall influence radius
        // is at most one cell, so the 27-cell neighbourhood covers it either way)
        const float inv = (float)(1.0 / (double)d.box.m_CellSize);
        cx = f2i((p.x - d.box.m_BufferedZone.m_MinBound.x) * inv);
        cy = f2i((p.y - d.box.m_BufferedZone.m_MinBound.y) * inv);
        cz = f2i((p.z - d.box.m_BufferedZone.m_MinBound.z) * inv);
    } else {
        const double cs = d.box.m_CellSize;
        cx = f2i(((double)p.x - (double)d.box.m_BufferedZone.m_MinBound.x) / cs);
        cy = f2i(((double)p.y - (double)d.box.m_BufferedZone.m_MinBound.y) / cs);
        cz = f2i(((double)p.z - (double)d.box.m_BufferedZone.m_MinBound.z) / cs);
    }
    // the triangles binned around the particle's cell (clamped to the grid): the halo
    // list of that cell, walls or drag bodies, each triangle once
    const Integer3 G = d.box.m_GridSize;
    cx = min(max(cx, 0), G.x - 1);
    cy = min(max(cy, 0), G.y - 1);
    cz = min(max(cz, 0), G.z - 1);
    const int key = 2 * cell_key(G, cx, cy, cz) + (drag_only ? 1 : 0);
    const int s = d.tcs[key];
    if (s < 0) return;
    const int e = d.tcs[2 * d.cells + key];
    for (int l = s; l < e; ++l) {
        const int t = d.tids[l];
        V3<T> q;
        if constexpr (sizeof(T) == 4) {
            const float* v = d.tri32 + 9 * (size_t)t;
            q = closest_on_tri<T>(p, v3<T>(v[0], v[1], v[2]), v3<T>(v[3], v[4], v[5]), v3<T>(v[6], v[7], v[8]));
        } else {
            const double* v = d.tri + 9 * (size_t)t;
            q = closest_on_tri<T>(p, v3<T>(v[0], v[1], v[2]), v3<T>(v[3], v[4], v[5]), v3<T>(v[6], v[7], v[8]));
        }
        const V3<T> dv = v3(p.x - q.x, p.y - q.y, p.z - q.z);
        const T dd = sqrt(dv.x * dv.x + dv.y * dv.y + dv.z * dv.z);
        if (dd < md - tol) {
            md = dd;
            mdir = dv;
            mid = t;
        }
    }
}

template <class T>
__device__ __forceinline__ V3<T> load_p(const Dev& d, int i) {
    if constexpr (sizeof(T) == 8) {
        const dbl4 p = d.pos[i];
        return v3<T>(p.x, p.y, p.z);
    } else {
        const float4 p = d.opos[i];
        return v3<T>(p.x, p.y, p.z);
    }
}
template <class T>
__device__ __forceinline__ V3<T> load_v(const Dev& d, int i) {
    if constexpr (sizeof(T) == 8) {
        const dbl4 p = d.vel[i];
        return v3<T>(p.x, p.y, p.z);
    } else {
        const float4 p = d.ovel[i];
        return v3<T>(p.x, p.y, p.z);
    }
}

template <class T>
__global__ void k_wall_distance(const __grid_constant__ Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    T md;
    V3<T> dir;
    int mid;
    nearest_tri<T>(d, load_p<T>(d, i), false, md, dir, mid);
    d.wdist[i] = md;
    d.wdir[3 * (size_t)i] = dir.x;
    d.wdir[3 * (size_t)i + 1] = dir.y;
    d.wdir[3 * (size_t)i + 2] = dir.z;
    d.wid[i] = mid;
}

// Per-body drag (CalcDragEffect_Kernel, DeviceProcess_Kernel.h:309-389, without the
// reference's sorted/original index mix-up): nearest drag-model triangle within the
// influence radius; 'E'+'V'/'B': velocity decrement k |u|^e n / permeability;
// 'C': constant velocity; 'F': velocity factor.
template <class T>
__global__ void k_drag(const __grid_constant__ Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    double dv[3] = {0, 0, 0};
    T md;
    V3<T> dir;
    int mid;
    nearest_tri<T>(d, load_p<T>(d, i), true, md, dir, mid);
    if (mid >= 0) {
        const DragParameter dp = d.drag[d.tparams[d.tmodel[mid]].DragTriangleID];
        if ((double)md <= (double)dp.CoefficientofInflueneRegion * d.c.l0) {
            dbl4 v = d.vel[i];
            if (dp.DragToken == 'E' && (dp.InputVelocityToken1 == 'V' || dp.InputVelocityToken1 == 'B')) {
                const double sv = sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
                const double pr = (double)dp.VelocityIndex * pow(sv, (double)dp.VelocityExponential);
                if (dp.VelocityDragPermiabilityConstant != 0) {
                    const double f = pr / (double)dp.VelocityDragPermiabilityConstant;
                    dv[0] = f * d.tnrm[3 * mid];
                    dv[1] = f * d.tnrm[3 * mid + 1];
                    dv[2] = f * d.tnrm[3 * mid + 2];
                }
            } else if (dp.DragToken == 'C' && (dp.InputVelocityToken1 == 'V' || dp.InputVelocityToken1 == 'v')) {
                v.x = dp.ConstantVx; v.y = dp.ConstantVy; v.z = dp.ConstantVz;
                d.vel[i] = v;
                d.ovel[i] = make_float4((float)v.x, (float)v.y, (float)v.z, 0.f);
            } else if (dp.DragToken == 'F' && (dp.InputVelocityToken1 == 'V' || dp.InputVelocityToken1 == 'v')) {
                const double f = dp.VelocityMagnitueFactor;
                v.x *= f; v.y *= f; v.z *= f;
                d.vel[i] = v;
                d.ovel[i] = make_float4((float)v.x, (float)v.y, (float)v.z, 0.f);
            }
        }
    }
    d.dragv[3 * (size_t)i] = dv[0];
    d.dragv[3 * (size_t)i + 1] = dv[1];
    d.dragv[3 * (size_t)i + 2] = dv[2];
}

// ---------------------------------------------------------------------------
// neighbour passes (shared-memory staged, warp per target)
// ---------------------------------------------------------------------------
// exact r (no contracted multiply-add) so FP64 neighbour sets equal the oracle's
__device__ __forceinline__ double exact_r(double dx, double dy, double dz) {
    return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

// Epilogue of one target of k_neighbours (run lane-parallel: each lane finishes the
// target it parked, so the FP64 state update uses every lane of the FP64 pipe).
template <class T, int MODE>
__device__ __forceinline__ void nb_epilogue(const Dev& d, int i, T a0, T a1, T a2, T a3, int cnt, int gcnt) {
    if constexpr (MODE == NB_PREDICT) {
        // wall friction term, viscosity, gravity, drag (CalcExplicitly_Kernel)
        const V3<T> vi = load_v<T>(d, i);
        double lx = a0, ly = a1, lz = a2;
        const int t = d.wid[i];
        const double wd = d.wdist[i];
        if (t >= 0 && wd > 0 && wd < d.c.re_lap) {
            const double ww = exact_z<double>(d.c.dim == 2 ? c_zlap2 : c_zlap3, d.c.dim == 2 ? 23 : 25, wd, d.c.l0);
            const Scalar3 vw = d.tparams[d.tmodel[t]].Velocity;
            lx += ((double)vw.x - (double)vi.x) * d.c.wall_fric * ww;
            ly += ((double)vw.y - (double)vi.y) * d.c.wall_fric * ww;
            lz += ((double)vw.z - (double)vi.z) * d.c.wall_fric * ww;
        }
        const double cf = d.c.coef_lap * (double)d.visc[i];
        const dbl4 v = d.vel[i];
        const dbl4 p = d.pos[i];
        const double dt = d.c.dt;
        dbl4 vn, pn;
        vn.x = v.x + (d.c.g[0] + lx * cf) * dt - d.dragv[3 * (size_t)i];
        vn.y = v.y + (d.c.g[1] + ly * cf) * dt - d.dragv[3 * (size_t)i + 1];
        vn.z = v.z + (d.c.g[2] + lz * cf) * dt - d.dragv[3 * (size_t)i + 2];
        vn.w = 0.0;
        pn.x = p.x + vn.x * dt;
        pn.y = p.y + vn.y * dt;
        pn.z = p.z + vn.z * dt;
        pn.w = 0.0;
        if (!(isfinite(vn.x) && isfinite(vn.y) && isfinite(vn.z))) {
            atomicOr(d.err, MPS_ERR_NONFINITE);
            vn = v;
            pn = p;
        }
        d.vel2[i] = vn;
        d.pos2[i] = pn;
    } else {
        if (cnt > d.K || gcnt > d.KG) atomicOr(d.err, MPS_ERR_NEIGHBOUR_CAP);
        atomicMax(d.istat, cnt);
        d.nbr_cnt[i] = cnt < d.K ? cnt : d.K;
        d.gcnt[i] = gcnt < d.KG ? gcnt : d.KG;
        double pnd = (double)a2;
        const double riw = d.wdist[i];
        if (d.wid[i] >= 0 && riw >= 0 && riw <= d.c.re_grad)
            pnd += exact_z<double>(d.c.dim == 2 ? c_zgrad2 : c_zgrad3, d.c.dim == 2 ? 23 : 21, riw, d.c.l0);
        d.pnd[i] = pnd;
        d.sumw[i] = (double)a0;
    }
}

// FP32 squared distance and Laplacian weight of one pair, every rounding explicit:
// the neighbour pass that stores the weights and the matrix-free SpMV that
// recomputes them from the same positions get the same bits.
__device__ __forceinline__ float dist2_f32(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}
// w = re / max(r, mind) - 1 from one reciprocal square root; rinv = 1 / r, rr = r
__device__ __forceinline__ float lap_weight_f32(float d2, float re, float mind, float wmax, float& rinv, float& rr) {
    rinv = rsqrtf(fmaxf(d2, 1e-30f));
    rr = __fmul_rn(d2, rinv);
    return rr > mind ? __fmaf_rn(re, rinv, -1.f) : wmax;
}

// Neighbour passes, CTA per non-empty cell.  The 9 (x, y) columns of the 27-cell
// neighbourhood are contiguous z-runs in the sorted order; their positions are
// staged in shared memory (float4), a warp takes one target particle at a time and
// its lanes test 32 candidates per round, in a z window of each run found by binary
// search on the global z bin (w of opos).  MODE:
//   NB_PREDICT    Laplacian of the velocity -> viscosity/gravity/drag predictor
//   NB_LIST       Laplacian rows (row-major staging), gradient rows, PND, sum of weights
// The warp's butterfly sums are parked in lane k%32 for its k-th target and the
// epilogues run lane-parallel.
template <class T, int MODE>
__global__ void __launch_bounds__(kNbThreads) k_neighbours(const __grid_constant__ Dev d) {
    __shared__ __align__(16) float4 spos[kStageCap];
    __shared__ __align__(8) unsigned long long stage_bar;
    __shared__ int rs[9], rl[9], rp[10];
    // per-warp queues of accepted candidates (FP32 path): index and squared distance;
    // a round adds at most 32 to fewer than 32 waiting entries
    __shared__ int nb_qj[kNbThreads / 32][64];
    __shared__ float nb_qd[kNbThreads / 32][64];
    const int ci = blockIdx.x;
    if (ci >= *d.cell_count) return;
    const int cell = d.cell_list[ci];
    const int s0 = d.cstart[cell], e0 = d.cend[cell];
    const Integer3 G = d.box.m_GridSize;
    const int cx = cell / (G.y * G.z), cy = (cell / G.z) % G.y, cz = cell % G.z;
    if (threadIdx.x < 9) {
        const int x = cx + (int)threadIdx.x / 3 - 1, y = cy + (int)threadIdx.x % 3 - 1;
        int first = -1, last = -1;
        if (x >= 0 && x < G.x && y >= 0 && y < G.y) {
            for (int z = max(cz - 1, 0); z <= min(cz + 1, G.z - 1); ++z) {
                const int c = cell_key(G, x, y, z);
                const int st = d.cstart[c];
                if (st >= 0) {
                    if (first < 0) first = st;
                    last = d.cend[c];
                }
            }
        }
        rs[threadIdx.x] = first < 0 ? 0 : first;
        rl[threadIdx.x] = first < 0 ? 0 : last - first;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        rp[0] = 0;
        for (int r = 0; r < 9; ++r) rp[r + 1] = rp[r] + rl[r];
    }
    __syncthreads();
    const int S = rp[9];
    bool staged = S <= kStageCap;
    if (staged && S > 0) {
        // the 9 runs are contiguous float4 ranges: one bulk copy each (16-byte aligned
        // addresses, sizes multiples of 16 bytes), completed on one mbarrier
        if (threadIdx.x == 0) {
            mbar_init(&stage_bar, 1);
            mbar_arrive_expect_tx(&stage_bar, (unsigned)S * (unsigned)sizeof(float4));
            for (int r = 0; r < 9; ++r)
                if (rl[r] > 0)
                    bulk_copy_g2s(&spos[rp[r]], d.opos + rs[r], (unsigned)rl[r] * (unsigned)sizeof(float4), &stage_bar);
        }
        __syncthreads();
        if (!mbar_wait_bounded(&stage_bar, 1ll << 22)) {
            // the copies did not land in time: flag it, wait (bounded) for the copies
            // still in flight into this CTA's shared memory, and use global loads
            if (threadIdx.x == 0) atomicOr(d.err, MPS_ERR_STAGE_TIMEOUT);
            mbar_wait_bounded(&stage_bar, 1ll << 26);
            staged = false;
        }
    }
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const T re = (T)d.c.re_lap, reg = (T)d.c.re_grad, mind = (T)d.c.mind_lap, mindg = (T)d.c.mind_grad;
    const float re2f = (float)(d.c.re_lap * d.c.re_lap) * 1.0001f;
    // FP32 path: one reciprocal square root per accepted pair gives r and both weights
    const float re2s = (float)d.c.re_lap * (float)d.c.re_lap;
    const float wmax = (float)(d.c.re_lap / d.c.mind_lap) - 1.f, wgmax = (float)(d.c.re_grad / d.c.mind_grad) - 1.f;
    // target parked in this lane for the lane-parallel epilogue
    int my_i = -1, my_cnt = 0, my_gcnt = 0;
    T m0 = 0, m1 = 0, m2 = 0, m3 = 0;
    int k = 0;
    for (int i = s0 + warp; i < e0; i += nwarp, ++k) {
        const float4 pf = d.opos[i];
        const V3<T> pi = load_p<T>(d, i);
        const V3<T> vi = load_v<T>(d, i);
        T a0 = 0, a1 = 0, a2 = 0, a3 = 0;   // mode-specific accumulators
        int cnt = 0, gcnt = 0;
        // the row's entries are stored contiguously (row i at i*K; k_rows_sell turns the
        // interior rows into SELL-32), so a batch of 32 accepted entries is one line
        int* const nrow = d.rnbr + (size_t)i * d.K;
        T* const wrow = (T*)d.rw + (size_t)i * d.K;
        int* const grow = d.gnbr + (size_t)i * d.KG;
        T* const grrow = (T*)d.gnbrr + (size_t)i * d.KG;
        // z window of each run for this target: the run (3 cells stacked in z) is sorted
        // by z bin; the bins a neighbour can occupy are those within +-sqrt(re^2 - dxy^2)
        // of the target, dxy its distance to the run's column in x-y (re^2 with a 2e-4
        // margin, bounds widened by one bin: no neighbour is cut by FP32 round-off).
        // Lanes 0..8 find the first candidate of run `lane`, lanes 16..24 the end.
        int bound = 0;
        {
            const int r = lane & 15;
            const bool upper = lane >= 16;
            if (r < 9) {
                const int len = rl[r];
                bound = upper ? len : 0;
                if (d.zbits && len > 0) {
                    const float cs = d.box.m_CellSize;
                    const float xlo = d.box.m_BufferedZone.m_MinBound.x + (float)(cx + r / 3 - 1) * cs;
                    const float ylo = d.box.m_BufferedZone.m_MinBound.y + (float)(cy + r % 3 - 1) * cs;
                    const float ddx = fmaxf(0.f, fmaxf(xlo - pf.x, pf.x - (xlo + cs)));
                    const float ddy = fmaxf(0.f, fmaxf(ylo - pf.y, pf.y - (ylo + cs)));
                    const float rem = re2f * 1.0001f - (ddx * ddx + ddy * ddy);
                    if (rem <= 0.f) {
                        bound = 0;
                    } else {
                        const float reff = sqrtf(rem);
                        const float scale = 64.f / cs;
                        const float zrel = pf.z - d.box.m_BufferedZone.m_MinBound.z;
                        const float tb = upper ? floorf((zrel + reff) * scale) + 1.f : floorf((zrel - reff) * scale) - 1.f;
                        int lo = 0, hi = len;
                        while (lo < hi) {
                            const int mid = (lo + hi) >> 1;
                            const float w = staged ? spos[rp[r] + mid].w : d.opos[rs[r] + mid].w;
                            if (upper ? (w <= tb) : (w < tb)) lo = mid + 1;
                            else hi = mid;
                        }
                        bound = lo;
                    }
                }
            }
        }
        if constexpr (sizeof(T) == 4) {
            // FP32: the candidates a round accepts queue up in candidate order; the
            // weight, the sums and the row stores run on full batches of 32 entries,
            // so the expensive path executes ~accepted/32 times per target instead of
            // once per 32-candidate round.  Entry order (hence every row) is unchanged.
            int* const qj = nb_qj[warp];
            float* const qd = nb_qd[warp];
            int qn = 0;
            auto flush = [&](int nq) {   // the first nq <= 32 entries (nq warp-uniform)
                const bool on = lane < nq;
                const int j = on ? qj[lane] : 0;
                float rinv = 0.f, rrf = 0.f, w = 0.f;
                if (on) w = lap_weight_f32(qd[lane], (float)re, (float)mind, wmax, rinv, rrf);
                bool gacc = false;
                if constexpr (MODE == NB_PREDICT) {
                    if (on) {
                        const float4 v = d.ovel[j];
                        a0 += (v.x - vi.x) * w;
                        a1 += (v.y - vi.y) * w;
                        a2 += (v.z - vi.z) * w;
                    }
                } else {
                    if (on) {
                        const int slot = cnt + lane;
                        if (slot < d.K) {
                            nrow[slot] = j;
                            wrow[slot] = w;
                        }
                        a0 += w;                                   // sum of Laplacian weights
                        if (rrf < reg) {
                            gacc = true;
                            a2 += rrf > mindg ? __fmaf_rn(reg, rinv, -1.f) : wgmax;   // PND
                        }
                    }
                    const unsigned gb = __ballot_sync(0xffffffffu, gacc);
                    if (gb != 0u && gacc) {
                        const int slot = gcnt + __popc(gb & lt);
                        if (slot < d.KG) {
                            grow[slot] = j;
                            grrow[slot] = rrf;
                        }
                    }
                    gcnt += __popc(gb);
                }
                cnt += nq;
            };
            for (int r = 0; r < 9; ++r) {
                const int kb = __shfl_sync(0xffffffffu, bound, r);
                const int len = max(kb, __shfl_sync(0xffffffffu, bound, 16 + r));
                const int rsr = rs[r], rpr = rp[r];   // run start (global) and stage offset
                for (int b = kb; b < len; b += 32) {
                    const int o = b + lane;
                    const int j = rsr + o;
                    bool acc = false;
                    float d2f = 0.f;
                    if (o < len && j != i) {
                        const float4 q = staged ? spos[rpr + o] : d.opos[j];
                        d2f = dist2_f32(q.x - pf.x, q.y - pf.y, q.z - pf.z);
                        acc = d2f < re2s;
                    }
                    const unsigned bal = __ballot_sync(0xffffffffu, acc);
                    if (acc) {
                        const int pos = qn + __popc(bal & lt);
                        qj[pos] = j;
                        qd[pos] = d2f;
                    }
                    qn += __popc(bal);
                    if (qn >= 32) {
                        __syncwarp();
                        flush(32);
                        // the entries past the batch move to the front of the queue
                        const int rest = qn - 32;
                        int mj = 0;
                        float md = 0.f;
                        if (lane < rest) {
                            mj = qj[32 + lane];
                            md = qd[32 + lane];
                        }
                        __syncwarp();
                        if (lane < rest) {
                            qj[lane] = mj;
                            qd[lane] = md;
                        }
                        __syncwarp();
                        qn = rest;
                    }
                }
            }
            __syncwarp();
            if (qn > 0) flush(qn);
            __syncwarp();   // the queue is reused for the warp's next target
        } else {
            // FP64: the FP32 distance screens, the exact FP64 distance decides
            for (int r = 0; r < 9; ++r) {
                const int kb = __shfl_sync(0xffffffffu, bound, r);
                const int len = max(kb, __shfl_sync(0xffffffffu, bound, 16 + r));
                const int rsr = rs[r], rpr = rp[r];   // run start (global) and stage offset
                for (int b = kb; b < len; b += 32) {
                    const int o = b + lane;
                    const bool valid = o < len;
                    const int j = rsr + o;
                    bool acc = false, gacc = false;
                    T rr = T(0);
                    if (valid && j != i) {
                        const float4 q = staged ? spos[rpr + o] : d.opos[j];
                        const float d2f = dist2_f32(q.x - pf.x, q.y - pf.y, q.z - pf.z);
                        if (d2f < re2f) {
                            const dbl4 pj = d.pos[j];
                            const double rd = exact_r(pj.x - pi.x, pj.y - pi.y, pj.z - pi.z);
                            if (rd < re) {
                                acc = true;
                                rr = rd;
                            }
                        }
                    }
                    const unsigned bal = __ballot_sync(0xffffffffu, acc);
                    if (acc) {
                        const T w = wdiv<T>(re, rr > mind ? rr : mind) - T(1);
                        if constexpr (MODE == NB_PREDICT) {
                            const dbl4 v = d.vel[j];
                            a0 += (v.x - vi.x) * w;
                            a1 += (v.y - vi.y) * w;
                            a2 += (v.z - vi.z) * w;
                        } else {
                            const int slot = cnt + __popc(bal & lt);
                            if (slot < d.K) {
                                nrow[slot] = j;
                                wrow[slot] = w;
                            }
                            a0 += w;                                   // sum of Laplacian weights
                            if (rr < reg) {
                                gacc = true;
                                a2 += wdiv<T>(reg, rr > mindg ? rr : mindg) - T(1);   // PND
                            }
                        }
                    }
                    cnt += __popc(bal);
                    if constexpr (MODE != NB_PREDICT) {
                        const unsigned gb = __ballot_sync(0xffffffffu, gacc);
                        if (gb != 0u && gacc) {
                            const int slot = gcnt + __popc(gb & lt);
                            if (slot < d.KG) {
                                grow[slot] = j;
                                grrow[slot] = rr;
                            }
                        }
                        gcnt += __popc(gb);
                    }
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a0 += __shfl_xor_sync(0xffffffffu, a0, o);
            a1 += __shfl_xor_sync(0xffffffffu, a1, o);
            a2 += __shfl_xor_sync(0xffffffffu, a2, o);
            a3 += __shfl_xor_sync(0xffffffffu, a3, o);
        }
        if (lane == (k & 31)) {
            my_i = i; m0 = a0; m1 = a1; m2 = a2; m3 = a3; my_cnt = cnt; my_gcnt = gcnt;
        }
        if ((k & 31) == 31) {
            if (my_i >= 0) nb_epilogue<T, MODE>(d, my_i, m0, m1, m2, m3, my_cnt, my_gcnt);
            my_i = -1;
        }
    }
    if (my_i >= 0) nb_epilogue<T, MODE>(d, my_i, m0, m1, m2, m3, my_cnt, my_gcnt);
}

// FP64 checksum of the neighbour ids of every row (neighbour-set comparison in tests)
__global__ void k_row_idsum(const __grid_constant__ Dev d, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    double s = 0.0;
    const int cnt = d.nbr_cnt[i];
    for (int k = 0; k < cnt; ++k) s += (double)d.id[d.rnbr[(size_t)i * d.K + k]];
    out[i] = s;
}

// ---------------------------------------------------------------------------
// PPE assembly, explicit pressure
// ---------------------------------------------------------------------------
__global__ void k_ppe_setup(const __grid_constant__ Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const double pnd = d.pnd[i];
    const bool in = pnd > d.c.beta * d.c.n0_pnd;
    d.inner[i] = in ? 1 : 0;
    if (in) {
        const double dg = d.c.coef_lap * d.sumw[i] + d.c.kappa;
        d.diag[i] = dg;
        d.rhs[i] = d.c.gamma * d.c.rho / (d.c.dt * d.c.dt) * (pnd - d.c.n0_pnd) / d.c.n0_pnd;
        d.minv[i] = 1.0 / dg;
    } else {
        d.diag[i] = 1.0;
        d.rhs[i] = 0.0;
        d.minv[i] = 0.0;
        d.press[i] = 0.0;
    }
}

// The reference's equation of state (CalcExplicitPressure_Kernel :1043-1047)
__global__ void k_eos(const __grid_constant__ Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const double pnd = d.pnd[i];
    const double p = pnd > d.c.beta * d.c.n0_pnd ? d.c.sonic2 * d.c.rho / d.c.n0_pnd * (pnd - d.c.n0_pnd) : 0.0;
    d.press[i] = p;
    d.pf32[i] = (float)p;
}

// ---------------------------------------------------------------------------
// CG machinery: warp-per-row SpMV over the neighbour rows, vector updates with
// fused FP64 dot products, convergence decided on the device.
// ---------------------------------------------------------------------------
// Column index of SELL entry e: a signed 16-bit offset from the slice's first row,
// or the 32-bit index
template <bool NARROW>
__device__ __forceinline__ int sell_col(const Dev& d, size_t e, int sb) {
    if constexpr (NARROW) return sb + (int)(short)__ldcs(d.nbr16 + e);
    return __ldcs(d.nbr + e);
}

// SELL-32 rows of the interior rows from the list pass's row-major rows, one read
// pass: warp per 32-row slice; each 32-entry chunk of the slice's rows is loaded one
// 128-byte line per row into a [32][33] shared-memory tile and written back transposed,
// so entry k of the slice's 32 rows is again one contiguous store per array.
// flags bit 0: 16-bit column offsets j - 32*slice (sbase / skmax; a slice with an offset
// outside [-32768, 32767] keeps 32-bit columns, sbase = -1); bit 1: the FP16 copy of each
// FP32 weight (round to nearest) and the diagonal of that operator, coef * (sum of the
// FP16 weights in entry order, in FP32) + kappa, so the FP16-weight operator is again a
// Laplacian plus kappa; bit 2: 32-bit columns for every slice (the wide streamed SpMV,
// uncompressed rows); bit 3: leave the wide-entry count alone (a repeated transpose).
// The weights (T) are always written.  A row's columns ascend (its candidates are
// visited run by run in cell-key order, each run in index order), so its first and last
// entries decide whether the slice fits 16 bits; every offset is still checked as it is
// written, and an offset that breaks that order sets MPS_ERR_NEIGHBOUR_CAP.
template <class T>
constexpr int rows_sell_warps() { return sizeof(T) == 4 ? 4 : 2; }

template <class T>
__global__ void __launch_bounds__(rows_sell_warps<T>() * 32) k_rows_sell(const __grid_constant__ Dev d, int flags) {
    constexpr int WARPS = rows_sell_warps<T>();
    __shared__ int tj[WARPS][32][33];
    __shared__ T tw[WARPS][32][33];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int sl = blockIdx.x * WARPS + wl;
    if (sl >= (d.n + 31) >> 5) return;   // warp-uniform
    const bool narrow = (flags & 1) != 0, w16 = sizeof(T) == 4 && (flags & 2) != 0, full32 = (flags & 4) != 0;
    const int r0 = sl * 32, i = r0 + lane;
    const int cnt = (i < d.n && d.inner[i]) ? min(d.nbr_cnt[i], d.K) : 0;
    const int kmax = __reduce_max_sync(0xffffffffu, cnt);
    const int* __restrict__ rj = d.rnbr + (size_t)r0 * d.K;
    const T* __restrict__ rwt = (const T*)d.rw + (size_t)r0 * d.K;
    bool fit = true;
    if (cnt > 0) {
        const int lo = __ldcs(rj + (size_t)lane * d.K) - r0, hi = __ldcs(rj + (size_t)lane * d.K + cnt - 1) - r0;
        fit = lo >= -32768 && hi <= 32767;
    }
    const bool n16 = narrow && __all_sync(0xffffffffu, fit);
    const bool c32 = full32 || !n16;
    const size_t e0 = (size_t)sl * d.K * 32 + lane;   // SELL position of this lane's entry 0
    T* __restrict__ ws = (T*)d.nbrw;
    float sw16 = 0.f;
    bool bad = false;
    for (int c = 0; c < kmax; c += 32) {
#pragma unroll 8
        for (int r = 0; r < 32; ++r) {
            const int cr = __shfl_sync(0xffffffffu, cnt, r);
            if (c + lane < cr) {
                tj[wl][r][lane] = __ldcs(rj + (size_t)r * d.K + c + lane);
                tw[wl][r][lane] = __ldcs(rwt + (size_t)r * d.K + c + lane);
            }
        }
        __syncwarp();
        const int m = min(32, kmax - c);
        for (int k = 0; k < m; ++k) {
            if (c + k < cnt) {
                const int j = tj[wl][lane][k];
                const T w = tw[wl][lane][k];
                const size_t e = e0 + (size_t)(c + k) * 32;
                ws[e] = w;
                if (c32) d.nbr[e] = j;
                if (n16) {
                    const int off = j - r0;
                    bad = bad || off < -32768 || off > 32767;
                    d.nbr16[e] = (unsigned short)(short)off;
                }
                if (w16) {
                    const __half h = __float2half_rn((float)w);
                    d.w16[e] = h;
                    sw16 += __half2float(h);
                }
            }
        }
        __syncwarp();   // the tile is refilled for the next chunk
    }
    if (w16 && cnt > 0) d.diag16[i] = d.c.coef_lap * (double)sw16 + d.c.kappa;
    if (bad) atomicOr(d.err, MPS_ERR_NEIGHBOUR_CAP);
    if (lane == 0) {
        d.sbase[sl] = n16 ? r0 : -1;
        d.skmax[sl] = n16 ? kmax : -1 - kmax;
    }
    if (narrow && !(flags & 8)) {
        // interior entries kept at 32 bits (counted for the bytes-per-launch figure)
        int wide = n16 ? 0 : cnt;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) wide += __shfl_down_sync(0xffffffffu, wide, o);
        if (lane == 0 && wide) atomicAdd(d.istat + 1, wide);
    }
}

// FP32 rows (the step's default): the same transpose with the chunks moved global ->
// shared by 16-byte cp.async pieces, double-buffered so that the next chunk's copies
// are in flight while the current chunk is written out.  A warp per slice, 2 warps per
// CTA (32 KB: 2 stages x columns and weights x 32 rows x 128 B).  Piece q (entries
// 4q..4q+3) of row r sits at piece position q ^ (r & 7) of the row's 128 bytes, so the
// 16-byte reads of lanes 0..7 (rows 0..7, one piece each) cover the 32 banks.  Pieces
// of a chunk past a row's count copy stale staging entries inside the row's capacity
// (K is a multiple of 128) and are never read.  Same outputs as k_rows_sell<float>.
constexpr int kRsWarps = 2;
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__global__ void __launch_bounds__(kRsWarps * 32) k_rows_sell_async(const __grid_constant__ Dev d, int flags) {
    __shared__ __align__(128) unsigned char tiles[kRsWarps][2][2][32 * 128];   // [warp][stage][cols, weights]
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int sl = blockIdx.x * kRsWarps + wl;
    if (sl >= (d.n + 31) >> 5) return;   // warp-uniform
    const bool narrow = (flags & 1) != 0, w16 = (flags & 2) != 0, full32 = (flags & 4) != 0;
    const int r0 = sl * 32, i = r0 + lane;
    const int cnt = (i < d.n && d.inner[i]) ? min(d.nbr_cnt[i], d.K) : 0;
    const int kmax = __reduce_max_sync(0xffffffffu, cnt);
    const int* __restrict__ rj = d.rnbr + (size_t)r0 * d.K;
    const float* __restrict__ rwt = (const float*)d.rw + (size_t)r0 * d.K;
    bool fit = true;
    if (cnt > 0) {
        const int lo = __ldcs(rj + (size_t)lane * d.K) - r0, hi = __ldcs(rj + (size_t)lane * d.K + cnt - 1) - r0;
        fit = lo >= -32768 && hi <= 32767;
    }
    const bool n16 = narrow && __all_sync(0xffffffffu, fit);
    const bool c32 = full32 || !n16;
    const size_t e0 = (size_t)sl * d.K * 32 + lane;
    float* __restrict__ ws = (float*)d.nbrw;
    // lane t copies piece t & 7 of rows 4u + t / 8, u = 0..7
    const int cq = lane & 7, crow = lane >> 3;
    auto issue = [&](int c, int st) {
        unsigned char* tj = tiles[wl][st][0];
        unsigned char* tw = tiles[wl][st][1];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int r = 4 * u + crow;
            const int cr = __shfl_sync(0xffffffffu, cnt, r);
            if (c < cr) {
                const size_t g = (size_t)r * d.K + c + 4 * cq;
                const int pos = r * 128 + ((cq ^ (r & 7)) << 4);
                cp_async16(tj + pos, rj + g);
                cp_async16(tw + pos, rwt + g);
            }
        }
        cp_async_commit();
    };
    const int nch = (kmax + 31) >> 5;
    if (nch > 0) issue(0, 0);
    float sw16 = 0.f;
    bool bad = false;
    for (int ci = 0; ci < nch; ++ci) {
        if (ci + 1 < nch) {
            issue((ci + 1) * 32, (ci + 1) & 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncwarp();   // every lane's pieces of chunk ci have landed
        const unsigned char* tj = tiles[wl][ci & 1][0];
        const unsigned char* tw = tiles[wl][ci & 1][1];
        const int c = ci * 32;
        for (int q = 0; q < 8 && c + 4 * q < kmax; ++q) {
            const int pos = lane * 128 + ((q ^ (lane & 7)) << 4);
            const int4 jv = *(const int4*)(tj + pos);
            const float4 wv = *(const float4*)(tw + pos);
            const int jj[4] = {jv.x, jv.y, jv.z, jv.w};
            const float wf[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int k = c + 4 * q + u;
                if (k < cnt) {
                    const size_t e = e0 + (size_t)k * 32;
                    ws[e] = wf[u];
                    if (c32) d.nbr[e] = jj[u];
                    if (n16) {
                        const int off = jj[u] - r0;
                        bad = bad || off < -32768 || off > 32767;
                        d.nbr16[e] = (unsigned short)(short)off;
                    }
                    if (w16) {
                        const __half h = __float2half_rn(wf[u]);
                        d.w16[e] = h;
                        sw16 += __half2float(h);
                    }
                }
            }
        }
        __syncwarp();   // stage ci & 1 is refilled by the next iteration's copies
    }
    if (w16 && cnt > 0) d.diag16[i] = d.c.coef_lap * (double)sw16 + d.c.kappa;
    if (bad) atomicOr(d.err, MPS_ERR_NEIGHBOUR_CAP);
    if (lane == 0) {
        d.sbase[sl] = n16 ? r0 : -1;
        d.skmax[sl] = n16 ? kmax : -1 - kmax;
    }
    if (narrow && !(flags & 8)) {
        int wide = n16 ? 0 : cnt;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) wide += __shfl_down_sync(0xffffffffu, wide, o);
        if (lane == 0 && wide) atomicAdd(d.istat + 1, wide);
    }
}

// a stored weight as a float or double (FP16 weights widen to float)
__device__ __forceinline__ float to_wt(float v) { return v; }
__device__ __forceinline__ double to_wt(double v) { return v; }
__device__ __forceinline__ float to_wt(__half v) { return __half2float(v); }
// acc + a * b with one rounding (no contraction left to the compiler)
__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }

// Dot of one SELL row with x (lane = row), evict-first loads.  U entries' loads are
// in flight before their gathers: 8 for 16-bit columns (6 B per entry, so a warp
// keeps about as many bytes in flight as with 4 entries of 8 B), 4 otherwise.
template <bool NARROW, class TA, class TW, class TX>
__device__ __forceinline__ TA sell_row_dot(const Dev& d, const TW* __restrict__ w, const TX* __restrict__ x,
                                           size_t base, int cnt, int kmax, int sb) {
    constexpr int U = NARROW ? 8 : 4;
    TA acc = TA(0);
    int k = 0;
    for (; k + U <= kmax; k += U) {
        int id[U];
        TW wv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            id[u] = sell_col<NARROW>(d, base + (size_t)(k + u) * 32, sb);
            wv[u] = __ldcs(w + base + (size_t)(k + u) * 32);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (k + u < cnt) acc = fma_t((TA)to_wt(wv[u]), (TA)x[id[u]], acc);
    }
    for (; k < kmax; ++k) {
        const int idk = sell_col<NARROW>(d, base + (size_t)k * 32, sb);
        const TW wk = __ldcs(w + base + (size_t)k * 32);
        if (k < cnt) acc = fma_t((TA)to_wt(wk), (TA)x[idk], acc);
    }
    return acc;
}

// Matrix-free FP32 row dot (lane = row): only the columns are streamed; each weight
// is recomputed from the FP32 positions the neighbour pass used, by the same
// expression (dist2_f32, lap_weight_f32), so the sum is bit-identical to the
// stored-weight walk.  U entries' columns are loaded, then their position and x
// gathers (a padded entry gathers the row itself and is not accumulated).
template <bool NARROW, int U>
__device__ __forceinline__ float sell_row_dot_mf(const Dev& d, const float* __restrict__ x, size_t base, int cnt,
                                                 int kmax, int sb, int i, float4 pi, float re, float mind,
                                                 float wmax) {
    float acc = 0.f;
    int k = 0;
    for (; k + U <= kmax; k += U) {
        int id[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            id[u] = sell_col<NARROW>(d, base + (size_t)(k + u) * 32, sb);
            if (k + u >= cnt) id[u] = i;
        }
        float4 q[U];
        float xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            q[u] = __ldg(d.opos + id[u]);
            xv[u] = __ldg(x + id[u]);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            float rinv, rr;
            const float wk = lap_weight_f32(dist2_f32(__fsub_rn(q[u].x, pi.x), __fsub_rn(q[u].y, pi.y),
                                                      __fsub_rn(q[u].z, pi.z)),
                                            re, mind, wmax, rinv, rr);
            if (k + u < cnt) acc = __fmaf_rn(wk, xv[u], acc);
        }
    }
    for (; k < kmax; ++k) {
        int j = sell_col<NARROW>(d, base + (size_t)k * 32, sb);
        if (k >= cnt) j = i;
        const float4 q = __ldg(d.opos + j);
        const float xj = __ldg(x + j);
        float rinv, rr;
        const float wk = lap_weight_f32(dist2_f32(__fsub_rn(q.x, pi.x), __fsub_rn(q.y, pi.y), __fsub_rn(q.z, pi.z)),
                                        re, mind, wmax, rinv, rr);
        if (k < cnt) acc = __fmaf_rn(wk, xj, acc);
    }
    return acc;
}

// y = A x for interior rows (y = 0 elsewhere); A = diag - coef * W.  MODE 0: plain
// (+ dot x.y -> S_PQ, alpha = rz / pq); MODE 1: residual r = b - A x (FP64 out),
// norms -> S_RR, S_BNORM; MODE 2: y = A x with dots x.y -> S_LS0 and x.b -> S_LS1.
// SELL-32: one warp per slice of 32 consecutive rows, one lane per row; entry k of
// the slice is 32 consecutive words, so every index / weight load of a warp is one
// full 128-byte line (256 for FP64 weights) and no cross-lane reduction is needed.
// The k loop runs to the slice's longest row, unrolled 4x so that eight line loads
// are in flight per warp before the gathers; matrix loads are evict-first.
// MF > 0 (FP32 weights, FP32 x): matrix-free rows, MF entries per unrolled group; the
// weight array is not read.
template <class TW, class TX, class TY, int MODE, int MF = 0>
__global__ void __launch_bounds__(256, MF == 0 ? 8 : (MF <= 4 ? 5 : 3))
    k_spmv(const __grid_constant__ Dev d, const TW* __restrict__ w, const TX* __restrict__ x, TY* __restrict__ y,
           const double* __restrict__ b, int slot) {
    static_assert(MF == 0 || (sizeof(TW) == 4 && sizeof(TX) == 4 && MODE != 1), "matrix-free rows: FP32 only");
    if (MODE == 0 && d.scal[S_CONV] != 0.0) return;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int nslices = (d.n + 31) >> 5;
    double part0 = 0.0, part1 = 0.0;
    const double coef = d.c.coef_lap;
    // entry arithmetic: FP32 unless a weight or x is FP64, or the FP64 residual (MODE 1)
    using TA = typename std::conditional<(sizeof(TX) == 8 || sizeof(TW) == 8 || MODE == 1), double, float>::type;
    TA partw = TA(0);   // MODE 0 partial dot, in the arithmetic type
    for (int sl = gw; sl < nslices; sl += nw) {
        const int i = sl * 32 + lane;
        const bool row = i < d.n;
        const bool in = row && d.inner[i];
        const int cnt = in ? d.nbr_cnt[i] : 0;
        const int kmax = __reduce_max_sync(0xffffffffu, cnt);
        const size_t base = (size_t)sl * d.K * 32 + lane;
        const int sb = (sizeof(TW) == 4 && d.rows16) ? d.sbase[sl] : -1;
        TA acc;
        if constexpr (MF > 0) {
            const float4 pi = in ? d.opos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float re = (float)d.c.re_lap, mind = (float)d.c.mind_lap;
            const float wmax = (float)(d.c.re_lap / d.c.mind_lap) - 1.f;
            const int ii = row ? i : 0;
            acc = sb >= 0 ? sell_row_dot_mf<true, MF>(d, (const float*)x, base, cnt, kmax, sb, ii, pi, re, mind, wmax)
                          : sell_row_dot_mf<false, MF>(d, (const float*)x, base, cnt, kmax, sb, ii, pi, re, mind, wmax);
        } else {
            acc = sb >= 0 ? sell_row_dot<true, TA>(d, w, x, base, cnt, kmax, sb)
                          : sell_row_dot<false, TA>(d, w, x, base, cnt, kmax, sb);
        }
        if (!row) continue;
        if (!in) {
            y[i] = TY(0);
            continue;
        }
        const double yi = d.diag[i] * (double)x[i] - coef * (double)acc;
        if (MODE == 0) {
            y[i] = (TY)yi;
            partw += (TA)x[i] * (TA)(TY)yi;
        } else if (MODE == 2) {
            y[i] = (TY)yi;
            part0 += (double)x[i] * yi;
            part1 += (double)x[i] * b[i];
        } else {
            const double ri = b[i] - yi;
            y[i] = (TY)ri;
            part0 += ri * ri;
            part1 += b[i] * b[i];
        }
    }
    if (MODE == 0) part0 = (double)partw;
    double v[2] = {part0, part1}, out[2];
    if (grid_reduce<2, typename std::conditional<MODE == 0, TA, double>::type>(v, d.red, d.red_count + slot, out) &&
        threadIdx.x == 0) {
        if (MODE == 0) {
            d.scal[S_PQ] = out[0];
            d.scal[S_ALPHA] = out[0] != 0.0 ? d.scal[S_RZ] / out[0] : 0.0;
        } else if (MODE == 2) {
            d.scal[S_LS0] = out[0];
            d.scal[S_LS1] = out[1];
        } else {
            d.scal[S_RR] = out[0];
            d.scal[S_RNORM] = sqrt(out[0]);
            d.scal[S_BNORM] = sqrt(out[1]);
        }
    }
}

// FP32 copy of the wall vertices (after the walls moved)
__global__ void k_tri_to_float(const __grid_constant__ Dev d) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < 9 * d.tri_n) d.tri32[k] = (float)d.tri[k];
}

// FP32 copy of the pressure (neighbour-pressure feature)
__global__ void k_to_float_p(int n, const double* __restrict__ p, float* __restrict__ q) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) q[i] = (float)p[i];
}

// x = xs.x + xs.y: the FP64 pressure split into two floats (representation error
// about 2^-48 |x|) for the double-float residual
__global__ void k_split_x(int n, const double* __restrict__ x, float2* __restrict__ xs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    const float h = (float)v;
    xs[i] = make_float2(h, (float)(v - (double)h));
}

// (S, C) += p + lo in double-float: TwoSum of the high words, low words added
__device__ __forceinline__ void df_add(float& S, float& C, float p, float lo) {
    const float s = __fadd_rn(S, p);
    const float bb = __fsub_rn(s, S);
    const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    S = s;
    C = __fadd_rn(C, __fadd_rn(err, lo));
}

// double-float sum of w * (xh + xl) over one SELL row (lane = row), see k_residual_df.
// Two independent (hi, lo) accumulators (even / odd unrolled entries) so the TwoSum
// chains overlap, merged with TwoSum at the end (a fixed order); two rather than four
// keep the kernel at 32 registers (8 CTAs of 256 per SM).
// x_j as its (hi, lo) words: the split FP64 iterate, or an FP32 vector (lo = 0)
__device__ __forceinline__ void x_hl(const float2* __restrict__ x, int j, float& h, float& l) {
    const float2 v = x[j];
    h = v.x;
    l = v.y;
}
__device__ __forceinline__ void x_hl(const float* __restrict__ x, int j, float& h, float& l) {
    h = x[j];
    l = 0.f;
}
template <bool NARROW, class TX>
__device__ __forceinline__ void df_row_sum(const Dev& d, const float* __restrict__ w, const TX* __restrict__ xs,
                                           size_t base, int cnt, int kmax, int sb, float& S_out, float& C_out) {
    float S0 = 0.f, C0 = 0.f, S1 = 0.f, C1 = 0.f;
    for (int k = 0; k < kmax; k += 4) {
        int id[4];
        float wv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const bool a = k + u < kmax;
            const size_t e = base + (size_t)(a ? k + u : k) * 32;
            id[u] = sell_col<NARROW>(d, e, sb);
            wv[u] = __ldcs(w + e);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (k + u < cnt) {
                float h, l;
                x_hl(xs, id[u], h, l);
                const float p = __fmul_rn(wv[u], h);
                const float pe = __fmaf_rn(wv[u], h, -p);
                if (u & 1) df_add(S1, C1, p, __fmaf_rn(wv[u], l, pe));
                else df_add(S0, C0, p, __fmaf_rn(wv[u], l, pe));
            }
        }
    }
    df_add(S0, C0, S1, C1);
    S_out = S0;
    C_out = C0;
}

// Refinement residual r = b - A x with FP32 weights, in double-float arithmetic:
// every product w*xh is kept exactly as the pair (p, fma(w, xh, -p)), w*xl joins
// the low word, and the row sum is a (hi, lo) float pair updated by TwoSum
// (Knuth; rounding-explicit intrinsics so nothing is contracted).  Only the row
// term diag*x and the final difference are FP64, so the FP64 pipe does per-row
// work instead of per-entry work.  Error: about 2^-44 of sum |w x| per row.
// Norms ||r||^2 -> S_RR / S_RNORM and ||b|| -> S_BNORM as in k_spmv MODE 1.
__global__ void __launch_bounds__(256, 8) k_residual_df(const __grid_constant__ Dev d, const float* __restrict__ w,
                                                     const double* __restrict__ x, double* __restrict__ r,
                                                     const double* __restrict__ b, int slot) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int nslices = (d.n + 31) >> 5;
    const float2* __restrict__ xs = d.xs;
    double part0 = 0.0, part1 = 0.0;
    for (int sl = gw; sl < nslices; sl += nw) {
        const int i = sl * 32 + lane;
        const bool row = i < d.n;
        const bool in = row && d.inner[i];
        const int cnt = in ? d.nbr_cnt[i] : 0;
        const int kmax = __reduce_max_sync(0xffffffffu, cnt);
        const size_t base = (size_t)sl * d.K * 32 + lane;
        float S, C;
        // 32-bit columns: the residual is compute-heavy per entry, and the 16-bit
        // form measured slower here than in the SpMV
        df_row_sum<false>(d, w, xs, base, cnt, kmax, -1, S, C);
        if (!row) continue;
        if (!in) {
            r[i] = 0.0;
            continue;
        }
        const double acc = (double)S + (double)C;
        const double ri = b[i] - (d.diag[i] * x[i] - d.c.coef_lap * acc);
        r[i] = ri;
        part0 += ri * ri;
        part1 += b[i] * b[i];
    }
    double v[2] = {part0, part1}, out[2];
    if (grid_reduce<2>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        d.scal[S_RR] = out[0];
        d.scal[S_RNORM] = sqrt(out[0]);
        d.scal[S_BNORM] = sqrt(out[1]);
    }
}

// ---------------------------------------------------------------------------
// Streamed SELL rows: the 16-bit columns and FP32 weights of each slice reach shared
// memory by bulk (TMA) copies, so the loads in flight hold no registers and the
// matrix does not pass through L1 (the x gathers keep it).  Every warp owns a ring of
// SS stages of SC entries (SC x 64 B of columns + SC x 128 B of weights per stage,
// one mbarrier each); lane 0 keeps the ring full, running ahead across the warp's
// slices (gw, gw + nw, ...), and all lanes consume a stage in entry order.  The
// copies carry an L2 evict-first policy (the CG vectors and the multilevel data stay
// resident).  A stage that does not land within the poll limit sets
// MPS_ERR_STAGE_TIMEOUT; the warp then waits (bounded) for its copies in flight and
// finishes on the register walk.  32-bit slices (skmax = -1) take the register walk.
// ---------------------------------------------------------------------------
// stage: SC x 32 columns (16-bit offsets, or 32-bit indices when WIDE), then SC x 32
// weights of type TW
template <int SC, class TW = float, bool WIDE = false> constexpr int stream_stage_bytes() {
    return SC * ((WIDE ? 128 : 64) + 32 * (int)sizeof(TW));
}
template <int SC, int SS, int W, class TW = float, bool WIDE = false> constexpr int stream_smem_bytes() {
    return W * SS * stream_stage_bytes<SC, TW, WIDE>();
}
// longest interior row of a slice from skmax (kmax for a 16-bit slice, -1 - kmax for
// a 32-bit one)
__device__ __forceinline__ int slice_kmax(int v) { return v >= 0 ? v : -1 - v; }
__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(__half v) { return __half2float(v); }

template <int SC, int SS, class TW = float, bool WIDE = false>
struct SliceRing {
    static constexpr int SB = stream_stage_bytes<SC, TW, WIDE>();
    static constexpr unsigned CB = WIDE ? 128u : 64u;            // column bytes per entry
    static constexpr unsigned WB = (unsigned)sizeof(TW) * 32u;   // weight bytes per entry
    unsigned char* ring;
    unsigned long long* bar;
    const unsigned char* cols;
    const TW* w;
    const int* skmax;
    unsigned* err;
    int nsl, nw, K, lane;
    int ps, pc, pk, pn;          // producer: next chunk pc of slice ps (pk entries, pn chunks)
    unsigned q_issue, q_cons;
    bool streaming;
    unsigned long long pol;

    __device__ void init(const Dev& d, const TW* w_, unsigned char* ring_, unsigned long long* bar_, int gw,
                         int nw_) {
        ring = ring_;
        bar = bar_;
        cols = WIDE ? (const unsigned char*)d.nbr : (const unsigned char*)d.nbr16;
        w = w_;
        skmax = d.skmax;
        err = d.err;
        nsl = (d.n + 31) >> 5;
        nw = nw_;
        K = d.K;
        lane = threadIdx.x & 31;
        if (lane == 0)
            for (int st = 0; st < SS; ++st) mbar_init(&bar[st], 1);
        __syncwarp();
        ps = gw - nw;
        q_issue = q_cons = 0;
        streaming = true;
        pol = l2_evict_first_policy();
        next_slice();
    }
    __device__ void next_slice() {
        do {
            ps += nw;
            pk = ps < nsl ? skmax[ps] : 0;
            if (WIDE) pk = slice_kmax(pk);   // every slice; else 16-bit slices only
        } while (ps < nsl && pk <= 0);
        pc = 0;
        pn = (pk + SC - 1) / SC;
    }
    // issue copies until SS stages are in flight or the warp's slices are exhausted
    __device__ void refill() {
        while (streaming && ps < nsl && q_issue - q_cons < (unsigned)SS) {
            const int st = (int)(q_issue % SS);
            const int k0 = pc * SC;
            const int ne = min(SC, pk - k0);
            if (lane == 0) {
                const size_t e0 = ((size_t)ps * K + k0) * 32;
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(&bar[st], (unsigned)ne * (CB + WB));
                bulk_copy_g2s_hint(ring + st * SB, cols + e0 * (CB / 32u), (unsigned)ne * CB, &bar[st], pol);
                bulk_copy_g2s_hint(ring + st * SB + SC * CB, w + e0, (unsigned)ne * WB, &bar[st], pol);
            }
            ++q_issue;
            if (++pc == pn) next_slice();
        }
    }
    // waits for the next stage; false: streaming abandoned (the caller recomputes the
    // slice on the register walk)
    __device__ bool acquire(const unsigned char*& cs, const TW*& ws) {
        refill();
        const int st = (int)(q_cons % SS);
        if (!__all_sync(0xffffffffu, mbar_wait_parity_bounded(&bar[st], (q_cons / SS) & 1u, 1ll << 20))) {
            if (lane == 0) atomicOr(err, MPS_ERR_STAGE_TIMEOUT);
            for (unsigned q = q_cons; q != q_issue; ++q)
                mbar_wait_parity_bounded(&bar[q % SS], (q / SS) & 1u, 1ll << 24);
            streaming = false;
            q_cons = q_issue;
            return false;
        }
        cs = ring + st * SB;
        ws = (const TW*)(ring + st * SB + SC * CB);
        return true;
    }
    // the warp is done reading the stage
    __device__ void release() {
        __syncwarp();
        ++q_cons;
    }
};

// FP32 SpMV of the inner CG over streamed rows, MODE 0 / 2 as in k_spmv.  Each row
// accumulates its entries in order with one FMA each, so every row value is
// bit-identical to the register walk.  TW = __half: the FP16-weight operator (w16,
// diag16), accumulated in FP32.
template <int MODE, int SC, int SS, int W, int MINB, class TW = float, bool WIDE = false>
__global__ void __launch_bounds__(W * 32, MINB) k_spmv_stream(const __grid_constant__ Dev d,
                                                             const TW* __restrict__ w,
                                                             const float* __restrict__ x, float* __restrict__ y,
                                                             const double* __restrict__ b, int slot) {
    static_assert(MODE == 0 || MODE == 2, "FP32 modes only");
    static_assert(SC % 8 == 0, "stages hold whole groups of 8 entries");
    pdl_wait();
    pdl_trigger();
    if (MODE == 0 && d.scal[S_CONV] != 0.0) return;
    extern __shared__ __align__(128) unsigned char stream_smem[];
    __shared__ __align__(8) unsigned long long bars[W][SS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gw = blockIdx.x * W + warp, nw = gridDim.x * W;
    SliceRing<SC, SS, TW, WIDE> R;
    R.init(d, w, stream_smem + warp * SS * SliceRing<SC, SS, TW, WIDE>::SB, bars[warp], gw, nw);
    const double* __restrict__ diag = sizeof(TW) == 2 ? d.diag16 : d.diag;

    const double coef = d.c.coef_lap;
    double part0 = 0.0, part1 = 0.0;
    float partw = 0.f;
    for (int sl = gw; sl < R.nsl; sl += nw) {
        const int i = sl * 32 + lane;
        const bool row = i < d.n;
        const bool in = row && d.inner[i];
        const int cnt = in ? d.nbr_cnt[i] : 0;
        const int km = d.skmax[sl];
        float acc = 0.f;
        bool done = false;
        if ((WIDE || km >= 0) && R.streaming) {
            const int kms = slice_kmax(km);
            const int nc = (kms + SC - 1) / SC;
            const int r0 = sl * 32;
            for (int c = 0; c < nc; ++c) {
                const unsigned char* cs;
                const TW* ws;
                if (!R.acquire(cs, ws)) break;
                const int k0 = c * SC;
#pragma unroll
                for (int g = 0; g < SC; g += 8) {
                    int j[8];
                    float wv[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        if constexpr (WIDE) j[u] = ((const int*)cs)[(g + u) * 32 + lane];
                        else j[u] = r0 + (int)(short)((const unsigned short*)cs)[(g + u) * 32 + lane];
                        wv[u] = to_f32(ws[(g + u) * 32 + lane]);
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u)
                        if (k0 + g + u < cnt) acc = __fmaf_rn(wv[u], __ldg(x + j[u]), acc);
                }
                R.release();
            }
            done = R.streaming;
        }
        if (!done) {
            // 32-bit slice, or streaming given up: the register walk
            const int kmax = __reduce_max_sync(0xffffffffu, cnt);
            const size_t base = (size_t)sl * d.K * 32 + lane;
            acc = km >= 0 ? sell_row_dot<true, float>(d, w, x, base, cnt, kmax, sl * 32)
                          : sell_row_dot<false, float>(d, w, x, base, cnt, kmax, -1);
        }
        if (!row) continue;
        if (!in) {
            y[i] = 0.f;
            continue;
        }
        const double yi = diag[i] * (double)x[i] - coef * (double)acc;
        y[i] = (float)yi;
        if (MODE == 0) {
            partw += x[i] * (float)yi;
        } else {
            part0 += (double)x[i] * yi;
            part1 += (double)x[i] * b[i];
        }
    }
    if (MODE == 0) part0 = (double)partw;
    double v[2] = {part0, part1}, out[2];
    if (grid_reduce<2, typename std::conditional<MODE == 0, float, double>::type>(v, d.red, d.red_count + slot, out) &&
        threadIdx.x == 0) {
        if (MODE == 0) {
            d.scal[S_PQ] = out[0];
            d.scal[S_ALPHA] = out[0] != 0.0 ? d.scal[S_RZ] / out[0] : 0.0;
        } else {
            d.scal[S_LS0] = out[0];
            d.scal[S_LS1] = out[1];
        }
    }
}

// FP64 SpMV of the plain FP64 solver over streamed rows: the columns (16-bit offsets,
// or 32-bit indices when WIDE) and FP64 weights of each slice reach shared memory by
// bulk copies as in k_spmv_stream, and every row accumulates its entries in order with
// one FP64 FMA each, so every row value is bit-identical to the register walk
// k_spmv<double, double, double, MODE>.  MODE 0: y = A x (CG, S_CONV early exit) and
// x.y -> S_PQ / S_ALPHA; MODE 1: y = b - A x with ||y||^2 -> S_RR / S_RNORM and ||b||
// -> S_BNORM.
template <int MODE, int SC, int SS, int W, int MINB, bool WIDE = false>
__global__ void __launch_bounds__(W * 32, MINB) k_spmv_stream64(const __grid_constant__ Dev d,
                                                               const double* __restrict__ w,
                                                               const double* __restrict__ x, double* __restrict__ y,
                                                               const double* __restrict__ b, int slot) {
    static_assert(MODE == 0 || MODE == 1, "CG product or residual");
    static_assert(SC % 4 == 0, "stages hold whole groups of 4 entries");
    if (MODE == 0 && d.scal[S_CONV] != 0.0) return;
    extern __shared__ __align__(128) unsigned char stream_smem[];
    __shared__ __align__(8) unsigned long long bars[W][SS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gw = blockIdx.x * W + warp, nw = gridDim.x * W;
    SliceRing<SC, SS, double, WIDE> R;
    R.init(d, w, stream_smem + warp * SS * SliceRing<SC, SS, double, WIDE>::SB, bars[warp], gw, nw);
    const double coef = d.c.coef_lap;
    double part0 = 0.0, part1 = 0.0;
    for (int sl = gw; sl < R.nsl; sl += nw) {
        const int i = sl * 32 + lane;
        const bool row = i < d.n;
        const bool in = row && d.inner[i];
        const int cnt = in ? d.nbr_cnt[i] : 0;
        const int km = d.skmax[sl];
        double acc = 0.0;
        bool done = false;
        if ((WIDE || km >= 0) && R.streaming) {
            const int nc = (slice_kmax(km) + SC - 1) / SC;
            const int r0 = sl * 32;
            for (int c = 0; c < nc; ++c) {
                const unsigned char* cs;
                const double* ws;
                if (!R.acquire(cs, ws)) break;
                const int k0 = c * SC;
#pragma unroll
                for (int g = 0; g < SC; g += 4) {
                    int j[4];
                    double wv[4], xv[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        if constexpr (WIDE) j[u] = ((const int*)cs)[(g + u) * 32 + lane];
                        else j[u] = r0 + (int)(short)((const unsigned short*)cs)[(g + u) * 32 + lane];
                        wv[u] = ws[(g + u) * 32 + lane];
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) xv[u] = k0 + g + u < cnt ? __ldg(x + j[u]) : 0.0;
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (k0 + g + u < cnt) acc = __fma_rn(wv[u], xv[u], acc);
                }
                R.release();
            }
            done = R.streaming;
        }
        if (!done) {
            // 32-bit slice (16-bit ring), or streaming given up: the register walk
            const int kmax = __reduce_max_sync(0xffffffffu, cnt);
            const size_t base = (size_t)sl * d.K * 32 + lane;
            acc = sell_row_dot<false, double>(d, w, x, base, cnt, kmax, -1);
        }
        if (!row) continue;
        if (!in) {
            y[i] = 0.0;
            continue;
        }
        const double yi = d.diag[i] * x[i] - coef * acc;
        if (MODE == 0) {
            y[i] = yi;
            part0 += x[i] * yi;
        } else {
            const double ri = b[i] - yi;
            y[i] = ri;
            part0 += ri * ri;
            part1 += b[i] * b[i];
        }
    }
    double v[2] = {part0, part1}, out[2];
    if (grid_reduce<2, double>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        if (MODE == 0) {
            d.scal[S_PQ] = out[0];
            d.scal[S_ALPHA] = out[0] != 0.0 ? d.scal[S_RZ] / out[0] : 0.0;
        } else {
            d.scal[S_RR] = out[0];
            d.scal[S_RNORM] = sqrt(out[0]);
            d.scal[S_BNORM] = sqrt(out[1]);
        }
    }
}

// Refinement residual r = b - A x over streamed rows in double-float arithmetic, the
// same per-entry operations and accumulator order as k_residual_df (entries of even
// index into the first (hi, lo) pair, odd into the second, merged at the end), so r
// is bit-identical to it.  Norms -> S_RR / S_RNORM and ||b|| -> S_BNORM.
template <int SC, int SS, int W, int MINB, bool WIDE = false>
__global__ void __launch_bounds__(W * 32, MINB) k_residual_stream(const __grid_constant__ Dev d,
                                                                 const float* __restrict__ w,
                                                                 const double* __restrict__ x,
                                                                 double* __restrict__ r,
                                                                 const double* __restrict__ b, int slot) {
    static_assert(SC % 8 == 0, "stages hold whole groups of 8 entries");
    extern __shared__ __align__(128) unsigned char stream_smem[];
    __shared__ __align__(8) unsigned long long bars[W][SS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gw = blockIdx.x * W + warp, nw = gridDim.x * W;
    SliceRing<SC, SS, float, WIDE> R;
    R.init(d, w, stream_smem + warp * SS * SliceRing<SC, SS, float, WIDE>::SB, bars[warp], gw, nw);
    const float2* __restrict__ xs = d.xs;

    double part0 = 0.0, part1 = 0.0;
    for (int sl = gw; sl < R.nsl; sl += nw) {
        const int i = sl * 32 + lane;
        const bool row = i < d.n;
        const bool in = row && d.inner[i];
        const int cnt = in ? d.nbr_cnt[i] : 0;
        const int km = d.skmax[sl];
        float S0 = 0.f, C0 = 0.f, S1 = 0.f, C1 = 0.f;
        bool done = false;
        if ((WIDE || km >= 0) && R.streaming) {
            const int nc = (slice_kmax(km) + SC - 1) / SC;
            const int r0 = sl * 32;
            for (int c = 0; c < nc; ++c) {
                const unsigned char* cs;
                const float* ws;
                if (!R.acquire(cs, ws)) break;
                const int k0 = c * SC;
#pragma unroll
                for (int g = 0; g < SC; g += 8) {
                    int j[8];
                    float wv[8], h[8], l[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        if constexpr (WIDE) j[u] = ((const int*)cs)[(g + u) * 32 + lane];
                        else j[u] = r0 + (int)(short)((const unsigned short*)cs)[(g + u) * 32 + lane];
                        wv[u] = ws[(g + u) * 32 + lane];
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const bool a = k0 + g + u < cnt;
                        const float2 v = a ? xs[j[u]] : make_float2(0.f, 0.f);
                        h[u] = v.x;
                        l[u] = v.y;
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        if (k0 + g + u < cnt) {
                            const float p = __fmul_rn(wv[u], h[u]);
                            const float pe = __fmaf_rn(wv[u], h[u], -p);
                            if (u & 1) df_add(S1, C1, p, __fmaf_rn(wv[u], l[u], pe));
                            else df_add(S0, C0, p, __fmaf_rn(wv[u], l[u], pe));
                        }
                    }
                }
                R.release();
            }
            if (R.streaming) {
                df_add(S0, C0, S1, C1);
                done = true;
            }
        }
        if (!done) {
            const int kmax = __reduce_max_sync(0xffffffffu, cnt);
            const size_t base = (size_t)sl * d.K * 32 + lane;
            if (km >= 0) df_row_sum<true>(d, w, xs, base, cnt, kmax, sl * 32, S0, C0);
            else df_row_sum<false>(d, w, xs, base, cnt, kmax, -1, S0, C0);
        }
        if (!row) continue;
        if (!in) {
            r[i] = 0.0;
            continue;
        }
        const double acc = (double)S0 + (double)C0;
        const double ri = b[i] - (d.diag[i] * x[i] - d.c.coef_lap * acc);
        r[i] = ri;
        part0 += ri * ri;
        part1 += b[i] * b[i];
    }
    double v[2] = {part0, part1}, out[2];
    if (grid_reduce<2>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        d.scal[S_RR] = out[0];
        d.scal[S_RNORM] = sqrt(out[0]);
        d.scal[S_BNORM] = sqrt(out[1]);
    }
}

// The refinement residual after a pass, from the pass's own correction: with the FP32
// solution d of the pass and its scale s, x += s d and r -= s A d on interior rows (A
// the FP32-weight operator, A d in double-float as in k_residual_stream: each product
// exact as (p, fma(w, d_j, -p)); d is FP32, so there is no low word to gather), and
// r.r to the scalars (S_RR, S_RNORM; S_BNORM stays the first residual's).  Against
// b - A x recomputed, this adds the FP64 rounding of the x update, 2^-53 |x_i| per row,
// well inside the double-float residual's own 2^-44 of sum |w x|.  Non-interior rows keep
// r = 0 and x.
template <int SC, int SS, int W, int MINB, bool WIDE = false>
__global__ void __launch_bounds__(W * 32, MINB) k_residual_update_stream(const __grid_constant__ Dev d,
                                                                        const float* __restrict__ w,
                                                                        const float* __restrict__ dv, double s,
                                                                        double* __restrict__ x,
                                                                        double* __restrict__ r, int slot) {
    static_assert(SC % 8 == 0, "stages hold whole groups of 8 entries");
    extern __shared__ __align__(128) unsigned char stream_smem[];
    __shared__ __align__(8) unsigned long long bars[W][SS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gw = blockIdx.x * W + warp, nw = gridDim.x * W;
    SliceRing<SC, SS, float, WIDE> R;
    R.init(d, w, stream_smem + warp * SS * SliceRing<SC, SS, float, WIDE>::SB, bars[warp], gw, nw);

    double part0 = 0.0;
    for (int sl = gw; sl < R.nsl; sl += nw) {
        const int i = sl * 32 + lane;
        const bool row = i < d.n;
        const bool in = row && d.inner[i];
        const int cnt = in ? d.nbr_cnt[i] : 0;
        const int km = d.skmax[sl];
        float S0 = 0.f, C0 = 0.f, S1 = 0.f, C1 = 0.f;
        bool done = false;
        if ((WIDE || km >= 0) && R.streaming) {
            const int nc = (slice_kmax(km) + SC - 1) / SC;
            const int r0 = sl * 32;
            for (int c = 0; c < nc; ++c) {
                const unsigned char* cs;
                const float* ws;
                if (!R.acquire(cs, ws)) break;
                const int k0 = c * SC;
#pragma unroll
                for (int g = 0; g < SC; g += 8) {
                    int j[8];
                    float wv[8], h[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        if constexpr (WIDE) j[u] = ((const int*)cs)[(g + u) * 32 + lane];
                        else j[u] = r0 + (int)(short)((const unsigned short*)cs)[(g + u) * 32 + lane];
                        wv[u] = ws[(g + u) * 32 + lane];
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) h[u] = k0 + g + u < cnt ? dv[j[u]] : 0.f;
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        if (k0 + g + u < cnt) {
                            const float p = __fmul_rn(wv[u], h[u]);
                            const float pe = __fmaf_rn(wv[u], h[u], -p);
                            if (u & 1) df_add(S1, C1, p, pe);
                            else df_add(S0, C0, p, pe);
                        }
                    }
                }
                R.release();
            }
            if (R.streaming) {
                df_add(S0, C0, S1, C1);
                done = true;
            }
        }
        if (!done) {
            const int kmax = __reduce_max_sync(0xffffffffu, cnt);
            const size_t base = (size_t)sl * d.K * 32 + lane;
            if (km >= 0) df_row_sum<true>(d, w, dv, base, cnt, kmax, sl * 32, S0, C0);
            else df_row_sum<false>(d, w, dv, base, cnt, kmax, -1, S0, C0);
        }
        if (!in) continue;
        const double acc = (double)S0 + (double)C0;
        const double di = (double)dv[i];
        const double ri = r[i] - s * (d.diag[i] * di - d.c.coef_lap * acc);
        r[i] = ri;
        x[i] += s * di;
        part0 += ri * ri;
    }
    double v[1] = {part0}, out[1];
    if (grid_reduce<1>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        d.scal[S_RR] = out[0];
        d.scal[S_RNORM] = sqrt(out[0]);
    }
}

// CG start: z = M r, p = z, rz = r.z, plus the convergence test on ||r||.
// r / z / p of type TV; TR the type r is read from (FP64 residual for FP32 inner).
template <class TV>
__global__ void __launch_bounds__(256) k_cg_start(const __grid_constant__ Dev d, TV* r, TV* z, TV* p, const double* r64,
                                                  double scale, const double* m64, const float* m32, TV* xd, int slot,
                                                  double tol_abs, int maxit) {
    // element arithmetic in TV (FP32 for the inner solve: GB300's FP64 pipe is narrow);
    // per-thread partial dots in TV over <= a few rows, cross-thread sums in FP64
    TV prz = TV(0), prr = TV(0);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x) {
        TV rv = r64 ? (TV)(r64[i] * scale) : r[i];
        if (!d.inner[i]) rv = TV(0);
        const TV mi = m32 ? (TV)m32[i] : (TV)m64[i];
        const TV zv = rv * mi;
        r[i] = rv;
        z[i] = zv;
        p[i] = zv;
        if (xd) xd[i] = TV(0);
        prz += rv * zv;
        prr += rv * rv;
    }
    double v[2] = {(double)prz, (double)prr}, out[2];
    if (grid_reduce<2, TV>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        d.scal[S_RZ] = out[0];
        d.scal[S_RNORM] = sqrt(out[1]);
        d.scal[S_R0NORM] = sqrt(out[1]);
        d.scal[S_TOL] = tol_abs;
        d.scal[S_ITER] = 0.0;
        d.scal[S_MAXIT] = (double)maxit;
        d.scal[S_CONV] = (sqrt(out[1]) <= tol_abs || maxit <= 0) ? 1.0 : 0.0;
    }
}

// x += alpha p; r -= alpha q; z = M r; rz, rr; then beta, convergence.
// with_z = 0: the preconditioner is applied by separate kernels (z, rz and beta
// are theirs); only x, r and the convergence test here.
// flexible (with_z only): beta = -(z.q) / (p.q) of flexible CG instead of the ratio of
// successive r.z.
template <class TV, class TXA>
__global__ void __launch_bounds__(256) k_cg_update(const __grid_constant__ Dev d, TXA* x, TV* r, TV* z, const TV* p,
                                                   const TV* q, const double* m64, const float* m32, int slot,
                                                   int with_z, int flexible = 0) {
    if (d.scal[S_CONV] != 0.0) return;
    const TV alpha = (TV)d.scal[S_ALPHA];
    TV prz = TV(0), prr = TV(0), pzq = TV(0);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x) {
        if (!d.inner[i]) continue;
        x[i] = x[i] + (TXA)alpha * (TXA)p[i];
        const TV ri = r[i] - alpha * q[i];
        r[i] = ri;
        if (with_z) {
            const TV mi = m32 ? (TV)m32[i] : (TV)m64[i];
            const TV zi = ri * mi;
            z[i] = zi;
            prz += ri * zi;
            if (flexible) pzq += zi * q[i];
        }
        prr += ri * ri;
    }
    double v[3] = {(double)prz, (double)prr, (double)pzq}, out[3];
    if (grid_reduce<3, TV>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        if (with_z && flexible) {
            const double pq = d.scal[S_PQ];
            d.scal[S_BETA] = pq != 0.0 ? -out[2] / pq : 0.0;
            d.scal[S_RZ] = out[0];
        } else if (with_z) {
            const double rz = d.scal[S_RZ];
            d.scal[S_BETA] = rz != 0.0 ? out[0] / rz : 0.0;
            d.scal[S_RZ] = out[0];
        }
        const double rn = sqrt(out[1]);
        d.scal[S_RNORM] = rn;
        const double it = d.scal[S_ITER] + 1.0;
        d.scal[S_ITER] = it;
        if (rn <= d.scal[S_TOL] || it >= d.scal[S_MAXIT] || !(rn == rn)) d.scal[S_CONV] = 1.0;
    }
}

template <class TV>
__global__ void k_cg_p(const __grid_constant__ Dev d, TV* p, const TV* z) {
    pdl_wait();
    pdl_trigger();
    if (d.scal[S_CONV] != 0.0) return;
    const TV beta = (TV)d.scal[S_BETA];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x)
        p[i] = z[i] + beta * p[i];
}

// neighbour-entry counts of interior rows (PPE matrix) and all rows; interior rows
__global__ void __launch_bounds__(256) k_count_nnz(const __grid_constant__ Dev d, int slot) {
    double a = 0.0, b = 0.0, m = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x) {
        const double c = (double)d.nbr_cnt[i];
        b += c;
        if (d.inner[i]) {
            a += c;
            m += 1.0;
        }
    }
    double v[3] = {a, b, m}, out[3];
    if (grid_reduce<3>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        d.scal[S_NNZ0] = out[0];
        d.scal[S_NNZ1] = out[1];
        d.scal[S_NINT] = out[2];
    }
}

// host state exchange (SoA doubles <-> packed device state)
__global__ void k_pack_state(const __grid_constant__ Dev d, const double* p3, const double* v3, const double* pr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    d.pos[i] = make_dbl4(p3[3 * (size_t)i], p3[3 * (size_t)i + 1], p3[3 * (size_t)i + 2], 0.0);
    d.vel[i] = make_dbl4(v3[3 * (size_t)i], v3[3 * (size_t)i + 1], v3[3 * (size_t)i + 2], 0.0);
    d.press[i] = pr[i];
}
// particle inflow (CMultiGPUHandler::InsertBucket, MultiGPUHandler.cpp:1163-1210): the
// IDs below the extent that no particle carries are the holes, filled in increasing
// order; the rest of a bucket goes on at the extent
__global__ void k_fill_u32(unsigned* a, int n, unsigned v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}
__global__ void k_clear_present(const __grid_constant__ Dev d, unsigned* hole, int idext) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const int id = d.id[i];
    if (id >= 0 && id < idext) hole[id] = 0u;
}
__global__ void k_hole_list(const unsigned* hole, const unsigned* rank, int idext, int* holes) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id < idext && hole[id]) holes[rank[id]] = id;
}
// bucket particle j -> state slot d.n + j with the j-th hole's ID, or the extent + (j - holes)
__global__ void k_insert(const __grid_constant__ Dev d, const CParticle* __restrict__ b, int added, int nholes,
                         const int* __restrict__ holes, int idext) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= added) return;
    const size_t s = (size_t)d.n + (size_t)j;
    const CParticle q = b[j];
    d.pos[s] = make_dbl4(q.Position.x, q.Position.y, q.Position.z, 0.0);
    d.vel[s] = make_dbl4(q.Velocity.x, q.Velocity.y, q.Velocity.z, 0.0);
    d.press[s] = q.Pressure;
    d.visc[s] = q.KineticViscosity;
    d.type[s] = (int)q.Type;
    d.id[s] = j < nholes ? holes[j] : idext + (j - nholes);
    d.dph1[s] = 0.f;
    d.dph2[s] = 0.f;
}

// output frames in particle-ID order: mark the IDs present (the exclusive scan of the
// marks is each ID's row), then pack position, velocity, pressure, PND, viscosity
// (FP32) and type at that row: out = [pos 3n | vel 3n | press n | pnd n | visc n]
__global__ void k_frame_mark(const __grid_constant__ Dev d, unsigned* flag, int idcap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const int id = d.id[i];
    if (id >= 0 && id < idcap) flag[id] = 1u;
}
__global__ void k_frame_pack(const __grid_constant__ Dev d, const unsigned* rank, int idcap, float* out, int* otype) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const int id = d.id[i];
    if (id < 0 || id >= idcap) return;
    const size_t n = (size_t)d.n, r = rank[id];
    if (r >= n) return;
    const dbl4 p = d.pos[i], v = d.vel[i];
    out[3 * r] = (float)p.x; out[3 * r + 1] = (float)p.y; out[3 * r + 2] = (float)p.z;
    out[3 * n + 3 * r] = (float)v.x; out[3 * n + 3 * r + 1] = (float)v.y; out[3 * n + 3 * r + 2] = (float)v.z;
    out[6 * n + r] = (float)d.press[i];
    out[7 * n + r] = (float)d.pnd[i];
    out[8 * n + r] = d.visc[i];
    otype[r] = d.type[i];
}
__global__ void k_unpack_state(const __grid_constant__ Dev d, double* p3, double* v3, double* pr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const dbl4 p = d.pos[i], v = d.vel[i];
    p3[3 * (size_t)i] = p.x; p3[3 * (size_t)i + 1] = p.y; p3[3 * (size_t)i + 2] = p.z;
    v3[3 * (size_t)i] = v.x; v3[3 * (size_t)i + 1] = v.y; v3[3 * (size_t)i + 2] = v.z;
    pr[i] = d.press[i];
}

// ---------------------------------------------------------------------------
// learned initial guess / scaling
// ---------------------------------------------------------------------------
// pressure scale of the step: max(rms of the warm start over interior rows, rho |g| l0)
__global__ void __launch_bounds__(256) k_pressure_scale(const __grid_constant__ Dev d, int slot) {
    double a = 0.0, b = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x)
        if (d.inner[i]) {
            a += d.press[i] * d.press[i];
            b += 1.0;
        }
    double v[2] = {a, b}, out[2];
    if (grid_reduce<2>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        const double g = sqrt(d.c.g[0] * d.c.g[0] + d.c.g[1] * d.c.g[1] + d.c.g[2] * d.c.g[2]);
        const double floor_p = d.c.rho * (g > 0 ? g : 1.0) * d.c.l0;
        const double rms = out[1] > 0 ? sqrt(out[0] / out[1]) : 0.0;
        d.scal[S_PSCALE] = rms > floor_p ? rms : floor_p;
    }
}

// 12 features per particle (FP32); r holds the FP64 initial residual b - A p0 of the warm start p0
// The network's neighbour aggregates come from the gradient-radius rows (index,
// distance): mean previous pressure and velocity divergence
// sum (v_j - v_i).(x_j - x_i) w_g / r^2 * d / n0 over the PND neighbours.
template <class T>
__global__ void k_features(const __grid_constant__ Dev d) {
    // A warp takes 32 consecutive particles: for each, the lanes read its gradient
    // row together (coalesced) and the sums are shuffle-reduced and parked in the
    // particle's lane; then every lane assembles its own particle's features (FP32
    // arithmetic, FP64 only for the PND deviation), so nothing runs on one lane alone.
    const int lane = threadIdx.x & 31;
    const int base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
    const float reg = (float)d.c.re_grad, mindg = (float)d.c.mind_grad;
    float my_psum = 0.f, my_div = 0.f;
    for (int q = 0; q < 32 && base + q < d.n; ++q) {   // warp-uniform
        const int iq = base + q;
        const float4 pi = d.opos[iq], vi = d.ovel[iq];
        const int gc = d.gcnt[iq];
        float psum = 0.f, div = 0.f;
        for (int k = lane; k < gc; k += 32) {
            const size_t e = (size_t)iq * d.KG + k;
            const int j = d.gnbr[e];
            const float r = (float)((const T*)d.gnbrr)[e];
            const float4 pj = d.opos[j], vj = d.ovel[j];
            const float rg = r > mindg ? r : mindg;
            const float wg = reg / rg - 1.f;
            psum += d.pf32[j];
            div += ((vj.x - vi.x) * (pj.x - pi.x) + (vj.y - vi.y) * (pj.y - pi.y) + (vj.z - vi.z) * (pj.z - pi.z)) *
                   wg / (rg * rg);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            psum += __shfl_xor_sync(0xffffffffu, psum, o);
            div += __shfl_xor_sync(0xffffffffu, div, o);
        }
        if (lane == q) {
            my_psum = psum;
            my_div = div;
        }
    }
    const int i = base + lane;
    if (i >= d.n) return;
    const float psum = my_psum, div = my_div;
    const int gc = d.gcnt[i];
    const float4 vi = d.ovel[i];
    const float ips = (float)(1.0 / d.scal[S_PSCALE]);
    float* f = d.feat + 12 * (size_t)i;
    const float idg = 1.f / (float)d.diag[i];
    f[0] = (float)(d.pnd[i] - d.c.n0_pnd) * (float)(10.0 / d.c.n0_pnd);
    f[1] = div * (float)(d.c.dim / d.c.n0_pnd * d.c.dt * 10.0);
    const int t = d.wid[i];
    const float wd = (float)d.wdist[i];
    if (t >= 0 && wd < (float)d.c.re_lap) {
        const double* w = d.wdir + 3 * (size_t)i;
        const float wx = (float)w[0], wy = (float)w[1], wz = (float)w[2];
        const float l = sqrtf(wx * wx + wy * wy + wz * wz);
        const float il = l > 0.f ? 1.f / l : 0.f;
        f[2] = wd * (float)(1.0 / d.c.re_lap);
        f[3] = wx * il;
        f[4] = wy * il;
        f[5] = wz * il;
    } else {
        f[2] = 1.f; f[3] = 0.f; f[4] = 0.f; f[5] = 0.f;
    }
    f[6] = (float)d.press[i] * ips;
    f[7] = gc > 0 ? psum / (float)gc * ips : 0.f;
    f[8] = (float)d.rhs[i] * idg * ips;
    f[9] = (float)d.nbr_cnt[i] * (1.f / 250.f);
    f[10] = d.inner[i] ? (float)d.r[i] * idg * ips : 0.f;
    f[11] = sqrtf(vi.x * vi.x + vi.y * vi.y + vi.z * vi.z) * (float)(d.c.dt / d.c.l0 * 100.0);
}

// Extrapolated pressure increment of particle i from its last two increments: order 1
// repeats the last one (linear in time), order 2 adds its change (quadratic:
// P_n ~ 3 P_{n-1} - 3 P_{n-2} + P_{n-3}); order 0: none.
__device__ __forceinline__ double warm_increment(const Dev& d, int i, int order) {
    if (order <= 0) return 0.0;
    const double a = (double)d.dph1[i];
    return order >= 2 ? 2.0 * a - (double)d.dph2[i] : a;
}

// Warm start of the PPE solve: pprev = P_{n-1}, the particle's pressure after the last
// step, and the start p0 = P_{n-1} + the extrapolated increment on interior rows.
__global__ void k_warm_start(const __grid_constant__ Dev d, int order) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const double p = d.press[i];
    d.pprev[i] = p;
    if (order > 0 && d.inner[i]) d.press[i] = p + warm_increment(d, i, order);
}

// CalcPoisson's start: p0 of each particle from the caller's ID-indexed array (an ID at
// or above `cap` sets MPS_ERR_KEY_RANGE and keeps the particle's own pressure)
__global__ void k_poisson_start(const __grid_constant__ Dev d, int cap, const float* __restrict__ x0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const int id = d.id[i];
    if (id < 0 || id >= cap) {
        atomicOr(d.err, MPS_ERR_KEY_RANGE);
        return;
    }
    d.press[i] = (double)x0[id];
}
// CalcPoisson's outputs, ID-indexed: diagonal and right-hand side of the PPE row (0 for
// particles outside the PPE: free surface, Dirichlet P = 0) and the solved pressure
__global__ void k_poisson_out(const __grid_constant__ Dev d, int cap, float* a, float* b, float* x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const int id = d.id[i];
    if (id < 0 || id >= cap) {
        atomicOr(d.err, MPS_ERR_KEY_RANGE);
        return;
    }
    const bool in = d.inner[i] != 0;
    if (a) a[id] = in ? (float)d.diag[i] : 0.f;
    if (b) b[id] = in ? (float)d.rhs[i] : 0.f;
    if (x) x[id] = (float)d.press[i];
}

// after the solve: shift the increment history (P_n - P_{n-1} on interior rows, else 0)
__global__ void k_history(const __grid_constant__ Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    d.dph2[i] = d.dph1[i];
    d.dph1[i] = d.inner[i] ? (float)(d.press[i] - d.pprev[i]) : 0.f;
    d.pf32[i] = (float)d.press[i];   // FP32 copy for the correction's pair terms
}

// predicted increment dp = scale * y0 (into z), preconditioner M^-1 = exp(y1) / diag
// when the scaling output is used (else Jacobi)
__global__ void k_learned_apply(const __grid_constant__ Dev d, int use_scaling) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    if (!d.inner[i]) {
        d.z[i] = 0.0;
        d.z32[i] = 0.f;
        d.minv[i] = 0.0;
        return;
    }
    const float y0 = d.mlp_out[2 * (size_t)i], y1 = d.mlp_out[2 * (size_t)i + 1];
    const double inc = (double)fminf(fmaxf(y0, -50.f), 50.f) * d.scal[S_PSCALE];
    d.z[i] = isfinite(inc) ? inc : 0.0;
    d.z32[i] = (float)d.z[i];
    const double s = use_scaling ? exp((double)fminf(fmaxf(isfinite(y1) ? y1 : 0.f, -2.3f), 2.3f)) : 1.0;
    d.minv[i] = s / d.diag[i];
}

// p = p0 + alpha dp with alpha = (dp . r0) / (dp . A dp), the A-norm-optimal step
// along the predicted increment (so the start is never worse than the warm start p0)
__global__ void k_learned_finish(const __grid_constant__ Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const double dad = d.scal[S_LS0], dr = d.scal[S_LS1];
    double a = (dad > 0.0 && isfinite(dr / dad)) ? dr / dad : 0.0;
    if (i == 0) d.scal[S_IRTOL] = a;
    d.press[i] = d.inner[i] ? d.press[i] + a * d.z[i] : 0.0;
}

// FP32 path: the same update, and the refinement residual of the new start without a
// second residual pass: r = r0 - alpha (A dp), with r0 = b - A p0 (FP64-accurate,
// already in d.r) and A dp the line search's FP32 product (q32); ||r|| -> S_RR, S_RNORM
// (S_BNORM is r0's).  The FP32 error of alpha (A dp) only perturbs the first
// refinement pass, which is followed by a freshly computed residual.
__global__ void __launch_bounds__(256) k_learned_finish_r(const __grid_constant__ Dev d, int slot) {
    const double dad = d.scal[S_LS0], dr = d.scal[S_LS1];
    const double a = (dad > 0.0 && isfinite(dr / dad)) ? dr / dad : 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        d.scal[S_IRTOL] = a;
        d.scal[S_TMP1] = d.scal[S_RNORM];   // ||r|| of the warm start, before the update
    }
    double rr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x) {
        if (!d.inner[i]) {
            d.press[i] = 0.0;
            d.r[i] = 0.0;
            continue;
        }
        d.press[i] = d.press[i] + a * d.z[i];
        const double ri = d.r[i] - a * (double)d.q32[i];
        d.r[i] = ri;
        rr += ri * ri;
    }
    double v[1] = {rr}, out[1];
    if (grid_reduce<1>(v, d.red, d.red_count + slot, out) && threadIdx.x == 0) {
        d.scal[S_RR] = out[0];
        d.scal[S_RNORM] = sqrt(out[0]);
    }
}

// training targets after a plain solve: (p - p0) / scale, p0 the warm start the features
// were computed at (P_{n-1} + the extrapolated increment of `order`), and the log of the
// diagonal scale that maps the initial residual onto the error, clamped to [0.1, 10]
__global__ void k_targets(const __grid_constant__ Dev d, int order) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    float* t = d.targets + 2 * (size_t)i;
    if (!d.inner[i]) {
        t[0] = nanf("");
        t[1] = nanf("");
        return;
    }
    const double ps = d.scal[S_PSCALE];
    const double e = d.press[i] - (d.pprev[i] + warm_increment(d, i, order));
    t[0] = (float)(e / ps);
    const double r0n = (double)d.feat[12 * (size_t)i + 10];   // r0 / (diag ps)
    const double en = e / ps;
    double ls = 0.0;
    if (fabs(r0n) > 1e-6) {
        double s = en / r0n;
        s = s < 0.1 ? 0.1 : (s > 10.0 ? 10.0 : s);
        ls = log(s);
    }
    t[1] = (float)ls;
}

__global__ void k_restore_plain(const __grid_constant__ Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    d.press[i] = d.inner[i] ? d.pprev[i] : 0.0;
    d.minv[i] = d.inner[i] ? 1.0 / d.diag[i] : 0.0;
}

__global__ void k_to_float(int n, const double* a, float* b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// x (FP64) += s * dx (FP32), interior only
__global__ void k_axpy_ir(const __grid_constant__ Dev d, double* x, const float* dx, double s) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x)
        if (d.inner[i]) x[i] += s * (double)dx[i];
}

// ---------------------------------------------------------------------------
// pressure-gradient correction (CalcExplicitPressureGradient_Kernel semantics)
// ---------------------------------------------------------------------------
template <class T>
__device__ void correct_finish(const Dev& d, int i, T gx, T gy, T gz);

template <class T>
__global__ void k_correct(const __grid_constant__ Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    const V3<T> pi = load_p<T>(d, i);
    const double Pi = d.press[i];
    const T reg = (T)d.c.re_grad, mindg = (T)d.c.mind_grad;
    T gx = 0, gy = 0, gz = 0;
    const int cnt = d.gcnt[i];
    const size_t base = (size_t)i * d.KG;
    for (int k = 0; k < cnt; ++k) {
        const int j = d.gnbr[base + k];
        const T r = ((const T*)d.gnbrr)[base + k];
        const V3<T> pj = load_p<T>(d, j);
        const T rr = r > mindg ? r : mindg;
        const T pc = (T)(0.5 * (d.press[j] + Pi)) * (reg / rr - T(1)) / (rr * rr);
        gx += (pj.x - pi.x) * pc;
        gy += (pj.y - pi.y) * pc;
        gz += (pj.z - pi.z) * pc;
    }
    correct_finish<T>(d, i, gx, gy, gz);
}

// FP32 path of the correction: a warp takes 32 consecutive particles; for each, the
// lanes read its gradient row together (coalesced) with the pair pressures from the
// FP32 copy of the solved pressure (no FP64 arithmetic per pair: GB300's FP64 pipe is
// narrow), the sums are shuffle-reduced and parked in the particle's lane, and every
// lane then finishes its own particle (correct_finish, FP64 state update).
__global__ void k_correct_warp(const __grid_constant__ Dev d) {
    const int lane = threadIdx.x & 31;
    const int base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
    const float reg = (float)d.c.re_grad, mindg = (float)d.c.mind_grad;
    float mx = 0.f, my = 0.f, mz = 0.f;
    for (int q = 0; q < 32 && base + q < d.n; ++q) {   // warp-uniform
        const int iq = base + q;
        const float4 pi = d.opos[iq];
        const float Pi = d.pf32[iq];
        const int gc = d.gcnt[iq];
        float gx = 0.f, gy = 0.f, gz = 0.f;
        for (int k = lane; k < gc; k += 32) {
            const size_t e = (size_t)iq * d.KG + k;
            const int j = d.gnbr[e];
            const float r = ((const float*)d.gnbrr)[e];
            const float4 pj = d.opos[j];
            const float rr = r > mindg ? r : mindg;
            const float pc = 0.5f * (d.pf32[j] + Pi) * (reg / rr - 1.f) / (rr * rr);
            gx += (pj.x - pi.x) * pc;
            gy += (pj.y - pi.y) * pc;
            gz += (pj.z - pi.z) * pc;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            gx += __shfl_xor_sync(0xffffffffu, gx, o);
            gy += __shfl_xor_sync(0xffffffffu, gy, o);
            gz += __shfl_xor_sync(0xffffffffu, gz, o);
        }
        if (lane == q) {
            mx = gx;
            my = gy;
            mz = gz;
        }
    }
    const int i = base + lane;
    if (i < d.n) correct_finish<float>(d, i, mx, my, mz);
}

// the per-particle end of the correction: FP64 gradient with the wall terms, velocity
// update with the Courant clamp, position update (CalcExplicitPressureGradient_Kernel)
template <class T>
__device__ void correct_finish(const Dev& d, int i, T gx, T gy, T gz) {
    const double Pi = d.press[i];
    double g[3] = {(double)gx * d.c.c1, (double)gy * d.c.c1, (double)gz * d.c.c1};
    if (d.wid[i] >= 0) {
        const double m = d.wdist[i];
        const double* dir = d.wdir + 3 * (size_t)i;
        if (m > 0 && m <= d.c.re_grad) {
            const double ww = exact_z<double>(c_zgrad3, 21, m, d.c.l0);
            const double wc = 0.5 * d.c.c1 * ww * Pi / (m * m);
            for (int a = 0; a < 3; ++a) g[a] -= wc * dir[a];
        }
        if (m > 0 && m <= d.c.offset_l0) {
            const double mc = d.c.c2 * (d.c.offset_l0 - m) / m;
            for (int a = 0; a < 3; ++a) g[a] -= mc * dir[a];
        }
    }
    const dbl4 v = d.vel[i];
    const dbl4 p = d.pos[i];
    const double c3 = -d.c.dt / d.c.rho;
    dbl4 vn = make_dbl4(v.x + c3 * g[0], v.y + c3 * g[1], v.z + c3 * g[2], 0.0);
    const double a = sqrt(vn.x * vn.x + vn.y * vn.y + vn.z * vn.z);
    if (a > d.c.vmax) {
        const double s = d.c.vmax / a;
        vn.x *= s; vn.y *= s; vn.z *= s;
    }
    if (!(isfinite(vn.x) && isfinite(vn.y) && isfinite(vn.z))) {
        atomicOr(d.err, MPS_ERR_NONFINITE);
        vn = v;
    }
    d.vel2[i] = vn;
    d.pos2[i] = make_dbl4(p.x + (vn.x - v.x) * d.c.dt, p.y + (vn.y - v.y) * d.c.dt, p.z + (vn.z - v.z) * d.c.dt, 0.0);
}

// Wall motion: translation + incremental rotation with linear ramp, FP64, exactly
// normalised axis (RotateTrianglePosition_Kernel semantics).
__global__ void k_walls_move(const __grid_constant__ Dev d, int step) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.tri_n) return;
    const CTriangleParameters tp = d.tparams[d.tmodel[t]];
    double* v = d.tri + 9 * (size_t)t;
    const double dt = d.c.dt;
    for (int q = 0; q < 3; ++q) {
        v[3 * q] += (double)tp.Velocity.x * dt;
        v[3 * q + 1] += (double)tp.Velocity.y * dt;
        v[3 * q + 2] += (double)tp.Velocity.z * dt;
    }
    if (!tp.RotatingOrNot) return;
    const double tpass = dt * step;
    if (tpass < tp.RotationStartTime || tp.AngleOfRotationInDegree == 0) return;
    double ang;
    if (tpass < tp.TimeToReachRPM) {
        const int req = (int)((tp.TimeToReachRPM - tp.RotationStartTime) / dt);
        ang = ((double)tp.AngleOfRotationInDegree / (double)(req + 1)) * (step - tp.RotationStartTime / dt);
    } else {
        ang = tp.AngleOfRotationInDegree;
    }
    if (ang == 0) return;
    const double cx = tp.CenterOfRotation.x, cy = tp.CenterOfRotation.y, cz = tp.CenterOfRotation.z;
    double ax = tp.SecondPointOfRotation.x - cx, ay = tp.SecondPointOfRotation.y - cy, az = tp.SecondPointOfRotation.z - cz;
    const double al = sqrt(ax * ax + ay * ay + az * az);
    if (!(al > 0)) return;
    ax /= al; ay /= al; az /= al;
    const double th = ang * 3.14159265358979323846 / 180.0;
    double st, ct;
    sincos(th, &st, &ct);
    for (int q = 0; q < 3; ++q) {
        const double px = v[3 * q] - cx, py = v[3 * q + 1] - cy, pz = v[3 * q + 2] - cz;
        const double kx = ay * pz - az * py, ky = az * px - ax * pz, kz = ax * py - ay * px;
        const double kv = ax * px + ay * py + az * pz;
        v[3 * q] = cx + px * ct + kx * st + ax * kv * (1.0 - ct);
        v[3 * q + 1] = cy + py * ct + ky * st + ay * kv * (1.0 - ct);
        v[3 * q + 2] = cz + pz * ct + kz * st + az * kv * (1.0 - ct);
    }
    const double e1x = v[3] - v[0], e1y = v[4] - v[1], e1z = v[5] - v[2];
    const double e2x = v[6] - v[0], e2y = v[7] - v[1], e2z = v[8] - v[2];
    double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
    const double nl = sqrt(nx * nx + ny * ny + nz * nz);
    if (nl > 0) {
        d.tnrm[3 * t] = nx / nl;
        d.tnrm[3 * t + 1] = ny / nl;
        d.tnrm[3 * t + 2] = nz / nl;
    }
}

}  // namespace mps
