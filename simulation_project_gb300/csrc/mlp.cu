// mlp.cu - BF16 tensor-core GEMM and the learned-preconditioner MLP (forward,
// backward, Adam) of the GB300 MPS library (include/mps_learned.h).
//
// GEMM (training): k_gemm_tc on the 5th-generation tensor cores (tcgen05.mma into
// TMEM, see below).  Cross-check variant k_gemm_bf16: one CTA of 4 warps computes a
// 64x64 FP32 tile of C with warp-level
// mma.sync.m16n8k16 (BF16 in, FP32 accumulate); each warp owns a 32x32 sub-tile
// (2 x 4 MMA tiles).  K advances 32 at a time through padded shared-memory tiles
// As[m][k] and Bs[n][k], so every A and B fragment register is one 32-bit shared
// load of two consecutive k.  Transposed operands are handled by the tile loader.
// The epilogue adds a bias, optionally keeps the FP32 pre-activation, applies SiLU
// and writes FP32 and/or BF16; split-K CTAs accumulate with FP32 atomics.
// The network is tiny (69 kFLOP per particle per forward), so these kernels are a
// small part of a solver step; they exist so the network is trained on the GPU by
// this library's own kernels.  The solver's inference runs on the 5th-generation
// tensor cores in FP16 (k_mlp_infer_tc: tcgen05.mma into TMEM, four 128-row tiles in
// flight per SM, weights staged by one bulk copy, biases inside the MMAs, SiLU in
// packed FP16); the fused mma.sync inference kernel (k_mlp_infer, BF16 and FP32 like
// training) is kept as its cross-check.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <math.h>
#include <stdio.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "mps_common.cuh"
#include "mps_internal.h"
#include "../../include/mps_learned.h"
#include "../../include/mps_solver.h"

namespace mps {

typedef __nv_bfloat16 bf16;
constexpr int GT_M = 64, GT_N = 64, GT_K = 32, GT_PAD = 8;
constexpr int H = 128;      // hidden width
constexpr int FIN = 12;     // input features
constexpr int FINP = 16;    // padded input width
constexpr int FOUT = 2;     // outputs
constexpr int FOUTP = 16;   // padded output width
static_assert(MPS_MLP_PARAMS == FIN * H + H + 2 * (H * H + H) + H * FOUT + FOUT,
              "parameter vector length must match the layer layout");

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

__global__ void __launch_bounds__(128) k_gemm_bf16(int M, int N, int K, const bf16* __restrict__ A, int lda, int ta,
                                                  const bf16* __restrict__ B, int ldb, int tb, float* C, int ldc,
                                                  bf16* Cb, int ldcb, float* Cz, const float* __restrict__ bias, int act,
                                                  float beta, int kchunk) {
    __shared__ __align__(16) bf16 As[GT_M][GT_K + GT_PAD];
    __shared__ __align__(16) bf16 Bs[GT_N][GT_K + GT_PAD];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, c = lane & 3;
    const int m0 = blockIdx.y * GT_M, n0 = blockIdx.x * GT_N;
    const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[a][b][q] = 0.f;
    const bf16 zero = __float2bfloat16(0.f);
    for (int k0 = kbeg; k0 < kend; k0 += GT_K) {
        for (int e = tid; e < GT_M * GT_K; e += 128) {
            int mm, kk;
            if (ta == 0) { mm = e / GT_K; kk = e % GT_K; } else { kk = e / GT_M; mm = e % GT_M; }
            const int m = m0 + mm, k = k0 + kk;
            bf16 v = zero;
            if (m < M && k < kend) v = ta == 0 ? A[(size_t)m * lda + k] : A[(size_t)k * lda + m];
            As[mm][kk] = v;
        }
        for (int e = tid; e < GT_N * GT_K; e += 128) {
            int nn, kk;
            if (tb == 0) { kk = e / GT_N; nn = e % GT_N; } else { nn = e / GT_K; kk = e % GT_K; }
            const int n = n0 + nn, k = k0 + kk;
            bf16 v = zero;
            if (n < N && k < kend) v = tb == 0 ? B[(size_t)k * ldb + n] : B[(size_t)n * ldb + k];
            Bs[nn][kk] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GT_K; kk += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const int r = wm + mt * 16 + g;
                af[mt][0] = *(const uint32_t*)&As[r][kk + 2 * c];
                af[mt][1] = *(const uint32_t*)&As[r + 8][kk + 2 * c];
                af[mt][2] = *(const uint32_t*)&As[r][kk + 2 * c + 8];
                af[mt][3] = *(const uint32_t*)&As[r + 8][kk + 2 * c + 8];
            }
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int r = wn + nt * 8 + g;
                bfr[nt][0] = *(const uint32_t*)&Bs[r][kk + 2 * c];
                bfr[nt][1] = *(const uint32_t*)&Bs[r][kk + 2 * c + 8];
            }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], af[mt], bfr[nt]);
        }
        __syncthreads();
    }
    const bool split = gridDim.z > 1;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int row = m0 + wm + mt * 16 + g + (q >= 2 ? 8 : 0);
                const int col = n0 + wn + nt * 8 + 2 * c + (q & 1);
                if (row >= M || col >= N) continue;
                float v = acc[mt][nt][q];
                if (split) {
                    atomicAdd(C + (size_t)row * ldc + col, v);
                    continue;
                }
                if (bias) v += bias[col];
                if (Cz) Cz[(size_t)row * ldc + col] = v;
                if (act == 1) v = silu(v);
                if (C) C[(size_t)row * ldc + col] = beta != 0.f ? beta * C[(size_t)row * ldc + col] + v : v;
                if (Cb) Cb[(size_t)row * ldcb + col] = __float2bfloat16(v);
            }
}

// the mma.sync GEMM (variant 1, a cross-check of the tcgen05 one)
cudaError_t gemm_mma_sync(int M, int N, int K, const bf16* A, int lda, int ta, const bf16* B, int ldb, int tb, float* C,
                          int ldc, bf16* Cb, int ldcb, float* Cz, const float* bias, int act, float beta, int split,
                          cudaStream_t st) {
    if (M <= 0 || N <= 0 || K <= 0) return cudaErrorInvalidValue;
    split = max(1, split);
    int kchunk = (K + split - 1) / split;
    kchunk = (kchunk + GT_K - 1) / GT_K * GT_K;
    split = (K + kchunk - 1) / kchunk;
    dim3 grid(div_up(N, GT_N), div_up(M, GT_M), split);
    MPS_COUNT_LAUNCH k_gemm_bf16<<<grid, 128, 0, st>>>(M, N, K, A, lda, ta, B, ldb, tb, C, ldc, Cb, ldcb, Cz, bias, act, beta, kchunk);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// elementwise helpers of the MLP
// ---------------------------------------------------------------------------
__global__ void k_pack_input(int M, const float* __restrict__ X, bf16* __restrict__ Xb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * FINP) return;
    const int r = i / FINP, c = i % FINP;
    Xb[i] = __float2bfloat16(c < FIN ? X[(size_t)r * FIN + c] : 0.f);
}
// FP32 master parameters -> padded BF16 weights and FP32 biases
struct Layers {
    bf16 *W1, *W2, *W3, *W4;      // [16][128], [128][128], [128][128], [128][16]
    float *b1, *b2, *b3, *b4;     // [128] x3, [16]
    unsigned char* tc;            // shared-memory image of the tcgen05 inference kernel:
                                  // W1^T .. W4^T (canonical K-major) and the biases
};
__global__ void k_params_to_layers(const float* __restrict__ p, Layers L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int o1 = FIN * H, o2 = o1 + H, o3 = o2 + H * H, o4 = o3 + H, o5 = o4 + H * H, o6 = o5 + H, o7 = o6 + H * FOUT;
    if (i < FINP * H) {
        const int k = i / H, n = i % H;
        L.W1[i] = __float2bfloat16(k < FIN ? p[k * H + n] : 0.f);
    }
    if (i < H) {
        L.b1[i] = p[o1 + i];
        L.b2[i] = p[o3 + i];
        L.b3[i] = p[o5 + i];
    }
    if (i < H * H) {
        L.W2[i] = __float2bfloat16(p[o2 + i]);
        L.W3[i] = __float2bfloat16(p[o4 + i]);
    }
    if (i < H * FOUTP) {
        const int k = i / FOUTP, n = i % FOUTP;
        L.W4[i] = __float2bfloat16(n < FOUT ? p[o6 + k * FOUT + n] : 0.f);
    }
    if (i < FOUTP) L.b4[i] = i < FOUT ? p[o7 + i] : 0.f;
}
__global__ void k_unpad_output(int M, const float* __restrict__ Yp, float* __restrict__ Y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * FOUT) return;
    Y[i] = Yp[(size_t)(i / FOUT) * FOUTP + (i % FOUT)];
}

// ---------------------------------------------------------------------------
// Fused inference: the whole 12 -> 128 -> 128 -> 128 -> 2 network in one
// persistent kernel.  Each CTA stages the four weight matrices once in shared
// memory, transposed to [n][k] with padded rows (conflict-free B fragments); each
// warp takes 16 rows at a time through all layers with mma.m16n8k16 (BF16 in, FP32
// accumulate).  Bias and SiLU are applied to the accumulator fragments in
// registers, which are repacked directly as the next layer's BF16 A fragments
// (the m16n8 accumulator of n-tiles 2k, 2k+1 is the m16k16 A tile of k-step k), so
// activations never leave the registers.  Same rounding points as the layer-by-
// layer path: FP32 sum + bias, SiLU in FP32, BF16 activations.
// ---------------------------------------------------------------------------
constexpr int kMiWarps = 16;
constexpr int kMiS1 = 24;    // padded row (elements) of W1^T [128][16]
constexpr int kMiS = 136;    // padded row of W2^T, W3^T [128][128] and W4^T [8][128]
constexpr size_t kMiSmem = sizeof(bf16) * (128 * kMiS1 + 2 * 128 * kMiS + 8 * kMiS) + sizeof(float) * (3 * H + 8);

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// 16 x 128 accumulator (16 n-tiles) -> bias + SiLU -> A fragments of the next layer
__device__ __forceinline__ void mi_activate(float (&acc)[16][4], const float* __restrict__ bias, int c,
                                            uint32_t (&a)[8][4]) {
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
        const float b0 = bias[nt * 8 + 2 * c], b1 = bias[nt * 8 + 2 * c + 1];
        acc[nt][0] = silu(acc[nt][0] + b0);
        acc[nt][1] = silu(acc[nt][1] + b1);
        acc[nt][2] = silu(acc[nt][2] + b0);
        acc[nt][3] = silu(acc[nt][3] + b1);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        a[k][0] = pack_bf16(acc[2 * k][0], acc[2 * k][1]);
        a[k][1] = pack_bf16(acc[2 * k][2], acc[2 * k][3]);
        a[k][2] = pack_bf16(acc[2 * k + 1][0], acc[2 * k + 1][1]);
        a[k][3] = pack_bf16(acc[2 * k + 1][2], acc[2 * k + 1][3]);
    }
}

// four 8x8 BF16 matrices from shared memory; lane l gives the address of row l % 8 of
// matrix l / 8 (16-byte aligned).  With W^T stored [n][k], an 8 (n) x 8 (k) matrix is
// exactly one register of an m16n8k16 B fragment.
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const bf16* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"((unsigned)__cvta_generic_to_shared(p)));
}

// hidden layer 128 -> 128 with weights W^T [128][kMiS] in shared memory; one ldmatrix
// brings the B fragments of two n-tiles
__device__ __forceinline__ void mi_hidden(const uint32_t (&a)[8][4], const bf16* __restrict__ wt, int lane,
                                          float (&acc)[16][4]) {
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
    const int m = lane >> 3, rr = lane & 7;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
#pragma unroll
        for (int np = 0; np < 8; ++np) {
            uint32_t b[4];
            ldsm_x4(b, wt + ((2 * np + (m >> 1)) * 8 + rr) * kMiS + 16 * k + 8 * (m & 1));
            const uint32_t b0[2] = {b[0], b[1]}, b1[2] = {b[2], b[3]};
            mma_bf16(acc[2 * np], a[k], b0);
            mma_bf16(acc[2 * np + 1], a[k], b1);
        }
    }
}

__global__ void __launch_bounds__(kMiWarps * 32, 1) k_mlp_infer(int M, const float* __restrict__ X, float* __restrict__ Y,
                                                            Layers L) {
    extern __shared__ __align__(16) unsigned char mi_smem[];
    bf16* w1 = reinterpret_cast<bf16*>(mi_smem);   // [128][kMiS1]
    bf16* w2 = w1 + 128 * kMiS1;                    // [128][kMiS]
    bf16* w3 = w2 + 128 * kMiS;
    bf16* w4 = w3 + 128 * kMiS;                     // [8][kMiS]
    float* bs = reinterpret_cast<float*>(w4 + 8 * kMiS);   // b1, b2, b3 [128], b4 [8]
    const bf16 zero = __float2bfloat16(0.f);
    for (int e = threadIdx.x; e < 128 * kMiS1; e += blockDim.x) {
        const int n = e / kMiS1, k = e % kMiS1;
        w1[e] = k < FINP ? L.W1[k * H + n] : zero;
    }
    for (int e = threadIdx.x; e < H * H; e += blockDim.x) {
        const int k = e / H, n = e % H;   // W[k][n]
        w2[n * kMiS + k] = L.W2[e];
        w3[n * kMiS + k] = L.W3[e];
    }
    for (int e = threadIdx.x; e < 8 * H; e += blockDim.x) {
        const int n = e / H, k = e % H;
        w4[n * kMiS + k] = L.W4[k * FOUTP + n];
    }
    for (int e = threadIdx.x; e < 3 * H + 8; e += blockDim.x)
        bs[e] = e < H ? L.b1[e] : e < 2 * H ? L.b2[e - H] : e < 3 * H ? L.b3[e - 2 * H] : L.b4[e - 3 * H];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, c = lane & 3;
    const int tiles = (M + 15) / 16;
    for (int t = blockIdx.x * kMiWarps + warp; t < tiles; t += gridDim.x * kMiWarps) {
        const int r0 = t * 16 + g, r1 = r0 + 8;
        // layer 1: A = features (12 of 16 columns), one k-step
        auto feat2 = [&](int r, int col) -> uint32_t {
            if (r >= M || col >= FIN) return 0u;
            const float2 v = *reinterpret_cast<const float2*>(X + (size_t)r * FIN + col);
            return pack_bf16(v.x, v.y);
        };
        const uint32_t a1[4] = {feat2(r0, 2 * c), feat2(r1, 2 * c), feat2(r0, 2 * c + 8), feat2(r1, 2 * c + 8)};
        float acc[16][4];
        const int m = lane >> 3, rr = lane & 7;
#pragma unroll
        for (int np = 0; np < 8; ++np) {
            uint32_t b[4];
            ldsm_x4(b, w1 + ((2 * np + (m >> 1)) * 8 + rr) * kMiS1 + 8 * (m & 1));
            const uint32_t b0[2] = {b[0], b[1]}, b1[2] = {b[2], b[3]};
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[2 * np][q] = acc[2 * np + 1][q] = 0.f;
            mma_bf16(acc[2 * np], a1, b0);
            mma_bf16(acc[2 * np + 1], a1, b1);
        }
        uint32_t a[8][4];
        mi_activate(acc, bs, c, a);
        mi_hidden(a, w2, lane, acc);
        mi_activate(acc, bs + H, c, a);
        mi_hidden(a, w3, lane, acc);
        mi_activate(acc, bs + 2 * H, c, a);
        // output layer: one n-tile (columns 0..7, of which 0 and 1 are used); one
        // ldmatrix brings the B fragments of two k-steps
        float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kp = 0; kp < 4; ++kp) {
            uint32_t b[4];
            ldsm_x4(b, w4 + rr * kMiS + 16 * (2 * kp + (m >> 1)) + 8 * (m & 1));
            const uint32_t b0[2] = {b[0], b[1]}, b1[2] = {b[2], b[3]};
            mma_bf16(o, a[2 * kp], b0);
            mma_bf16(o, a[2 * kp + 1], b1);
        }
        if (c == 0) {
            const float b0 = bs[3 * H], b1 = bs[3 * H + 1];
            if (r0 < M) *reinterpret_cast<float2*>(Y + (size_t)r0 * FOUT) = make_float2(o[0] + b0, o[1] + b1);
            if (r1 < M) *reinterpret_cast<float2*>(Y + (size_t)r1 * FOUT) = make_float2(o[2] + b0, o[3] + b1);
        }
    }
}
// ---------------------------------------------------------------------------
// Fused inference on the 5th-generation tensor cores (tcgen05).  A persistent CTA
// keeps kTcSlots 128-row tiles in flight, each with its own TMEM accumulator (128
// columns), its own layer input in shared memory and its own 4 warps (warp w reads
// TMEM lanes 32 (w % 4) ..): the slot's first thread issues the MMAs of a layer and
// commits them to the slot's mbarrier mma_done[s]; the 4 warps wait on it, read their
// rows of the accumulator with tcgen05.ld, apply SiLU and write the FP16 activations as
// the next layer's A operand, meet at the slot's named barrier, and the first thread
// issues the next layer.  The slots run independently, so the tensor cores work on
// one slot's layer while other slots' epilogues run.
// Operands use the canonical K-major layout without swizzle (core matrices of 8 rows
// x 16 bytes; the two core matrices of one 16-wide k-step 128 bytes apart, 8-row
// groups K/8 x 128 bytes apart): the weights W^T [n][k], staged once per CTA by one
// bulk copy of an image prepared from the FP32 parameters at each update
// (k_layers_to_tc), and the layer input [row][k] (one [128][144] buffer per slot; the
// 12 features of layer 1, two ones and two zeros sit in its first 16 columns, read as
// a K = 16 operand).  MMAs:
// tcgen05.mma.cta_group::1.kind::f16 with FP16 A and B, FP32 accumulate, M = 128,
// N = 128 (hidden layers) or 16 (output), one per k-step of 16.
// The biases ride in the MMAs: every layer input carries two columns of ones (input
// columns 12 and 13; hidden columns 128 and 129, K = 144) against the bias split into
// an FP16 high part and the FP16 rounding of its remainder (about 21 significant
// bits).  The hidden layers accumulate in FP16 (9 k-steps: the partial sums are
// rounded to 11 significant bits 9 times, about the error of the BF16 activations the
// FP32-accumulating kernels keep), read two per register (tcgen05.ld .pack::16b); the
// output layer accumulates in FP32.  SiLU(z) = h (1 + tanh h) with h = z / 2: the
// image holds the hidden layers' weights and biases times 1/2, so the accumulator is
// h; tanh is the hardware approximation on two values at once (tanh.approx.f16x2) and
// h + h tanh h one packed FP16 multiply-add: two instructions per pair of activations
// and no conversion (the SFU pipe runs only the tanh), FP16 activations.  Every
// mbarrier wait is bounded; a slot whose wait ran out (any of its threads: the
// outcome is made uniform with a barrier reduction) sets g_mlp_tc_timeout and the
// caller's error word and stops, its first thread waiting (bounded) for the MMAs it
// issued before TMEM is freed.
// ---------------------------------------------------------------------------
constexpr int kTcRows = 128;
constexpr int kTcSlots = 4;
constexpr int kTcK = H + 16;   // hidden layer input: 128 activations, 2 ones, 14 zeros
// the weight image (FP16, byte offsets)
constexpr int kImW1 = 0;                           // W1^T [128][16]  (x 1/2, bias in k = 12, 13)
constexpr int kImW2 = kImW1 + 128 * FINP * 2;      // W2^T [128][144] (x 1/2, bias in k = 128, 129)
constexpr int kImW3 = kImW2 + 128 * kTcK * 2;      // W3^T [128][144] (x 1/2)
constexpr int kImW4 = kImW3 + 128 * kTcK * 2;      // W4^T [16][144]
constexpr int kTcImage = kImW4 + FOUTP * kTcK * 2; // bytes of the image
constexpr int kTcABytes = 128 * kTcK * 2;          // one slot's layer input [128][144]
// shared memory and launch shape of the kernel with NS slots: the slots' layer inputs
// (the features of layer 1 in the first 16 columns), the image, the mbarriers and the
// TMEM address; 4 warps per slot
template <int NS>
struct TcShape {
    static constexpr int W = NS * kTcABytes;
    static constexpr int Bar = W + kTcImage;
    static constexpr size_t Smem = Bar + 128 + 1024;   // + room to align the base to 1024 B
    static constexpr int Threads = 4 * NS * 32;
    static constexpr unsigned TmemCols = 128 * NS <= 256 ? 256u : 512u;   // a power of 2
    static_assert(kTcImage % 16 == 0 && W % 16 == 0 && Bar % 8 == 0, "bulk copy and mbarrier alignment");
    static_assert(Smem <= 227 * 1024 && 128 * NS <= 512, "shared memory and TMEM of one CTA");
};

__device__ unsigned g_mlp_tc_timeout;   // set when an MMA completion wait ran out
// polls of the inference kernel's MMA completion waits (mps_mlp_debug_wait_spins)
constexpr long long kMlpWaitSpins = 1ll << 22;
__device__ long long g_mlp_tc_wait_spins = kMlpWaitSpins;

// canonical K-major offset (bytes) of element (r, k) of an operand with K columns
__device__ __forceinline__ int tc_off(int r, int k, int K) {
    return (r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}
// shared-memory matrix descriptor: start address, leading (K) and stride (8-row)
// byte offsets, fixed version bits 46..48 = 0b001, no swizzle
__device__ __forceinline__ unsigned long long tc_desc(unsigned saddr, unsigned lbo, unsigned sbo) {
    return (unsigned long long)((saddr & 0x3FFFFu) >> 4) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
           ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: FP32 D, BF16 A and B, both K-major, N, M
__host__ __device__ constexpr unsigned tc_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}
// FP16 A and B (format 0), D FP32 (f32acc) or FP16
__host__ __device__ constexpr unsigned tc_idesc_f16(int M, int N, bool f32acc) {
    return (f32acc ? (1u << 4) : 0u) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}
__device__ __forceinline__ unsigned tc_smem(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void tc_mma(unsigned tmem_d, unsigned long long a, unsigned long long b, unsigned idesc,
                                       int accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void tc_commit(unsigned long long* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(bar))
                 : "memory");
}
__device__ __forceinline__ bool tc_bar_test(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(tc_smem(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool tc_bar_wait(unsigned long long* bar, unsigned parity, long long spins) {
    for (long long k = 0; k < spins; ++k)
        if (tc_bar_test(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy writes of shared memory -> visible to the tensor cores (async proxy)
__device__ __forceinline__ void tc_fence_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// 32 consecutive TMEM columns of this thread's lane
__device__ __forceinline__ void tc_ld32(unsigned taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_ld2(unsigned taddr, uint32_t& a, uint32_t& b) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];" : "=r"(a), "=r"(b) : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_ld16(unsigned taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---------------------------------------------------------------------------
// BF16 GEMM on the 5th-generation tensor cores, the training path of the MLP:
// C[M x N] (+)= op(A)[M x K] op(B)[K x N], FP32 accumulate, with the epilogue of
// k_gemm_bf16 (bias, FP32 pre-activation Cz, SiLU, FP32 C with beta, BF16 Cb;
// split-K CTAs add into C with FP32 atomics).  A CTA of 4 warps owns a 128 x BN tile
// (BN = 16..64, a multiple of 16) whose accumulator lives in TMEM (128 lanes x BN
// FP32 columns).  K advances 64 at a time through two shared-memory stages holding
// the A tile [128][64] and the B^T tile [BN][64] in the canonical K-major layout
// without swizzle (tc_off); every thread loads one row of each (rows of A and of B^T
// that are K-contiguous in memory as 16-byte vectors, transposed operands element by
// element, coalesced across the warp), zero-filling outside the matrix.  One thread
// issues the four tcgen05.mma (M = 128, N = BN, K = 16 each) of a stage and commits
// them to the stage's mbarrier; a stage is refilled only after its MMAs completed
// (bounded wait).  The epilogue reads each warp's 32 TMEM lanes (= rows) with
// tcgen05.ld.  Bounded waits that run out set g_mlp_tc_timeout, wait (bounded) for
// the MMAs in flight and skip the epilogue.
// ---------------------------------------------------------------------------
// BN at most 64: twice the CTAs of 128-column tiles on the MLP's 128-wide layers (the
// training GEMMs are small, so their time is latency, not tensor throughput)
constexpr int kGtBM = 128, kGtBK = 64, kGtMaxBN = 64, kGtThreads = 128;
constexpr int kGtStageA = kGtBM * kGtBK * 2;                 // 16 KB
constexpr int kGtStageB = kGtMaxBN * kGtBK * 2;              // 8 KB
constexpr int kGtStage = kGtStageA + kGtStageB;
constexpr size_t kGtSmem = 2 * kGtStage + 64 + 1024;         // 2 stages, barriers, TMEM slot, alignment

// A tile [R][64 k] (K-major, canonical) of a matrix whose rows r0.. (`rows` in all)
// are K-contiguous in memory (trans = 0: X[row*ld + k]) or row-contiguous (trans = 1:
// X[k*ld + row]); zero outside the matrix and beyond kend.  The CTA's threads take
// 16-byte pieces: K-contiguous rows as 8 lanes per 128-byte row piece (coalesced),
// transposed ones as 8 consecutive rows at one k (coalesced along the rows) written to
// the 8 rows' K-major slots; pieces that leave the matrix or are misaligned go element
// by element.
template <int R>
__device__ __forceinline__ void gt_load_tile(unsigned char* tile, const bf16* __restrict__ X, int ld, int trans, int r0,
                                             int rows, int k0, int kend) {
    const bf16 zero = __float2bfloat16(0.f);
    auto elem = [&](int row, int k) -> bf16 {
        return (row < rows && k < kend) ? (trans ? X[(size_t)k * ld + row] : X[(size_t)row * ld + k]) : zero;
    };
    constexpr int kPieces = R * kGtBK / 8;   // 16-byte pieces of the tile
#pragma unroll 1
    for (int pc = threadIdx.x; pc < kPieces; pc += kGtThreads) {
        if (!trans) {
            const int r = pc >> 3, c = pc & 7;   // row r, k chunk c of 8
            const int row = r0 + r, kb = k0 + 8 * c;
            uint4 o = make_uint4(0u, 0u, 0u, 0u);
            if (row < rows && kb < kend) {
                const bf16* src = X + (size_t)row * ld + kb;
                if (kb + 8 <= kend && (((uintptr_t)src) & 15u) == 0) {
                    o = *reinterpret_cast<const uint4*>(src);
                } else {
                    uint32_t w[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        w[q] = (uint32_t)__bfloat16_as_ushort(elem(row, kb + 2 * q)) |
                               ((uint32_t)__bfloat16_as_ushort(elem(row, kb + 2 * q + 1)) << 16);
                    o = make_uint4(w[0], w[1], w[2], w[3]);
                }
            }
            *reinterpret_cast<uint4*>(tile + tc_off(r, 8 * c, kGtBK)) = o;
        } else {
            const int k = pc / (R / 8), g = pc % (R / 8);   // k, group of 8 rows
            const int row = r0 + 8 * g, kk = k0 + k;
            uint16_t v[8];
            const bf16* src = X + (size_t)kk * ld + row;
            if (kk < kend && row + 8 <= rows && (((uintptr_t)src) & 15u) == 0) {
                const uint4 o = *reinterpret_cast<const uint4*>(src);
                v[0] = (uint16_t)(o.x & 0xFFFFu); v[1] = (uint16_t)(o.x >> 16);
                v[2] = (uint16_t)(o.y & 0xFFFFu); v[3] = (uint16_t)(o.y >> 16);
                v[4] = (uint16_t)(o.z & 0xFFFFu); v[5] = (uint16_t)(o.z >> 16);
                v[6] = (uint16_t)(o.w & 0xFFFFu); v[7] = (uint16_t)(o.w >> 16);
            } else {
#pragma unroll
                for (int q = 0; q < 8; ++q) v[q] = __bfloat16_as_ushort(elem(row + q, kk));
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) *reinterpret_cast<uint16_t*>(tile + tc_off(8 * g + q, k, kGtBK)) = v[q];
        }
    }
}

__global__ void __launch_bounds__(kGtThreads) k_gemm_tc(int M, int N, int K, const bf16* __restrict__ A, int lda, int ta,
                                                        const bf16* __restrict__ B, int ldb, int tb, float* C, int ldc,
                                                        bf16* Cb, int ldcb, float* Cz, const float* __restrict__ bias,
                                                        int act, float beta, int kchunk, int BN) {
    extern __shared__ unsigned char gt_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)gt_raw + 1023) & ~(uintptr_t)1023);
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(sm + 2 * kGtStage);   // [2]
    unsigned* tmem_slot = reinterpret_cast<unsigned*>(sm + 2 * kGtStage + 16);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.y * kGtBM, n0 = blockIdx.x * BN;
    const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
    const unsigned cols = BN <= 32 ? 32u : (BN <= 64 ? 64u : 128u);   // TMEM columns: a power of 2 >= 32
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(bar)) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(bar + 1)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        __syncwarp();
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tmem_slot)),
                     "r"(cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tmem_slot;
    const unsigned idesc = tc_idesc(kGtBM, BN);
    const int nk = kend > kbeg ? (kend - kbeg + kGtBK - 1) / kGtBK : 0;
    unsigned phases = 0u;   // bit s: parity of the next completion of stage s's barrier
    bool timed_out = false;
    for (int kt = 0; kt < nk; ++kt) {
        const int s = kt & 1;
        unsigned char* As = sm + s * kGtStage;
        unsigned char* Bs = As + kGtStageA;
        if (kt >= 2) {   // the MMAs that read this stage two tiles ago are done
            const bool ok = tc_bar_wait(bar + s, (phases >> s) & 1u, 1ll << 22);
            if (__syncthreads_or(!ok)) {
                if (tid == 0) atomicOr(&g_mlp_tc_timeout, 1u);
                tc_bar_wait(bar + s, (phases >> s) & 1u, 1ll << 24);
                tc_bar_wait(bar + (s ^ 1), (phases >> (s ^ 1)) & 1u, 1ll << 24);
                timed_out = true;
                break;
            }
            phases ^= 1u << s;
        }
        const int k0 = kbeg + kt * kGtBK;
        gt_load_tile<kGtBM>(As, A, lda, ta, m0, M, k0, kend);
        // B^T tile: rows are the n of op(B); B[k*ldb + n] (transB = 0) is row-contiguous
        switch (BN) {
            case 16: gt_load_tile<16>(Bs, B, ldb, tb ? 0 : 1, n0, N, k0, kend); break;
            case 32: gt_load_tile<32>(Bs, B, ldb, tb ? 0 : 1, n0, N, k0, kend); break;
            case 48: gt_load_tile<48>(Bs, B, ldb, tb ? 0 : 1, n0, N, k0, kend); break;
            case 64: gt_load_tile<64>(Bs, B, ldb, tb ? 0 : 1, n0, N, k0, kend); break;
            case 80: gt_load_tile<80>(Bs, B, ldb, tb ? 0 : 1, n0, N, k0, kend); break;
            case 96: gt_load_tile<96>(Bs, B, ldb, tb ? 0 : 1, n0, N, k0, kend); break;
            case 112: gt_load_tile<112>(Bs, B, ldb, tb ? 0 : 1, n0, N, k0, kend); break;
            default: gt_load_tile<128>(Bs, B, ldb, tb ? 0 : 1, n0, N, k0, kend); break;
        }
        tc_fence_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const unsigned aa = tc_smem(As), ba = tc_smem(Bs);
#pragma unroll
            for (int q = 0; q < kGtBK / 16; ++q)
                tc_mma(tmem, tc_desc(aa + 256 * q, 128, 1024), tc_desc(ba + 256 * q, 128, 1024), idesc,
                       (kt > 0 || q > 0) ? 1 : 0);
            tc_commit(bar + s);
        }
    }
    // all MMAs done: the last stage's commit tracks every earlier MMA of this thread
    if (!timed_out && nk > 0) {
        const int s = (nk - 1) & 1;
        const bool ok = tc_bar_wait(bar + s, (phases >> s) & 1u, 1ll << 22);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(&g_mlp_tc_timeout, 1u);
            tc_bar_wait(bar + s, (phases >> s) & 1u, 1ll << 24);
            timed_out = true;
        }
    }
    tc_fence_after();
    __syncwarp();
    if (!timed_out) {
        // each warp's 32 rows x 16 columns go through a padded shared-memory block (the
        // stage buffers are free now) so that a store instruction writes two 16-column
        // row pieces (64 B each) instead of 32 rows one column apart
        const bool split = gridDim.z > 1;
        const int lane = tid & 31;
        float* blk = reinterpret_cast<float*>(sm) + warp * 32 * 17;
        const unsigned trow = tmem + ((unsigned)(32 * warp) << 16);
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            uint32_t v[16];
            if (nk > 0) tc_ld16(trow + c0, v);
            else
#pragma unroll
                for (int q = 0; q < 16; ++q) v[q] = 0u;
#pragma unroll
            for (int q = 0; q < 16; ++q) blk[lane * 17 + q] = __uint_as_float(v[q]);
            __syncwarp();
            const int cq = lane & 15, col = n0 + c0 + cq;
#pragma unroll 4
            for (int rr = lane >> 4; rr < 32; rr += 2) {
                const int row = m0 + 32 * warp + rr;
                if (row >= M || col >= N) continue;
                float x = blk[rr * 17 + cq];
                if (split) {
                    atomicAdd(C + (size_t)row * ldc + col, x);
                    continue;
                }
                if (bias) x += bias[col];
                if (Cz) Cz[(size_t)row * ldc + col] = x;
                if (act == 1) x = silu(x);
                if (C) C[(size_t)row * ldc + col] = beta != 0.f ? beta * C[(size_t)row * ldc + col] + x : x;
                if (Cb) Cb[(size_t)row * ldcb + col] = __float2bfloat16(x);
            }
            __syncwarp();
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols) : "memory");
    }
}

// the training GEMM on tcgen05 (variant 0): BN = N rounded up to 16, at most 64
cudaError_t gemm(int M, int N, int K, const bf16* A, int lda, int ta, const bf16* B, int ldb, int tb, float* C, int ldc,
                 bf16* Cb, int ldcb, float* Cz, const float* bias, int act, float beta, int split, cudaStream_t st) {
    if (M <= 0 || N <= 0 || K <= 0) return cudaErrorInvalidValue;
    static bool smem_set = false;
    if (!smem_set) {
        const cudaError_t e = cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGtSmem);
        if (e) return e;
        smem_set = true;
    }
    split = max(1, split);
    int kchunk = (K + split - 1) / split;
    kchunk = (kchunk + kGtBK - 1) / kGtBK * kGtBK;
    split = (K + kchunk - 1) / kchunk;
    const int BN = std::min(kGtMaxBN, (N + 15) / 16 * 16);
    dim3 grid(div_up(N, BN), div_up(M, kGtBM), split);
    MPS_COUNT_LAUNCH k_gemm_tc<<<grid, kGtThreads, kGtSmem, st>>>(M, N, K, A, lda, ta, B, ldb, tb, C, ldc, Cb, ldcb, Cz,
                                                                  bias, act, beta, kchunk, BN);
    return cudaGetLastError();
}

// the shared-memory image of the tcgen05 inference (W^T in the canonical layout, FP16,
// the biases as high and low FP16 parts in the ones columns), built from the FP32
// parameters once per update so every CTA stages it with one bulk copy
__device__ __forceinline__ void put_f16(unsigned char* img, int off, float v) {
    *reinterpret_cast<__half*>(img + off) = __float2half_rn(v);
}
__device__ __forceinline__ void put_bias_f16(unsigned char* img, int off_hi, int off_lo, float b) {
    const __half hi = __float2half_rn(b);
    *reinterpret_cast<__half*>(img + off_hi) = hi;
    *reinterpret_cast<__half*>(img + off_lo) = __float2half_rn(b - __half2float(hi));
}
__global__ void k_layers_to_tc(const float* __restrict__ p, Layers L) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int o1 = FIN * H, o2 = o1 + H, o3 = o2 + H * H, o4 = o3 + H, o5 = o4 + H * H, o6 = o5 + H, o7 = o6 + H * FOUT;
    unsigned char* img = L.tc;
    if (e < FINP * H) {   // W1^T [n][k]
        const int n = e / FINP, k = e % FINP;
        const int off = kImW1 + tc_off(n, k, FINP);
        if (k < FIN) put_f16(img, off, 0.5f * p[k * H + n]);
        else if (k == FIN) put_bias_f16(img, off, kImW1 + tc_off(n, k + 1, FINP), 0.5f * p[o1 + n]);
        else if (k > FIN + 1) put_f16(img, off, 0.f);
    }
    if (e < kTcK * H) {   // W2^T, W3^T [n][k]
        const int n = e / kTcK, k = e % kTcK;
        const int off2 = kImW2 + tc_off(n, k, kTcK), off3 = kImW3 + tc_off(n, k, kTcK);
        if (k < H) {
            put_f16(img, off2, 0.5f * p[o2 + k * H + n]);
            put_f16(img, off3, 0.5f * p[o4 + k * H + n]);
        } else if (k == H) {
            put_bias_f16(img, off2, kImW2 + tc_off(n, k + 1, kTcK), 0.5f * p[o3 + n]);
            put_bias_f16(img, off3, kImW3 + tc_off(n, k + 1, kTcK), 0.5f * p[o5 + n]);
        } else if (k > H + 1) {
            put_f16(img, off2, 0.f);
            put_f16(img, off3, 0.f);
        }
    }
    if (e < kTcK * FOUTP) {   // W4^T [n][k], outputs n >= 2 zero
        const int n = e / kTcK, k = e % kTcK;
        const int off = kImW4 + tc_off(n, k, kTcK);
        if (n >= FOUT) put_f16(img, off, 0.f);
        else if (k < H) put_f16(img, off, p[o6 + k * FOUT + n]);
        else if (k == H) put_bias_f16(img, off, kImW4 + tc_off(n, k + 1, kTcK), p[o7 + n]);
        else if (k > H + 1) put_f16(img, off, 0.f);
    }
}

// SiLU of two FP16 pre-activations given as h = z / 2: h (1 + tanh h) with
// tanh.approx.f16x2 and one FP16x2 multiply-add
__device__ __forceinline__ uint32_t silu2_f16(uint32_t h) {
    uint32_t t;
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(h));
    asm("fma.rn.f16x2 %0, %1, %2, %1;" : "=r"(t) : "r"(h), "r"(t));
    return t;
}

// 64 consecutive FP16 TMEM columns of this thread's lane, two per register, without
// waiting (tcgen05.wait::ld before the registers are read)
__device__ __forceinline__ void tc_ld32_pack16_nowait(unsigned taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.pack::16b.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
        "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
}
// The same SiLU on the FMA pipe, for a share of the columns while the SFU runs the
// others: tanh |h| from a degree-8 polynomial in v = min(|h|, 4.5) - 2.25, the
// least-squares fit of tanh on [0, 4.5] at 4000 Chebyshev nodes, coefficients rounded to
// FP16 and evaluated by FP16x2 Horner (|error| <= 1.9e-3 over every FP16 input; tanh
// 4.5 rounds to 1 in FP16); the sign bits of h give tanh h, then h + h tanh h.  SiLU
// error <= 3.6e-3 absolute, 2.3e-3 relative beyond 1 (an exactly rounded FP16 tanh:
// 2.9e-3 / 1.1e-3).  Eleven FP16x2 instructions on the FMA pipe and two logic ops.
__device__ __forceinline__ uint32_t hfma2(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t d;
    asm("fma.rn.f16x2 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}
__device__ __forceinline__ uint32_t silu2_f16_poly(uint32_t h) {
    uint32_t a = h & 0x7FFF7FFFu, v;
    asm("min.f16x2 %0, %1, %2;" : "=r"(a) : "r"(a), "r"(0x44804480u));   // 4.5
    asm("add.f16x2 %0, %1, %2;" : "=r"(v) : "r"(a), "r"(0xC080C080u));   // -2.25
    uint32_t t = hfma2(0x09230923u, v, 0x91A791A7u);
    t = hfma2(t, v, 0x855C855Cu);
    t = hfma2(t, v, 0x1D6F1D6Fu);
    t = hfma2(t, v, 0xA33BA33Bu);
    t = hfma2(t, v, 0x26AD26ADu);
    t = hfma2(t, v, 0xA944A944u);
    t = hfma2(t, v, 0x29962996u);
    t = hfma2(t, v, 0x3BD33BD3u);
    t ^= h & 0x80008000u;   // tanh(-a) = -tanh(a)
    return hfma2(h, t, h);
}
// pair u (0..3) of every group of four on the FMA pipe when bit u of POLY is set
template <int POLY>
__device__ __forceinline__ uint32_t silu2_mixed(uint32_t h, int u) {
    return (POLY >> u) & 1 ? silu2_f16_poly(h) : silu2_f16(h);
}

// hidden-layer epilogue: this thread's row of the 128 FP16 accumulator columns (both
// halves loaded before one wait), SiLU -> FP16 A operand of the next layer (row r,
// canonical K-major, K = 144)
template <int POLY>
__device__ __forceinline__ void tc_epilogue_hidden(unsigned tmem_row, unsigned char* __restrict__ A, int r) {
    uint32_t v[2][32];
    tc_ld32_pack16_nowait(tmem_row, v[0]);
    tc_ld32_pack16_nowait(tmem_row + 64, v[1]);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int c = 0; c < 2; ++c) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const uint4 o = make_uint4(silu2_mixed<POLY>(v[c][4 * q], 0), silu2_mixed<POLY>(v[c][4 * q + 1], 1),
                                       silu2_mixed<POLY>(v[c][4 * q + 2], 2), silu2_mixed<POLY>(v[c][4 * q + 3], 3));
            *reinterpret_cast<uint4*>(A + tc_off(r, 64 * c + 8 * q, kTcK)) = o;
        }
    }
}
// two features -> FP16 pair (saturating: the input stays finite)
__device__ __forceinline__ uint32_t pack_f16(float lo, float hi) {
    uint32_t h;
    asm("cvt.rn.satfinite.f16x2.f32 %0, %1, %2;" : "=r"(h) : "f"(hi), "f"(lo));
    return h;
}

// the 128 threads of a slot: a named barrier (ids 1.. ; 0 is __syncthreads) and the
// same with an OR over a predicate
__device__ __forceinline__ void slot_sync(int id) { asm volatile("barrier.cta.sync %0, 128;" ::"r"(id) : "memory"); }
__device__ __forceinline__ bool slot_any(int id, bool v) {
    unsigned r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n barrier.cta.red.or.pred p, %2, 128, q;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"((unsigned)v), "r"(id)
        : "memory");
    return r != 0;
}

template <int NS, int POLY>
__global__ void __launch_bounds__(TcShape<NS>::Threads, 1) k_mlp_infer_tc(int M, const float* __restrict__ X,
                                                                          float* __restrict__ Y, Layers L,
                                                                          unsigned* err) {
    using S = TcShape<NS>;
    extern __shared__ unsigned char tc_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)tc_raw + 1023) & ~(uintptr_t)1023);
    unsigned long long* mma_done = reinterpret_cast<unsigned long long*>(sm + S::Bar);   // [NS]
    unsigned long long* drain = mma_done + NS;                                          // [NS]
    unsigned long long* wbar = mma_done + 2 * NS;
    unsigned* tmem_slot = reinterpret_cast<unsigned*>(sm + S::Bar + 8 * (2 * NS + 1));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < NS; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(mma_done + s)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(drain + s)) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(wbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // the weight image: one bulk copy (16-byte aligned, a multiple of 16 bytes),
        // completed on wbar
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc_smem(wbar)),
                     "r"((unsigned)kTcImage)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(tc_smem(sm + S::W)), "l"(L.tc), "r"((unsigned)kTcImage), "r"(tc_smem(wbar))
                     : "memory");
    }
    if (warp == 0) {
        __syncwarp();   // .aligned: the whole warp, converged (thread 0 just left its branch)
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tmem_slot)),
                     "r"(S::TmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    __syncthreads();   // barriers initialised before anyone polls them
    bool failed = !tc_bar_wait(wbar, 0, 1ll << 22);
    if (__syncthreads_or(failed)) {
        if (tid == 0) {
            atomicOr(&g_mlp_tc_timeout, 1u);
            if (err) atomicOr(err, MPS_ERR_STAGE_TIMEOUT);
        }
        tc_bar_wait(wbar, 0, 1ll << 24);   // the copy may still land: wait (bounded) for it
        failed = true;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tmem_slot;
    const int tiles = (M + kTcRows - 1) / kTcRows;
    const int stride = NS * gridDim.x;   // tiles t = NS * blockIdx.x + s + k * stride
    constexpr unsigned sbo = kTcK / 8 * 128;   // 8-row group stride of the [128][144] operands

    const int s = warp >> 2, r = 32 * (warp & 3) + lane, bar_id = 1 + s;
    const bool leader = r == 0;   // issues the slot's MMAs
    const unsigned tslot = tmem + 128u * (unsigned)s;
    const unsigned trow = tslot + ((unsigned)(32 * (warp & 3)) << 16);
    unsigned char* As = sm + s * kTcABytes;
    const unsigned aa = tc_smem(As);
    // hidden layers accumulate in FP16, the output layer in FP32
    const unsigned id128 = tc_idesc_f16(128, 128, false), id16 = tc_idesc_f16(128, 16, true);
    auto issue = [&](int layer) {   // by the leader, after the slot's barrier
        tc_fence_after();
        if (layer == 0) {
            tc_mma(tslot, tc_desc(aa, 128, sbo), tc_desc(tc_smem(sm + S::W + kImW1), 128, 256), id128, 0);
        } else {
            const unsigned wa = tc_smem(sm + S::W + (layer == 1 ? kImW2 : layer == 2 ? kImW3 : kImW4));
            const unsigned idesc = layer == 3 ? id16 : id128;
#pragma unroll
            for (int k = 0; k < kTcK / 16; ++k)
                tc_mma(tslot, tc_desc(aa + 256 * k, 128, sbo), tc_desc(wa + 256 * k, 128, sbo), idesc, k > 0);
        }
        tc_commit(mma_done + s);
    };
    // the ones columns of the hidden inputs (written once)
    *reinterpret_cast<uint4*>(As + tc_off(r, H, kTcK)) = make_uint4(0x3C003C00u, 0u, 0u, 0u);
    *reinterpret_cast<uint4*>(As + tc_off(r, H + 8, kTcK)) = make_uint4(0u, 0u, 0u, 0u);
    unsigned ph = 0u;   // parity of the next phase of mma_done[s]
    auto load_row = [&](int t, float4 (&x)[3]) {
        const int row = t * kTcRows + r;
        if (t < tiles && row < M) {
            const float4* xr = reinterpret_cast<const float4*>(X + (size_t)row * FIN);
#pragma unroll
            for (int q = 0; q < 3; ++q) x[q] = xr[q];
        } else {
#pragma unroll
            for (int q = 0; q < 3; ++q) x[q] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    float4 xn[3];
    int t = NS * blockIdx.x + s;
    load_row(t, xn);
    // a wait of this warp ran out: the slot stops at its next barrier (the barriers
    // carry the OR of the flag, so every warp of the slot stops there)
    bool bad = failed;
    bool stop = false;   // uniform over the slot: taken from a barrier's OR
    for (; t < tiles && !stop; t += stride) {
        const int row = t * kTcRows + r;
        // layer-1 input in the first 16 columns: 12 features (FP16), two ones, two zeros
        {
            uint4 o0, o1;
            o0.x = pack_f16(xn[0].x, xn[0].y);
            o0.y = pack_f16(xn[0].z, xn[0].w);
            o0.z = pack_f16(xn[1].x, xn[1].y);
            o0.w = pack_f16(xn[1].z, xn[1].w);
            o1.x = pack_f16(xn[2].x, xn[2].y);
            o1.y = pack_f16(xn[2].z, xn[2].w);
            o1.z = 0x3C003C00u;
            o1.w = 0u;
            load_row(t + stride, xn);
            *reinterpret_cast<uint4*>(As + tc_off(r, 0, kTcK)) = o0;
            *reinterpret_cast<uint4*>(As + tc_off(r, 8, kTcK)) = o1;
        }
        tc_fence_smem();
        tc_fence_before();
        if ((stop = slot_any(bar_id, bad))) break;
        if (leader) issue(0);
        for (int layer = 0; layer < 4; ++layer) {
            const bool ok = __all_sync(0xffffffffu, tc_bar_wait(mma_done + s, ph, g_mlp_tc_wait_spins));
            if (!ok) {
                if (lane == 0) {
                    atomicOr(&g_mlp_tc_timeout, 1u);
                    if (err) atomicOr(err, MPS_ERR_STAGE_TIMEOUT);
                }
                bad = true;
            } else {
                ph ^= 1u;
                tc_fence_after();
                if (layer < 3) {
                    tc_epilogue_hidden<POLY>(trow, As, r);
                } else {
                    uint32_t y0, y1;
                    tc_ld2(trow, y0, y1);
                    if (row < M)
                        *reinterpret_cast<float2*>(Y + (size_t)row * FOUT) =
                            make_float2(__uint_as_float(y0), __uint_as_float(y1));
                }
            }
            tc_fence_smem();
            tc_fence_before();   // the next MMAs overwrite the accumulator these warps read
            if (layer < 3) {
                if ((stop = slot_any(bar_id, bad))) break;
                if (leader) issue(layer + 1);
            }
        }
    }
    if (leader) {
        // every MMA this thread issued has completed before TMEM is freed
        tc_commit(drain + s);
        tc_bar_wait(drain + s, 0, 1ll << 26);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(S::TmemCols) : "memory");
    }
}

// dY = d loss / d y for loss = mean((y0 - t0)^2 + w1 (y1 - t1)^2); loss partial sums
__global__ void k_loss_grad(int M, const float* __restrict__ Yp, const float* __restrict__ T, float w1,
                            bf16* __restrict__ dYb, float* __restrict__ dY, double* __restrict__ loss) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (i < M) {
        const float e0 = Yp[(size_t)i * FOUTP] - T[2 * (size_t)i];
        const float e1 = Yp[(size_t)i * FOUTP + 1] - T[2 * (size_t)i + 1];
        l = (double)e0 * e0 + (double)w1 * e1 * e1;
        const float s = 2.0f / (float)M;
        for (int c = 0; c < FOUTP; ++c) {
            const float gv = c == 0 ? s * e0 : (c == 1 ? s * w1 * e1 : 0.f);
            dY[(size_t)i * FOUTP + c] = gv;
            dYb[(size_t)i * FOUTP + c] = __float2bfloat16(gv);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}
__global__ void k_silu_back(int n, const float* __restrict__ dH, const float* __restrict__ Z, float* __restrict__ dZ,
                            bf16* __restrict__ dZb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = dH[i] * silu_grad(Z[i]);
    dZ[i] = v;
    dZb[i] = __float2bfloat16(v);
}
// column sums (bias gradients), FP32 -> out[c]
__global__ void k_colsum(int M, int N, const float* __restrict__ A, float* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    float s = 0.f;
    for (int r = 0; r < M; ++r) s += A[(size_t)r * N + c];
    out[c] = s;
}
// gradient buffers (padded layer shapes) -> parameter-vector layout
__global__ void k_grad_to_vec(const float* __restrict__ dW1, const float* __restrict__ db1, const float* __restrict__ dW2,
                              const float* __restrict__ db2, const float* __restrict__ dW3, const float* __restrict__ db3,
                              const float* __restrict__ dW4, const float* __restrict__ db4, float* __restrict__ g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int o1 = FIN * H, o2 = o1 + H, o3 = o2 + H * H, o4 = o3 + H, o5 = o4 + H * H, o6 = o5 + H, o7 = o6 + H * FOUT;
    if (i < FIN * H) g[i] = dW1[i];
    if (i < H) {
        g[o1 + i] = db1[i];
        g[o3 + i] = db2[i];
        g[o5 + i] = db3[i];
    }
    if (i < H * H) {
        g[o2 + i] = dW2[i];
        g[o4 + i] = dW3[i];
    }
    if (i < H * FOUT) g[o6 + i] = dW4[(i / FOUT) * FOUTP + (i % FOUT)];
    if (i < FOUT) g[o7 + i] = db4[i];
}
__global__ void k_adam(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1t, float b2t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = 0.9f * m[i] + 0.1f * gi;
    const float vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.f - b1t), vh = vi / (1.f - b2t);
    p[i] -= lr * mh / (sqrtf(vh) + 1e-8f);
}

}  // namespace mps

using namespace mps;

struct MpsMlp {
    int maxb = 0;
    int nparams = MPS_MLP_PARAMS;
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    Layers L{};
    bf16 *Xb = nullptr, *H1 = nullptr, *H2 = nullptr, *H3 = nullptr, *dYb = nullptr, *dZb = nullptr;
    float *Z1 = nullptr, *Z2 = nullptr, *Z3 = nullptr, *Yp = nullptr, *dY = nullptr, *dH = nullptr, *dZ = nullptr;
    float *dW1 = nullptr, *dW2 = nullptr, *dW3 = nullptr, *dW4 = nullptr, *db = nullptr;
    double* loss = nullptr;
    double* h_loss = nullptr;
    int t = 0;
    std::vector<void*> allocs;

    template <class T>
    cudaError_t mk(T** ptr, size_t count) {
        cudaError_t e = cudaMalloc((void**)ptr, sizeof(T) * (count ? count : 1));
        if (e == cudaSuccess) allocs.push_back(*ptr);
        return e;
    }
    cudaError_t init(int b) {
        maxb = (b + 63) / 64 * 64;
        const size_t B = maxb;
        cudaError_t e = cudaSuccess;
        e = e ? e : mk(&p, nparams); e = e ? e : mk(&g, nparams); e = e ? e : mk(&m, nparams); e = e ? e : mk(&v, nparams);
        e = e ? e : mk(&L.W1, FINP * H); e = e ? e : mk(&L.W2, H * H); e = e ? e : mk(&L.W3, H * H);
        e = e ? e : mk(&L.W4, H * FOUTP);
        e = e ? e : mk(&L.b1, H); e = e ? e : mk(&L.b2, H); e = e ? e : mk(&L.b3, H); e = e ? e : mk(&L.b4, FOUTP);
        e = e ? e : mk(&L.tc, (size_t)kTcImage);
        e = e ? e : mk(&Xb, B * FINP); e = e ? e : mk(&H1, B * H); e = e ? e : mk(&H2, B * H); e = e ? e : mk(&H3, B * H);
        e = e ? e : mk(&Z1, B * H); e = e ? e : mk(&Z2, B * H); e = e ? e : mk(&Z3, B * H);
        e = e ? e : mk(&Yp, B * FOUTP); e = e ? e : mk(&dY, B * FOUTP); e = e ? e : mk(&dYb, B * FOUTP);
        e = e ? e : mk(&dH, B * H); e = e ? e : mk(&dZ, B * H); e = e ? e : mk(&dZb, B * H);
        e = e ? e : mk(&dW1, FINP * H); e = e ? e : mk(&dW2, H * H); e = e ? e : mk(&dW3, H * H);
        e = e ? e : mk(&dW4, H * FOUTP); e = e ? e : mk(&db, 4 * H);
        e = e ? e : mk(&loss, 1);
        if (e) return e;
        if ((e = cudaMallocHost((void**)&h_loss, sizeof(double)))) return e;
        cudaMemset(m, 0, sizeof(float) * nparams);
        cudaMemset(v, 0, sizeof(float) * nparams);
        return cudaDeviceSynchronize();
    }
    void release() {
        cudaDeviceSynchronize();
        for (void* a : allocs) cudaFree(a);
        allocs.clear();
        if (h_loss) cudaFreeHost(h_loss);
        h_loss = nullptr;
    }
    cudaError_t sync_layers(cudaStream_t st) {
        MPS_COUNT_LAUNCH k_params_to_layers<<<div_up(H * H, 256), 256, 0, st>>>(p, L);
        MPS_COUNT_LAUNCH k_layers_to_tc<<<div_up(kTcK * H, 256), 256, 0, st>>>(p, L);
        return cudaGetLastError();
    }
    // forward over M rows (M <= maxb); keep pre-activations when train
    cudaError_t forward(int M, const float* X, cudaStream_t st, bool train) {
        MPS_COUNT_LAUNCH k_pack_input<<<div_up(M * FINP, 256), 256, 0, st>>>(M, X, Xb);
        cudaError_t e = gemm(M, H, FINP, Xb, FINP, 0, L.W1, H, 0, nullptr, H, H1, H, train ? Z1 : nullptr, L.b1, 1,
                             0.f, 1, st);
        if (!e) e = gemm(M, H, H, H1, H, 0, L.W2, H, 0, nullptr, H, H2, H, train ? Z2 : nullptr, L.b2, 1, 0.f, 1, st);
        if (!e) e = gemm(M, H, H, H2, H, 0, L.W3, H, 0, nullptr, H, H3, H, train ? Z3 : nullptr, L.b3, 1, 0.f, 1, st);
        if (!e) e = gemm(M, FOUTP, H, H3, H, 0, L.W4, FOUTP, 0, Yp, FOUTP, nullptr, 0, nullptr, L.b4, 0, 0.f, 1, st);
        return e;
    }
    cudaError_t backward(int M, const float* T, float w1, cudaStream_t st) {
        cudaError_t e = cudaSuccess;
#define MLP_STEP(label, call)                       \
    do {                                             \
        call;                                        \
        if ((e = cudaGetLastError())) {              \
            note_error(label, e);                    \
            return e;                                \
        }                                            \
    } while (0)
#define MLP_GEMM(label, ...)                         \
    do {                                             \
        if ((e = gemm(__VA_ARGS__))) {               \
            note_error(label, e);                    \
            return e;                                \
        }                                            \
    } while (0)
        MLP_STEP("loss reset", cudaMemsetAsync(loss, 0, sizeof(double), st));
        MLP_STEP("k_loss_grad", (MPS_COUNT_LAUNCH k_loss_grad<<<div_up(M, 256), 256, 0, st>>>(M, Yp, T, w1, dYb, dY, loss)));
        const int split = max(1, min(64, M / 512));
        MLP_STEP("grad reset", cudaMemsetAsync(dW4, 0, sizeof(float) * H * FOUTP, st));
        MLP_STEP("grad reset", cudaMemsetAsync(dW3, 0, sizeof(float) * H * H, st));
        MLP_STEP("grad reset", cudaMemsetAsync(dW2, 0, sizeof(float) * H * H, st));
        MLP_STEP("grad reset", cudaMemsetAsync(dW1, 0, sizeof(float) * FINP * H, st));
        const int Kb = M;   // batch as K; the tile loader zero-fills k >= K
        MLP_GEMM("dW4", H, FOUTP, Kb, H3, H, 1, dYb, FOUTP, 0, dW4, FOUTP, nullptr, 0, nullptr, nullptr, 0, 1.f, split, st);
        MLP_STEP("db4", (MPS_COUNT_LAUNCH k_colsum<<<1, 128, 0, st>>>(M, FOUTP, dY, db + 3 * H)));
        MLP_GEMM("dH3", M, H, FOUTP, dYb, FOUTP, 0, L.W4, FOUTP, 1, dH, H, nullptr, 0, nullptr, nullptr, 0, 0.f, 1, st);
        MLP_STEP("silu3", (MPS_COUNT_LAUNCH k_silu_back<<<div_up(M * H, 256), 256, 0, st>>>(M * H, dH, Z3, dZ, dZb)));
        MLP_GEMM("dW3", H, H, Kb, H2, H, 1, dZb, H, 0, dW3, H, nullptr, 0, nullptr, nullptr, 0, 1.f, split, st);
        MLP_STEP("db3", (MPS_COUNT_LAUNCH k_colsum<<<1, 128, 0, st>>>(M, H, dZ, db + 2 * H)));
        MLP_GEMM("dH2", M, H, H, dZb, H, 0, L.W3, H, 1, dH, H, nullptr, 0, nullptr, nullptr, 0, 0.f, 1, st);
        MLP_STEP("silu2", (MPS_COUNT_LAUNCH k_silu_back<<<div_up(M * H, 256), 256, 0, st>>>(M * H, dH, Z2, dZ, dZb)));
        MLP_GEMM("dW2", H, H, Kb, H1, H, 1, dZb, H, 0, dW2, H, nullptr, 0, nullptr, nullptr, 0, 1.f, split, st);
        MLP_STEP("db2", (MPS_COUNT_LAUNCH k_colsum<<<1, 128, 0, st>>>(M, H, dZ, db + 1 * H)));
        MLP_GEMM("dH1", M, H, H, dZb, H, 0, L.W2, H, 1, dH, H, nullptr, 0, nullptr, nullptr, 0, 0.f, 1, st);
        MLP_STEP("silu1", (MPS_COUNT_LAUNCH k_silu_back<<<div_up(M * H, 256), 256, 0, st>>>(M * H, dH, Z1, dZ, dZb)));
        MLP_GEMM("dW1", FINP, H, Kb, Xb, FINP, 1, dZb, H, 0, dW1, H, nullptr, 0, nullptr, nullptr, 0, 1.f, split, st);
        MLP_STEP("db1", (MPS_COUNT_LAUNCH k_colsum<<<1, 128, 0, st>>>(M, H, dZ, db)));
        MLP_STEP("grad vec", (MPS_COUNT_LAUNCH k_grad_to_vec<<<div_up(H * H, 256), 256, 0, st>>>(dW1, db, dW2, db + H, dW3, db + 2 * H,
                                                                                 dW4, db + 3 * H, g)));
#undef MLP_STEP
#undef MLP_GEMM
        return cudaSuccess;
    }
};

namespace mps {
// the tcgen05 inference kernel with POLY's columns on the FMA pipe
template <int POLY>
cudaError_t mlp_forward_tc(MpsMlp* m, int M, const float* X, float* Y, cudaStream_t st, unsigned* err, int sms) {
    static bool tc_set = false;   // the attribute is per function, set once
    if (!tc_set) {
        const cudaError_t e = cudaFuncSetAttribute(k_mlp_infer_tc<kTcSlots, POLY>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)TcShape<kTcSlots>::Smem);
        if (e) return e;
        tc_set = true;
    }
    const int tiles = (M + kTcRows - 1) / kTcRows;
    const int grid = std::max(1, std::min(div_up(tiles, kTcSlots), std::max(sms, 1)));   // one CTA per SM
    MPS_COUNT_LAUNCH k_mlp_infer_tc<kTcSlots, POLY>
        <<<grid, TcShape<kTcSlots>::Threads, TcShape<kTcSlots>::Smem, st>>>(M, X, Y, m->L, err);
    return cudaGetLastError();
}
// share of the SiLU pairs the solver's inference kernel runs on the FMA pipe (bit u:
// pair u of every four)
constexpr int kTcPolyDefault = 0x8;

// forward of a created MLP on M rows of features: variant 0 the tcgen05 kernel (the
// solver's), 1 the mma.sync kernel (kept as a cross-check of the former), 2..5 the
// tcgen05 kernel with 0, 1, 2, 3 of every 4 SiLU pairs on the FMA pipe (the rest on the
// SFU's tanh)
cudaError_t mlp_forward_variant(MpsMlp* m, int M, const float* X, float* Y, cudaStream_t st, int variant,
                                unsigned* err) {
    if (M <= 0) return cudaSuccess;
    static bool smem_set = false;   // the attribute is per function, set once
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    switch (variant) {
        case 0: return mlp_forward_tc<kTcPolyDefault>(m, M, X, Y, st, err, sms);
        case 2: return mlp_forward_tc<0x0>(m, M, X, Y, st, err, sms);
        case 3: return mlp_forward_tc<0x8>(m, M, X, Y, st, err, sms);
        case 4: return mlp_forward_tc<0xA>(m, M, X, Y, st, err, sms);
        case 5: return mlp_forward_tc<0xE>(m, M, X, Y, st, err, sms);
        default: break;
    }
    if (!smem_set) {
        const cudaError_t e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMiSmem);
        if (e) return e;
        smem_set = true;
    }
    const int tiles = (M + 15) / 16;
    const int grid = std::max(1, std::min(div_up(tiles, kMiWarps), 2 * std::max(sms, 1)));
    MPS_COUNT_LAUNCH k_mlp_infer<<<grid, kMiWarps * 32, kMiSmem, st>>>(M, X, Y, m->L);
    return cudaGetLastError();
}
// used by the solver (err: its error word)
cudaError_t mlp_forward(MpsMlp* m, int M, const float* X, float* Y, cudaStream_t st, unsigned* err) {
    return mlp_forward_variant(m, M, X, Y, st, 0, err);
}
}  // namespace mps

extern "C" {

CCTStatusType mps_gemm_bf16(int M, int N, int K, const void* A, int lda, int transA, const void* B, int ldb,
                            int transB, float* C, int ldc, void* Cb, int ldcb, float* Cz, const float* bias, int act,
                            float beta, int split_k, void* stream) {
    if (split_k > 1 && (act != 0 || beta != 1.f || !C)) return CCT_PARAMERR;
    cudaError_t e = gemm(M, N, K, (const bf16*)A, lda, transA, (const bf16*)B, ldb, transB, C, ldc, (bf16*)Cb, ldcb, Cz,
                         bias, act, beta, split_k, (cudaStream_t)stream);
    return e == cudaErrorInvalidValue ? CCT_PARAMERR : cuda_status(e);
}

CCTStatusType mps_gemm_bf16_variant(int M, int N, int K, const void* A, int lda, int transA, const void* B, int ldb,
                                    int transB, float* C, int ldc, void* Cb, int ldcb, float* Cz, const float* bias,
                                    int act, float beta, int split_k, int variant, void* stream) {
    if (variant < 0 || variant > 1) return CCT_PARAMERR;
    if (variant == 0)
        return mps_gemm_bf16(M, N, K, A, lda, transA, B, ldb, transB, C, ldc, Cb, ldcb, Cz, bias, act, beta, split_k,
                             stream);
    if (split_k > 1 && (act != 0 || beta != 1.f || !C)) return CCT_PARAMERR;
    cudaError_t e = gemm_mma_sync(M, N, K, (const bf16*)A, lda, transA, (const bf16*)B, ldb, transB, C, ldc, (bf16*)Cb,
                                  ldcb, Cz, bias, act, beta, split_k, (cudaStream_t)stream);
    return e == cudaErrorInvalidValue ? CCT_PARAMERR : cuda_status(e);
}

CCTStatusType mps_mlp_create(int max_batch, unsigned long long seed, MpsMlp** out) {
    if (max_batch <= 0 || !out) return CCT_PARAMERR;
    MpsMlp* m = new MpsMlp();
    if (m->init(max_batch) != cudaSuccess) {
        m->release();
        delete m;
        return CCT_MEMERR;
    }
    // PyTorch-Linear-style uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)), last layer x0.1
    std::vector<float> p(MPS_MLP_PARAMS);
    unsigned long long s = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto rnd = [&]() {
        s = s * 6364136223846793005ULL + 1442695040888963407ULL;
        return (float)((s >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
    };
    size_t o = 0;
    const int fan[4] = {FIN, H, H, H}, outs[4] = {H, H, H, FOUT};
    for (int l = 0; l < 4; ++l) {
        const float b = 1.f / sqrtf((float)fan[l]) * (l == 3 ? 0.1f : 1.f);
        for (int i = 0; i < fan[l] * outs[l]; ++i) p[o++] = b * rnd();
        for (int i = 0; i < outs[l]; ++i) p[o++] = b * rnd();
    }
    if (mps_mlp_set_params(m, p.data()) != CCT_NOERR) {
        m->release();
        delete m;
        return CCT_CUDAERR;
    }
    *out = m;
    return CCT_NOERR;
}

void mps_mlp_destroy(MpsMlp* m) {
    if (!m) return;
    m->release();
    delete m;
}

CCTStatusType mps_mlp_set_params(MpsMlp* m, const float* host_params) {
    if (!m || !host_params) return CCT_PARAMERR;
    cudaError_t e = cudaMemcpy(m->p, host_params, sizeof(float) * MPS_MLP_PARAMS, cudaMemcpyHostToDevice);
    if (!e) e = m->sync_layers(0);
    if (!e) e = cudaDeviceSynchronize();
    m->t = 0;
    cudaMemset(m->m, 0, sizeof(float) * MPS_MLP_PARAMS);
    cudaMemset(m->v, 0, sizeof(float) * MPS_MLP_PARAMS);
    return cuda_status(e);
}

CCTStatusType mps_mlp_get_params(MpsMlp* m, float* host_params) {
    if (!m || !host_params) return CCT_PARAMERR;
    return cuda_status(cudaMemcpy(host_params, m->p, sizeof(float) * MPS_MLP_PARAMS, cudaMemcpyDeviceToHost));
}

CCTStatusType mps_mlp_forward(MpsMlp* m, int M, const float* X, float* Y, void* stream) {
    if (!m || M < 0) return CCT_PARAMERR;
    if (M == 0) return CCT_NOERR;
    return cuda_status(mlp_forward(m, M, X, Y, (cudaStream_t)stream, nullptr));
}

CCTStatusType mps_mlp_forward_variant(MpsMlp* m, int M, const float* X, float* Y, int variant, void* stream) {
    if (!m || M < 0 || variant < 0 || variant > 5) return CCT_PARAMERR;
    if (M == 0) return CCT_NOERR;
    return cuda_status(mlp_forward_variant(m, M, X, Y, (cudaStream_t)stream, variant, nullptr));
}

CCTStatusType mps_mlp_tc_timeouts(unsigned* out) {
    if (!out) return CCT_PARAMERR;
    return cuda_status(cudaMemcpyFromSymbol(out, g_mlp_tc_timeout, sizeof(unsigned)));
}

CCTStatusType mps_mlp_debug_wait_spins(long long spins) {
    const long long v = spins < 0 ? kMlpWaitSpins : spins;
    const unsigned zero = 0;
    cudaError_t e = cudaDeviceSynchronize();
    if (!e) e = cudaMemcpyToSymbol(g_mlp_tc_wait_spins, &v, sizeof(v));
    if (!e) e = cudaMemcpyToSymbol(g_mlp_tc_timeout, &zero, sizeof(zero));
    return cuda_status(e);
}

CCTStatusType mps_mlp_loss_grad(MpsMlp* m, int M, const float* X, const float* T, float w1, float* grad,
                                float* host_loss, void* stream) {
    if (!m || M <= 0 || M > m->maxb) return CCT_PARAMERR;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaGetLastError();
    if (e) { note_error("mps_mlp_loss_grad: pending error on entry", e); return CCT_CUDAERR; }
    if ((e = m->forward(M, X, st, true))) { note_error("mlp forward", e); return CCT_CUDAERR; }
    if ((e = m->backward(M, T, w1, st))) return CCT_CUDAERR;   // backward names the failing launch
    if (grad && (e = cudaMemcpyAsync(grad, m->g, sizeof(float) * MPS_MLP_PARAMS, cudaMemcpyDeviceToDevice, st))) {
        char what[96];
        snprintf(what, sizeof(what), "gradient copy %p <- %p", (void*)grad, (void*)m->g);
        note_error(what, e);
        return CCT_CUDAERR;
    }
    if ((e = cudaMemcpyAsync(m->h_loss, m->loss, sizeof(double), cudaMemcpyDeviceToHost, st))) {
        note_error("loss copy", e);
        return CCT_CUDAERR;
    }
    if ((e = cudaStreamSynchronize(st))) { note_error("mps_mlp_loss_grad sync", e); return CCT_CUDAERR; }
    if (host_loss) *host_loss = (float)(*m->h_loss / M);
    return CCT_NOERR;
}

CCTStatusType mps_mlp_train_step(MpsMlp* m, int M, const float* X, const float* T, float w1, float lr,
                                 float* host_loss, void* stream) {
    if (!m || M <= 0 || M > m->maxb) return CCT_PARAMERR;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = m->forward(M, X, st, true);
    if (!e) e = m->backward(M, T, w1, st);
    if (e) return cuda_status(e);
    m->t += 1;
    const float b1t = powf(0.9f, (float)m->t), b2t = powf(0.999f, (float)m->t);
    MPS_COUNT_LAUNCH k_adam<<<div_up(MPS_MLP_PARAMS, 256), 256, 0, st>>>(MPS_MLP_PARAMS, m->p, m->g, m->m, m->v, lr, b1t, b2t);
    e = m->sync_layers(st);
    if (!e && host_loss) {
        e = cudaMemcpyAsync(m->h_loss, m->loss, sizeof(double), cudaMemcpyDeviceToHost, st);
        if (!e) e = cudaStreamSynchronize(st);
        if (!e) *host_loss = (float)(*m->h_loss / M);
    }
    return cuda_status(e ? e : cudaGetLastError());
}

}  // extern "C"
