/*
 * mps_learned.h - the learned PPE initial guess / preconditioner scaling (BF16 MLP).
 *
 * No counterpart in the reference (its NJPCG solver is declared only:
 * solver/MPS_SOLVER_WITH_ROTATION/PMMultiGPU/Source/CGPUCellSet.h:224-225, 239).
 *
 * Network: 12 features -> 128 -> 128 -> 128 (SiLU) -> 2 outputs (pressure increment
 * in units of the step's pressure scale, log of the diagonal preconditioner scale).
 * Training (forward with kept pre-activations, backward, Adam) runs on the
 * 5th-generation tensor cores (tcgen05) with BF16 weights and activations, FP32
 * accumulation and an FP32 master copy.  Inference (mps_mlp_forward) runs on them too,
 * in FP16: weights, activations and the hidden layers' accumulators FP16 (11
 * significant bits against BF16's 8), the biases carried in the MMA through columns of
 * ones (split into two FP16 parts), the output layer accumulated in FP32.
 * Parameter vector layout (FP32, MPS_MLP_PARAMS = 34,946 floats):
 *   W1[12][128] b1[128] W2[128][128] b2[128] W3[128][128] b3[128] W4[128][2] b4[2]
 * (W[k][n]: input k, output n).
 *
 * All array arguments are DEVICE pointers unless stated; `stream` is a cudaStream_t
 * (NULL = legacy default stream).  Every call returns a CCTStatusType.
 */
#ifndef MPS_LEARNED_H
#define MPS_LEARNED_H

#include "mps_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* C[m][n] = act(sum_k A(m,k) B(k,n) + bias[n]) (+ beta * C) with BF16 A, B and FP32
 * accumulation on the tensor cores.  A(m,k) = A[m*lda + k] (transA = 0) or
 * A[k*lda + m] (transA = 1); B(k,n) = B[k*ldb + n] (transB = 0) or B[n*ldb + k]
 * (transB = 1).  Any K (tiles are zero-filled).  C (FP32, ldc) and/or Cb (BF16, ldcb)
 * may be NULL.  act: 0 none, 1 SiLU (Cz, if given, receives the pre-activation FP32).
 * split_k > 1 splits the K loop over CTAs and accumulates into C with atomics
 * (beta must be 1 and act 0 then).  Runs on the 5th-generation tensor cores
 * (tcgen05.mma into TMEM, 128 x 16..64 tiles, K in stages of 64); the MLP's forward
 * and backward passes of training use it. */
CCTStatusType mps_gemm_bf16(int M, int N, int K, const void* A, int lda, int transA, const void* B, int ldb,
                            int transB, float* C, int ldc, void* Cb, int ldcb, float* Cz, const float* bias, int act,
                            float beta, int split_k, void* stream);
/* the same with a chosen kernel: 0 the tcgen05 kernel of mps_gemm_bf16, 1 the
 * warp-level mma.sync kernel (a cross-check) */
CCTStatusType mps_gemm_bf16_variant(int M, int N, int K, const void* A, int lda, int transA, const void* B, int ldb,
                                    int transB, float* C, int ldc, void* Cb, int ldcb, float* Cz, const float* bias,
                                    int act, float beta, int split_k, int variant, void* stream);

typedef struct MpsMlp MpsMlp;
CCTStatusType mps_mlp_create(int max_batch, unsigned long long seed, MpsMlp** out);
void mps_mlp_destroy(MpsMlp* m);
/* host FP32 parameter vector in / out (MPS_MLP_PARAMS floats) */
CCTStatusType mps_mlp_set_params(MpsMlp* m, const float* host_params);
CCTStatusType mps_mlp_get_params(MpsMlp* m, float* host_params);
/* Y[M][2] = MLP(X[M][12]) (device FP32) */
CCTStatusType mps_mlp_forward(MpsMlp* m, int M, const float* X, float* Y, void* stream);
/* the same with a chosen kernel: 0 the tcgen05 FP16 kernel mps_mlp_forward uses, 1 the
 * warp-level mma.sync kernel with the BF16 / FP32 rounding points of training (a
 * cross-check), 2..5 the tcgen05 kernel with 0, 1, 2 or 3 of every 4 pairs of hidden
 * activations computed on the FMA pipe (a polynomial tanh) and the rest on the SFU */
CCTStatusType mps_mlp_forward_variant(MpsMlp* m, int M, const float* X, float* Y, int variant, void* stream);
/* nonzero if an MMA completion wait of the tcgen05 kernel ever ran out (the kernel then
 * stops early; its outputs are incomplete) */
CCTStatusType mps_mlp_tc_timeouts(unsigned* out);
/* debugging and tests: the number of polls of the inference kernel's MMA completion
 * waits (negative: the default, 4,194,304; 0: every such wait runs out at once, so the
 * kernel's stop path runs: each 128-row tile stops after issuing its first layer and
 * writes no output, the MMAs in flight drain before TMEM is freed).  Synchronises the
 * device and clears the mps_mlp_tc_timeouts flag. */
CCTStatusType mps_mlp_debug_wait_spins(long long spins);
/* loss = mean over rows of (y0-t0)^2 + w1 (y1-t1)^2 and the gradient of every
 * parameter (device FP32, MPS_MLP_PARAMS floats) by the tensor-core backward pass */
CCTStatusType mps_mlp_loss_grad(MpsMlp* m, int M, const float* X, const float* T, float w1, float* grad,
                                float* host_loss, void* stream);
/* one Adam step (lr, beta1 0.9, beta2 0.999, eps 1e-8) on a mini-batch */
CCTStatusType mps_mlp_train_step(MpsMlp* m, int M, const float* X, const float* T, float w1, float lr,
                                 float* host_loss, void* stream);

#ifdef __cplusplus
}
#endif

#endif
