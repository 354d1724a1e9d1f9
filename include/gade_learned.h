/*
 * gade_learned.h - kernels of the learned initial guess (no counterpart in
 * the reference, whose BiCGSTAB always starts from the previous solution,
 * tools/dirac_solver.c:533-551) and of the eigenstate projection that turns
 * states into bound / ionised populations.
 *
 * A POD basis U (R complex64 rows of length n, orthonormal) spans the part
 * of the next state that linear extrapolation misses; an MLP with two hidden
 * layers maps the projections of the last K states and the pulse factors
 * f_a(t) to R coefficients c, and a mixed-precision step starts from
 * x_n + (x_n - x_{n-1}) + U c (gade_batch_use_guess).  All pointers are
 * device pointers; every call is asynchronous on `stream` (a cudaStream_t as
 * void*, NULL: the default stream) and allocates nothing.  BF16 values are
 * stored as 16-bit words (bfloat16).
 */
#ifndef GADE_LEARNED_H
#define GADE_LEARNED_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* C = epi(A B + bias) on the tensor cores (tcgen05.mma, BF16 operands,
 * FP32 accumulation in tensor memory).  A(i,k) = A[i*sa0 + k*sa1] (M x K),
 * B(k,j) = B[k*sb0 + j*sb1] (K x N), so either operand may be read
 * transposed.  bias [N] may be NULL.  mask (M x N, row stride ldm) may be
 * NULL; where mask <= 0 the result is 0 (ReLU backward).  act: 0 none,
 * 1 ReLU.  C (FP32, row stride ldc) and C16 (BF16, row stride ldc16) may
 * each be NULL, not both.  Operands that are 16-byte aligned, unit-stride
 * along one dimension and with a row stride of a multiple of 8 elements are
 * staged by tensor copies (TMA); others by plain loads.  Both stagings give
 * the same bits. */
int gade_gemm_bf16(int32_t M, int32_t N, int32_t K, const void *A, int64_t sa0, int64_t sa1,
                   const void *B, int64_t sb0, int64_t sb1, const float *bias, const float *mask,
                   int64_t ldm, int32_t act, float *C, int64_t ldc, void *C16, int64_t ldc16, void *stream);

/* 1 when gade_gemm_bf16 with these operands stages them by tensor copies,
 * 0 when by plain loads (host only, no GPU work). */
int gade_gemm_bf16_path(int32_t M, int32_t N, int32_t K, const void *A, int64_t sa0, int64_t sa1,
                        const void *B, int64_t sb0, int64_t sb1);

/* Process-wide GEMM options (tests): path 0 automatic, 1 plain loads only;
 * wait_limit = mbarrier polls before a CTA gives up (0: the default, ~2^24);
 * withhold_copies = 1 makes the tensor-copy stager issue nothing, so that
 * the MMA thread's wait runs out and the status word is set. */
int gade_learned_set_gemm_options(int32_t path, uint32_t wait_limit, int32_t withhold_copies);

/* Status of the learned-model kernels since the last call (synchronous,
 * clears it): bit 0 = a tensor-core wait of gade_gemm_bf16 ran out (the
 * tile it was computing was not written). */
int gade_learned_status(int32_t *flags);

/* mean squared error of out against target (M x N, FP32): gradient
 * 2 (out - target)/(M N) into grad (FP32, may be NULL) and grad16 (BF16);
 * rowloss[i] = sum_j (out - target)^2 (FP64). */
int gade_mse_grad(int32_t M, int32_t N, const float *out, const float *target, float *grad, void *grad16,
                  double *rowloss, void *stream);

/* db[j] = sum_i G[i*ldg + j] (bias gradient), fixed summation order. */
int gade_colsum(int32_t M, int32_t N, const float *G, int64_t ldg, float *db, void *stream);

/* One Adam step (step = 1, 2, ...) on n FP32 master weights w with moments
 * m, v; w16 (BF16 copy, may be NULL) is refreshed. */
int gade_adam(int64_t n, float *w, void *w16, const float *g, float *m, float *v, float lr, float beta1,
              float beta2, float eps, int32_t step, void *stream);

/* y[i] = bf16(x[i]). */
int gade_to_bf16(int64_t n, const float *x, void *y, void *stream);

/* coef[p][r] = sum_i conj(U[r][i]) x_p[i] for p < npulse: U complex64
 * [R][n], x complex128 with pulse stride ldx, coef complex128 [npulse][R].
 * FP32 products of U and x's FP32 part, summed in FP32 over chunks of 1024
 * elements and the chunks in FP64, in a fixed order (relative error
 * ~1e-7: the network's BF16 inputs need no more).  scratch: device bytes,
 * at least gade_pod_project_scratch(n, R, npulse). */
int gade_pod_project(int64_t n, int32_t R, const void *U, const void *x, int64_t ldx, int32_t npulse,
                     void *coef, void *scratch, int64_t scratch_bytes, void *stream);
int64_t gade_pod_project_scratch(int64_t n, int32_t R, int32_t npulse);
/* The same with FP64 products and sums in a fixed order (relative error
 * ~1e-15): for training targets, second differences of projections. */
int gade_pod_project_fp64(int64_t n, int32_t R, const void *U, const void *x, int64_t ldx, int32_t npulse,
                          void *coef, void *scratch, int64_t scratch_bytes, void *stream);

/* y_p = scale[p] * U c_p (complex64 U [R][n] and c [npulse][R], complex128
 * y with pulse stride ldy); scale may be NULL (1). */
int gade_pod_expand(int64_t n, int32_t R, const void *U, const void *c, const float *scale, int32_t npulse,
                    void *y, int64_t ldy, void *stream);

/* Network input rows (BF16, and FP32 when out32 is not NULL), one per
 * pulse, length K*2R + 12: the projections of the last K states, newest
 * first, from the ring hist [K][npulse][R] complex128 whose newest slot is
 * head, as (re, im) pairs, then the 12 reals of f(t) (ft [npulse][12]); each
 * value normalised as (v - mu[e]) / sd[e]. */
int gade_learned_features(int32_t npulse, int32_t R, int32_t K, int32_t head, const void *hist, const double *ft,
                          const float *mu, const float *sd, void *out16, float *out32, void *stream);

/* Network outputs (FP32 [npulse][2R], normalised) -> complex64 coefficients
 * c = out * sd + mu; scale[p] = 1 while |c_p| <= limit * |h_0 - h_1| (the
 * projection of the last state change, from hist), else 0: an implausible
 * prediction falls back to plain extrapolation. */
int gade_learned_outputs(int32_t npulse, int32_t R, int32_t K, int32_t head, const float *out, const float *mu,
                         const float *sd, const void *hist, float limit, void *c, float *scale, void *stream);

/* The learned guess of a batch, one step in one call: every pointer a
 * device address fixed for the batch's lifetime (set once by the caller). */
typedef struct {
    int32_t n, R, npulse, K;        /* state length, POD rank, pulses, history length */
    int32_t din, dh, dout;          /* network widths: K*2R + 12 -> dh -> dh -> 2R */
    const void *U;                  /* complex64 POD basis [R][n] */
    void *hist;                     /* complex128 projection ring [K][npulse][R] */
    const void *x;                  /* complex128 states, pulse stride ldx */
    int64_t ldx;
    void *scratch;                  /* >= gade_pod_project_scratch(n, R, npulse) bytes */
    int64_t scratch_bytes;
    const float *mu_in, *sd_in, *mu_out, *sd_out;   /* input / output normalisation */
    void *x16;                      /* BF16 network inputs [npulse][din] */
    const void *W16[3];             /* BF16 weights [din][dh], [dh][dh], [dh][dout] */
    const float *bias[3];
    float *H1, *H2, *out;           /* FP32 activations [npulse][dh], [npulse][dh], outputs [npulse][dout] */
    void *H1_16, *H2_16;            /* their BF16 copies */
    void *c;                        /* complex64 coefficients [npulse][R] */
    float *scale;                   /* [npulse] */
    void *corr;                     /* complex128 guess correction, pulse stride ldcorr */
    int64_t ldcorr;
    float limit;                    /* gade_learned_outputs' plausibility limit */
} gade_learned_guess_plan;

/* Project the current states into hist[head] (gade_pod_project); when ft
 * (device, [npulse][12] reals: the next step's pulse factors) is not NULL,
 * also run the network on the K newest projections (gade_learned_features,
 * three gade_gemm_bf16, gade_learned_outputs) and write U c into corr
 * (gade_pod_expand).  Every kernel on stream, nothing synchronises. */
int gade_learned_guess_step(const gade_learned_guess_plan *plan, int32_t head, const double *ft, void *stream);

/* Eigenstate projection of states (the populations of src/process_output.cpp
 * with src/hamiltonian.h:1246-1330): for every pulse p < npulse and block
 * row r, coef[p][r][j] = sum_i conj(x_p[r*B + i]) W[k_r][i][j] with
 * W = S(k) V(k) (real, [nk][B][B], j fastest) from the per-kappa eigenpairs
 * of (H0(k), S(k)), k_r = block_kidx[r] (device).  classes[p][r][0..2] =
 * sum_j |coef|^2 over eigenvalues E < e_lo (negative-energy), e_lo <= E < 0
 * (bound) and E >= 0 (continuum) of evals [nk][B]; classes[..][3] = total.
 * x complex128 with pulse stride ldx; coef (may be NULL) complex128
 * [npulse][nblk][B]; classes double [npulse][nblk][4]; B <= 2048. */
int gade_eigproj(int32_t npulse, int32_t nblk, int32_t B, const int32_t *block_kidx, const double *W,
                 const double *evals, double e_lo, const void *x, int64_t ldx, void *coef, double *classes,
                 void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GADE_LEARNED_H */
