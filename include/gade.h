/*
 * gade.h — C ABI of the GB300-native Crank-Nicolson step of GaDE
 * (JVembe/dirac_hydrogen_code, tools/ solver).
 *
 * One process, one GPU (sm_103a).  Plain C types only: complex numbers are
 * interleaved (re, im) doubles, indices are int32/int64, streams are passed
 * as void*.  Every entry point returns GADE_OK (0) or an error code; the
 * message of the last error on the calling thread is gade_last_error().
 * Nothing here calls exit(): the reference's ERROR()/CHECK_GPU() exits
 * (tools/utils.h:42-46, tools/cuda_translate.h:100-125) become status codes.
 *
 * Each function cites the reference interface it replaces.
 */
#ifndef GADE_H
#define GADE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GADE_OK            0
#define GADE_ERR_IO        1   /* file cannot be opened                        */
#define GADE_ERR_FORMAT    2   /* malformed input file                         */
#define GADE_ERR_CUDA      3   /* CUDA runtime / launch failure                */
#define GADE_ERR_ARG       4   /* invalid argument or size                     */
#define GADE_ERR_NUMERIC   5   /* zero pivot, non-finite residual              */
#define GADE_ERR_STATE     6   /* call order violated                          */

/* precision of the time step */
#define GADE_PREC_FP64     0   /* complex128 everywhere (reference parity)     */
#define GADE_PREC_MIXED    1   /* complex64 inner BiCGSTAB in FP64 refinement  */

typedef struct gade_problem gade_problem;   /* host copy of the input files  */
typedef struct gade_solver  gade_solver;    /* device state of one pulse     */

typedef struct {
    int32_t lmax, nblk, blkdim, blk_nnz;
    int64_t n;            /* state dimension nblk*blkdim                       */
    int64_t hall_nnz;     /* non-zero blocks of H.csr                          */
    int64_t nnz_full;     /* non-zeros of the assembled operator (reference)   */
    int32_t real_coupling;/* 1: g real, H0l/H1l imaginary (fast path)          */
    int32_t dkb_zero;     /* 1: g has the DKB zero blocks (the operator skips them) */
} gade_problem_info;

typedef struct {
    int32_t iters;        /* reference semantics: index of breaking iteration  */
    double  tol_error;    /* sqrt(|r|^2/|b|^2) of the recursive residual       */
    int32_t restarts;     /* BiCGSTAB restarts (|rho| tiny)                     */
    int32_t refinements;  /* outer FP64 refinement sweeps (mixed precision)    */
    int32_t inner_iters;  /* total inner complex64 iterations (mixed)          */
    double  true_residual;/* |b - A x|/|b| at exit (mixed precision only)      */
    double  snorm;        /* x^H S x before the step, FP64 (mixed precision)  */
    double  init_residual;/* |b - A x0|/|b| of the initial guess, FP64 (mixed)  */
} gade_step_stats;

/* Message of the last failing call on this thread ("" if none). */
const char *gade_last_error(void);

/* Reads H.csr, H0l<l>/H1l<l>.csr, g<q>a<a>l<l>.csr, h0<n>.csr, s<n>.csr and
 * psi0.vec from dir, like tools/dirac_solver.c:223-388 (csr_read,
 * csr_conj_transpose, vec_read, vec_read_perm). */
int gade_problem_load(const char *dir, int32_t lmax, gade_problem **out);
int gade_problem_get_info(const gade_problem *p, gade_problem_info *info);
/* psi0.vec contents: psi (2n doubles) and perm (n int32), either may be NULL.
 * Replaces vec_read/vec_read_perm (tools/dirac_solver.c:68-108). */
int gade_problem_get_psi0(const gade_problem *p, double *psi, int32_t *perm);
/* kappa[r] and the original angular index ang[r] of every block row r
 * (nblk entries each; either may be NULL): the rows of H.csr map to angular
 * indices through its perm array, kappa = ik(index) (tools/dirac_solver.c:
 * 396-431, tools/solver_common.c:30-37). */
int gade_problem_get_blocks(const gade_problem *p, int32_t *kappa, int32_t *ang);
void gade_problem_free(gade_problem *p);

/* Builds the device solver for a fixed time step dt (and h, always 1 in the
 * reference): uploads the radial and angular tables, the stationary blocks
 * and the block-LU preconditioner.  Replaces gpu_init_model_matrices +
 * gpu_compute_row_col (tools/gpu_solver.cu:137-236, 288-327),
 * compute_stationary_matrices + compute_preconditioner
 * (tools/solver.c:409-485), slu_compute_ilu (tools/superlu.c:154-266),
 * gpu_put_csr(L,U,S) + gpu_lu_analyze (tools/gpu_sparse.c:60-109,162-233)
 * and gpu_sparse_init/gpu_blas_init.  x is set to psi0.
 * precision: GADE_PREC_FP64 or GADE_PREC_MIXED. device: CUDA ordinal. */
int gade_solver_create(const gade_problem *p, double dt, double h, int32_t precision,
                       int32_t device, gade_solver **out);
void gade_solver_free(gade_solver *s);

/* State vector in the solver's (permuted) order; 2n doubles.
 * Replaces gpu_put_vec / gpu_get_vec (tools/gpu_sparse.c:120-152). */
int gade_solver_set_x(gade_solver *s, const double *x, int64_t n);
int gade_solver_get_x(gade_solver *s, double *x, int64_t n);
/* Starts a new pulse on the same solver (no reference counterpart: the
 * reference runs one pulse per process): sets the state like
 * gade_solver_set_x and clears what carries over from one step to the next
 * (BiCGSTAB's p and v, tools/bicgstab.c:28-31, and the previous state that
 * mixed precision extrapolates from), so the following steps are those of a
 * new solver with the same operator choice and partition. */
int gade_solver_restart(gade_solver *s, const double *x, int64_t n);

/* One Crank-Nicolson step at time t with pulse factors ft (6 complex, i.e.
 * 12 doubles, beoyndDipolePulse_axialPart at t): fills this step's operator
 * (the assembled real coupling values, or the matrix-free radial tables,
 * whichever was chosen at creation), then forms
 * rhs = S x - H(t) x and solves (S + H(t)) x' = rhs with right-block-LU-
 * preconditioned BiCGSTAB warm-started at x.  Replaces the loop body
 * tools/dirac_solver.c:503-551 (gpu_compute_timedep_matrices, gpu_spmv,
 * gpu_spmv_local, gpu_bicgstab of tools/gpu_bicgstab.c:133-307).
 * maxit/tol: the reference hard-codes 500 and 1e-16 (dirac_solver.c:506-507).
 * stats may be NULL. */
int gade_solver_step(gade_solver *s, const double *ft, int32_t maxit, double tol,
                     gade_step_stats *stats);
/* The same step with the state in host memory (no reference counterpart;
 * the reference keeps psi on the device between steps): x_in (2n doubles,
 * solver order, may be NULL to continue from the device state) is copied in
 * as by gade_solver_set_x, the step runs, and the new state is copied to
 * x_out (may be NULL, may equal x_in).  The copy-out is queued with the
 * step's convergence read-back, so a step that converges in one graph
 * replay waits for the device once.  x_out is undefined on error. */
int gade_solver_step_host(gade_solver *s, const double *x_in, const double *ft, int32_t maxit, double tol,
                          double *x_out, gade_step_stats *stats);

/* Sets the time-dependent radial tables for pulse factors ft without solving
 * (the pgsum part of gpu_compute_timedep_matrices, tools/gpu_solver.cu:50-82). */
int gade_solver_set_time(gade_solver *s, const double *ft);

/* y = S x + H(t) x for host vectors (2n doubles each), with the tables of
 * the last set_time/step.  Replaces gpu_HS_spmv_fun
 * (tools/dirac_solver.c:141-156) with alpha=1, beta=0.  Sx and Hx may be
 * NULL; when given they receive the two parts separately
 * (gpu_spmv_local(S) and gpu_spmv(Hfull), tools/gpu_sparse.c:267-313). */
int gade_solver_apply(gade_solver *s, const double *x, double *y, double *Sx, double *Hx);

/* z = (P^T)^{-1} b with P = S + i h dt/2 h0 block diagonal.  Replaces
 * gpu_LU_precond_fun / gpu_lu_solve (tools/dirac_solver.c:158-165,
 * tools/gpu_sparse.c:235-263) and slu_lu_solve (tools/superlu.c:268-290). */
int gade_solver_precond(gade_solver *s, const double *b, double *z);

/* Device-resident variants: x, y are device pointers to n complex128 values
 * in HBM, stream is a cudaStream_t passed as void* (NULL: the solver's
 * stream).  No host synchronisation. */
int gade_solver_apply_device(gade_solver *s, const void *x_dev, void *y_dev, void *stream);

/* Number of this library's kernel launches since creation (instrumentation). */
int64_t gade_solver_launch_count(const gade_solver *s);

/* Device time of the last apply issued by gade_solver_time_apply, and a
 * helper that times `reps` back-to-back operator applies with CUDA events on
 * the solver's stream; ms receives the average. */
int gade_solver_time_apply(gade_solver *s, int32_t reps, double *ms);
int gade_solver_time_precond(gade_solver *s, int32_t reps, double *ms);
/* The same for the complex64 operator apply of a mixed-precision solver's
 * inner BiCGSTAB (with its <r0, v> reduction); no reference counterpart. */
int gade_solver_time_apply_mixed(gade_solver *s, int32_t reps, double *ms);

/* The cudaStream_t (as void*) on which every call of this solver is ordered;
 * callers record their own CUDA events on it. */
void *gade_solver_stream(const gade_solver *s);

/* Device time of this solver's kernels, measured with CUDA events around each
 * launch while enabled (off by default; no reference counterpart — the
 * reference times whole BiCGSTAB calls with gettimeofday, tools/dirac_solver.c:547-551). */
typedef struct {
    int64_t apply_launches;   double apply_ms;     /* matrix-free operator      */
    int64_t precond_launches; double precond_ms;   /* block-LU solves           */
    int64_t other_launches;   double other_ms;     /* tables, vector updates    */
} gade_kernel_times;
int gade_solver_profile(gade_solver *s, int32_t enable);
/* Synchronises, returns the accumulated times and resets them. */
int gade_solver_kernel_times(gade_solver *s, gade_kernel_times *out);

/* Partition of the operator kernel's work chosen at creation (no reference
 * counterpart).  The work units are (row chunk, block row) pairs.  nsplit
 * 1-4: order split, nsplit CTAs share each unit, each with a part of the
 * Bessel orders; nsplit 0: balanced segments, the units' work cut by a cost
 * model into one equal share per resident CTA (a unit may be cut into
 * pieces).  A unit in several pieces is combined by its last piece in a fixed
 * order.  split_ms (4 floats, may be NULL) receives the timed apply for 1-4
 * splits (0 where not timed). */
int gade_solver_split(const gade_solver *s, int32_t *nsplit, float *split_ms);
/* Forces the partition (0 balanced, 1-4 order split) instead of the timed
 * choice; results differ from the plain layout only by the order of
 * summation. */
int gade_solver_set_split(gade_solver *s, int32_t nsplit);
/* The balanced partition of the FP64 BiCGSTAB operator: its CTAs (segments),
 * pieces, timed apply ms (0 where not built or not timed) and the weight of
 * the gather in its cost model, chosen by timing (any pointer may be NULL). */
int gade_solver_balanced(const gade_solver *s, int32_t *segments, int32_t *pieces, float *ms,
                         double *gather_weight);

/* Operator of a single pulse with real couplings, FP64 or mixed precision
 * (no reference counterpart): matrix-free (0) or assembled (1).  The couplings of H(t) are
 * linear in the six pulse factors, so the solver can store the coupling
 * values of each unit factor once (K_a, built from the radial tables) and
 * form this step's values as sum_a w_a(t) K_a; an apply then streams the
 * values (2 FMAs each); in mixed precision the complex64 inner solve
 * streams the values rounded to float.  gade_solver_create times both (the
 * step's tables and three applies) and keeps the faster (the assembled one
 * needs 32 bytes of device memory per stored coupling value, 36 in mixed
 * precision).  gade_solver_operator reports the choice and, in ms (5
 * floats, may be NULL), the timed matrix-free apply, the assembled one with
 * the plain and the balanced partition, and the step's matrix-free radial
 * tables and assembly (0 where not timed).  After
 * gade_solver_set_operator the next gade_solver_set_time or step fills the
 * chosen operator's tables. */
int gade_solver_set_operator(gade_solver *s, int32_t assembled);
int gade_solver_operator(const gade_solver *s, int32_t *assembled, float *ms);

/* FP64 flops (2 per FMA) executed by one operator apply and one
 * preconditioner solve, counted exactly from the set-up structure. */
int gade_solver_flops(const gade_solver *s, double *apply_flops, double *precond_flops);
/* Compulsory DRAM bytes of one FP64 BiCGSTAB operator apply (no reference
 * counterpart).  Matrix-free: the radial-table slabs of the distinct (order,
 * kappa) pairs the block rows use, the diagonal blocks, the angular terms
 * and slot maps, and the vectors read and written (x, r0 in; v out).
 * Assembled: the stored coupling values, the diagonal blocks and the
 * vectors. */
int gade_solver_apply_bytes(const gade_solver *s, double *bytes);
/* FP64 flops and compulsory DRAM bytes of one step's assembly of the
 * coupling values (0 with the matrix-free operator); no reference
 * counterpart.  gade_solver_flops and gade_solver_apply_bytes describe the
 * operator in use. */
int gade_solver_assembly_cost(const gade_solver *s, double *flops, double *bytes);

/* y = (S + H(t)) x and dot = sum_i conj(r0_i) y_i (2 doubles, re and im), all
 * device pointers in HBM, with the tables of the last set_time/step; no
 * counterpart in the reference.  For callers that may not allocate device
 * memory once they are running: frameworks that own all GPU memory through
 * their own pool and forbid other allocations after start-up, or loops on
 * pipelined streams where cudaMalloc's implicit device synchronisation would
 * stall them.  This entry point calls no cudaMalloc/cudaFree and no allocating
 * library routine: its cross-block reduction scratch is a fixed 512 KB device
 * array inside the library (16384 partial-sum slots), which every GPU that
 * loads the library keeps until exit.  Problems that need more than 16384
 * row-chunk x block work units are rejected with GADE_ERR_ARG.  The first call
 * on each device looks up that array's device address and keeps it for the
 * life of the process; make that first call before any stream capture, and
 * do not call cudaDeviceReset (or otherwise tear down the device's primary
 * context) after it.  All calls share the array, so calls whose kernels
 * overlap on the GPU race: order them on one stream.  The call reads the
 * operator (radial tables or assembled values) that set_time and step write
 * asynchronously on the solver's stream (gade_solver_stream): on another
 * stream, order it after them with an event.  Asynchronous on `stream`
 * (NULL: the solver's stream). */
int gade_solver_apply_dot_noalloc(gade_solver *s, const void *x_dev, const void *r0_dev, void *y_dev,
                                  void *dot_dev, void *stream);

/* Arithmetic of the FP64 refinement residual of a mixed-precision step (no
 * reference counterpart): 0 the FP64 units; 1 (the default where available)
 * double-float on the FP32 units, each value a pair of floats (about 48
 * significant bits: products split exactly by FMA, sums by two-sum), which
 * keeps the residual accurate to ~1e-13 of |b| and runs on GB300's 64-times
 * larger FP32 rate.  Available for mixed-precision solvers with real
 * couplings on the matrix-free operator; the assembled operator's residual
 * stays FP64.  gade_solver_residual_precision reports the setting and
 * whether the double-float pass is the one steps use.  Takes effect at the
 * next step. */
int gade_solver_set_residual_precision(gade_solver *s, int32_t mode);
int gade_solver_residual_precision(const gade_solver *s, int32_t *mode, int32_t *in_use);

/* Polls of each shared-memory stage wait of the block-LU preconditioner
 * kernel before it gives up (no reference counterpart: the reference's
 * cuSPARSE solves have no waits of their own).  0 restores the default,
 * 2^22.  A wait that runs out sets an error bit, the kernel lets its copies
 * in flight land (with the default limit) and returns; the step then
 * returns GADE_ERR_CUDA, clears BiCGSTAB's carried vectors p and v
 * (tools/bicgstab.c:28-31) and leaves the state undefined: set it again
 * before the next step.  The device stays usable.  Takes effect at the next
 * step (captured graphs are rebuilt). */
int gade_solver_set_wait_limit(gade_solver *s, uint32_t polls);
/* Warps per block row of the FP64 block-LU solves (replacing the cuSPARSE
 * triangular solves of tools/gpu_sparse.c:235-263): 8 (the default; two
 * per SM sub-partition, the triangle products of a chunk pair split over
 * two warps) or 4.  The two differ only in the order of FP64 additions.
 * The complex64 solves of the mixed-precision inner iterations always use
 * 4.  Takes effect at the next step. */
int gade_solver_set_precond_warps(gade_solver *s, int32_t warps);
/* Failure injection for tests of that path (no reference counterpart): the
 * preconditioner kernel does not issue the copy of stage `stage` (0 is the
 * first; -1 turns the injection off), so the wait for it runs out after the
 * wait limit and the step returns GADE_ERR_CUDA.  Nothing is read or written
 * out of place: the kernel only skips that copy and the wait for it. */
int gade_solver_inject_wait_timeout(gade_solver *s, int32_t stage);

/* Measured FP64 FMA throughput of a device in TFLOP/s (2 flops per DFMA),
 * from a dependent-chain-free FMA kernel timed with CUDA events. */
int gade_probe_fp64_peak(int32_t device, double *tflops);

/* ---- batched pulses (no counterpart in the reference) ----------------
 * Many independent pulses advance together: the reference runs one
 * dirac_solver process per pulse (tools/dirac_solver.c:496-636), each with
 * its own dt = T/Ntime and its own radial tables g (they depend on Omega and
 * Cycles through the Bessel arguments), on the same angular tables, h0 and S.
 * A batch holds all of them on one GPU; every kernel of a step runs over all
 * pulses still in the launch list, and each step is replayed from captured
 * CUDA graphs with BiCGSTAB's control on the device.  Results of pulse k are
 * those of a gade_solver made with dt[k] and g slice k. */
typedef struct gade_batch gade_batch;

typedef struct {
    int32_t chunk_splines;     /* operator row-chunk size in splines, 16..64; 0: autotune */
    int32_t iters_per_launch;  /* BiCGSTAB iterations per graph replay, 1..64; 0: adaptive */
    int32_t use_graphs;        /* nonzero: replay captured CUDA graphs; 0: direct launches */
} gade_batch_options;

typedef struct {
    int32_t npulse, active;    /* pulses held; pulses in the current launch list */
    int32_t chunk_splines;     /* row-chunk size in use */
    int32_t iters_per_launch;  /* current iterations per graph replay */
    int64_t graph_replays, steps;
    int32_t ntune;             /* autotuner candidates timed */
    int32_t tune_cs[4];        /* candidate chunk sizes */
    float tune_ms[4];          /* their batched operator-apply times */
    double apply_flops;        /* FP64 flops of one operator apply of one pulse */
} gade_batch_info;

/* npulse pulses on problem p.  dt[k]: time step of pulse k.  g: NULL (every
 * pulse uses p's radial tables) or npulse slices of the loader's layout,
 * [k][a<6][l<lmax][q<4][blk_nnz] complex128 (re, im), q = g0..g3 of
 * g<q>a<a>l<l>.csr in the base pattern's CSR order; they must be real when
 * p's are.  precision: GADE_PREC_FP64.  opt may be NULL (autotune, adaptive,
 * graphs).  Every pulse starts from psi0. */
int gade_batch_create(const gade_problem *p, int32_t npulse, const double *dt, const double *g, double h,
                      int32_t precision, int32_t device, const gade_batch_options *opt, gade_batch **out);
/* The operator of a batch (no reference counterpart): chosen by timing at
 * creation like gade_solver_operator, ms as there (the assembled values take 8 bytes per
 * stored coupling value and pulse, 12 in mixed precision, plus 24 per value
 * for each distinct set of radial tables); gade_batch_set_operator forces it
 * (the next step fills the chosen operator's tables). */
int gade_batch_operator(const gade_batch *b, int32_t *assembled, float *ms);
int gade_batch_set_operator(gade_batch *b, int32_t assembled);
void gade_batch_free(gade_batch *b);
int gade_batch_set_x(gade_batch *b, int32_t pulse, const double *x, int64_t n);
int gade_batch_get_x(gade_batch *b, int32_t pulse, double *x, int64_t n);

/* One CN step of every pulse k with active[k] != 0 (active NULL: all), with
 * pulse factors ft[k*12 .. k*12+11] as in gade_solver_step.  Pulses that
 * leave the active set leave the launch list (retired pulses cost nothing).
 * stats (may be NULL) receives npulse records; inactive pulses get zeros.
 * Returns the first failing pulse's error. */
int gade_batch_step(gade_batch *b, const int32_t *active, const double *ft, int32_t maxit, double tol,
                    gade_step_stats *stats);
int gade_batch_get_info(const gade_batch *b, gade_batch_info *info);

/* Device address of the pulse states (complex128, pulse k at x_dev + k*ld
 * elements), for projections and copies on gade_batch_stream.  Valid until
 * gade_batch_free. */
int gade_batch_state_device(gade_batch *b, void **x_dev, int64_t *ld);

/* Initial-guess correction of mixed-precision batches: a device buffer of
 * npulse complex128 vectors (pulse k at corr_dev + k*ld elements), made on
 * the first call.  While enabled, a step starts pulse k from
 * x_n + (x_n - x_{n-1}) + corr_k (the learned guess, gade_learned.h) instead
 * of the linear extrapolation alone; a pulse without an x_{n-1} starts from
 * x_n.  The FP64 refinement still certifies every step. */
int gade_batch_guess_buffer(gade_batch *b, void **corr_dev, int64_t *ld);
int gade_batch_use_guess(gade_batch *b, int32_t enable);
/* The cudaStream_t (as void*) on which the batch's work is ordered. */
void *gade_batch_stream(const gade_batch *b);
/* gade_solver_set_wait_limit for the pulses of a batch. */
int gade_batch_set_wait_limit(gade_batch *b, uint32_t polls);
/* gade_solver_set_residual_precision for a batch. */
int gade_batch_set_residual_precision(gade_batch *b, int32_t mode);

#ifdef __cplusplus
}
#endif
#endif /* GADE_H */
