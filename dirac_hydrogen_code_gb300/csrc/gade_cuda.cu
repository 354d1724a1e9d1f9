/*
 * GB300 (sm_103a) Crank-Nicolson step of GaDE: matrix-free operator,
 * block-LU preconditioner, fused BiCGSTAB.  Exposes the C ABI of
 * include/gade.h.
 *
 * Operator (replaces assembly + SpMV, tools/gpu_solver.cu:50-135 and
 * tools/gpu_sparse.c:267-313).  Block (r,c) of S + H(t) is
 *   delta_rc [S(k_r) + i h dt/2 h0(k_r)]
 *   + sum_l H0l(r,c) (pg_l0 + k_r pg_l1 + k_c pg_l2 + k_r k_c pg_l3)
 *          + H1l(r,c) (pgt_l0 + k_c pgt_l1 + k_r pgt_l2 + k_r k_c pgt_l3)
 * (tools/solver.c:328-383).  Factoring the column kappa out,
 *   y_r = D(k_r) x_r + sum_l [ M0_l(k_r) u_l + M1_l(k_r) w_l
 *                            + M2_l(k_r) u'_l + M3_l(k_r) w'_l ]
 * with u_l = sum_c H0l(r,c) x_c, w_l = sum_c H0l(r,c) k_c x_c (u', w' with
 * H1l) and the per-step radial tables
 *   M0 = pg0 + k pg1, M1 = pg2 + k pg3, M2 = pgt0 + k pgt2, M3 = pgt1 + k pgt3
 * built once per step for every distinct kappa.  Nothing of size nnz(A) is
 * ever stored.  When g is real and H0l/H1l imaginary (always true for the
 * dumpCouplings physics) the coupling is real: tables and angular factors
 * are stored as real numbers and each term costs 2 FMAs instead of 4.
 *
 * Preconditioner: exact LU of each distinct diagonal block of P^T,
 * P = S + i h dt/2 h0, in a banded ordering; one warp per block row solves
 * 32 rows at a time with the pre-inverted 32x32 diagonal blocks.
 *
 * BiCGSTAB (tools/bicgstab.c:125-295): 5 kernels per iteration; the update
 * of p and s is fused into the preconditioner, dots into the operator and
 * the x/r update; every scalar lives on the device and reductions are
 * deterministic (per-CTA partials summed in a fixed order by the last CTA).
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <algorithm>
#include <utility>
#include <vector>

#include "gade_internal.h"
#include "../../include/gade.h"

#define SOL 137.035999084

/* ------------------------------------------------------------------ */
/* errors                                                              */
/* ------------------------------------------------------------------ */
static thread_local char g_err[1024];

static int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

extern "C" const char *gade_last_error(void) { return g_err; }

/* error reporting of the other translation units of the library */
extern "C" int gade_set_error(int code, const char *msg) { return fail(code, "%s", msg); }

#define CK(call)                                                                     \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess)                                                       \
            return fail(GADE_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,    \
                        cudaGetErrorString(e_));                                     \
    } while (0)

#define CKL()                                                                        \
    do {                                                                             \
        cudaError_t e_ = cudaGetLastError();                                         \
        if (e_ != cudaSuccess)                                                       \
            return fail(GADE_ERR_CUDA, "%s:%d launch: %s", __FILE__, __LINE__,       \
                        cudaGetErrorString(e_));                                     \
        s->launches++;                                                               \
    } while (0)

/* ------------------------------------------------------------------ */
/* complex helpers                                                     */
/* ------------------------------------------------------------------ */
template <typename R> struct Cx;
template <> struct Cx<double> { typedef double2 T; };
template <> struct Cx<float> { typedef float2 T; };

template <typename C> __device__ __forceinline__ C mk(double re, double im) { C c; c.x = re; c.y = im; return c; }
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C c; c.x = a.x + b.x; c.y = a.y + b.y; return c; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C c; c.x = a.x - b.x; c.y = a.y - b.y; return c; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b)
{
    C c; c.x = a.x * b.x - a.y * b.y; c.y = a.x * b.y + a.y * b.x; return c;
}
/* acc += a*b */
template <typename C> __device__ __forceinline__ void cfma(C &acc, C a, C b)
{
    acc.x = fma(a.x, b.x, acc.x); acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y); acc.y = fma(a.y, b.x, acc.y);
}
/* acc += a*b, a real */
template <typename C, typename R> __device__ __forceinline__ void rfma(C &acc, R a, C b)
{
    acc.x = fma(a, b.x, acc.x); acc.y = fma(a, b.y, acc.y);
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b)
{
    /* Smith's algorithm (robust complex division) */
    double2 q;
    if (fabs(b.x) >= fabs(b.y)) {
        double r = b.y / b.x, d = b.x + b.y * r;
        q.x = (a.x + a.y * r) / d; q.y = (a.y - a.x * r) / d;
    } else {
        double r = b.x / b.y, d = b.x * r + b.y;
        q.x = (a.x * r + a.y) / d; q.y = (a.y * r - a.x) / d;
    }
    return q;
}
struct alignas(32) R4d { double a, b, c, d; };
struct alignas(16) R4f { float a, b, c, d; };
template <typename R> struct R4;
template <> struct R4<double> { typedef R4d T; };
template <> struct R4<float> { typedef R4f T; };
template <typename C> struct alignas(16) C4 { C a, b, c, d; };
/* cache-global load of a complex value (the partial sums of pieces) */
template <typename C> __device__ __forceinline__ C ldcg_c(const C *p) { return __ldcg(p); }

/*
 * Double-float ("dd") arithmetic for the refinement residual of mixed
 * precision.  A value is hi + lo in two floats, |lo| <= ulp(hi)/2 when
 * normalised, about 48 significant bits.  A product a b is split exactly
 * into p = fl(a.hi b.hi) and its error by one FMA (the FMA form of Dekker's
 * two-product, with the a.hi b.lo + a.lo b.hi terms added to the error);
 * the high parts of a running sum are added by Knuth's two-sum, which is
 * exact, and the rounding errors collect in the low part.  The relative
 * error of a sum of n products is about n 2^-46 of the terms' magnitudes,
 * against n 2^-53 in FP64: residuals of the refinement are then accurate
 * to ~1e-13 of |b|, far below the tolerances (>= 1e-12) they decide.  All
 * of it runs on the FP32 pipes, which GB300 has 64 times as many of as
 * FP64 units.
 */
struct __align__(8) dd { float hi, lo; };
struct __align__(16) cdd { dd x, y; };
struct alignas(32) R4dd { dd a, b, c, d; };
template <> struct Cx<dd> { typedef cdd T; };
template <> struct R4<dd> { typedef R4dd T; };

__host__ __device__ inline dd dd_from(double v)
{
    dd r;
    r.hi = (float)v;
    r.lo = (float)(v - (double)r.hi);
    return r;
}
__device__ __forceinline__ double dd_to(dd a) { return (double)a.hi + (double)a.lo; }
/* the same split without double -> float conversions (which run at the FP64
   rate on GB300): hi keeps the sign, exponent and top 23 stored mantissa
   bits (truncation, exact), lo the remaining 29 bits as a float (one
   integer -> float conversion and a power-of-two scale), so hi + lo is v
   within 2^-47 relative.  Below 2^-74 lo is dropped (float precision) and
   below 2^-126 the value is 0: terms that small do not register in sums of
   the tables' magnitudes. */
__device__ __forceinline__ dd dd_from_bits(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int e11 = (int)((b >> 52) & 0x7FF);
    const int e8 = e11 - 1023 + 127;
    dd r;
    if (e8 <= 0) { r.hi = 0.f; r.lo = 0.f; return r; }
    r.hi = __uint_as_float(sign | ((unsigned)e8 << 23) | (unsigned)((b >> 29) & 0x7FFFFF));
    const unsigned rem = (unsigned)(b & 0x1FFFFFFFull);   /* units of 2^(e11 - 1075) */
    const int t = e11 - 1075 + 127;
    r.lo = (t > 0 && rem) ? (float)rem * __uint_as_float(sign | ((unsigned)t << 23)) : 0.f;
    return r;
}
__device__ __forceinline__ dd dd_neg(dd a) { dd r; r.hi = -a.hi; r.lo = -a.lo; return r; }
/* acc += a b */
__device__ __forceinline__ void dd_fma(dd &acc, dd a, dd b)
{
    const float p = a.hi * b.hi;
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    const float sum = acc.hi + p;
    const float bv = sum - acc.hi;
    const float err = (acc.hi - (sum - bv)) + (p - bv);
    acc.hi = sum;
    acc.lo += err + e;
}
__device__ __forceinline__ dd dd_add(dd a, dd b)
{
    const float sum = a.hi + b.hi;
    const float bv = sum - a.hi;
    const float err = (a.hi - (sum - bv)) + (b.hi - bv);
    dd r;
    r.hi = sum;
    r.lo = a.lo + b.lo + err;
    return r;
}
/* renormalise (fast two-sum of hi and lo) */
__device__ __forceinline__ dd dd_norm(dd a)
{
    dd r;
    r.hi = a.hi + a.lo;
    r.lo = a.lo - (r.hi - a.hi);
    return r;
}
template <> __device__ __forceinline__ cdd mk<cdd>(double re, double im)
{
    cdd c; c.x = dd_from(re); c.y = dd_from(im); return c;
}
template <> __device__ __forceinline__ cdd cadd<cdd>(cdd a, cdd b)
{
    cdd c; c.x = dd_add(a.x, b.x); c.y = dd_add(a.y, b.y); return c;
}
template <> __device__ __forceinline__ cdd csub<cdd>(cdd a, cdd b)
{
    cdd c; c.x = dd_add(a.x, dd_neg(b.x)); c.y = dd_add(a.y, dd_neg(b.y)); return c;
}
template <> __device__ __forceinline__ void cfma<cdd>(cdd &acc, cdd a, cdd b)
{
    dd_fma(acc.x, a.x, b.x); dd_fma(acc.x, dd_neg(a.y), b.y);
    dd_fma(acc.y, a.x, b.y); dd_fma(acc.y, a.y, b.x);
}
__device__ __forceinline__ void rfma(cdd &acc, dd a, cdd b)
{
    dd_fma(acc.x, a, b.x); dd_fma(acc.y, a, b.y);
}
template <> __device__ __forceinline__ cdd ldcg_c<cdd>(const cdd *p)
{
    const float4 v = __ldcg((const float4 *)p);
    cdd c; c.x.hi = v.x; c.x.lo = v.y; c.y.hi = v.z; c.y.lo = v.w; return c;
}
__device__ __forceinline__ cdd cdd_norm(cdd a) { cdd c; c.x = dd_norm(a.x); c.y = dd_norm(a.y); return c; }
/* a sum about to be used as a factor: renormalised for double-float, as is otherwise */
template <typename C> __device__ __forceinline__ C norm_c(C a) { return a; }
template <> __device__ __forceinline__ cdd norm_c<cdd>(cdd a) { return cdd_norm(a); }
__device__ __forceinline__ double2 cdd_to(cdd a) { return make_double2(dd_to(a.x), dd_to(a.y)); }
__device__ __forceinline__ cdd cdd_from(double2 v) { cdd c; c.x = dd_from(v.x); c.y = dd_from(v.y); return c; }

/* ------------------------------------------------------------------ */
/* device scalars of one BiCGSTAB solve                                */
/* ------------------------------------------------------------------ */
struct DevScal {
    double2 rho_prev, rho, alpha, w;
    double r0_sqnorm, rhs_sqnorm, rr;
    double2 r0v, ts;
    double tt;
    unsigned int err;      /* bit 0: a bounded mbarrier wait timed out */
    unsigned int pad0;
    double snorm;          /* x^H S x (mixed precision conservation check) */
    /* device-side iteration control (batched pulses; ctl = 1): the reduction
       epilogues advance state / iter exactly as the host loop of the single
       solver does, and every predicated kernel of a pulse whose state is not
       the one it waits for returns at entry */
    double tol2rel;        /* tol^2: converged when rr < tol2rel * rhs_sqnorm */
    int ctl;               /* 0 host control; 1 BiCGSTAB / refinement record; 2 inner-solve record */
    int state, iter, maxit, restarts;
    /* mixed precision, refinement record: the inner solve's pending
       correction, sweeps and FP64 residual passes so far, inner iterations
       summed over sweeps, inner iteration limit, stall flag */
    int pending, sweeps, refinements, inner_total, maxit_in, stalled;
    double tol2abs;        /* inner-solve record: absolute target for |r|^2 */
    double rr_init;        /* refinement record: |r|^2 of the initial guess */
};

enum { ST_RUN = 0, ST_DONE, ST_ZERO, ST_RESTART, ST_BAD };
/* launch predicates on a pulse's records: a = the refinement / BiCGSTAB
   record, b = the inner-solve record */
enum { PRED_NONE = 0, PRED_RUN, PRED_RESTART, PRED_MIX, PRED_FIN, PRED_DONE };

#define MIXED_MAX_SWEEPS 8

/* Programmatic dependent launch: the step's kernels are launched so that the
   next one's CTAs may become resident while the previous kernel drains; every
   kernel waits for its predecessor's completion (and memory) before it reads
   or writes anything a kernel produced, and only then lets its own successor
   launch.  Both are no-ops for a kernel launched without the attribute. */
#ifndef GADE_PDL
#define GADE_PDL 1
#endif
__device__ __forceinline__ void pdl_enter()
{
#if GADE_PDL
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

__device__ __forceinline__ bool pred_ok(int pred, const DevScal *a, const DevScal *b)
{
    if (pred == PRED_NONE) return true;
    const int st = *(volatile const int *)&a->state;
    switch (pred) {
    case PRED_RUN: return st == ST_RUN;
    case PRED_RESTART: return st == ST_RESTART;
    case PRED_MIX: return st == ST_RUN && *(volatile const int *)&a->pending == 0;
    case PRED_FIN: return *(volatile const int *)&a->pending != 0 && *(volatile const int *)&b->state != ST_RUN;
    default: return st == ST_DONE;
    }
}

/* predicate of kernels without a reduction */
struct BPred {
    const int *plist;              /* grid y -> pulse (NULL: pulse 0) */
    DevScal *a, *b;                /* [pulse] records */
    int pred;
};

enum { RED_RHS = 0, RED_RESTART, RED_R0V, RED_TS, RED_UPDATE, RED_NONE, RED_DOT_OUT, RED_MIX };
enum { AX_PLAIN = 0, AX_PARTS, AX_R0V, AX_TS, AX_RHS, AX_RESTART, AX_MIX };
enum { PC_PLAIN = 0, PC_P, PC_S };

#define NRED 4   /* values per partial: up to 4 doubles */
#define APPLY_G64 3   /* Bessel orders per gather phase of the FP64 operator */
#ifndef APPLY_G32
#define APPLY_G32 4   /* ... of the complex64 operator */
#endif
#ifndef APPLY_GDD
#define APPLY_GDD 3   /* ... of the double-float residual pass */
#endif

/* ------------------------------------------------------------------ */
/* operator parameters                                                 */
/* ------------------------------------------------------------------ */
struct OpP {
    int nblk, B, lmax, W, nk, RM, CM, AM;   /* AM: max angular terms of one block row */
    const int *row_kidx, *act_ptr, *act_l, *ang_ptr, *ang_c;
    const void *ang_a0, *ang_a0k, *ang_a1, *ang_a1k;
    const int *chunk_nrows, *chunk_ncols, *chunk_rows, *chunk_cols, *chunk_lcol;
    const unsigned short *chunk_acol;   /* [nchunk][W][RM] column within the block of each ELL slot (B: empty) */
    const void *M;             /* [pulse][lmax][nk][W][B] */
    const void *S_ell;         /* [nk][W][B], shared by all pulses */
    const void *Hst_ell, *D_ell;   /* [pulse][nk][W][B] (depend on dt) */
    const int *plist;          /* grid x -> pulse (NULL: pulse 0) */
    long long vstride;         /* complex elements per pulse of every vector */
    size_t mstride, dstride;   /* elements per pulse of M and of Hst / D */
    /* partition of the work: unit u = (block row u / nchunk, chunk u % nchunk);
       CTA y runs pieces seg_ptr[y] .. seg_ptr[y+1]-1 in order, a piece being
       {unit, first active order, end, index within the unit | pieces of the
       unit << 16}.  A unit cut into pieces leaves partial row sums in
       piece_acc [piece][3][RM]; the last piece to arrive (unit_tick [unit])
       sums them in piece order and runs the epilogue */
    int nchunk;
    const int *seg_ptr;
    const int4 *pieces;
    void *piece_acc;
    unsigned int *unit_tick;
    /* assembled operator (k_apply_asm): this step's coupling values
       A[pair][W][B] and the coupled block of every (block row, block) pair;
       a piece's order range is then a pair range */
    const void *A;                 /* double, or float for the complex64 instance */
    const int *pair_c;
    size_t astride;                /* values per pulse of A */
};

struct VecP {
    void *out0, *out1, *out2;      /* outputs by mode */
    const void *in0, *in1;         /* r0 / s / rhs by mode */
    const void *in0dd, *in1dd;     /* double-float residual pass: x_n and delta as double-float */
};

struct RedP {
    double *part;                  /* [pulse][nCTA][NRED] */
    unsigned int *ticket;          /* [pulse] */
    DevScal *sc;                   /* [pulse] */
    int kind;
    double *out;                   /* RED_DOT_OUT: receives (re, im) of the dot */
    size_t pstride;                /* partials per pulse */
    int pred;                      /* PRED_*: which pulse state the launch works on */
    DevScal *pa, *pb;              /* [pulse] predicate record (NULL: sc) and second record */
};

/* Move the reduction targets to pulse `pulse`; false when the pulse's state
   says this launch has nothing to do (uniform over the CTA). */
__device__ __forceinline__ bool red_select(RedP &red, int pulse)
{
    red.sc += pulse;
    red.ticket += pulse;
    red.part += (size_t)pulse * red.pstride;
    if (red.pa) red.pa += pulse;
    if (red.pb) red.pb += pulse;
    return pred_ok(red.pred, red.pa ? red.pa : red.sc, red.pb ? red.pb : red.sc);
}

/* Block-wide deterministic sum of NV doubles; result valid in thread 0. */
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *sh)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int k = 0; k < NV; k++) sh[k * nt + tid] = v[k];
    __syncthreads();
    for (int s = 1; s < nt; s <<= 1) {
        /* pairwise in fixed order: thread tid (multiple of 2s) adds tid+s */
        if ((tid % (2 * s)) == 0 && tid + s < nt)
            for (int k = 0; k < NV; k++) sh[k * nt + tid] += sh[k * nt + tid + s];
        __syncthreads();
    }
    for (int k = 0; k < NV; k++) v[k] = sh[k * nt];
    __syncthreads();
}

/* The CTA's block sum of v into partial slot idx (written by thread 0). */
__device__ __forceinline__ void reduce_part(RedP red, double (&v)[NRED], double *sh, unsigned idx)
{
    block_sum<NRED>(v, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < NRED; k++) red.part[(size_t)idx * NRED + k] = v[k];
}

/* Arrival of one CTA (narrive CTAs per pulse); the last to arrive sums the
   npart partial slots in index order and finalises the reduction. */
__device__ void reduce_tail(RedP red, double *sh, unsigned narrive, unsigned npart)
{
    __shared__ bool am_last;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (tid == 0) {
        __threadfence();
        unsigned t = atomicAdd(red.ticket, 1u);
        am_last = (t == narrive - 1);
    }
    __syncthreads();
    if (!am_last) return;
    __threadfence();
    double acc[NRED] = {0, 0, 0, 0};
    for (unsigned j = tid; j < npart; j += nt)
        for (int k = 0; k < NRED; k++) acc[k] += __ldcg(&red.part[(size_t)j * NRED + k]);
    block_sum<NRED>(acc, sh);
    if (tid == 0) {
        DevScal *sc = red.sc;
        switch (red.kind) {
        case RED_RHS:
            sc->r0_sqnorm = acc[0];
            sc->rr = acc[0];
            sc->rhs_sqnorm = acc[1];
            sc->rho = make_double2(acc[0], 0.0);
            sc->rho_prev = make_double2(1.0, 0.0);
            sc->alpha = make_double2(1.0, 0.0);
            sc->w = make_double2(1.0, 0.0);
            if (sc->ctl == 1) {
                /* the early exits of the host loop (tools/bicgstab.c:176-189) */
                sc->iter = 0;
                sc->restarts = 0;
                if (!isfinite(acc[0]) || !isfinite(acc[1])) sc->state = ST_BAD;
                else if (acc[1] == 0.0) sc->state = ST_ZERO;
                else if (acc[0] < sc->tol2rel * acc[1] || sc->maxit <= 0) sc->state = ST_DONE;
                else sc->state = ST_RUN;
            } else if (sc->ctl == 2) {
                /* inner solve started from the refinement residual; its
                   correction is now pending on the refinement record */
                sc->iter = 0;
                red.pa->pending = 1;
                sc->state = (sc->maxit <= 0 || fabs(acc[0]) < (1e-12 * 1e-12) * acc[0]) ? ST_DONE : ST_RUN;
            }
            break;
        case RED_RESTART:
            sc->r0_sqnorm = acc[0];
            sc->rr = acc[0];
            sc->rho = make_double2(acc[0], 0.0);
            if (sc->ctl == 1) { sc->restarts++; sc->state = ST_RUN; }
            break;
        case RED_R0V:
            sc->r0v = make_double2(acc[0], acc[1]);
            sc->alpha = cdiv(sc->rho, sc->r0v);
            break;
        case RED_TS:
            sc->tt = acc[0];
            sc->ts = make_double2(acc[1], acc[2]);
            sc->w = acc[0] > 0 ? make_double2(acc[1] / acc[0], acc[2] / acc[0]) : make_double2(0.0, 0.0);
            break;
        case RED_UPDATE:
            sc->rr = acc[0];
            sc->rho_prev = sc->rho;
            sc->rho = make_double2(acc[1], acc[2]);
            if (sc->ctl == 1) {
                /* convergence, iteration limit, then the restart test that
                   opens the next iteration (tools/bicgstab.c:205-212,287-293) */
                if (!isfinite(acc[0])) sc->state = ST_BAD;
                else if (acc[0] < sc->tol2rel * sc->rhs_sqnorm) sc->state = ST_DONE;
                else if (++sc->iter >= sc->maxit) sc->state = ST_DONE;
                else if (fabs(acc[1]) < (1e-12 * 1e-12) * sc->r0_sqnorm) sc->state = ST_RESTART;
            } else if (sc->ctl == 2) {
                /* inner solve: stop at the target (or a non-finite value),
                   at the iteration limit, or on breakdown; refinement follows */
                sc->iter++;
                if (!(acc[0] >= sc->tol2abs)) sc->state = ST_DONE;
                else if (sc->iter >= sc->maxit) sc->state = ST_DONE;
                else if (fabs(acc[1]) < (1e-12 * 1e-12) * sc->r0_sqnorm) sc->state = ST_DONE;
            }
            break;
        case RED_DOT_OUT:
            red.out[0] = acc[0];
            red.out[1] = acc[1];
            break;
        case RED_MIX:
            if (sc->ctl != 1) {
                sc->rhs_sqnorm = acc[0];
                sc->rr = acc[1];
                sc->snorm = acc[2];
            } else {
                /* the refinement loop's tests after each FP64 residual pass */
                const int first = sc->refinements == 0;
                sc->refinements++;
                sc->rr = acc[1];
                if (first) { sc->rhs_sqnorm = acc[0]; sc->snorm = acc[2]; sc->rr_init = acc[1]; }
                const double b2 = sc->rhs_sqnorm, tol2 = sc->tol2rel * b2;
                if (first && !isfinite(b2)) sc->state = ST_BAD;
                else if (first && b2 == 0.0) sc->state = ST_ZERO;
                else if (!isfinite(acc[1])) sc->state = ST_BAD;
                else if (acc[1] < tol2) sc->state = ST_DONE;
                else if (sc->sweeps >= MIXED_MAX_SWEEPS || sc->maxit_in <= 0) {
                    sc->state = ST_DONE;
                    sc->stalled = sc->maxit_in > 0;
                } else {
                    sc->sweeps++;
                    red.pb->tol2abs = 0.25 * tol2;
                }
            }
            break;
        }
        *red.ticket = 0u;
    }
}

/* Per-CTA partials + last-CTA finalisation (fixed summation order).
   ncta / cta: the CTAs of one pulse and this CTA's index among them. */
__device__ void reduce_finish(RedP red, double (&v)[NRED], double *sh, unsigned ncta, unsigned cta)
{
    reduce_part(red, v, sh, cta);
    reduce_tail(red, sh, ncta, ncta);
}

/* ------------------------------------------------------------------ */
/* per-step radial tables                                              */
/* ------------------------------------------------------------------ */
struct TabP {
    int lmax, nk, W, B;
    const double *kvals;
    const void *g, *gt;           /* [pulse][lmax][3][4][W][B]: ELL slot layout, zero on empty slots
                                     (a in the l-parity set) */
    void *M, *M32, *Mdd;          /* [pulse][lmax][nk][W][B]: FP64 tables, complex64 and double-float copies */
    const int *plist;             /* grid z -> pulse (NULL: pulse 0) */
    size_t gstride, mstride;      /* elements per pulse of g / gt and of M */
};

/* coef[l*3 + ia]: SoL * i h dt/2 * f_a for a = (l%2+1)%2 + 2 ia.
 * RC: imaginary parts only (pg is imaginary, the stored table is -Im M). */
/* grid (slot blocks, order l, pulse slot): no integer division, so the FP64
   pipe only carries the table arithmetic */
template <bool RC, int OUT>
__global__ void k_tables(TabP T, const double2 *__restrict__ coef)
{
    /* OUT: bit 1 the FP64 tables M, bit 2 the complex64 copies M32 (rounded
       from the same FP64 values), bit 4 the double-float copies Mdd (real
       couplings), any combination from one pass */
    const int per_l = T.W * T.B;
    const int l = blockIdx.y;
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;     /* j*B + i: consecutive threads stream g, gt and M */
    if (slot >= per_l) return;
    const int pulse = T.plist ? T.plist[blockIdx.z] : 0;
    coef += (size_t)pulse * T.lmax * 3;
    const size_t mo = (size_t)pulse * T.mstride;
    if (RC) {
        double pg[4] = {0, 0, 0, 0}, pgt[4] = {0, 0, 0, 0};
        {
            const double *g = (const double *)T.g + (size_t)pulse * T.gstride;
            const double *gt = (const double *)T.gt + (size_t)pulse * T.gstride;
            for (int ia = 0; ia < 3; ia++) {
                const double c = -coef[l * 3 + ia].y;     /* the stored table is -Im M */
                for (int q = 0; q < 4; q++) {
                    const size_t off = (((size_t)l * 3 + ia) * 4 + q) * per_l + slot;
                    pg[q] = fma(c, g[off], pg[q]);
                    pgt[q] = fma(c, gt[off], pgt[q]);
                }
            }
        }
        for (int kk = 0; kk < T.nk; kk++) {
            const double kap = T.kvals[kk];
            R4<double>::T m;
            m.a = fma(kap, pg[1], pg[0]);
            m.b = fma(kap, pg[3], pg[2]);
            m.c = fma(kap, pgt[2], pgt[0]);
            m.d = fma(kap, pgt[3], pgt[1]);
            const size_t e = mo + ((size_t)l * T.nk + kk) * per_l + slot;
            if (OUT & 1) ((R4<double>::T *)T.M)[e] = m;
            if (OUT & 4) {
                /* double-float split by bit operations; the complex64 copy is
                   its high part (truncated rather than rounded to float) */
                R4dd f;
                f.a = dd_from_bits(m.a); f.b = dd_from_bits(m.b); f.c = dd_from_bits(m.c); f.d = dd_from_bits(m.d);
                ((R4dd *)T.Mdd)[e] = f;
                if (OUT & 2) {
                    R4<float>::T h;
                    h.a = f.a.hi; h.b = f.b.hi; h.c = f.c.hi; h.d = f.d.hi;
                    ((R4<float>::T *)T.M32)[e] = h;
                }
            } else if (OUT & 2) {
                R4<float>::T f;
                f.a = (float)m.a; f.b = (float)m.b; f.c = (float)m.c; f.d = (float)m.d;
                ((R4<float>::T *)T.M32)[e] = f;
            }
        }
    } else {
        double2 pg[4], pgt[4];
        for (int q = 0; q < 4; q++) { pg[q] = make_double2(0, 0); pgt[q] = make_double2(0, 0); }
        {
            const double2 *g = (const double2 *)T.g + (size_t)pulse * T.gstride;
            const double2 *gt = (const double2 *)T.gt + (size_t)pulse * T.gstride;
            for (int ia = 0; ia < 3; ia++) {
                const double2 c = coef[l * 3 + ia];
                for (int q = 0; q < 4; q++) {
                    const size_t off = (((size_t)l * 3 + ia) * 4 + q) * per_l + slot;
                    cfma(pg[q], c, g[off]);
                    cfma(pgt[q], c, gt[off]);
                }
            }
        }
        for (int kk = 0; kk < T.nk; kk++) {
            const double kap = T.kvals[kk];
            C4<double2> m;
            m.a = make_double2(fma(kap, pg[1].x, pg[0].x), fma(kap, pg[1].y, pg[0].y));
            m.b = make_double2(fma(kap, pg[3].x, pg[2].x), fma(kap, pg[3].y, pg[2].y));
            m.c = make_double2(fma(kap, pgt[2].x, pgt[0].x), fma(kap, pgt[2].y, pgt[0].y));
            m.d = make_double2(fma(kap, pgt[3].x, pgt[1].x), fma(kap, pgt[3].y, pgt[1].y));
            const size_t e = mo + ((size_t)l * T.nk + kk) * per_l + slot;
            if (OUT & 1) ((C4<double2> *)T.M)[e] = m;
            if (OUT & 2) {
                C4<float2> f;
                f.a = make_float2((float)m.a.x, (float)m.a.y); f.b = make_float2((float)m.b.x, (float)m.b.y);
                f.c = make_float2((float)m.c.x, (float)m.c.y); f.d = make_float2((float)m.d.x, (float)m.d.y);
                ((C4<float2> *)T.M32)[e] = f;
            }
        }
    }
}

/* Outputs and dot partials of one row of the operator kernels, by mode:
   accH = A x (or H x where S x is apart in accS), accD = S delta (AX_MIX). */
template <typename C, bool SEP>
__device__ __forceinline__ void apply_epilogue(int mode, const VecP &V, size_t gi, C accS, C accH, C accD,
                                               double (&v)[NRED])
{
    const C ax = SEP ? cadd(accH, accS) : accH;
    switch (mode) {
    case AX_PLAIN:
        ((C *)V.out0)[gi] = ax;
        break;
    case AX_PARTS:
        ((C *)V.out0)[gi] = accS;
        ((C *)V.out1)[gi] = accH;
        break;
    case AX_R0V: {          /* v = A y ; <r0, v> */
        ((C *)V.out0)[gi] = ax;
        const C r0 = ((const C *)V.in0)[gi];
        v[0] = (double)r0.x * ax.x + (double)r0.y * ax.y;
        v[1] = (double)r0.x * ax.y - (double)r0.y * ax.x;
        break;
    }
    case AX_TS: {           /* t = A z ; <t,t>, <t,s> */
        ((C *)V.out0)[gi] = ax;
        const C sv = ((const C *)V.in0)[gi];
        v[0] = (double)ax.x * ax.x + (double)ax.y * ax.y;
        v[1] = (double)ax.x * sv.x + (double)ax.y * sv.y;
        v[2] = (double)ax.x * sv.y - (double)ax.y * sv.x;
        break;
    }
    case AX_RHS: {          /* rhs = -Hx + Sx ; r = rhs - (Hx + Sx) ; r0 = r */
        const C rhs = csub(accS, accH);
        const C rv = csub(rhs, ax);
        ((C *)V.out0)[gi] = rhs;
        ((C *)V.out1)[gi] = rv;
        ((C *)V.out2)[gi] = rv;
        v[0] = (double)rv.x * rv.x + (double)rv.y * rv.y;
        v[1] = (double)rhs.x * rhs.x + (double)rhs.y * rhs.y;
        break;
    }
    case AX_MIX: {          /* r = -S delta - H w ; b = S x_n - H w / 2 ; x_n^H S x_n */
        const C rv = mk<C>(-accD.x - accH.x, -accD.y - accH.y);
        ((C *)V.out0)[gi] = rv;
        const C b = mk<C>(accS.x - 0.5 * accH.x, accS.y - 0.5 * accH.y);
        v[0] = (double)b.x * b.x + (double)b.y * b.y;
        v[1] = (double)rv.x * rv.x + (double)rv.y * rv.y;
        const C xi = ((const C *)V.in0)[gi];
        v[2] = (double)xi.x * accS.x + (double)xi.y * accS.y;
        break;
    }
    case AX_RESTART: {      /* r = rhs - A x ; r0 = r */
        const C rhs = ((const C *)V.in0)[gi];
        const C rv = csub(rhs, ax);
        ((C *)V.out1)[gi] = rv;
        ((C *)V.out2)[gi] = rv;
        v[0] = (double)rv.x * rv.x + (double)rv.y * rv.y;
        break;
    }
    }
}

/* ------------------------------------------------------------------ */
/* matrix-free operator                                                */
/* ------------------------------------------------------------------ */
/* Shared-memory carve-up of k_apply, computed the same way on the host
   (launch size) and in the kernel: every piece starts on a 32-byte boundary. */
struct ApplySmem {
    unsigned xr, ub, xs, ds, lcs, angc, ang, ord, shred, total;
};

__host__ __device__ __forceinline__ unsigned up32(unsigned o) { return (o + 31u) & ~31u; }

__host__ __device__ __forceinline__ ApplySmem apply_smem(int CS, int W, int RM, int AM, int G, unsigned elem,
                                                         unsigned ang4, int nt, int lmax)
{
    ApplySmem s;
    unsigned o = 0;
    s.xr = o;    o = up32(o + elem * CS);
    s.ub = o;    o = up32(o + 4u * elem * G * CS);
    s.xs = o;    o = up32(o + elem * CS);
    s.ds = o;    o = up32(o + elem * CS);
    s.lcs = o;   o = up32(o + 4u * W * RM);
    s.angc = o;  o = up32(o + 4u * AM);
    s.ang = o;   o = up32(o + ang4 * AM);
    s.ord = o;   o = up32(o + 16u * lmax);
    s.shred = o; o = up32(o + 8u * NRED * nt);
    s.total = o;
    return s;
}

/*
 * grid (pulse slot, segment): a unit is (block row, row chunk) and a segment
 * a run of pieces of units (see OpP); one piece per unit and one unit per
 * segment is the plain layout.  Two threads per output row (HJ ELL slots
 * each: HJ = (W+1)/2).  Per thread the local columns of its HJ slots stay in
 * registers for a piece; empty slots point to a zero
 * column, so the table loops carry no branch and unroll completely.  The four
 * contracted vectors u, w, u', w' of a column are interleaved (one 32- or
 * 64-byte record) and so are the four angular factors of a term.
 */
#ifndef GADE_TABLE_PF
#define GADE_TABLE_PF 1    /* bulk L2 prefetch of each order group's table rows (double-float instance) */
#endif
#ifndef GADE_DD_MINB
#define GADE_DD_MINB 2     /* resident CTAs per SM the double-float instance is compiled for */
#endif
template <typename R, bool RC, bool SEP, bool Z>
__global__ void __launch_bounds__(256, std::is_same<R, dd>::value ? GADE_DD_MINB : ((sizeof(R) == 8 && SEP) ? 2 : 3))
    k_apply(OpP P, const typename Cx<R>::T *__restrict__ x, int mode, VecP V, RedP red)
{
    /* Z: the DKB zero blocks hold (slots laid out by column half): the
       first-half columns (this row's slots 0..14, thread half 0) have M3 = 0
       and need no w', the second-half columns (slots 15..29, half 1) have
       M1 = 0 and need no w */
    /* SEP: modes that need S x and H x apart (AX_RHS, AX_PARTS, AX_MIX, three
       accumulators); the BiCGSTAB modes use D = S + i h dt/2 h0 and one
       accumulator, which lets the FP64 instance fit three CTAs per SM */
    constexpr int HJ = 15;                    /* slots per thread: W in {29, 30} */
    typedef typename Cx<R>::T C;
    typedef typename std::conditional<RC, typename R4<R>::T, C4<C>>::type A4;   /* a0, a0 k_c, a1, a1 k_c */
    extern __shared__ __align__(32) unsigned char smem_raw[];
    /* G orders per gather phase: 3 (FP64, double-float) or 4 (FP32); with
       ~150 columns a chunk's G x columns gather items fill the CTA's threads
       twice (2, 4 and 6, 8 measured no faster) */
    constexpr int G = std::is_same<R, dd>::value ? APPLY_GDD : (sizeof(R) == 8 ? APPLY_G64 : APPLY_G32);
    const int CS = (P.CM + 2) & ~1;           /* column stride: CM + the zero column, even */
    const ApplySmem L = apply_smem(CS, P.W, P.RM, P.AM, G, sizeof(C), sizeof(A4), blockDim.x, P.lmax);
    C *xr = (C *)(smem_raw + L.xr);           /* [CS] */
    /* [G][4][CS] u, w, u', w' of a column, one array per vector: a warp
       reads one vector of neighbouring columns, 16 or 8 bytes apart, free of
       bank conflicts */
    C *ub = (C *)(smem_raw + L.ub);
    C *xs = (C *)(smem_raw + L.xs);           /* [CS] AX_MIX: x_n slice   */
    C *ds = (C *)(smem_raw + L.ds);           /* [CS] AX_MIX: delta slice */
    int *lcs = (int *)(smem_raw + L.lcs);     /* [W][RM] local column of each ELL slot (CM: empty) */
    int *angc = (int *)(smem_raw + L.angc);   /* [AM] coupled block of each angular term of row r */
    A4 *ang = (A4 *)(smem_raw + L.ang);       /* [AM] */
    int4 *oinf = (int4 *)(smem_raw + L.ord);  /* [lmax] the piece's orders: l, first and end angular term */
    double *shred = (double *)(smem_raw + L.shred); /* [NRED * blockDim] */

    /* grid (pulse slot, segment): the slots of one segment run side by side,
       so the shared maps and angular tables come from L2 for all but one */
    const int pulse = P.plist ? P.plist[blockIdx.x] : 0;
    if (!red_select(red, pulse)) return;
    /* the pulse's vectors and tables: offsets applied where they are used,
       so the pointers stay in the parameter space across the pieces */
    x += (long long)pulse * P.vstride;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int B = P.B, W = P.W, CM = P.CM;
    if (tid == 0) {                           /* the zero column: empty slots and columns past a chunk */
        const C z = mk<C>(0, 0);
        xr[CM] = z; xs[CM] = z; ds[CM] = z;
        C4<C> z4; z4.a = z; z4.b = z; z4.c = z; z4.d = z;
        for (int g = 0; g < G; g++)
            for (int q4 = 0; q4 < 4; q4++) ub[(g * 4 + q4) * CS + CM] = z4.a;
    }
    /* this CTA's segment: pieces (unit, order range) in sequence order.  The
       piece's scalars are kept in shared memory and read back after the
       order loop, which leaves the loop its registers */
    __shared__ int s_pc, s_pw;
    for (int pc = P.seg_ptr[blockIdx.y]; pc < P.seg_ptr[blockIdx.y + 1]; pc = *(volatile int *)&s_pc + 1) {
    const int4 pd = P.pieces[pc];
    const int u = pd.x, r = u / P.nchunk, q = u - r * P.nchunk;
    const int kk = P.row_kidx[r];
    const int nrows = P.chunk_nrows[q], ncols = P.chunk_ncols[q];
    /* two threads per output row, each with half of the ELL slots */
    const int half = tid / P.RM, trow = tid - half * P.RM;
    const int i = (half < 2 && trow < nrows) ? P.chunk_rows[q * P.RM + trow] : -1;
    const int jb = half == 0 ? 0 : (W + 1) / 2, je = half == 0 ? (W + 1) / 2 : W;
    const int nj = je - jb;                   /* <= HJ */
    const int *cols = P.chunk_cols + (size_t)q * CM;
    const C *xb = x + (size_t)r * B;
    __syncthreads();                          /* the previous piece is done with shared memory */
    if (tid == 0) { s_pc = pc; s_pw = pd.w; } /* read back after the next barrier */
    {
        const int *gl = P.chunk_lcol + (size_t)q * W * P.RM;
        for (int e = tid; e < W * P.RM; e += nt) { const int v = gl[e]; lcs[e] = v < 0 ? CM : v; }
    }
    const int ea = P.ang_ptr[r * P.lmax], eb = P.ang_ptr[r * P.lmax + P.lmax];
    for (int e = tid; e < eb - ea; e += nt) {
        angc[e] = P.ang_c[ea + e];
        if constexpr (RC) {
            A4 a;
            a.a = ((const R *)P.ang_a0)[ea + e];
            a.b = ((const R *)P.ang_a0k)[ea + e];
            a.c = ((const R *)P.ang_a1)[ea + e];
            a.d = ((const R *)P.ang_a1k)[ea + e];
            ang[e] = a;
        } else {
            A4 a;
            a.a = ((const C *)P.ang_a0)[ea + e];
            a.b = ((const C *)P.ang_a0k)[ea + e];
            a.c = ((const C *)P.ang_a1)[ea + e];
            a.d = ((const C *)P.ang_a1k)[ea + e];
            ang[e] = a;
        }
    }

    for (int k = tid; k < pd.z - pd.y; k += nt) {
        const int l = P.act_l[pd.y + k];
        oinf[k] = make_int4(l, P.ang_ptr[r * P.lmax + l] - ea, P.ang_ptr[r * P.lmax + l + 1] - ea, 0);
    }
    for (int c = tid; c < ncols; c += nt) xr[c] = xb[cols[c]];
    if (mode == AX_MIX) {
        /* x_n and delta (double-float instance: their double-float copies) */
        constexpr bool DD = std::is_same<R, dd>::value;
        const size_t vo = (size_t)pulse * P.vstride + (size_t)r * B;
        const C *xn = (const C *)(DD ? V.in0dd : V.in0) + vo, *dn = (const C *)(DD ? V.in1dd : V.in1) + vo;
        for (int c = tid; c < ncols; c += nt) { xs[c] = xn[cols[c]]; ds[c] = dn[cols[c]]; }
    }
    __syncthreads();

    /* this thread's slots: local column (CM when empty or past the half);
       table rows advance by B per slot and stay on the half's last slot
       past its end (the product is zero there) */
    /* two 16-bit local columns per register (CM < 2^16) */
    unsigned lcp[(HJ + 1) / 2];
#pragma unroll
    for (int t = 0; t < HJ; t += 2) {
        const unsigned c0 = (t < nj && trow < P.RM) ? lcs[(jb + t) * P.RM + trow] : CM;
        const unsigned c1 = (t + 1 < HJ && t + 1 < nj && trow < P.RM) ? lcs[(jb + t + 1) * P.RM + trow] : CM;
        lcp[t / 2] = c0 | (c1 << 16);
    }
#define LCO(t) ((int)(((t) & 1) ? (lcp[(t) >> 1] >> 16) : (lcp[(t) >> 1] & 0xffffu)))
    const int jB = jb * B;

    C accS = mk<C>(0, 0), accH = mk<C>(0, 0), accD = mk<C>(0, 0);
    if (i >= 0 && (pd.w & 0xffff) == 0) {     /* diagonal blocks: the unit's first piece */
        if (SEP && mode == AX_MIX) {
            /* x = w = 2 x_n + delta: S x_n, S delta and (i h dt/2 h0) w */
            const C *Se = (const C *)P.S_ell + (size_t)kk * W * B + i + jB;
            const C *He = (const C *)P.Hst_ell + (size_t)pulse * P.dstride + (size_t)kk * W * B + i + jB;
#pragma unroll
            for (int t = 0; t < HJ; t++) {
                const int lc = LCO(t);
                const C sv = *Se;
                cfma(accS, sv, xs[lc]);
                cfma(accD, sv, ds[lc]);
                cfma(accH, *He, xr[lc]);
                if (t + 1 < nj) { Se += B; He += B; }
            }
        } else if (SEP) {
            const C *Se = (const C *)P.S_ell + (size_t)kk * W * B + i + jB;
            const C *He = (const C *)P.Hst_ell + (size_t)pulse * P.dstride + (size_t)kk * W * B + i + jB;
#pragma unroll
            for (int t = 0; t < HJ; t++) {
                const C xv = xr[LCO(t)];
                cfma(accS, *Se, xv);
                cfma(accH, *He, xv);
                if (t + 1 < nj) { Se += B; He += B; }
            }
        } else {
            const C *De = (const C *)P.D_ell + (size_t)pulse * P.dstride + (size_t)kk * W * B + i + jB;
#pragma unroll
            for (int t = 0; t < HJ; t++) {
                cfma(accH, *De, xr[LCO(t)]);
                if (t + 1 < nj) De += B;
            }
        }
    }

    const int a_end = pd.z;
    for (int ag = pd.y; ag < a_end; ag += G) {
        const int ng = a_end - ag < G ? a_end - ag : G;
        __syncthreads();     /* staging done / previous group's apply done */
#if GADE_TABLE_PF
        if constexpr (std::is_same<R, dd>::value) {
            /* the group's table rows into L2 while the gather below runs: per
               (order, slot) the chunk's rows are two contiguous runs, the
               first and second half of the sorted chunk_rows (splines s and
               their partners s + B/2).  Double-float instance only: it lifted
               the mixed NKappa=16 step 650 -> 673 steps/s; the complex64
               instance measured slower at N = 53,040 (tables L2-resident,
               70 -> 77 us) and the FP64 one unchanged */
            typedef typename std::conditional<RC, typename R4<R>::T, C4<C>>::type Q4;
            const int n0 = nrows >> 1;
            for (int it = tid; it < ng * W * 2; it += nt) {
                const int g = it / (2 * W), rem = it - g * 2 * W, w = rem >> 1, h = rem & 1;
                const int len = h ? nrows - n0 : n0;
                if (len <= 0) continue;
                const int rs = P.chunk_rows[q * P.RM + (h ? n0 : 0)];
                const int l = oinf[ag - pd.y + g].x;
                const Q4 *src = (const Q4 *)P.M + (size_t)pulse * P.mstride +
                                ((size_t)l * P.nk + kk) * W * B + (size_t)w * B + rs;
                asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src),
                             "r"((unsigned)(len * sizeof(Q4))) : "memory");
            }
        }
#endif
        /* gather u, w, u', w' of ng orders at once: (order, column) items */
        for (int item = tid; item < ng * ncols; item += nt) {
            const int g = item / ncols, c = item - g * ncols;
            const int4 oi = oinf[ag - pd.y + g];
            const int e0 = oi.y, e1 = oi.z;
            const int gc = cols[c];
            const C *xc = x + gc;
            /* with the DKB zero blocks a first-half column needs no w' and a
               second-half column no w */
            const bool qcol = gc >= (B >> 1);
            const bool need_b = !Z || !qcol, need_d = !Z || qcol;
            C4<C> uv;
            uv.a = mk<C>(0, 0); uv.b = uv.a; uv.c = uv.a; uv.d = uv.a;
#pragma unroll 4
            for (int e = e0; e < e1; e++) {
                const C xv = xc[(size_t)angc[e] * B];
                const A4 a = ang[e];
                if constexpr (RC) {
                    rfma(uv.a, a.a, xv);
                    if (need_b) rfma(uv.b, a.b, xv);
                    rfma(uv.c, a.c, xv);
                    if (need_d) rfma(uv.d, a.d, xv);
                } else {
                    cfma(uv.a, a.a, xv);
                    if (need_b) cfma(uv.b, a.b, xv);
                    cfma(uv.c, a.c, xv);
                    if (need_d) cfma(uv.d, a.d, xv);
                }
            }
            C *u4 = ub + (size_t)g * 4 * CS + c;
            u4[0] = norm_c(uv.a); u4[CS] = norm_c(uv.b); u4[2 * CS] = norm_c(uv.c); u4[3 * CS] = norm_c(uv.d);
        }
        __syncthreads();
        if (i >= 0) {
            for (int g = 0; g < ng; g++) {
                const int l = oinf[ag - pd.y + g].x;
                const C *ua = ub + (size_t)g * 4 * CS, *uw = ua + CS, *uc = ua + 2 * CS, *ud = ua + 3 * CS;
                const bool second = half == 1;
                const C *u3 = second ? ud : uw;          /* with the DKB zero blocks: the half's third vector */
                if constexpr (RC) {
                    typedef typename R4<R>::T Q4;
                    const Q4 *Mt = (const Q4 *)P.M + (size_t)pulse * P.mstride + ((size_t)l * P.nk + kk) * W * B + i + jB;
#pragma unroll
                    for (int t = 0; t < HJ; t++) {
                        const Q4 m = *Mt;
                        const int lc = LCO(t);
                        rfma(accH, m.a, ua[lc]);
                        rfma(accH, m.c, uc[lc]);
                        if (Z) {
                            rfma(accH, second ? m.d : m.b, u3[lc]);
                        } else {
                            rfma(accH, m.b, uw[lc]);
                            rfma(accH, m.d, ud[lc]);
                        }
                        if (t + 1 < nj) Mt += B;
                    }
                } else {
                    const C4<C> *Mt = (const C4<C> *)P.M + (size_t)pulse * P.mstride + ((size_t)l * P.nk + kk) * W * B + i + jB;
#pragma unroll
                    for (int t = 0; t < HJ; t++) {
                        const C4<C> m = *Mt;
                        const int lc = LCO(t);
                        cfma(accH, m.a, ua[lc]);
                        cfma(accH, m.c, uc[lc]);
                        if (Z) {
                            cfma(accH, second ? m.d : m.b, u3[lc]);
                        } else {
                            cfma(accH, m.b, uw[lc]);
                            cfma(accH, m.d, ud[lc]);
                        }
                        if (t + 1 < nj) Mt += B;
                    }
                }
            }
        }
    }

#undef LCO
    /* combine the two halves of every row */
    __syncthreads();
    {
        C *xch = (C *)shred;                  /* 3 per row; fits in the reduction buffer */
        if (SEP) {
            if (half == 1 && i >= 0) { xch[3 * trow] = accS; xch[3 * trow + 1] = accH; xch[3 * trow + 2] = accD; }
            __syncthreads();
            if (half == 0 && i >= 0) {
                accS = cadd(accS, xch[3 * trow]);
                accH = cadd(accH, xch[3 * trow + 1]);
                accD = cadd(accD, xch[3 * trow + 2]);
            }
        } else {
            if (half == 1 && i >= 0) xch[trow] = accH;
            __syncthreads();
            if (half == 0 && i >= 0) accH = cadd(accH, xch[trow]);
        }
        __syncthreads();
    }
    const int pw = *(volatile int *)&s_pw;
    const int pi = pw & 0xffff, np = pw >> 16;          /* piece index within the unit, pieces of the unit */
    if (np > 1) {
        /* a unit cut into pieces: partial row sums per piece; the last piece
           to arrive sums them in piece order and runs the epilogue */
        const int pc = *(volatile int *)&s_pc;
        __shared__ int piece_last;
        C *acc = (C *)P.piece_acc;
        const size_t RM3 = (size_t)3 * P.RM;
        if (half == 0 && i >= 0) {
            acc[pc * RM3 + P.RM + trow] = accH;
            if (SEP) { acc[pc * RM3 + trow] = accS; acc[pc * RM3 + 2 * P.RM + trow] = accD; }
        }
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            const unsigned t = atomicAdd(&P.unit_tick[u], 1u);
            piece_last = (t == (unsigned)np - 1u);
        }
        __syncthreads();
        if (!piece_last) continue;
        __threadfence();
        if (half == 0 && i >= 0) {
            accS = mk<C>(0, 0); accH = accS; accD = accS;
            for (int k = 0; k < np; k++) {
                const size_t pk = (size_t)(pc - pi + k) * RM3;
                accH = cadd(accH, ldcg_c(&acc[pk + P.RM + trow]));
                if (SEP) {
                    accS = cadd(accS, ldcg_c(&acc[pk + trow]));
                    accD = cadd(accD, ldcg_c(&acc[pk + 2 * P.RM + trow]));
                }
            }
        }
        if (tid == 0) P.unit_tick[u] = 0u;
    }
    /* epilogue (the double-float instance writes FP64 outputs) */
    double v[NRED] = {0, 0, 0, 0};
    if (half == 0 && i >= 0) {
        const size_t gi = (size_t)pulse * P.vstride + (size_t)r * B + i;
        if constexpr (std::is_same<R, dd>::value)
            apply_epilogue<double2, SEP>(mode, V, gi, cdd_to(accS), cdd_to(accH), cdd_to(accD), v);
        else
            apply_epilogue<C, SEP>(mode, V, gi, accS, accH, accD, v);
    }
    /* the unit's dot partials, indexed by unit (not by CTA): the final sum
       has the same order for every partition */
    if (red.kind != RED_NONE) reduce_part(red, v, shred, (unsigned)u);
    }
    if (red.kind != RED_NONE) reduce_tail(red, shred, gridDim.y, (unsigned)(P.nchunk * P.nblk));
}


/* ------------------------------------------------------------------ */
/* assembled operator (one FP64 pulse, real couplings)                 */
/* ------------------------------------------------------------------ */
/*
 * The couplings of H(t) are linear in the six pulse factors, so for real
 * couplings every off-diagonal value is A(t) = sum_a w_a(t) K_a with K_a
 * the values for a unit factor a (built once from the matrix-free tables)
 * and w_a(t) the step's coefficient of a.  An apply then costs 2 FMAs per
 * stored value (a real value times a complex x) against ~4.4 in the
 * matrix-free form, for an assembly of 3 FMAs per value once per step (the
 * orders coupling a pair share a parity, which selects three of the six
 * factors).
 * Values are stored per (block row, coupled block) pair in the ELL slot
 * layout [pair][W][B] of the radial tables, so one slot map serves every
 * pair.
 */

/* K[pair][ia][slot][row] = sum over the pair's (order l, angular term e) of
   M0(l,k_r) a0[e] + M1 a0k[e] + M2 a1[e] + M3 a1k[e], from the tables of a
   unit factor a.  The orders coupling one pair share a parity (the angular
   selection rules), and order l uses the factors a = (l%2+1)%2 + 2 ia, so a
   pair stores three values per slot, ia = 0..2; the pairs of the other
   parity are skipped.  grid (slot blocks, pairs) */
__global__ void k_build_K(double *__restrict__ K, const R4<double>::T *__restrict__ M, int nk, int WB, int a,
                          const int *__restrict__ pair_r, const int *__restrict__ pair_par,
                          const int *__restrict__ row_kidx,
                          const int *__restrict__ le_ptr, const int *__restrict__ le_l, const int *__restrict__ le_e,
                          const double *__restrict__ a0, const double *__restrict__ a0k,
                          const double *__restrict__ a1, const double *__restrict__ a1k)
{
    const int p = blockIdx.y;
    const int e_in = blockIdx.x * blockDim.x + threadIdx.x;
    const int base = (pair_par[p] + 1) % 2;      /* the parity's first factor */
    if (e_in >= WB || base != a % 2) return;
    const int ia = (a - base) / 2;
    const int kk = row_kidx[pair_r[p]];
    double acc = 0.0;
    for (int k = le_ptr[p]; k < le_ptr[p + 1]; k++) {
        const int l = le_l[k], e = le_e[k];
        const R4<double>::T m = M[((size_t)l * nk + kk) * WB + e_in];
        acc = fma(m.a, a0[e], acc);
        acc = fma(m.b, a0k[e], acc);
        acc = fma(m.c, a1[e], acc);
        acc = fma(m.d, a1k[e], acc);
    }
    K[((size_t)p * 3 + ia) * WB + e_in] = acc;
}

/* this step's couplings A[pair] = sum_ia w_ia K[pair][ia], w_ia the
   imaginary part of the step's coefficient of order parity par(pair) and
   factor ia (coef[lpar * 3 + ia], lpar the first order of that parity).
   grid (element blocks of a pair, pairs); two values per thread */
struct A32Map {
    float *A32;                    /* NULL: no float copy */
    const int *row_pos;            /* [B]: chunk << 16 | row within the chunk */
    int B, W, RMp, npairs;
    size_t astride;                /* floats per pulse */
};

__global__ void k_assemble(double2 *__restrict__ A, A32Map F, const double2 *__restrict__ K, int WB2,
                           const int *__restrict__ pair_par, const double2 *__restrict__ coef, int2 lpar,
                           const int *__restrict__ plist, size_t astride2, size_t kstride2, int lmax)
{
    /* F.A32 (NULL: none): the values rounded to float for mixed precision,
       in the chunk-major layout of k_apply_asm32 ([q][pair][W][RMp]).
       grid z: pulse slot (plist: slot -> pulse); A per pulse, K per pulse
       (kstride2 0: shared by pulses with the same radial tables) */
    pdl_enter();
    const int pulse = plist ? plist[blockIdx.z] : 0;
    A += (size_t)pulse * astride2;
    float *A32 = F.A32 ? F.A32 + (size_t)pulse * F.astride : nullptr;
    K += (size_t)pulse * kstride2;
    coef += (size_t)pulse * lmax * 3;
    const int p = blockIdx.y;
    const int par = pair_par[p];
    const int cb = 3 * (par ? lpar.y : lpar.x);
    const double w0 = coef[cb].y, w1 = coef[cb + 1].y, w2 = coef[cb + 2].y;
    const double2 *Kp = K + (size_t)p * 3 * WB2;
    double2 *Ap = A + (size_t)p * WB2;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < WB2; e += gridDim.x * blockDim.x) {
        const double2 k0 = __ldcs(&Kp[e]), k1 = __ldcs(&Kp[WB2 + e]), k2 = __ldcs(&Kp[2 * WB2 + e]);
        double2 v;
        v.x = fma(w2, k2.x, fma(w1, k1.x, w0 * k0.x));
        v.y = fma(w2, k2.y, fma(w1, k1.y, w0 * k0.y));
        Ap[e] = v;
        if (A32) {
            /* values 2e and 2e+1 of the pair: slot t, rows i0 and i0 + 1 (B even) */
            const int e2 = 2 * e, t = e2 / F.B, i0 = e2 - t * F.B;
            const int rp0 = F.row_pos[i0], rp1 = F.row_pos[i0 + 1];
            float *d = A32 + ((size_t)p * F.W + t) * F.RMp;
            const size_t qs = (size_t)F.npairs * F.W * F.RMp;
            d[(size_t)(rp0 >> 16) * qs + (rp0 & 0xffff)] = (float)v.x;
            d[(size_t)(rp1 >> 16) * qs + (rp1 & 0xffff)] = (float)v.y;
        }
    }
}

#define ASM_GB 4   /* coupled blocks staged per phase */

/* shared memory of k_apply_asm: x slices (x_r, x_n, delta), the staged
   windows of ASM_GB coupled blocks, the slot map, the reduction buffer */
__host__ __device__ __forceinline__ unsigned asm_smem(int CS, int W, int RM, int nt, unsigned elem, unsigned *o_xw,
                                                      unsigned *o_lcs, unsigned *o_red)
{
    unsigned o = up32(3u * elem * CS);
    *o_xw = o;  o = up32(o + elem * ASM_GB * CS);
    *o_lcs = o; o = up32(o + 4u * W * RM);
    *o_red = o; o = up32(o + 8u * NRED * nt);
    return o;
}

/*
 * y = (S + H(t)) x with the assembled couplings: grid (pulse slot, segment)
 * over the same units and pieces as k_apply (a piece's range is a range of
 * (block row, coupled block) pairs).  Two threads per row, 15 ELL slots each
 * with their local columns in registers; per group of ASM_GB coupled blocks
 * the CTA stages the blocks' x windows in shared memory, then every thread
 * streams its rows' values and adds value x window[column].
 */
template <typename R, bool SEP>
__global__ void __launch_bounds__(256, 3)
    k_apply_asm(OpP P, const typename Cx<R>::T *__restrict__ x, int mode, VecP V, RedP red)
{
    /* R: double (FP64 values and vectors) or float (the complex64 inner solve
       of mixed precision, with the step's values rounded to float) */
    constexpr int HJ = 15;
    typedef typename Cx<R>::T C;
    extern __shared__ __align__(32) unsigned char smem_raw[];
    const int CS = (P.CM + 2) & ~1;
    unsigned oxw, olcs, ored;
    asm_smem(CS, P.W, P.RM, blockDim.x, sizeof(C), &oxw, &olcs, &ored);
    C *xr = (C *)smem_raw, *xs = xr + CS, *ds = xs + CS;
    C *xw = (C *)(smem_raw + oxw);
    int *lcs = (int *)(smem_raw + olcs);
    double *shred = (double *)(smem_raw + ored);

    pdl_enter();
    const int pulse = P.plist ? P.plist[blockIdx.x] : 0;
    if (!red_select(red, pulse)) return;
    x += (long long)pulse * P.vstride;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int B = P.B, W = P.W, CM = P.CM;
    if (tid == 0) {
        const C z = mk<C>(0, 0);
        xr[CM] = z; xs[CM] = z; ds[CM] = z;
        for (int g = 0; g < ASM_GB; g++) xw[g * CS + CM] = z;
    }
    __shared__ int s_pc, s_pw;
    for (int pc = P.seg_ptr[blockIdx.y]; pc < P.seg_ptr[blockIdx.y + 1]; pc = *(volatile int *)&s_pc + 1) {
    const int4 pd = P.pieces[pc];
    const int u = pd.x, r = u / P.nchunk, q = u - r * P.nchunk;
    const int kk = P.row_kidx[r];
    const int nrows = P.chunk_nrows[q], ncols = P.chunk_ncols[q];
    const int half = tid / P.RM, trow = tid - half * P.RM;
    const int i = (half < 2 && trow < nrows) ? P.chunk_rows[q * P.RM + trow] : -1;
    const int jb = half == 0 ? 0 : (W + 1) / 2, je = half == 0 ? (W + 1) / 2 : W;
    const int nj = je - jb;
    const int *cols = P.chunk_cols + (size_t)q * CM;
    const C *xb = x + (size_t)r * B;
    __syncthreads();                          /* the previous piece is done with shared memory */
    if (tid == 0) { s_pc = pc; s_pw = pd.w; } /* read back after the next barrier */
    {
        const int *gl = P.chunk_lcol + (size_t)q * W * P.RM;
        for (int e = tid; e < W * P.RM; e += nt) { const int v = gl[e]; lcs[e] = v < 0 ? CM : v; }
    }
    for (int c = tid; c < ncols; c += nt) xr[c] = xb[cols[c]];
    if (mode == AX_MIX) {
        const size_t vo = (size_t)pulse * P.vstride + (size_t)r * B;
        const C *xn = (const C *)V.in0 + vo, *dn = (const C *)V.in1 + vo;
        for (int c = tid; c < ncols; c += nt) { xs[c] = xn[cols[c]]; ds[c] = dn[cols[c]]; }
    }
    __syncthreads();
    unsigned lcp[(HJ + 1) / 2];
#pragma unroll
    for (int t = 0; t < HJ; t += 2) {
        const unsigned c0 = (t < nj && trow < P.RM) ? lcs[(jb + t) * P.RM + trow] : CM;
        const unsigned c1 = (t + 1 < HJ && t + 1 < nj && trow < P.RM) ? lcs[(jb + t + 1) * P.RM + trow] : CM;
        lcp[t / 2] = c0 | (c1 << 16);
    }
#define LCO(t) ((int)(((t) & 1) ? (lcp[(t) >> 1] >> 16) : (lcp[(t) >> 1] & 0xffffu)))
    const int jB = jb * B;
    C accS = mk<C>(0, 0), accH = accS, accD = accS;
    if (i >= 0 && (pd.w & 0xffff) == 0) {     /* diagonal blocks: the unit's first piece */
        if (SEP && mode == AX_MIX) {
            const C *Se = (const C *)P.S_ell + (size_t)kk * W * B + i + jB;
            const C *He = (const C *)P.Hst_ell + (size_t)pulse * P.dstride + (size_t)kk * W * B + i + jB;
#pragma unroll
            for (int t = 0; t < HJ; t++) {
                const int lc = LCO(t);
                const C sv = *Se;
                cfma(accS, sv, xs[lc]);
                cfma(accD, sv, ds[lc]);
                cfma(accH, *He, xr[lc]);
                if (t + 1 < nj) { Se += B; He += B; }
            }
        } else if (SEP) {
            const C *Se = (const C *)P.S_ell + (size_t)kk * W * B + i + jB;
            const C *He = (const C *)P.Hst_ell + (size_t)pulse * P.dstride + (size_t)kk * W * B + i + jB;
#pragma unroll
            for (int t = 0; t < HJ; t++) {
                const C xv = xr[LCO(t)];
                cfma(accS, *Se, xv);
                cfma(accH, *He, xv);
                if (t + 1 < nj) { Se += B; He += B; }
            }
        } else {
            const C *De = (const C *)P.D_ell + (size_t)pulse * P.dstride + (size_t)kk * W * B + i + jB;
#pragma unroll
            for (int t = 0; t < HJ; t++) {
                cfma(accH, *De, xr[LCO(t)]);
                if (t + 1 < nj) De += B;
            }
        }
    }
    const size_t WB = (size_t)W * B;
    for (int pg = pd.y; pg < pd.z; pg += ASM_GB) {
        const int ng = pd.z - pg < ASM_GB ? pd.z - pg : ASM_GB;
        __syncthreads();     /* staging done / previous group's products done */
        for (int item = tid; item < ng * ncols; item += nt) {
            const int g = item / ncols, c = item - g * ncols;
            xw[g * CS + c] = x[(size_t)P.pair_c[pg + g] * B + cols[c]];
        }
        __syncthreads();
        if (i >= 0) {
            const R *A0 = (const R *)P.A + (size_t)pulse * P.astride + (size_t)pg * WB + i + jB;
            if constexpr (sizeof(R) == 4) {
                /* complex64: latency-bound, so the next block's values are
                   loaded while this block's are used (two sets in flight) */
                R cur[HJ];
                {
                    const R *Av = A0;
#pragma unroll
                    for (int t = 0; t < HJ; t++) { cur[t] = __ldcs(Av); if (t + 1 < nj) Av += B; }
                }
                for (int g = 0; g < ng; g++) {
                    R nxt[HJ];
                    if (g + 1 < ng) {
                        const R *Av = A0 + (size_t)(g + 1) * WB;
#pragma unroll
                        for (int t = 0; t < HJ; t++) { nxt[t] = __ldcs(Av); if (t + 1 < nj) Av += B; }
                    }
                    const C *xg = xw + g * CS;
#pragma unroll
                    for (int t = 0; t < HJ; t++) rfma(accH, cur[t], xg[LCO(t)]);
#pragma unroll
                    for (int t = 0; t < HJ; t++) cur[t] = nxt[t];
                }
            } else {
                for (int g = 0; g < ng; g++) {
                    const R *Av = A0 + (size_t)g * WB;
                    const C *xg = xw + g * CS;
#pragma unroll
                    for (int t = 0; t < HJ; t++) {
                        rfma(accH, __ldcs(Av), xg[LCO(t)]);
                        if (t + 1 < nj) Av += B;
                    }
                }
            }
        }
    }
#undef LCO
    /* combine the two halves of every row */
    __syncthreads();
    {
        C *xch = (C *)shred;
        if (SEP) {
            if (half == 1 && i >= 0) { xch[3 * trow] = accS; xch[3 * trow + 1] = accH; xch[3 * trow + 2] = accD; }
            __syncthreads();
            if (half == 0 && i >= 0) {
                accS = cadd(accS, xch[3 * trow]);
                accH = cadd(accH, xch[3 * trow + 1]);
                accD = cadd(accD, xch[3 * trow + 2]);
            }
        } else {
            if (half == 1 && i >= 0) xch[trow] = accH;
            __syncthreads();
            if (half == 0 && i >= 0) accH = cadd(accH, xch[trow]);
        }
        __syncthreads();
    }
    const int pw = *(volatile int *)&s_pw;
    const int pi = pw & 0xffff, np = pw >> 16;
    if (np > 1) {
        const int pcc = *(volatile int *)&s_pc;
        __shared__ int piece_last;
        C *acc = (C *)P.piece_acc;
        const size_t RM3 = (size_t)3 * P.RM;
        if (half == 0 && i >= 0) {
            acc[pcc * RM3 + P.RM + trow] = accH;
            if (SEP) { acc[pcc * RM3 + trow] = accS; acc[pcc * RM3 + 2 * P.RM + trow] = accD; }
        }
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            const unsigned t = atomicAdd(&P.unit_tick[u], 1u);
            piece_last = (t == (unsigned)np - 1u);
        }
        __syncthreads();
        if (!piece_last) continue;
        __threadfence();
        if (half == 0 && i >= 0) {
            accS = mk<C>(0, 0); accH = accS; accD = accS;
            for (int k = 0; k < np; k++) {
                const size_t pk = (size_t)(pcc - pi + k) * RM3;
                accH = cadd(accH, __ldcg(&acc[pk + P.RM + trow]));
                if (SEP) {
                    accS = cadd(accS, __ldcg(&acc[pk + trow]));
                    accD = cadd(accD, __ldcg(&acc[pk + 2 * P.RM + trow]));
                }
            }
        }
        if (tid == 0) P.unit_tick[u] = 0u;
    }
    double v[NRED] = {0, 0, 0, 0};
    if (half == 0 && i >= 0) {
        const size_t gi = (size_t)pulse * P.vstride + (size_t)r * B + i;
        apply_epilogue<C, SEP>(mode, V, gi, accS, accH, accD, v);
    }
    if (red.kind != RED_NONE) reduce_part(red, v, shred, (unsigned)u);
    }
    if (red.kind != RED_NONE) reduce_tail(red, shred, gridDim.y, (unsigned)(P.nchunk * P.nblk));
}

/* ------------------------------------------------------------------ */
/* block-LU preconditioner, TMA-staged factors                          */
/* ------------------------------------------------------------------ */
/* Each sweep (L forward, then U backward) over the 32-row chunks c of a
 * block row is split into a part without dependences and a short chain:
 *   L:  x_c = Linv_c b_c + G_c  x_{c-1}[32-BWP .. 31],  G_c  = -Linv_c Lband_c
 *   U:  z_c = Uinv_c x_c + GU_c z_{c+1}[0 .. BWP-1],    GU_c = -Uinv_c Uband_c
 * (Lband_c / Uband_c: the band entries whose source row lies in the
 * neighbouring chunk; the band is at most BWP <= 32 wide).  Factor data of
 * one (pulse, kappa) and sweep is contiguous in HBM:
 *   [triangles: npair x 33 x 32][chain blocks: nch x BWP x 32]  (complex)
 * A triangle pair packs two chunks' inverse blocks so that lane i runs
 * 33 products with no zeros: for L, row i of chunk 2p (i+1 entries) then
 * row 31-i of chunk 2p+1 (32-i entries); for U, row i of chunk 2p (32-i
 * entries) then row 31-i of chunk 2p+1 (i+1 entries).  One elected lane
 * streams stage s+1 into shared memory with cp.async.bulk on an mbarrier
 * while the CTA computes stage s; every wait is bounded: on timeout the
 * kernel sets sc->err, drains its copies (bounded) and returns. */
struct PcT {
    int nblk, B, Bp, nch;
    const int *row_kidx, *ord;
    const void *FL, *FU;           /* [pulse][nk][sweep layout] complex of the kernel's precision */
    const int *plist;              /* grid x -> pulse (NULL: pulse 0) */
    long long vstride;             /* complex elements per pulse of every vector */
    size_t fstride;                /* complex elements per pulse of FL / FU */
    int pred;                      /* PRED_* */
    unsigned spin_limit;           /* polls of a stage wait before the kernel gives up */
    int withhold;                  /* failure injection: stage whose copy is not issued (-1: none) */
};

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ void tma_bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

#define MBAR_SPIN_LIMIT (1u << 22)

/* complex elements of one triangle pair and of one chunk's chain block */
#define PC_TP (33 * 32)
__host__ __device__ __forceinline__ size_t pc_sweep_elems(int nch, int bwp)
{
    return (size_t)((nch + 1) / 2) * PC_TP + (size_t)nch * 32 * bwp;
}
/* staging buffer of one stage: up to 4 triangle pairs or PC_GCH chain blocks */
#define PC_GCH 4
__host__ __device__ __forceinline__ int pc_stage_elems(int bwp)
{
    return 4 * PC_TP > PC_GCH * 32 * bwp ? 4 * PC_TP : PC_GCH * 32 * bwp;
}

/* NW (4 or 8) warps per block row, one or two per SM sub-partition (each
 * has its own FP64 unit).  Triangle stages: the stage's pair w % 4 goes to
 * warp w; with 8 warps warps w and w + 4 split its 33 products per lane
 * (products 0-16 and 17-32), each keeping the parts of the two output rows
 * apart, and the first adds the second's parts.  Chain steps: warp w
 * applies chain columns w BWP/NW .. (w+1) BWP/NW - 1 to every row; the
 * partial sums meet in shared memory and are combined once per row, spread
 * over all warps (two adds per lane, then a shuffle over NW/2 lanes). */
template <typename R, int NW, int Q0, int Q1>
__device__ __forceinline__ void pc_triangle_part(const typename Cx<R>::T *__restrict__ T,
                                                 const typename Cx<R>::T *buf, int lane, int c0, int c1, bool has1,
                                                 bool up, typename Cx<R>::T &p0, typename Cx<R>::T &p1)
{
    typedef typename Cx<R>::T C;
    const int sw = up ? 31 - lane : lane;      /* last product of the first row */
    C acc = mk<C>(0, 0), sav = acc;
#pragma unroll
    for (int q = Q0; q < Q1; q++) {
        int src;
        if (!up) src = q <= lane ? 32 * c0 + q : (has1 ? 32 * c1 + q - lane - 1 : 0);
        else src = q <= 31 - lane ? 32 * c0 + lane + q : (has1 ? 32 * c1 + q - 1 : 0);
        cfma(acc, T[q * 32 + lane], buf[src]);
        if (q == sw) { sav = acc; acc = mk<C>(0, 0); }
    }
    /* the products of row c0 are those up to sw */
    if (sw >= Q1) { p0 = acc; p1 = mk<C>(0, 0); }
    else if (sw >= Q0) { p0 = sav; p1 = acc; }
    else { p0 = mk<C>(0, 0); p1 = acc; }
}

template <typename R, int BWP, int NW>
__global__ void __launch_bounds__(NW * 32) k_precond_tma(PcT Q, int mode, const typename Cx<R>::T *__restrict__ in0,
                                                         const typename Cx<R>::T *__restrict__ in1,
                                                         typename Cx<R>::T *io, typename Cx<R>::T *__restrict__ out,
                                                         DevScal *sc)
{
    typedef typename Cx<R>::T C;
    static_assert(NW == 4 || NW == 8, "4 or 8 warps");
    constexpr int NT = NW * 32;
    constexpr int GC = 32 * BWP;                 /* complex elements of one chain block */
    constexpr int CPW = BWP / NW;                /* chain columns per warp */
    constexpr int PARTS = NW / 2;                /* lanes that combine one row component */
    const int SB = pc_stage_elems(BWP);
    extern __shared__ __align__(128) unsigned char smem_tma[];
    C *stg = (C *)smem_tma;                /* [2][SB] */
    C *buf = stg + 2 * SB;                 /* [Bp]    */
    C *pt = buf + Q.Bp;                    /* [NW][32] chain partial sums / [4][2][32] triangle parts */
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int all_ok;
    pdl_enter();
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    /* combining thread: row tid / NW, component (tid / PARTS) & 1, part tid % PARTS */
    const int crow = tid / NW, ccomp = (tid / PARTS) & 1, cpart = tid % PARTS;
    const int r = blockIdx.y;
    if (r >= Q.nblk) return;
    const int pulse = Q.plist ? Q.plist[blockIdx.x] : 0;
    sc += pulse;
    if (Q.pred != PRED_NONE) {
        const int st = *(volatile const int *)&sc->state;
        if (Q.pred == PRED_RUN ? st != ST_RUN : st != ST_RESTART) return;
    }
    {
        const long long vo = (long long)pulse * Q.vstride;
        in0 += vo;
        if (in1) in1 += vo;
        if (io) io += vo;
        out += vo;
    }
    const int B = Q.B, Bp = Q.Bp, nch = Q.nch;
    const int npair = (nch + 1) / 2;
    const int nsa = (npair + 3) / 4, nsg = (nch + PC_GCH - 1) / PC_GCH, nps = nsa + nsg;
    const int ns = 2 * nps;                 /* stages: L triangles, L chain, U triangles, U chain */
    const int kk = Q.row_kidx[r];
    const size_t off = (size_t)r * B;
    const size_t per = pc_sweep_elems(nch, BWP);
    const C *FL = (const C *)Q.FL + (size_t)pulse * Q.fstride + (size_t)kk * per;
    const C *FU = (const C *)Q.FU + (size_t)pulse * Q.fstride + (size_t)kk * per;
    /* source and size of stage k; the U chain runs its groups last to first */
    auto stage = [&](int k, const C **src, int *cnt) {
        const C *F = k < nps ? FL : FU;
        const int j = k < nps ? k : k - nps;
        if (j < nsa) {
            *cnt = min(4, npair - 4 * j);
            *src = F + (size_t)4 * j * PC_TP;
            return (unsigned)(*cnt * PC_TP * sizeof(C));
        }
        const int g = k < nps ? j - nsa : nsg - 1 - (j - nsa);
        *cnt = min(PC_GCH, nch - g * PC_GCH);
        *src = F + (size_t)npair * PC_TP + (size_t)g * PC_GCH * GC;
        return (unsigned)(*cnt * GC * sizeof(C));
    };

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        const C *src;
        int cnt;
        const unsigned bytes = stage(0, &src, &cnt);
        if (Q.withhold != 0) tma_bulk_load(stg, src, bytes, &bar[0]);
        all_ok = 1;
    }

    C beta = mk<C>(0, 0), negw = mk<C>(0, 0), nega = mk<C>(0, 0);
    if (mode == PC_P) {
        const double2 a = cdiv(sc->rho, sc->rho_prev);
        const double2 b = cdiv(sc->alpha, sc->w);
        beta = mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
        negw = mk<C>(-sc->w.x, -sc->w.y);
    } else if (mode == PC_S) {
        nega = mk<C>(-sc->alpha.x, -sc->alpha.y);
    }
    for (int o = tid; o < Bp; o += NT) {
        C val = mk<C>(0, 0);
        if (o < B) {
            const size_t gi = off + Q.ord[o];
            if (mode == PC_PLAIN) {
                val = in0[gi];
            } else if (mode == PC_P) {
                C t = io[gi];
                cfma(t, negw, in1[gi]);
                C pv = in0[gi];
                cfma(pv, beta, t);
                io[gi] = pv;
                val = pv;
            } else {
                C sv = in0[gi];
                cfma(sv, nega, in1[gi]);
                io[gi] = sv;
                val = sv;
            }
        }
        buf[o] = val;
    }
    __syncthreads();

    int k = 0;
    for (; k < ns; k++) {
        if (tid == 0 && k + 1 < ns && k + 1 != Q.withhold) {
            const C *src;
            int cnt;
            const unsigned bytes = stage(k + 1, &src, &cnt);
            tma_bulk_load(stg + ((k + 1) & 1) * SB, src, bytes, &bar[(k + 1) & 1]);
        }
        unsigned spins = 0;
        bool ok = true;
        while (!mbar_try_wait(&bar[k & 1], (k >> 1) & 1)) {
            if (++spins > Q.spin_limit) { ok = false; break; }
        }
        if (!ok) all_ok = 0;
        __syncthreads();
        if (!all_ok) break;
        const C *S = stg + (k & 1) * SB;
        const int up = k >= nps;                   /* U sweep */
        const int j = up ? k - nps : k;
        if (j < nsa) {
            /* triangle pair 4 j + wid % 4: chunks c0 = 2p, c1 = 2p + 1 */
            const int w4 = wid & 3, half = wid >> 2;
            const int p = 4 * j + w4;
            const bool act = p < npair;
            const int c0 = 2 * p, c1 = 2 * p + 1;
            const bool has1 = c1 < nch;
            C p0 = mk<C>(0, 0), p1 = p0;
            if (act) {
                const C *T = S + w4 * PC_TP;
                if (NW == 4) pc_triangle_part<R, NW, 0, 33>(T, buf, lane, c0, c1, has1, up, p0, p1);
                else if (half == 0) pc_triangle_part<R, NW, 0, 17>(T, buf, lane, c0, c1, has1, up, p0, p1);
                else pc_triangle_part<R, NW, 17, 33>(T, buf, lane, c0, c1, has1, up, p0, p1);
            }
            if (NW == 8) {
                if (half == 1 && act) {
                    pt[(w4 * 2) * 32 + lane] = p0;
                    pt[(w4 * 2 + 1) * 32 + lane] = p1;
                }
                __syncthreads();                   /* every read of buf of this stage is done */
                if (half == 0 && act) {
                    const C q0 = pt[(w4 * 2) * 32 + lane], q1 = pt[(w4 * 2 + 1) * 32 + lane];
                    p0 = mk<C>(p0.x + q0.x, p0.y + q0.y);
                    p1 = mk<C>(p1.x + q1.x, p1.y + q1.y);
                }
            } else {
                __syncwarp();
            }
            if (half == 0 && act) {
                /* row lane of chunk c0, row 31 - lane of chunk c1 */
                buf[32 * c0 + lane] = p0;
                if (has1) buf[32 * c1 + 31 - lane] = p1;
            }
            __syncthreads();
        } else {
            const int g = up ? nsg - 1 - (j - nsa) : j - nsa;
            const int cnt = min(PC_GCH, nch - g * PC_GCH);
            for (int e = 0; e < cnt; e++) {
                const int ci = up ? cnt - 1 - e : e;     /* U: last chunk first */
                const int c = g * PC_GCH + ci;
                if (up ? c == nch - 1 : c == 0) continue;  /* no neighbour: the triangle result stands */
                const C *G = S + ci * GC;
                const int base = up ? 32 * (c + 1) : 32 * c - BWP;
                C t = (wid == 0) ? buf[32 * c + lane] : mk<C>(0, 0);
#pragma unroll
                for (int q = 0; q < CPW; q++) {
                    const int col = wid * CPW + q;
                    cfma(t, G[col * 32 + lane], buf[base + col]);
                }
                pt[wid * 32 + lane] = t;
                __syncthreads();
                {
                    /* the row's sum over the NW partials, once: a thread adds two
                       partials of one component, a shuffle over PARTS lanes the rest */
                    const R *pr = (const R *)pt;
                    R sum = pr[((2 * cpart) * 32 + crow) * 2 + ccomp] + pr[((2 * cpart + 1) * 32 + crow) * 2 + ccomp];
#pragma unroll
                    for (int o = 1; o < PARTS; o <<= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
                    if (cpart == 0) ((R *)buf)[(32 * c + crow) * 2 + ccomp] = sum;
                }
                __syncthreads();
            }
        }
    }
    if (!all_ok) {
        if (tid == 0) {
            atomicOr(&sc->err, 1u);
            /* drain the copies still in flight (bounded) before exiting: the
               stage that timed out and the next one, both issued unless withheld */
            for (int k2 = k; k2 < k + 2 && k2 < ns; k2++) {
                if (k2 == Q.withhold) continue;
                unsigned spins = 0;
                while (!mbar_try_wait(&bar[k2 & 1], (k2 >> 1) & 1) && ++spins < MBAR_SPIN_LIMIT) {
                }
            }
        }
        __syncthreads();
        return;
    }
    for (int o = tid; o < B; o += NT) out[off + Q.ord[o]] = buf[o];
}

/* ------------------------------------------------------------------ */
/* assembled operator, complex64, values streamed by cp.async.bulk      */
/* ------------------------------------------------------------------ */
/*
 * The complex64 apply of the mixed step's inner solve (and of mixed
 * batches) with this step's values rounded to float.  The values are laid
 * out chunk-major, [pulse][chunk q][pair][slot W][row RMp], so that what one
 * unit (chunk q, block row r) needs of one coupled block is one contiguous
 * W x RMp run; with the coupled block's x (B complex64, contiguous) it forms
 * one stage.  One elected thread keeps A32_NST stages in flight with
 * cp.async.bulk on one mbarrier each while the CTA multiplies the oldest,
 * so the value stream no longer waits on per-thread load latency.  Threads,
 * rows, slots, pieces and epilogue are those of k_apply_asm (two threads per
 * row, 15 slots each, columns held in registers as indices into the staged
 * block; index B is a zero).  Every stage wait is bounded: on a timeout the
 * CTA sets bit 1 of the record's error word, waits (bounded) for the copies
 * it issued and finishes its pieces without the products, so the launch's
 * reductions stay consistent.
 */
#ifndef A32_NST
#define A32_NST 3
#endif

__host__ __device__ __forceinline__ unsigned up128(unsigned o) { return (o + 127u) & ~127u; }

/* shared memory of k_apply_asm32: stages [A32_NST][values | x block], the
   unit's own x block, the reduction buffer */
__host__ __device__ __forceinline__ unsigned a32_smem(int W, int RMp, int B, int nt, int mp, unsigned *o_vb,
                                                      unsigned *o_sb, unsigned *o_xr, unsigned *o_red, unsigned *o_pl)
{
    const unsigned vb = up128(4u * W * RMp), sb = vb + up128(8u * (B + 1));
    *o_vb = vb; *o_sb = sb;
    unsigned o = A32_NST * sb;
    *o_xr = o;  o += up128(8u * (B + 1));
    *o_red = o; o += up128(8u * NRED * nt);
    *o_pl = o;  o += up128(4u * mp);
    return o;
}

/* one stage: the W x RMp values of (chunk q, pair p) and the x block of the
   pair's coupled column block, both completing on bar */
__device__ __forceinline__ void a32_issue(unsigned char *dst, unsigned vb, const float *src_v, unsigned vbytes,
                                          const float2 *src_x, unsigned xbytes, uint64_t *bar)
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(vbytes + xbytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)), "l"(src_v), "r"(vbytes), "r"(smem_u32(bar))
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst + vb)), "l"(src_x), "r"(xbytes), "r"(smem_u32(bar))
                 : "memory");
}

__global__ void __launch_bounds__(256, 3)
    k_apply_asm32(OpP P, const float2 *__restrict__ x, int mode, VecP V, RedP red, int RMp, int npairs, int mp)
{
    constexpr int HJ = 15;
    typedef float2 C;
    extern __shared__ __align__(128) unsigned char smem_a32[];
    const int W = P.W, B = P.B;
    unsigned VB, SB, oxr, ored, opl;
    a32_smem(W, RMp, B, blockDim.x, mp, &VB, &SB, &oxr, &ored, &opl);
    C *xr = (C *)(smem_a32 + oxr);
    double *shred = (double *)(smem_a32 + ored);
    int *pcl = (int *)(smem_a32 + opl);       /* [mp] coupled block of each pair of the piece */
    __shared__ __align__(8) uint64_t bar[A32_NST];
    __shared__ int s_pc, s_pw, s_fail;

    pdl_enter();
    const int pulse = P.plist ? P.plist[blockIdx.x] : 0;
    if (!red_select(red, pulse)) return;
    x += (long long)pulse * P.vstride;
    const float *A = (const float *)P.A + (size_t)pulse * P.astride;
    const size_t qstride = (size_t)npairs * W * RMp;        /* floats of one chunk's pairs */
    const unsigned vbytes = 4u * W * RMp, xbytes = 8u * B;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (tid == 0) {
        for (int b = 0; b < A32_NST; b++) mbar_init(&bar[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
    }
    /* the zero column of every x block (index B; the copies fill 0..B-1) */
    if (tid < A32_NST) ((C *)(smem_a32 + tid * SB + VB))[B] = mk<C>(0, 0);
    if (tid == A32_NST) xr[B] = mk<C>(0, 0);
    unsigned gs = 0;                 /* stages this CTA has issued and consumed (uniform) */
    for (int pc = P.seg_ptr[blockIdx.y]; pc < P.seg_ptr[blockIdx.y + 1]; pc = *(volatile int *)&s_pc + 1) {
    const int4 pd = P.pieces[pc];
    const int u = pd.x, r = u / P.nchunk, q = u - r * P.nchunk;
    const int kk = P.row_kidx[r];
    const int nrows = P.chunk_nrows[q];
    const int half = tid / P.RM, trow = tid - half * P.RM;
    const int i = (half < 2 && trow < nrows) ? P.chunk_rows[q * P.RM + trow] : -1;
    const int jb = half == 0 ? 0 : (W + 1) / 2, je = half == 0 ? (W + 1) / 2 : W;
    const int nj = je - jb;
    const int p0 = pd.y, np = pd.z - pd.y;
    __syncthreads();                          /* the previous piece is done with shared memory */
    const bool failed = *(volatile int *)&s_fail != 0;
    if (tid == 0) {
        s_pc = pc; s_pw = pd.w;               /* read back after the next barrier */
        if (!failed)
            for (int k = 0; k < np && k < A32_NST; k++) {
                const unsigned g = gs + k, b = g % A32_NST;
                const int pp = p0 + k;
                a32_issue(smem_a32 + b * SB, VB, A + (size_t)q * qstride + (size_t)pp * W * RMp, vbytes,
                          x + (size_t)P.pair_c[pp] * B, xbytes, &bar[b]);
            }
    }
    /* the piece's coupled blocks (read by the refills), the unit's own x
       block (diagonal blocks) and the thread's slot columns */
    for (int k = tid; k < np; k += nt) pcl[k] = P.pair_c[p0 + k];
    {
        const C *xb = x + (size_t)r * B;
        for (int c = tid; c < B; c += nt) xr[c] = xb[c];
    }
    unsigned lcp[(HJ + 1) / 2];
    {
        const unsigned short *ac = P.chunk_acol + (size_t)q * W * P.RM;
#pragma unroll
        for (int t = 0; t < HJ; t += 2) {
            const unsigned c0 = (t < nj && trow < P.RM) ? ac[(jb + t) * P.RM + trow] : (unsigned)B;
            const unsigned c1 = (t + 1 < nj && trow < P.RM) ? ac[(jb + t + 1) * P.RM + trow] : (unsigned)B;
            lcp[t / 2] = c0 | (c1 << 16);
        }
    }
#define LCO(t) ((int)(((t) & 1) ? (lcp[(t) >> 1] >> 16) : (lcp[(t) >> 1] & 0xffffu)))
    __syncthreads();                          /* xr complete */
    C accH = mk<C>(0, 0);
    if (i >= 0 && (pd.w & 0xffff) == 0) {     /* diagonal blocks: the unit's first piece */
        const C *De = (const C *)P.D_ell + (size_t)pulse * P.dstride + (size_t)kk * W * B + i + (size_t)jb * B;
#pragma unroll
        for (int t = 0; t < HJ; t++) {
            if (t < nj) cfma(accH, *De, xr[LCO(t)]);
            if (t + 1 < nj) De += B;
        }
    }
    for (int k = 0; k < np && !failed; k++) {
        const unsigned g = gs + k, b = g % A32_NST;
        bool ok = true;
        {
            unsigned spins = 0;
            while (!mbar_try_wait(&bar[b], (g / A32_NST) & 1u)) {
                if (++spins > MBAR_SPIN_LIMIT) { ok = false; break; }
            }
        }
        if (ok && i >= 0) {
            const float *vs = (const float *)(smem_a32 + b * SB) + (size_t)jb * RMp + trow;
            const C *xs = (const C *)(smem_a32 + b * SB + VB);
#pragma unroll
            for (int t = 0; t < HJ; t++)
                if (t < nj) rfma(accH, vs[(size_t)t * RMp], xs[LCO(t)]);
        }
        if (__syncthreads_or(!ok)) {          /* uniform: some wait ran out */
            if (tid == 0) {
                atomicOr(&red.sc->err, 2u);
                /* the copies still in flight: stages k .. min(np, k + A32_NST) - 1 */
                for (int k2 = k; k2 < np && k2 < k + A32_NST; k2++) {
                    const unsigned g2 = gs + k2;
                    unsigned spins = 0;
                    while (!mbar_try_wait(&bar[g2 % A32_NST], (g2 / A32_NST) & 1u) && ++spins < MBAR_SPIN_LIMIT) {
                    }
                }
                s_fail = 1;
            }
            break;
        }
        if (tid == 0 && k + A32_NST < np) {     /* refill the freed buffer */
            const int kk2 = k + A32_NST;
            a32_issue(smem_a32 + b * SB, VB, A + (size_t)q * qstride + (size_t)(p0 + kk2) * W * RMp, vbytes,
                      x + (size_t)pcl[kk2] * B, xbytes, &bar[b]);
        }
    }
    gs += np;
#undef LCO
    /* combine the two halves of every row */
    __syncthreads();
    {
        C *xch = (C *)shred;
        if (half == 1 && i >= 0) xch[trow] = accH;
        __syncthreads();
        if (half == 0 && i >= 0) accH = cadd(accH, xch[trow]);
        __syncthreads();
    }
    const int pw = *(volatile int *)&s_pw;
    const int pi = pw & 0xffff, npc = pw >> 16;
    if (npc > 1) {
        const int pcc = *(volatile int *)&s_pc;
        __shared__ int piece_last;
        C *acc = (C *)P.piece_acc;
        const size_t RM3 = (size_t)3 * P.RM;
        if (half == 0 && i >= 0) acc[pcc * RM3 + P.RM + trow] = accH;
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            const unsigned t = atomicAdd(&P.unit_tick[u], 1u);
            piece_last = (t == (unsigned)npc - 1u);
        }
        __syncthreads();
        if (!piece_last) continue;
        __threadfence();
        if (half == 0 && i >= 0) {
            accH = mk<C>(0, 0);
            for (int k = 0; k < npc; k++)
                accH = cadd(accH, __ldcg(&acc[(size_t)(pcc - pi + k) * RM3 + P.RM + trow]));
        }
        if (tid == 0) P.unit_tick[u] = 0u;
    }
    double v[NRED] = {0, 0, 0, 0};
    if (half == 0 && i >= 0) {
        const size_t gi = (size_t)pulse * P.vstride + (size_t)r * B + i;
        apply_epilogue<C, false>(mode, V, gi, accH, accH, accH, v);
    }
    if (red.kind != RED_NONE) reduce_part(red, v, shred, (unsigned)u);
    }
    if (red.kind != RED_NONE) reduce_tail(red, shred, gridDim.y, (unsigned)(P.nchunk * P.nblk));
}

/* ------------------------------------------------------------------ */
/* x += alpha y + w z ; r = s - w t ; |r|^2, <r0, r>                    */
/* ------------------------------------------------------------------ */
/* grid (CTAs per pulse, pulse slot); plist maps the slot to the pulse and
   n is also the per-pulse vector stride */
template <typename R>
__global__ void k_update(long long n, typename Cx<R>::T *x, const typename Cx<R>::T *__restrict__ y,
                         const typename Cx<R>::T *__restrict__ z, typename Cx<R>::T *r,
                         const typename Cx<R>::T *__restrict__ s, const typename Cx<R>::T *__restrict__ t,
                         const typename Cx<R>::T *__restrict__ r0, RedP red, const int *plist)
{
    typedef typename Cx<R>::T C;
    extern __shared__ unsigned char smem_raw[];
    double *shred = (double *)smem_raw;
    pdl_enter();
    const int pulse = plist ? plist[blockIdx.y] : 0;
    if (!red_select(red, pulse)) return;
    {
        const long long vo = (long long)pulse * n;
        x += vo; y += vo; z += vo; r += vo; s += vo; t += vo; r0 += vo;
    }
    const double2 al = red.sc->alpha, w = red.sc->w;
    const C a = mk<C>(al.x, al.y), wc = mk<C>(w.x, w.y), nw = mk<C>(-w.x, -w.y);
    double v[NRED] = {0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        C zz = cmul(a, y[i]);
        cfma(zz, wc, z[i]);
        x[i] = cadd(x[i], zz);
        C rv = s[i];
        cfma(rv, nw, t[i]);
        r[i] = rv;
        const C q = r0[i];
        v[0] += (double)rv.x * rv.x + (double)rv.y * rv.y;
        v[1] += (double)q.x * rv.x + (double)q.y * rv.y;
        v[2] += (double)q.x * rv.y - (double)q.y * rv.x;
    }
    reduce_finish(red, v, shred, gridDim.x, blockIdx.x);
}

/* ------------------------------------------------------------------ */
/* mixed precision: complex64 inner solves inside FP64 refinement      */
/* ------------------------------------------------------------------ */
/* Per-pulse base of the mixed-precision vector kernels: grid (CTAs per
   pulse, pulse slot), n is also the per-pulse stride.  Returns the pulse or
   -1 when the predicate says the launch has nothing to do for it. */
__device__ __forceinline__ int bp_select(BPred &bp)
{
    const int pulse = bp.plist ? bp.plist[blockIdx.y] : 0;
    if (bp.a) bp.a += pulse;
    if (bp.b) bp.b += pulse;
    return pred_ok(bp.pred, bp.a, bp.b) ? pulse : -1;
}

/* delta = x - x_prev (linear extrapolation of the state) or 0; FP32 copies.
   hprev[pulse] says whether x_prev exists.
   Under device control the first CTA also opens the step's records. */
/* double-float copies of the residual pass's inputs (NULL: none) */
struct DdVec { cdd *x, *d, *w; };

__global__ void k_mixed_prep(long long n, const double2 *__restrict__ x, const double2 *__restrict__ xprev,
                             const int *__restrict__ hprev, double2 *__restrict__ d64,
                             float2 *__restrict__ d32, double2 *__restrict__ w, BPred bp,
                             const double2 *__restrict__ corr, DdVec Q)
{
    const int pulse = bp_select(bp);
    if (pulse < 0) return;
    {
        const long long vo = (long long)pulse * n;
        x += vo; xprev += vo; d64 += vo; d32 += vo; w += vo;
        if (corr) corr += vo;
        if (Q.x) { Q.x += vo; Q.d += vo; Q.w += vo; }
    }
    const int have_prev = hprev[pulse];
    if (blockIdx.x == 0 && threadIdx.x == 0 && bp.a && bp.a->ctl == 1) {
        DevScal *a = bp.a;
        a->state = ST_RUN; a->pending = 0; a->sweeps = 0; a->refinements = 0; a->inner_total = 0;
        a->stalled = 0;
        bp.b->state = ST_DONE;
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double2 xv = x[i];
        double2 d = make_double2(0, 0);
        if (have_prev) {
            const double2 xp = xprev[i];
            d = make_double2(xv.x - xp.x, xv.y - xp.y);
            if (corr) { const double2 c = corr[i]; d.x += c.x; d.y += c.y; }
        }
        d64[i] = d;
        d32[i] = make_float2((float)d.x, (float)d.y);
        const double2 wv = make_double2(2.0 * xv.x + d.x, 2.0 * xv.y + d.y);
        w[i] = wv;
        if (Q.x) { Q.x[i] = cdd_from(xv); Q.d[i] = cdd_from(d); Q.w[i] = cdd_from(wv); }
    }
}

/* inner BiCGSTAB start from the FP64 refinement residual:
   e = 0, r = r0 = (complex64) rin, p = v = 0, |r|^2 */
__global__ void k_inner_init(long long n, const double2 *__restrict__ rin, float2 *e, float2 *r, float2 *r0,
                             float2 *p, float2 *v, RedP red, const int *plist)
{
    extern __shared__ unsigned char smem_raw[];
    double *shred = (double *)smem_raw;
    const int pulse = plist ? plist[blockIdx.y] : 0;
    if (!red_select(red, pulse)) return;
    {
        const long long vo = (long long)pulse * n;
        rin += vo; e += vo; r += vo; r0 += vo; p += vo; v += vo;
    }
    double acc[NRED] = {0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double2 rd = rin[i];
        const float2 rv = make_float2((float)rd.x, (float)rd.y);
        r[i] = rv; r0[i] = rv;
        e[i] = make_float2(0, 0); p[i] = make_float2(0, 0); v[i] = make_float2(0, 0);
        acc[0] += (double)rv.x * rv.x + (double)rv.y * rv.y;
    }
    acc[1] = acc[0];
    reduce_finish(red, acc, shred, gridDim.x, blockIdx.x);
}

/* delta += e (FP64), refresh the FP32 copy and w = 2 x_n + delta */
__global__ void k_delta_add(long long n, double2 *__restrict__ d64, const float2 *__restrict__ e,
                            float2 *__restrict__ d32, const double2 *__restrict__ x, double2 *__restrict__ w,
                            BPred bp, DdVec Q)
{
    const int pulse = bp_select(bp);
    if (pulse < 0) return;
    {
        const long long vo = (long long)pulse * n;
        d64 += vo; e += vo; d32 += vo; x += vo; w += vo;
        if (Q.x) { Q.d += vo; Q.w += vo; }
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 ev = e[i];
        double2 d = d64[i];
        d.x += (double)ev.x; d.y += (double)ev.y;
        d64[i] = d;
        d32[i] = make_float2((float)d.x, (float)d.y);
        const double2 xv = x[i];
        const double2 wv = make_double2(2.0 * xv.x + d.x, 2.0 * xv.y + d.y);
        w[i] = wv;
        if (Q.x) { Q.d[i] = cdd_from(d); Q.w[i] = cdd_from(wv); }
    }
}

/* x_prev = x ; x += delta (FP64); the pulse now has an x_prev */
__global__ void k_mixed_finish(long long n, double2 *__restrict__ x, double2 *__restrict__ xprev,
                               const double2 *__restrict__ d64, int *hprev, BPred bp)
{
    const int pulse = bp_select(bp);
    if (pulse < 0) return;
    {
        const long long vo = (long long)pulse * n;
        x += vo; xprev += vo; d64 += vo;
    }
    if (hprev && blockIdx.x == 0 && threadIdx.x == 0) hprev[pulse] = 1;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double2 xv = x[i], d = d64[i];
        xprev[i] = xv;
        x[i] = make_double2(xv.x + d.x, xv.y + d.y);
    }
}

/* After an inner solve and its delta update (device control): the inner
   estimate of the outer residual certifies the step when it is below the
   tolerance with margin (the host rule of the single-pulse mixed step);
   otherwise the next FP64 residual pass decides.  grid (1, pulse slots). */
__global__ void k_mixed_ctl(BPred bp)
{
    if (threadIdx.x != 0) return;
    if (bp_select(bp) < 0) return;
    DevScal *a = bp.a;
    const DevScal *b = bp.b;
    a->pending = 0;
    a->inner_total += b->iter;
    const double rin = b->rr, est = 1e-14 * b->r0_sqnorm;
    const double tol2 = a->tol2rel * a->rhs_sqnorm;
    if (isfinite(rin) && rin + est < 0.25 * tol2) {
        a->rr = rin + est;
        a->state = ST_DONE;
    }
}

/* ------------------------------------------------------------------ */
/* solver object                                                       */
/* ------------------------------------------------------------------ */
/* one partition of the operator's units into CTA segments (see OpP) */
struct PartList {
    int nseg = 0, npieces = 0;
    int multi = 0;              /* some unit has more than one piece */
    int *d_seg_ptr = nullptr;
    int4 *d_pieces = nullptr;
};

struct gade_solver {
    int device;
    cudaStream_t stream;
    int prec, rc;
    long long n;                /* unknowns of one pulse (also the per-pulse vector stride) */
    int nblk, B, lmax, W, nk, RM, CM, nchunk, AM;
    int bw, Bp, nch;
    double dt, h;               /* dt of pulse 0 */
    /* pulses: every per-pulse array holds npulse slices; kernels run over
       the nslot pulses listed in d_plist (NULL: pulse 0 alone) */
    int npulse, nslot, cs;
    int *d_plist;
    size_t mstride, dstride, fstride, gstride, pstride;
    std::vector<double> dts;
    /* operator tables */
    int *d_row_kidx, *d_act_ptr, *d_act_l, *d_ang_ptr, *d_ang_c;
    void *d_ang_a0, *d_ang_a0k, *d_ang_a1, *d_ang_a1k;
    int *d_chunk_nrows, *d_chunk_ncols, *d_chunk_rows, *d_chunk_cols, *d_chunk_lcol;
    unsigned short *d_chunk_acol;
    void *d_M, *d_S_ell, *d_Hst_ell, *d_D_ell;
    double *d_kvals;            /* the distinct kappa values, as doubles for the table kernel */
    void *d_g, *d_gt;
    int blk_nnz;
    /* preconditioner */
    int *d_ord;
    double2 *d_FL, *d_FU;       /* chunk-packed factors for the TMA kernel */
    int bwp;
    /* vectors */
    double2 *x, *rhs, *r, *r0, *p, *v, *y, *z, *s, *t, *tmp0, *tmp1;
    /* reductions */
    double *d_part;
    size_t part_cap;            /* doubles allocated in d_part */
    unsigned int *d_ticket;
    DevScal *d_sc, *h_sc;
    double2 *d_coef, *h_coef;
    int upd_grid, upd_block;
    long long launches;
    int has_time;
    std::vector<void *> allocs;
    /* event-pair profiling: kind 0 apply, 1 precond, 2 other */
    int profile;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<int> ev_kind;
    size_t ev_used;
    long long prof_n[3];
    double prof_ms[3];
    double apply_flops, precond_flops;   /* FP64 flops of one launch */
    double apply_bytes;                  /* compulsory DRAM bytes of one FP64 BiCGSTAB apply */
    /* mixed precision (GADE_PREC_MIXED) */
    void *d_M32, *d_S32, *d_H32, *d_D32;
    void *d_a32[4];
    void *d_FL32, *d_FU32;
    float2 *x32, *d32, *q32, *r32, *e32, *ri32, *r032, *p32, *v32, *y32, *z32, *s32, *t32;
    double2 *xprev, *delta64;
    DevScal *d_sc2, *h_sc2;
    int *d_hprev;               /* [pulse] x_prev exists (batched mixed precision) */
    /* partition of the operator's work into CTAs (single-pulse solvers):
       order split 1-4 (nsplit) or balanced segments (nsplit 0, one list per
       resident-CTAs-per-SM count of the kernel instance) */
    int nsplit;
    int nsm;
    float split_ms[5];          /* timed FP64 (+ complex64) applies: [0] balanced, [1..4] order splits */
    PartList part_split[5];
    PartList part_bal[9];
    int occ[2][2];              /* resident CTAs per SM of the operator instances [complex64][sep] */
    void *d_piece_acc;
    size_t piece_cap;           /* pieces the partial-sum scratch holds */
    unsigned int *d_unit_tick;
    /* host copy of the work model: active orders per block row, their
       angular term counts, rows and columns per chunk */
    std::vector<int> h_act_ptr, h_act_ne, h_chunk_nrows, h_chunk_ncols;
    double bal_gamma;           /* weight of the gather in the balanced cost model (timed at creation) */
    int bal_waves;              /* balanced segments per resident CTA slot (timed at creation) */
    gade_batch *engine;         /* step engine of a single-pulse solver (device control, graphs) */
    int zskip;                  /* the DKB zero blocks hold for every pulse's tables */
    int g_ext;                  /* the pulses have their own radial tables */
    /* assembled operator (one FP64 pulse, real couplings): A(t) = sum_a w_a(t) K_a */
    int asm_ok;                 /* K_a built */
    int use_asm;                /* applies and steps use it */
    int asm_part;               /* its partition: 0 plain, 1 balanced */
    int npairs;                 /* (block row, coupled block) pairs */
    int *d_pair_c;
    double *d_K, *d_A;          /* [table set][pairs][3][W][B], [pulse][pairs][W][B] */
    size_t asm_kstride;         /* doubles per pulse of K (0: one set shared by all pulses) */
    int *d_pair_par;            /* [pairs] parity of the orders coupling the pair */
    int lpar[2];                /* first order of each parity (-1: none) */
    std::vector<int> h_pair_ptr, h_pair_r, h_pair_par, h_le_ptr, h_le_l, h_le_e;   /* pairs per block row; (order, term) per pair */
    void *d_A32;                /* mixed precision: the values rounded to float, chunk-major (k_apply_asm32) */
    int RMp;                    /* rows per chunk of that layout (RM rounded up to 4) */
    int max_row_pairs;          /* most coupled blocks of one block row */
    size_t a32_stride;          /* floats per pulse of d_A32 */
    int *d_row_pos;             /* [B] chunk << 16 | row within the chunk */
    PartList part_asm[1];       /* plain: one piece per unit */
    PartList part_asm_bal[9];   /* balanced, by resident CTAs per SM */
    int occ_asm[2][2];          /* resident CTAs per SM [complex64][sep] */
    float asm_ms[2];            /* timed FP64 apply: [0] plain, [1] balanced partition */
    double asm_flops, asm_bytes;          /* one assembled apply: FP64 flops, compulsory DRAM bytes */
    double asmb_flops, asmb_bytes;        /* one step's assembly */
    float mf_ms;                /* best timed matrix-free apply */
    float tab_ms[2];            /* timed step tables: matrix-free radial tables, assembly */
    unsigned pc_wait;           /* polls of a preconditioner stage wait (0: MBAR_SPIN_LIMIT) */
    /* double-float refinement residual (mixed precision, real couplings,
       matrix-free operator): tables, angular factors, S and i h dt/2 h0 and
       the pass's inputs as double-float */
    int mix_dd;                 /* 1: the residual pass runs in double-float on the FP32 pipes */
    int m64_stale;              /* the last step wrote no FP64 radial tables (refreshed on the next FP64 apply) */
    void *d_ang_dd[4], *d_Sdd, *d_Hdd, *d_Mdd;
    cdd *xdd, *ddd, *wdd;
    int pc_withhold;            /* failure injection: preconditioner stage whose copy is withheld (-1: none) */
    int pc_nw;                  /* warps per block row of the FP64 preconditioner solves (4 or 8) */
};

/* dynamic shared memory of k_precond_tma: two stage buffers, the block
   row's right-hand side, NW x 32 partial sums (complex of elem bytes) */
static size_t pc_smem_bytes(const gade_solver *s, size_t elem)
{
    return elem * ((size_t)2 * pc_stage_elems(s->bwp) + s->Bp + 8 * 32);
}


static int solver_engine_step(gade_solver *s, const double *ft, int32_t maxit, double tol, gade_step_stats *stats,
                              double *x_out = nullptr);
static void solver_engine_free(gade_solver *s);
static void batch_drop_graphs(gade_batch *b);

static void prof_begin(gade_solver *s, cudaStream_t st)
{
    if (!s->profile) return;
    if (s->ev_used + 2 > s->ev_pool.size()) {
        for (int k = 0; k < 64; k++) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) { s->profile = 0; return; }
            s->ev_pool.push_back(e);
        }
        s->ev_kind.resize(s->ev_pool.size() / 2 + 1);
    }
    cudaEventRecord(s->ev_pool[s->ev_used], st);
}

static void prof_end(gade_solver *s, cudaStream_t st, int kind)
{
    if (!s->profile) return;
    cudaEventRecord(s->ev_pool[s->ev_used + 1], st);
    s->ev_kind[s->ev_used / 2] = kind;
    s->ev_used += 2;
}

static void prof_collect(gade_solver *s)
{
    if (s->ev_used == 0) return;
    cudaEventSynchronize(s->ev_pool[s->ev_used - 1]);
    for (size_t k = 0; k < s->ev_used; k += 2) {
        float ms = 0;
        cudaEventElapsedTime(&ms, s->ev_pool[k], s->ev_pool[k + 1]);
        int kind = s->ev_kind[k / 2];
        s->prof_n[kind]++;
        s->prof_ms[kind] += ms;
    }
    s->ev_used = 0;
}

template <typename T>
static int dev_upload(gade_solver *s, T **d, const T *h, size_t count)
{
    size_t bytes = sizeof(T) * (count ? count : 1);
    void *p = nullptr;
    CK(cudaMalloc(&p, bytes));
    s->allocs.push_back(p);
    if (h && count) CK(cudaMemcpy(p, h, sizeof(T) * count, cudaMemcpyHostToDevice));
    else CK(cudaMemset(p, 0, bytes));
    *d = (T *)p;
    return GADE_OK;
}

/* frees one allocation made by dev_upload (used when re-chunking) */
static void dev_release(gade_solver *s, void *p)
{
    if (!p) return;
    for (size_t k = 0; k < s->allocs.size(); k++)
        if (s->allocs[k] == p) { cudaFree(p); s->allocs.erase(s->allocs.begin() + k); return; }
}

#define UP(dst, src, cnt) do { int rc_ = dev_upload(s, &(dst), (src), (size_t)(cnt)); if (rc_) { gade_solver_free(s); return rc_; } } while (0)

struct gade_problem_handle;   /* gade_problem is the host struct */

extern "C" int gade_problem_load(const char *dir, int32_t lmax, gade_problem **out)
{
    char err[1024] = {0};
    if (!dir || !out) return fail(GADE_ERR_ARG, "gade_problem_load: NULL argument");
    int rc = gade_problem_read(dir, lmax, out, err, sizeof(err));
    if (rc) return fail(rc, "%s", err);
    return GADE_OK;
}

extern "C" int gade_problem_get_info(const gade_problem *p, gade_problem_info *info)
{
    if (!p || !info) return fail(GADE_ERR_ARG, "gade_problem_get_info: NULL argument");
    info->lmax = p->lmax; info->nblk = p->nblk; info->blkdim = p->blkdim; info->blk_nnz = p->blk_nnz;
    info->n = p->n;
    info->hall_nnz = p->hall_Ap[p->nblk];
    info->nnz_full = (int64_t)info->hall_nnz * p->blk_nnz;
    info->real_coupling = p->real_coupling;
    info->dkb_zero = p->dkb_zero;
    return GADE_OK;
}

extern "C" int gade_problem_get_psi0(const gade_problem *p, double *psi, int32_t *perm)
{
    if (!p) return fail(GADE_ERR_ARG, "gade_problem_get_psi0: NULL problem");
    if (psi) memcpy(psi, p->psi0, sizeof(gc64) * (size_t)p->n);
    if (perm) memcpy(perm, p->xperm, sizeof(int32_t) * (size_t)p->n);
    return GADE_OK;
}

extern "C" int gade_problem_get_blocks(const gade_problem *p, int32_t *kappa, int32_t *ang)
{
    if (!p) return fail(GADE_ERR_ARG, "gade_problem_get_blocks: NULL problem");
    for (int r = 0; r < p->nblk; r++) {
        if (kappa) kappa[r] = p->kappa[r];
        if (ang) ang[r] = p->perm[r];
    }
    return GADE_OK;
}

extern "C" void gade_problem_free(gade_problem *p) { gade_problem_release(p); }

extern "C" void gade_solver_free(gade_solver *s)
{
    if (!s) return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    solver_engine_free(s);
    for (void *p : s->allocs) cudaFree(p);
    for (cudaEvent_t e : s->ev_pool) cudaEventDestroy(e);
    if (s->h_sc) cudaFreeHost(s->h_sc);
    if (s->h_sc2) cudaFreeHost(s->h_sc2);
    if (s->h_coef) cudaFreeHost(s->h_coef);
    if (s->stream) cudaStreamDestroy(s->stream);
    cudaSetDevice(cur);
    delete s;
}

static int part_reset(gade_solver *s);

static int choose_chunk_splines(int nblk, int B, int nsm)
{
    int half = (B % 2 == 0) ? B / 2 : B;
    int target = 2 * nsm;
    int nch = (target + nblk - 1) / nblk;
    if (nch < 1) nch = 1;
    int cs = (half + nch - 1) / nch;
    cs = ((cs + 15) / 16) * 16;
    if (cs < 16) cs = 16;
    if (cs > 64) cs = 64;
    return cs;
}

/* row-chunk layout of the operator kernel (pattern only: shared by all
   pulses); replaces an earlier layout */
static int set_chunking(gade_solver *s, const gade_setup *su)
{
    if (su->chunk_rows_max > 128 || su->chunk_cols_max > 256)
        return fail(GADE_ERR_ARG, "row chunk too large for the operator kernel (rows %d, columns %d)",
                    su->chunk_rows_max, su->chunk_cols_max);
    int *old[5] = {s->d_chunk_nrows, s->d_chunk_ncols, s->d_chunk_rows, s->d_chunk_cols, s->d_chunk_lcol};
    for (int *p : old) dev_release(s, p);
    s->RM = su->chunk_rows_max; s->CM = su->chunk_cols_max; s->nchunk = su->nchunk;
    int rc;
    if ((rc = dev_upload(s, &s->d_chunk_nrows, su->chunk_nrows, s->nchunk))) return rc;
    if ((rc = dev_upload(s, &s->d_chunk_ncols, su->chunk_ncols, s->nchunk))) return rc;
    if ((rc = dev_upload(s, &s->d_chunk_rows, su->chunk_rows, (size_t)s->nchunk * s->RM))) return rc;
    if ((rc = dev_upload(s, &s->d_chunk_cols, su->chunk_cols, (size_t)s->nchunk * s->CM))) return rc;
    if ((rc = dev_upload(s, &s->d_chunk_lcol, su->chunk_lcol, (size_t)s->nchunk * s->W * s->RM))) return rc;
    if (s->B > 65535) return fail(GADE_ERR_ARG, "block dimension %d exceeds the 16-bit column indices", s->B);
    {
        /* every ELL slot's column within the block (B when empty) */
        std::vector<unsigned short> ac((size_t)s->nchunk * s->W * s->RM);
        for (int q = 0; q < s->nchunk; q++)
            for (int j = 0; j < s->W; j++)
                for (int t = 0; t < s->RM; t++) {
                    const int lc = su->chunk_lcol[((size_t)q * s->W + j) * s->RM + t];
                    ac[((size_t)q * s->W + j) * s->RM + t] =
                        (unsigned short)(lc < 0 ? s->B : su->chunk_cols[(size_t)q * s->CM + lc]);
                }
        dev_release(s, s->d_chunk_acol);
        if ((rc = dev_upload(s, &s->d_chunk_acol, ac.data(), ac.size()))) return rc;
    }
    {
        /* position of every row in the chunk layout (chunk << 16 | row within the chunk) */
        std::vector<int> pos((size_t)s->B, 0);
        for (int q = 0; q < s->nchunk; q++)
            for (int t = 0; t < su->chunk_nrows[q]; t++)
                pos[su->chunk_rows[(size_t)q * s->RM + t]] = (q << 16) | t;
        dev_release(s, s->d_row_pos);
        if ((rc = dev_upload(s, &s->d_row_pos, pos.data(), pos.size()))) return rc;
    }
    /* reduction partials: one slot per CTA of a pulse */
    size_t max_cta = (size_t)s->nchunk * s->nblk;
    if ((size_t)s->upd_grid > max_cta) max_cta = s->upd_grid;
    s->pstride = max_cta * NRED;
    if (s->pstride * s->npulse > s->part_cap) {
        dev_release(s, s->d_part);
        s->d_part = nullptr;
        if ((rc = dev_upload(s, &s->d_part, (const double *)nullptr, s->pstride * s->npulse))) return rc;
        s->part_cap = s->pstride * s->npulse;
    }
    s->cs = su->chunk_splines;
    /* exact FP64 flop count of one operator apply (2 per FMA) */
    const double fma_c = s->rc ? 2.0 : 4.0;     /* FMAs of one coupling term */
    double fmas = 4.0 * (double)s->blk_nnz * s->nblk;             /* diagonal blocks (A x modes) */
    double cols = 0;
    for (int q = 0; q < s->nchunk; q++) cols += su->chunk_ncols[q];
    for (int r = 0; r < s->nblk; r++)
        for (int a = su->act_ptr[r]; a < su->act_ptr[r + 1]; a++) {
            int l = su->act_l[a];
            double ne = su->ang_ptr[r * s->lmax + l + 1] - su->ang_ptr[r * s->lmax + l];
            /* u, w, u', w' and their four tables; three of them per column
               and per entry with the DKB zero blocks */
            const double terms = s->zskip ? 3.0 : 4.0;
            fmas += terms * fma_c * ne * cols;                     /* gather */
            fmas += terms * fma_c * (double)s->blk_nnz;            /* radial tables */
        }
    s->apply_flops = 2.0 * fmas;
    {
        /* compulsory bytes of one apply (mode AX_R0V): the table slabs of the
           distinct (order, kappa) pairs the block rows use, the diagonal
           blocks, the angular terms, the slot maps and x, r0 in, v out */
        std::vector<char> used((size_t)s->lmax * s->nk, 0);
        for (int r = 0; r < s->nblk; r++)
            for (int a = su->act_ptr[r]; a < su->act_ptr[r + 1]; a++)
                used[(size_t)su->act_l[a] * s->nk + su->row_kidx[r]] = 1;
        double slabs = 0;
        for (char u : used) slabs += u;
        const double entry = s->rc ? 32.0 : 64.0;            /* four table values per ELL slot */
        const double nang = su->ang_ptr[(size_t)s->nblk * s->lmax];
        s->apply_bytes = slabs * s->W * s->B * entry + (double)s->nk * s->W * s->B * 16.0
                       + nang * (4.0 + (s->rc ? 32.0 : 64.0)) + (double)s->nchunk * s->W * s->RM * 4.0
                       + 48.0 * (double)s->n;
    }
    /* host copy of the work model for the partitions */
    s->h_act_ptr.assign(su->act_ptr, su->act_ptr + s->nblk + 1);
    s->h_act_ne.assign((size_t)su->act_ptr[s->nblk], 0);
    for (int r = 0; r < s->nblk; r++)
        for (int a = su->act_ptr[r]; a < su->act_ptr[r + 1]; a++) {
            const int l = su->act_l[a];
            s->h_act_ne[a] = su->ang_ptr[r * s->lmax + l + 1] - su->ang_ptr[r * s->lmax + l];
        }
    s->h_chunk_nrows.assign(su->chunk_nrows, su->chunk_nrows + s->nchunk);
    s->h_chunk_ncols.assign(su->chunk_ncols, su->chunk_ncols + s->nchunk);
    return part_reset(s);
}

/* block-LU factors of one pulse in the sweep layout of k_precond_tma:
   per kappa and sweep [triangle pairs][chain blocks]; the chain blocks
   G_c = -Linv_c Lband_c and GU_c = -Uinv_c Uband_c are formed here in FP64 */
static void pack_factors(const gade_setup *su, int nk, int nch, int bw, int bwp, int B, int Bp,
                         double2 *FL, double2 *FU)
{
    const int npair = (nch + 1) / 2;
    const size_t per = pc_sweep_elems(nch, bwp);
    auto cmac = [](double2 &acc, gc64 a, gc64 b) {
        acc.x += a.re * b.re - a.im * b.im;
        acc.y += a.re * b.im + a.im * b.re;
    };
    for (int kk = 0; kk < nk; kk++) {
        const gc64 *Li = su->Linv + (size_t)kk * nch * 1024, *Ui = su->Uinv + (size_t)kk * nch * 1024;
        double2 *fl = FL + (size_t)kk * per, *fu = FU + (size_t)kk * per;
        /* inverse blocks, column-major [j][i]: Linv_c(i, j) = Li[c 1024 + 32 j + i] */
        for (int p = 0; p < npair; p++) {
            const int c0 = 2 * p, c1 = 2 * p + 1;
            for (int q = 0; q < 33; q++)
                for (int i = 0; i < 32; i++) {
                    gc64 lv = {0, 0}, uv = {0, 0};
                    if (q <= i) lv = Li[(size_t)c0 * 1024 + q * 32 + i];
                    else if (c1 < nch) lv = Li[(size_t)c1 * 1024 + (q - i - 1) * 32 + (31 - i)];
                    if (q <= 31 - i) uv = Ui[(size_t)c0 * 1024 + (i + q) * 32 + i];
                    else if (c1 < nch) uv = Ui[(size_t)c1 * 1024 + (q - 1) * 32 + (31 - i)];
                    fl[(size_t)p * PC_TP + q * 32 + i] = make_double2(lv.re, lv.im);
                    fu[(size_t)p * PC_TP + q * 32 + i] = make_double2(uv.re, uv.im);
                }
        }
        double2 *gl = fl + (size_t)npair * PC_TP, *gu = fu + (size_t)npair * PC_TP;
        for (int c = 0; c < nch; c++)
            for (int col = 0; col < bwp; col++)
                for (int i = 0; i < 32; i++) {
                    double2 g = make_double2(0, 0), h = make_double2(0, 0);
                    for (int m = 0; m < 32; m++) {
                        const int row = 32 * c + m;
                        if (row >= B) break;
                        /* L(row, 32 c - bwp + col) */
                        const int cl = 32 * c - bwp + col, dl = row - cl;
                        if (c > 0 && dl >= 1 && dl <= bw && cl >= 0 && m <= i)
                            cmac(g, Li[(size_t)c * 1024 + m * 32 + i], su->Lb[((size_t)kk * bw + dl - 1) * Bp + row]);
                        /* U(row, 32 (c + 1) + col) */
                        const int cu = 32 * (c + 1) + col, du = cu - row;
                        if (c + 1 < nch && du >= 1 && du <= bw && cu < B && m >= i)
                            cmac(h, Ui[(size_t)c * 1024 + m * 32 + i], su->Ub[((size_t)kk * bw + du - 1) * Bp + row]);
                    }
                    gl[((size_t)c * bwp + col) * 32 + i] = make_double2(-g.x, -g.y);
                    gu[((size_t)c * bwp + col) * 32 + i] = make_double2(-h.x, -h.y);
                }
    }
}

/*
 * Shared by gade_solver_create (one pulse) and gade_batch_create (npulse
 * pulses on one set of angular tables, h0 and S).  Pulse k has its own time
 * step dts[k], radial tables (gext slice k, or the problem's own when gext is
 * NULL) and therefore its own D = S + i h dt/2 h0 and block-LU factors.
 */
static int solver_create(const gade_problem *p, int npulse, const double *dts, const double *gext, double h,
                         int32_t precision, int32_t device, int cs_req, gade_solver **out)
{
    if (!p || !out || !dts) return fail(GADE_ERR_ARG, "solver create: NULL argument");
    *out = nullptr;
    if (precision != GADE_PREC_FP64 && precision != GADE_PREC_MIXED)
        return fail(GADE_ERR_ARG, "unknown precision %d", precision);
    if (npulse < 1) return fail(GADE_ERR_ARG, "at least one pulse is needed");
    for (int k = 0; k < npulse; k++)
        if (!(dts[k] > 0) || !std::isfinite(dts[k])) return fail(GADE_ERR_ARG, "dt of pulse %d must be finite and > 0", k);
    int ndev = 0;
    CK(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(GADE_ERR_ARG, "no CUDA device %d", device);
    CK(cudaSetDevice(device));
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, device));

    const size_t bn = (size_t)p->blk_nnz;
    std::vector<int32_t> tpos;
    if (gext) {
        /* external radial tables: same class (real or complex) as the problem's,
           transposed on the shared pattern like the loader does */
        tpos.resize(bn);
        if (gade_problem_transpose_map(p, tpos.data()))
            return fail(GADE_ERR_FORMAT, "base pattern is not structurally symmetric");
        if (p->real_coupling) {
            const size_t cnt = (size_t)npulse * 6 * p->lmax * 4 * bn;
            for (size_t e = 0; e < cnt; e++)
                if (gext[2 * e + 1] != 0.0 || !std::isfinite(gext[2 * e]))
                    return fail(GADE_ERR_ARG, "radial tables of pulse %zu must be real and finite like the problem's",
                                e / ((size_t)6 * p->lmax * 4 * bn));
        }
    }

    char err[1024] = {0};
    gade_setup *su = nullptr;
    int cs = cs_req > 0 ? cs_req : choose_chunk_splines(p->nblk, p->blkdim, prop.multiProcessorCount);
    int rcode = gade_setup_build(p, dts[0], h, cs, &su, err, sizeof(err));
    if (rcode) return fail(rcode, "%s", err);
    if (su->W < 29 || su->W > 30) {
        /* two threads per row with 15 slots each: degree-7 radial bases give W = 30 */
        int w = su->W;
        gade_setup_release(su);
        return fail(GADE_ERR_ARG, "base pattern rows hold up to %d entries; the operator kernel takes 29 or 30", w);
    }
    {
        /* operator kernels may use more than the default 48 KB of dynamic shared memory */
        const int lim = 160 * 1024;
        cudaFuncSetAttribute(k_apply<double, true, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<double, true, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<double, false, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<double, false, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<float, true, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<float, true, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<float, false, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<float, false, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<double, true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<double, true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<double, false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<double, false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<float, true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<float, true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<float, false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<float, false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply_asm32, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<dd, true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        cudaFuncSetAttribute(k_apply<dd, true, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    }

    gade_solver *s = new gade_solver();
    s->pc_withhold = -1;
    s->pc_nw = 8;
    s->device = device;
    s->prec = precision;
    s->rc = p->real_coupling;
    s->n = p->n; s->nblk = p->nblk; s->B = p->blkdim; s->lmax = p->lmax;
    s->W = su->W; s->nk = su->nk;
    s->npulse = npulse; s->nslot = 1;
    s->dts.assign(dts, dts + npulse);
    s->AM = 1;
    for (int r = 0; r < p->nblk; r++) {
        int na = su->ang_ptr[(size_t)(r + 1) * p->lmax] - su->ang_ptr[(size_t)r * p->lmax];
        if (na > s->AM) s->AM = na;
    }
    s->bw = su->bw; s->Bp = su->Bp; s->nch = su->nch;
    s->dt = dts[0]; s->h = h; s->blk_nnz = p->blk_nnz;
    s->zskip = su->ell_halves && p->dkb_zero;
    s->g_ext = gext != nullptr;
    if (s->zskip && gext) {
        const size_t per = (size_t)6 * p->lmax * 4 * bn;
        for (int k = 0; k < npulse && s->zskip; k++)
            if (!gade_dkb_zero(p, (const gc64 *)(gext + 2 * per * k))) s->zskip = 0;
    }
    s->nsm = prop.multiProcessorCount;
    s->nsplit = 1;
    s->upd_block = 256;
    {
        /* vector kernels: at most two CTAs per SM, no more than one thread per element */
        long long need = (s->n + s->upd_block - 1) / s->upd_block;
        s->upd_grid = 2 * prop.multiProcessorCount;
        if (need < s->upd_grid) s->upd_grid = (int)(need > 0 ? need : 1);
    }
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        gade_setup_release(su); delete s; return fail(GADE_ERR_CUDA, "stream creation failed");
    }
#undef UP
#define UP(dst, src, cnt) do { int rc_ = dev_upload(s, &(dst), (src), (size_t)(cnt)); if (rc_) { gade_setup_release(su); gade_solver_free(s); return rc_; } } while (0)
    const size_t WB = (size_t)s->W * s->B;
    const size_t NP = (size_t)npulse;
    s->mstride = (size_t)s->lmax * s->nk * WB;
    s->dstride = (size_t)s->nk * WB;
    s->gstride = (size_t)s->lmax * 3 * 4 * WB;     /* radial tables in the ELL slot layout */
    s->bwp = s->bw <= 16 ? 16 : 32;
    if (s->bw > 32) { gade_setup_release(su); gade_solver_free(s); return fail(GADE_ERR_ARG, "preconditioner band %d wider than 32 is not supported", s->bw); }
    s->fstride = (size_t)s->nk * pc_sweep_elems(s->nch, s->bwp);

    if (npulse > 1) {
        std::vector<int> ident(npulse);
        for (int k = 0; k < npulse; k++) ident[k] = k;
        UP(s->d_plist, ident.data(), npulse);
        s->nslot = npulse;
    }
    UP(s->d_row_kidx, su->row_kidx, s->nblk);
    UP(s->d_act_ptr, su->act_ptr, s->nblk + 1);
    UP(s->d_act_l, su->act_l, su->n_act);
    UP(s->d_ang_ptr, su->ang_ptr, (size_t)s->nblk * s->lmax + 1);
    UP(s->d_ang_c, su->ang_c, su->n_ang);
    {
        const gc64 *src[4] = {su->ang_a0, su->ang_a0k, su->ang_a1, su->ang_a1k};
        void **dst[4] = {&s->d_ang_a0, &s->d_ang_a0k, &s->d_ang_a1, &s->d_ang_a1k};
        for (int k = 0; k < 4; k++) {
            if (s->rc) {
                std::vector<double> im((size_t)su->n_ang + 1);
                for (int64_t e = 0; e < su->n_ang; e++) im[e] = src[k][e].im;
                double *d; UP(d, im.data(), su->n_ang); *dst[k] = d;
            } else {
                double2 *d; UP(d, (const double2 *)src[k], su->n_ang); *dst[k] = d;
            }
        }
    }
    {
        int rc = set_chunking(s, su);
        if (rc) { gade_setup_release(su); gade_solver_free(s); return rc; }
    }
    {
        std::vector<double> kd(su->kvals, su->kvals + s->nk);
        UP(s->d_kvals, kd.data(), s->nk);
    }
    UP(s->d_ord, su->ord, s->B);
    {
        double2 *d;
        UP(d, (const double2 *)su->S_ell, (size_t)s->nk * WB); s->d_S_ell = d;
        UP(d, (const double2 *)nullptr, NP * s->dstride); s->d_Hst_ell = d;
        UP(d, (const double2 *)nullptr, NP * s->dstride); s->d_D_ell = d;
        UP(s->d_FL, (const double2 *)nullptr, NP * s->fstride);
        UP(s->d_FU, (const double2 *)nullptr, NP * s->fstride);
        if (s->rc) { double *g; UP(g, (const double *)nullptr, NP * s->gstride); s->d_g = g; UP(g, (const double *)nullptr, NP * s->gstride); s->d_gt = g; }
        else { double2 *g; UP(g, (const double2 *)nullptr, NP * s->gstride); s->d_g = g; UP(g, (const double2 *)nullptr, NP * s->gstride); s->d_gt = g; }
        if (s->rc) { R4d *m = nullptr; UP(m, (const R4d *)nullptr, NP * s->mstride); s->d_M = m; }
        else { C4<double2> *m = nullptr; UP(m, (const C4<double2> *)nullptr, NP * s->mstride); s->d_M = m; }
    }
    const bool mixed = precision == GADE_PREC_MIXED;
    if (mixed) {
        if (s->rc) { R4f *m = nullptr; UP(m, (const R4f *)nullptr, NP * s->mstride); s->d_M32 = m; }
        else { C4<float2> *m = nullptr; UP(m, (const C4<float2> *)nullptr, NP * s->mstride); s->d_M32 = m; }
        std::vector<float2> Sf((size_t)s->nk * WB);
        for (size_t e = 0; e < Sf.size(); e++) Sf[e] = make_float2((float)su->S_ell[e].re, (float)su->S_ell[e].im);
        float2 *d;
        UP(d, Sf.data(), Sf.size()); s->d_S32 = d;
        UP(d, (const float2 *)nullptr, NP * s->dstride); s->d_H32 = d;
        UP(d, (const float2 *)nullptr, NP * s->dstride); s->d_D32 = d;
        UP(d, (const float2 *)nullptr, NP * s->fstride); s->d_FL32 = d;
        UP(d, (const float2 *)nullptr, NP * s->fstride); s->d_FU32 = d;
        const gc64 *src[4] = {su->ang_a0, su->ang_a0k, su->ang_a1, su->ang_a1k};
        for (int k = 0; k < 4; k++) {
            if (s->rc) {
                std::vector<float> v((size_t)su->n_ang + 1);
                for (int64_t e = 0; e < su->n_ang; e++) v[e] = (float)src[k][e].im;
                float *dd; UP(dd, v.data(), su->n_ang); s->d_a32[k] = dd;
            } else {
                std::vector<float2> v((size_t)su->n_ang + 1);
                for (int64_t e = 0; e < su->n_ang; e++) v[e] = make_float2((float)src[k][e].re, (float)src[k][e].im);
                float2 *dd; UP(dd, v.data(), su->n_ang); s->d_a32[k] = dd;
            }
        }
        if (s->rc) {
            /* the double-float residual pass: angular factors, S, tables, inputs */
            for (int k = 0; k < 4; k++) {
                std::vector<dd> v((size_t)su->n_ang + 1);
                for (int64_t e = 0; e < su->n_ang; e++) v[e] = dd_from(src[k][e].im);
                dd *q; UP(q, v.data(), su->n_ang); s->d_ang_dd[k] = q;
            }
            std::vector<cdd> Sd((size_t)s->nk * WB);
            for (size_t e = 0; e < Sd.size(); e++) { Sd[e].x = dd_from(su->S_ell[e].re); Sd[e].y = dd_from(su->S_ell[e].im); }
            cdd *c;
            UP(c, Sd.data(), Sd.size()); s->d_Sdd = c;
            UP(c, (const cdd *)nullptr, NP * s->dstride); s->d_Hdd = c;
            R4dd *m = nullptr;
            UP(m, (const R4dd *)nullptr, NP * s->mstride); s->d_Mdd = m;
            UP(s->xdd, (const cdd *)nullptr, NP * s->n);
            UP(s->ddd, (const cdd *)nullptr, NP * s->n);
            UP(s->wdd, (const cdd *)nullptr, NP * s->n);
            s->mix_dd = 1;
        }
    }
    {
        size_t smem = pc_smem_bytes(s, sizeof(double2));
        if (smem > 220 * 1024) { gade_setup_release(su); gade_solver_free(s); return fail(GADE_ERR_ARG, "block dimension too large for the preconditioner"); }
        const int sm64 = (int)smem, sm32 = (int)pc_smem_bytes(s, sizeof(float2));
        cudaFuncSetAttribute(k_precond_tma<double, 16, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm64);
        cudaFuncSetAttribute(k_precond_tma<double, 32, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm64);
        cudaFuncSetAttribute(k_precond_tma<double, 16, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm64);
        cudaFuncSetAttribute(k_precond_tma<double, 32, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm64);
        cudaFuncSetAttribute(k_precond_tma<float, 16, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm32);
        cudaFuncSetAttribute(k_precond_tma<float, 32, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm32);
    }
    /* per-pulse slices: dt-dependent D, i h dt/2 h0 and LU factors; radial tables */
    {
        std::vector<double2> D(s->dstride), FL(s->fstride), FU(s->fstride);
        std::vector<float2> Hf, Df, FLf, FUf;
        if (mixed) { Hf.resize(s->dstride); Df.resize(s->dstride); FLf.resize(s->fstride); FUf.resize(s->fstride); }
        std::vector<double> gr, gtr;
        std::vector<double2> gc, gtc;
        if (s->rc) { gr.resize(s->gstride); gtr.resize(s->gstride); }
        else { gc.resize(s->gstride); gtc.resize(s->gstride); }
        std::vector<gc64> gtmp;
        for (int k = 0; k < npulse; k++) {
            gade_setup *sk = su;
            if (k > 0) {
                sk = nullptr;
                rcode = gade_setup_build(p, dts[k], h, cs, &sk, err, sizeof(err));
                if (rcode) { gade_setup_release(su); gade_solver_free(s); return fail(rcode, "pulse %d: %s", k, err); }
                if (sk->bw != su->bw || sk->nk != su->nk || sk->nch != su->nch ||
                    memcmp(sk->ord, su->ord, sizeof(int32_t) * s->B) != 0) {
                    gade_setup_release(sk); gade_setup_release(su); gade_solver_free(s);
                    return fail(GADE_ERR_ARG, "pulse %d: preconditioner ordering differs from pulse 0", k);
                }
            }
            for (size_t e = 0; e < s->dstride; e++)
                D[e] = make_double2(sk->S_ell[e].re + sk->Hst_ell[e].re, sk->S_ell[e].im + sk->Hst_ell[e].im);
            pack_factors(sk, s->nk, s->nch, s->bw, s->bwp, s->B, s->Bp, FL.data(), FU.data());
            cudaError_t ce = cudaMemcpy((double2 *)s->d_Hst_ell + k * s->dstride, sk->Hst_ell, sizeof(double2) * s->dstride, cudaMemcpyHostToDevice);
            if (ce == cudaSuccess) ce = cudaMemcpy((double2 *)s->d_D_ell + k * s->dstride, D.data(), sizeof(double2) * s->dstride, cudaMemcpyHostToDevice);
            if (ce == cudaSuccess) ce = cudaMemcpy(s->d_FL + k * s->fstride, FL.data(), sizeof(double2) * s->fstride, cudaMemcpyHostToDevice);
            if (ce == cudaSuccess) ce = cudaMemcpy(s->d_FU + k * s->fstride, FU.data(), sizeof(double2) * s->fstride, cudaMemcpyHostToDevice);
            if (ce == cudaSuccess && mixed) {
                for (size_t e = 0; e < s->dstride; e++) {
                    Hf[e] = make_float2((float)sk->Hst_ell[e].re, (float)sk->Hst_ell[e].im);
                    Df[e] = make_float2((float)D[e].x, (float)D[e].y);
                }
                for (size_t e = 0; e < s->fstride; e++) {
                    FLf[e] = make_float2((float)FL[e].x, (float)FL[e].y);
                    FUf[e] = make_float2((float)FU[e].x, (float)FU[e].y);
                }
                ce = cudaMemcpy((float2 *)s->d_H32 + k * s->dstride, Hf.data(), sizeof(float2) * s->dstride, cudaMemcpyHostToDevice);
                if (ce == cudaSuccess && s->d_Hdd) {
                    std::vector<cdd> Hd(s->dstride);
                    for (size_t e = 0; e < s->dstride; e++) {
                        Hd[e].x = dd_from(sk->Hst_ell[e].re);
                        Hd[e].y = dd_from(sk->Hst_ell[e].im);
                    }
                    ce = cudaMemcpy((cdd *)s->d_Hdd + k * s->dstride, Hd.data(), sizeof(cdd) * s->dstride,
                                    cudaMemcpyHostToDevice);
                }
                if (ce == cudaSuccess) ce = cudaMemcpy((float2 *)s->d_D32 + k * s->dstride, Df.data(), sizeof(float2) * s->dstride, cudaMemcpyHostToDevice);
                if (ce == cudaSuccess) ce = cudaMemcpy((float2 *)s->d_FL32 + k * s->fstride, FLf.data(), sizeof(float2) * s->fstride, cudaMemcpyHostToDevice);
                if (ce == cudaSuccess) ce = cudaMemcpy((float2 *)s->d_FU32 + k * s->fstride, FUf.data(), sizeof(float2) * s->fstride, cudaMemcpyHostToDevice);
            }
            if (sk != su) gade_setup_release(sk);
            /* radial tables of the three pulse components used by each l */
            const gc64 *g = p->g, *gt = p->gt;
            if (gext) {
                const size_t per = (size_t)6 * s->lmax * 4 * bn;
                g = (const gc64 *)(gext + 2 * per * k);
                gtmp.resize(per);
                for (size_t blk = 0; blk < (size_t)6 * s->lmax * 4; blk++)
                    for (size_t e = 0; e < bn; e++) {
                        const gc64 v = g[blk * bn + e];
                        gtmp[blk * bn + tpos[e]] = gc64{v.re, -v.im};
                    }
                gt = gtmp.data();
            }
            for (int l = 0; l < s->lmax; l++)
                for (int ia = 0; ia < 3; ia++) {
                    int a = (l % 2 + 1) % 2 + 2 * ia;
                    for (int q = 0; q < 4; q++)
                        for (size_t slot = 0; slot < WB; slot++) {
                            /* ELL slot layout: the table kernel streams them */
                            const int e = su->ell_pos[slot];
                            const size_t dst = (((size_t)l * 3 + ia) * 4 + q) * WB + slot;
                            if (e < 0) {
                                if (s->rc) { gr[dst] = 0.0; gtr[dst] = 0.0; }
                                else { gc[dst] = make_double2(0, 0); gtc[dst] = make_double2(0, 0); }
                                continue;
                            }
                            const size_t src = (((size_t)a * s->lmax + l) * 4 + q) * bn + e;
                            if (s->rc) { gr[dst] = g[src].re; gtr[dst] = gt[src].re; }
                            else { gc[dst] = make_double2(g[src].re, g[src].im); gtc[dst] = make_double2(gt[src].re, gt[src].im); }
                        }
                }
            if (ce == cudaSuccess) {
                if (s->rc) {
                    ce = cudaMemcpy((double *)s->d_g + k * s->gstride, gr.data(), sizeof(double) * s->gstride, cudaMemcpyHostToDevice);
                    if (ce == cudaSuccess) ce = cudaMemcpy((double *)s->d_gt + k * s->gstride, gtr.data(), sizeof(double) * s->gstride, cudaMemcpyHostToDevice);
                } else {
                    ce = cudaMemcpy((double2 *)s->d_g + k * s->gstride, gc.data(), sizeof(double2) * s->gstride, cudaMemcpyHostToDevice);
                    if (ce == cudaSuccess) ce = cudaMemcpy((double2 *)s->d_gt + k * s->gstride, gtc.data(), sizeof(double2) * s->gstride, cudaMemcpyHostToDevice);
                }
            }
            if (ce != cudaSuccess) {
                gade_setup_release(su); gade_solver_free(s);
                return fail(GADE_ERR_CUDA, "upload of pulse %d failed: %s", k, cudaGetErrorString(ce));
            }
        }
    }
    /* vectors: every pulse starts from psi0 */
    double2 **vecs[] = {&s->x, &s->rhs, &s->r, &s->r0, &s->p, &s->v, &s->y, &s->z, &s->s, &s->t, &s->tmp0, &s->tmp1};
    for (double2 **vp : vecs) UP(*vp, (const double2 *)nullptr, NP * s->n);
    for (int k = 0; k < npulse; k++)
        CK(cudaMemcpy(s->x + (size_t)k * s->n, p->psi0, sizeof(double2) * (size_t)s->n, cudaMemcpyHostToDevice));
    /* reductions */
    UP(s->d_ticket, (const unsigned *)nullptr, NP);
    UP(s->d_sc, (const DevScal *)nullptr, NP);
    UP(s->d_coef, (const double2 *)nullptr, NP * s->lmax * 3);
    if (cudaMallocHost((void **)&s->h_sc, sizeof(DevScal) * NP) != cudaSuccess ||
        cudaMallocHost((void **)&s->h_coef, sizeof(double2) * NP * s->lmax * 3) != cudaSuccess) {
        gade_setup_release(su); gade_solver_free(s); return fail(GADE_ERR_CUDA, "pinned allocation failed");
    }
    memset(s->h_sc, 0, sizeof(DevScal) * NP);
    if (mixed) {
        float2 **v32[] = {&s->x32, &s->d32, &s->q32, &s->r32, &s->e32, &s->ri32, &s->r032, &s->p32, &s->v32,
                          &s->y32, &s->z32, &s->s32, &s->t32};
        for (float2 **vp : v32) UP(*vp, (const float2 *)nullptr, NP * s->n);
        UP(s->xprev, (const double2 *)nullptr, NP * s->n);
        UP(s->delta64, (const double2 *)nullptr, NP * s->n);
        UP(s->d_sc2, (const DevScal *)nullptr, NP);
        UP(s->d_hprev, (const int *)nullptr, NP);
        if (cudaMallocHost((void **)&s->h_sc2, sizeof(DevScal) * NP) != cudaSuccess) {
            gade_setup_release(su); gade_solver_free(s); return fail(GADE_ERR_CUDA, "pinned allocation failed");
        }
        memset(s->h_sc2, 0, sizeof(DevScal) * NP);
    }
    /* block solves, 2 sweeps: the triangle pairs (33 products per lane) and
       the chain blocks of every chunk with a neighbour (BWP products per row) */
    s->precond_flops = 2.0 * 8.0 * (double)s->nblk *
                       (32.0 * 33.0 * ((s->nch + 1) / 2) + 32.0 * s->bwp * (s->nch - 1));
    if (s->rc) {
        /* (block row, coupled block) pairs and the (order, angular term) list
           of every pair, for the assembled operator */
        s->h_pair_ptr.assign(1, 0);
        for (int r = 0; r < s->nblk; r++) {
            std::vector<std::pair<int, std::pair<int, int>>> ent;   /* (c, (l, e)) */
            for (int l = 0; l < s->lmax; l++)
                for (int e = su->ang_ptr[r * s->lmax + l]; e < su->ang_ptr[r * s->lmax + l + 1]; e++)
                    ent.push_back({su->ang_c[e], {l, e}});
            std::stable_sort(ent.begin(), ent.end(),
                             [](const std::pair<int, std::pair<int, int>> &a, const std::pair<int, std::pair<int, int>> &b) {
                                 return a.first < b.first;
                             });
            for (size_t k = 0; k < ent.size(); k++) {
                if (k == 0 || ent[k].first != ent[k - 1].first) {
                    s->h_pair_r.push_back(r);
                    s->h_pair_par.push_back(ent[k].second.first % 2);
                    s->h_le_ptr.push_back((int)s->h_le_l.size());
                    s->npairs++;
                }
                if (ent[k].second.first % 2 != s->h_pair_par.back()) s->h_pair_par.back() = -1;   /* mixed parity */
                s->h_le_l.push_back(ent[k].second.first);
                s->h_le_e.push_back(ent[k].second.second);
            }
            s->h_pair_ptr.push_back(s->npairs);
            const int rp = s->h_pair_ptr.back() - s->h_pair_ptr[s->h_pair_ptr.size() - 2];
            if (rp > s->max_row_pairs) s->max_row_pairs = rp;
        }
        s->h_le_ptr.push_back((int)s->h_le_l.size());
        std::vector<int> pc;
        for (int r = 0; r < s->nblk; r++) {
            int last = -1;
            std::vector<int> cs;
            for (int e = su->ang_ptr[r * s->lmax]; e < su->ang_ptr[(r + 1) * s->lmax]; e++) cs.push_back(su->ang_c[e]);
            std::sort(cs.begin(), cs.end());
            for (int c : cs) if (c != last) { pc.push_back(c); last = c; }
        }
        UP(s->d_pair_c, pc.data(), pc.size());
    }
    gade_setup_release(su);
#undef UP
#define UP(dst, src, cnt) do { int rc_ = dev_upload(s, &(dst), (src), (size_t)(cnt)); if (rc_) { gade_solver_free(s); return rc_; } } while (0)
    *out = s;
    return GADE_OK;
}



static OpP op_params(const gade_solver *s)
{
    OpP P;
    P.nblk = s->nblk; P.B = s->B; P.lmax = s->lmax; P.W = s->W; P.nk = s->nk; P.RM = s->RM; P.CM = s->CM;
    P.AM = s->AM;
    P.row_kidx = s->d_row_kidx; P.act_ptr = s->d_act_ptr; P.act_l = s->d_act_l;
    P.ang_ptr = s->d_ang_ptr; P.ang_c = s->d_ang_c;
    P.ang_a0 = s->d_ang_a0; P.ang_a0k = s->d_ang_a0k; P.ang_a1 = s->d_ang_a1; P.ang_a1k = s->d_ang_a1k;
    P.chunk_nrows = s->d_chunk_nrows; P.chunk_ncols = s->d_chunk_ncols; P.chunk_rows = s->d_chunk_rows;
    P.chunk_cols = s->d_chunk_cols; P.chunk_lcol = s->d_chunk_lcol; P.chunk_acol = s->d_chunk_acol;
    P.M = s->d_M; P.S_ell = s->d_S_ell; P.Hst_ell = s->d_Hst_ell; P.D_ell = s->d_D_ell;
    P.plist = s->d_plist; P.vstride = s->n; P.mstride = s->mstride; P.dstride = s->dstride;
    P.nchunk = s->nchunk;
    P.seg_ptr = s->part_split[1].d_seg_ptr; P.pieces = s->part_split[1].d_pieces;
    P.piece_acc = s->d_piece_acc; P.unit_tick = s->d_unit_tick;
    return P;
}

static RedP make_red(const gade_solver *s, DevScal *sc, int kind, int pred, DevScal *pa = nullptr,
                     DevScal *pb = nullptr)
{
    RedP r;
    r.part = s->d_part; r.ticket = s->d_ticket; r.sc = sc; r.kind = kind; r.out = nullptr;
    r.pstride = s->pstride; r.pred = pred; r.pa = pa; r.pb = pb;
    return r;
}

/* k_apply launch shape: one thread per output row and per gathered column */
static void apply_dims(const gade_solver *s, size_t elem, int *nt, size_t *smem, bool ddinst = false)
{
    int t = 2 * s->RM > s->CM ? 2 * s->RM : s->CM;   /* two threads per row */
    t = (t + 31) / 32 * 32;
    *nt = t;
    const int G = ddinst ? APPLY_GDD : (elem == sizeof(double2) ? APPLY_G64 : APPLY_G32);
    const unsigned ang4 = s->rc ? (unsigned)(2 * elem) : (unsigned)(4 * elem);   /* four angular factors */
    const int CS = (s->CM + 2) & ~1;                 /* columns + the zero column, even */
    *smem = apply_smem(CS, s->W, s->RM, s->AM, G, (unsigned)elem, ang4, t, s->lmax).total;
}

/* the operator kernel instance for a precision, coupling class and mode class */
template <typename R>
static void k_apply_launch(const gade_solver *s, dim3 grid, int nt, size_t smem, cudaStream_t st, OpP P,
                           const typename Cx<R>::T *x, int mode, VecP V, RedP red)
{
    const bool sep = mode == AX_RHS || mode == AX_PARTS || mode == AX_MIX;
#define KA(RC_, SEP_, Z_) k_apply<R, RC_, SEP_, Z_><<<grid, nt, smem, st>>>(P, x, mode, V, red)
    if (s->zskip) {
        if (s->rc) { if (sep) KA(true, true, true); else KA(true, false, true); }
        else { if (sep) KA(false, true, true); else KA(false, false, true); }
    } else {
        if (s->rc) { if (sep) KA(true, true, false); else KA(true, false, false); }
        else { if (sep) KA(false, true, false); else KA(false, false, false); }
    }
#undef KA
}

/* resident CTAs per SM of the operator instance for a precision and mode class */
template <typename R>
static int apply_occupancy(const gade_solver *s, bool sep)
{
    int nt;
    size_t smem;
    apply_dims(s, sizeof(typename Cx<R>::T), &nt, &smem, std::is_same<R, dd>::value);
    int n = 0;
    cudaError_t e = cudaSuccess;
#define OC(RC_, SEP_, Z_) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_apply<R, RC_, SEP_, Z_>, nt, smem)
    if (s->zskip) {
        if (s->rc) { if (sep) OC(true, true, true); else OC(true, false, true); }
        else { if (sep) OC(false, true, true); else OC(false, false, true); }
    } else {
        if (s->rc) { if (sep) OC(true, true, false); else OC(true, false, false); }
        else { if (sep) OC(false, true, false); else OC(false, false, false); }
    }
#undef OC
    if (e != cudaSuccess || n < 1) { cudaGetLastError(); n = 1; }
    return n > 8 ? 8 : n;
}

static void part_release(gade_solver *s, PartList &pl)
{
    dev_release(s, pl.d_seg_ptr);
    dev_release(s, pl.d_pieces);
    pl = PartList();
}

static int part_upload(gade_solver *s, PartList &pl, const std::vector<int> &seg, const std::vector<int4> &pcs)
{
    part_release(s, pl);
    int rc;
    if ((rc = dev_upload(s, &pl.d_seg_ptr, seg.data(), seg.size()))) return rc;
    if ((rc = dev_upload(s, &pl.d_pieces, pcs.data(), pcs.size()))) return rc;
    pl.nseg = (int)seg.size() - 1;
    pl.npieces = (int)pcs.size();
    for (const int4 &pc : pcs)
        if ((pc.w >> 16) > 1) pl.multi = 1;
    if (pl.multi && (size_t)pl.npieces > s->piece_cap) {
        dev_release(s, s->d_piece_acc);
        s->d_piece_acc = nullptr;
        s->piece_cap = 0;
        double2 *acc = nullptr;
        if ((rc = dev_upload(s, &acc, (const double2 *)nullptr, (size_t)pl.npieces * 3 * s->RM))) return rc;
        s->d_piece_acc = acc;
        s->piece_cap = (size_t)pl.npieces;
    }
    return GADE_OK;
}

/* Order split: ns pieces per unit, each with a share of the active orders
   (whole FP64 gather groups), one piece per segment. */
static int part_build_split(gade_solver *s, int ns)
{
    std::vector<int> seg(1, 0);
    std::vector<int4> pcs;
    const int nunit = s->nchunk * s->nblk;
    for (int u = 0; u < nunit; u++) {
        const int r = u / s->nchunk;
        const int a0 = s->h_act_ptr[r], a1 = s->h_act_ptr[r + 1], na = a1 - a0;
        const int per = ((na + ns - 1) / ns + APPLY_G64 - 1) / APPLY_G64 * APPLY_G64;
        for (int sp = 0; sp < ns; sp++) {
            const int b0 = std::min(a0 + sp * per, a1), b1 = std::min(b0 + per, a1);
            pcs.push_back(make_int4(u, b0, b1, sp | (ns << 16)));
            seg.push_back((int)pcs.size());
        }
    }
    return part_upload(s, s->part_split[ns], seg, pcs);
}

/* Balanced segments: the units' work, in unit order, laid on one line by a
   cost model (FMAs of the gather and the table products of every active
   order, the diagonal blocks and the staging of a unit) and cut into nseg
   equal lengths, one (or a few) segments per resident CTA slot; an order goes
   to the segment that holds its midpoint, so a unit's orders fall into
   consecutive pieces.  With one segment per slot every segment is resident at
   once and the SMs finish together; with more, the block scheduler gives the
   later segments to the slots that free first. */
static int part_build_balanced(gade_solver *s, int nseg, PartList &pl)
{
    const int nunit = s->nchunk * s->nblk;
    const double terms = s->zskip ? 3.0 : 4.0, fc = s->rc ? 2.0 : 4.0;
    const double gw = s->bal_gamma > 0 ? s->bal_gamma : 1.0;
    auto ocost = [&](int a, int q) {
        return terms * fc * (gw * s->h_act_ne[a] * s->h_chunk_ncols[q] + (double)s->h_chunk_nrows[q] * s->W);
    };
    auto ufix = [&](int q) { return 6.0 * s->h_chunk_nrows[q] * s->W; };
    double total = 0;
    for (int u = 0; u < nunit; u++) {
        const int r = u / s->nchunk, q = u - r * s->nchunk;
        total += ufix(q);
        for (int a = s->h_act_ptr[r]; a < s->h_act_ptr[r + 1]; a++) total += ocost(a, q);
    }
    const double T = total / nseg;
    auto seg_of = [&](double mid) { int k = (int)(mid / T); return k < 0 ? 0 : (k >= nseg ? nseg - 1 : k); };
    std::vector<int4> pcs;
    std::vector<int> pseg;                 /* segment of each piece */
    double pos = 0;
    for (int u = 0; u < nunit; u++) {
        const int r = u / s->nchunk, q = u - r * s->nchunk;
        const int a0 = s->h_act_ptr[r], a1 = s->h_act_ptr[r + 1];
        const double f = ufix(q);
        const size_t first = pcs.size();
        if (a0 == a1) {
            pcs.push_back(make_int4(u, a0, a0, 0));
            pseg.push_back(seg_of(pos + 0.5 * f));
        }
        pos += f;
        int cur = -1, b0 = a0;
        for (int a = a0; a < a1; a++) {
            const double c = ocost(a, q);
            const int sg = seg_of(pos + 0.5 * c);
            pos += c;
            if (sg != cur) {
                if (cur >= 0) { pcs.push_back(make_int4(u, b0, a, 0)); pseg.push_back(cur); }
                cur = sg;
                b0 = a;
            }
        }
        if (a1 > a0) { pcs.push_back(make_int4(u, b0, a1, 0)); pseg.push_back(cur); }
        const int np = (int)(pcs.size() - first);
        for (int k = 0; k < np; k++) pcs[first + k].w = k | (np << 16);
    }
    std::vector<int> seg((size_t)nseg + 1, 0);
    for (int sg : pseg) seg[sg + 1]++;
    for (int k = 0; k < nseg; k++) seg[k + 1] += seg[k];
    return part_upload(s, pl, seg, pcs);
}

/* the balanced lists of every operator instance the solver launches */
static int part_build_balanced_all(gade_solver *s)
{
    for (int f = 0; f < 2; f++) {
        if (f == 1 && s->prec != GADE_PREC_MIXED) continue;
        for (int sep = 0; sep < 2; sep++) {
            const int o = s->occ[f][sep];
            if (s->part_bal[o].nseg) continue;
            int rc = part_build_balanced(s, o * s->nsm * (s->bal_waves > 0 ? s->bal_waves : 1), s->part_bal[o]);
            if (rc) return rc;
        }
    }
    return GADE_OK;
}

/* after (re)chunking: the plain one-piece-per-unit list, nothing else */
static int part_reset(gade_solver *s)
{
    for (PartList &pl : s->part_split) part_release(s, pl);
    for (PartList &pl : s->part_bal) part_release(s, pl);
    dev_release(s, s->d_piece_acc);
    s->d_piece_acc = nullptr;
    s->piece_cap = 0;
    dev_release(s, s->d_unit_tick);
    s->d_unit_tick = nullptr;
    int rc;
    if ((rc = dev_upload(s, &s->d_unit_tick, (const unsigned *)nullptr, (size_t)s->nchunk * s->nblk))) return rc;
    for (int f = 0; f < 2; f++)
        for (int sep = 0; sep < 2; sep++)
            s->occ[f][sep] = f ? apply_occupancy<float>(s, sep) : apply_occupancy<double>(s, sep);
    s->nsplit = 1;
    return part_build_split(s, 1);
}

/* the partition a launch uses: its segment list in P, the segment count returned */
static int op_partition(const gade_solver *s, OpP &P, bool fp32, int mode)
{
    const bool sep = mode == AX_RHS || mode == AX_PARTS || mode == AX_MIX;
    const PartList *pl = &s->part_split[1];
    if (s->nsplit >= 2 && s->nsplit <= 4 && s->part_split[s->nsplit].nseg) pl = &s->part_split[s->nsplit];
    else if (s->nsplit == 0 && s->part_bal[s->occ[fp32][sep]].nseg) pl = &s->part_bal[s->occ[fp32][sep]];
    P.seg_ptr = pl->d_seg_ptr;
    P.pieces = pl->d_pieces;
    return pl->nseg;
}

static int launch_table_kernels(gade_solver *s, int which, cudaStream_t st);

/* the assembled operator's partitions: plain (one piece per unit) and
   balanced (units laid on a line by work: 2 FMAs per stored value, plus the
   staging of a coupled block's x window and a unit's diagonal blocks) */
static int asm_partitions(gade_solver *s)
{
    const int nunit = s->nchunk * s->nblk;
    int rc;
    {
        std::vector<int> seg(1, 0);
        std::vector<int4> pcs;
        for (int u = 0; u < nunit; u++) {
            const int r = u / s->nchunk;
            pcs.push_back(make_int4(u, s->h_pair_ptr[r], s->h_pair_ptr[r + 1], 0 | (1 << 16)));
            seg.push_back((int)pcs.size());
        }
        if ((rc = part_upload(s, s->part_asm[0], seg, pcs))) return rc;
    }
    auto pcost = [&](int q) { return 2.0 * s->h_chunk_nrows[q] * s->W + 2.0 * s->h_chunk_ncols[q]; };
    auto ufix = [&](int q) { return 4.0 * s->h_chunk_nrows[q] * s->W; };
    for (int cls = 0; cls < 4; cls++) {
        const int f = cls / 2, o = s->occ_asm[f][cls % 2];
        if (f == 1 && s->prec != GADE_PREC_MIXED) continue;
        if (s->part_asm_bal[o].nseg) continue;
        const int nseg = o * s->nsm;
        double total = 0;
        for (int u = 0; u < nunit; u++) {
            const int r = u / s->nchunk, q = u - r * s->nchunk;
            total += ufix(q) + pcost(q) * (s->h_pair_ptr[r + 1] - s->h_pair_ptr[r]);
        }
        const double T = total / nseg;
        auto seg_of = [&](double mid) { int k = (int)(mid / T); return k < 0 ? 0 : (k >= nseg ? nseg - 1 : k); };
        std::vector<int4> pcs;
        std::vector<int> pseg;
        double pos = 0;
        for (int u = 0; u < nunit; u++) {
            const int r = u / s->nchunk, q = u - r * s->nchunk;
            const int a0 = s->h_pair_ptr[r], a1 = s->h_pair_ptr[r + 1];
            const size_t first = pcs.size();
            if (a0 == a1) { pcs.push_back(make_int4(u, a0, a0, 0)); pseg.push_back(seg_of(pos + 0.5 * ufix(q))); }
            pos += ufix(q);
            int cur = -1, b0 = a0;
            for (int a = a0; a < a1; a++) {
                const int sg = seg_of(pos + 0.5 * pcost(q));
                pos += pcost(q);
                if (sg != cur) {
                    if (cur >= 0) { pcs.push_back(make_int4(u, b0, a, 0)); pseg.push_back(cur); }
                    cur = sg;
                    b0 = a;
                }
            }
            if (a1 > a0) { pcs.push_back(make_int4(u, b0, a1, 0)); pseg.push_back(cur); }
            const int np = (int)(pcs.size() - first);
            for (int k = 0; k < np; k++) pcs[first + k].w = k | (np << 16);
        }
        std::vector<int> seg((size_t)nseg + 1, 0);
        for (int sg : pseg) seg[sg + 1]++;
        for (int k = 0; k < nseg; k++) seg[k + 1] += seg[k];
        if ((rc = part_upload(s, s->part_asm_bal[o], seg, pcs))) return rc;
    }
    return GADE_OK;
}

static size_t asm_smem_bytes(const gade_solver *s, size_t elem)
{
    unsigned a, b, c;
    return asm_smem((s->CM + 2) & ~1, s->W, s->RM, 256, (unsigned)elem, &a, &b, &c);
}

/* dynamic shared memory of k_apply_asm32 */
static size_t asm32_smem_bytes(const gade_solver *s)
{
    unsigned a, b, c, d, e;
    return a32_smem(s->W, (s->RM + 3) & ~3, s->B, 256, s->max_row_pairs, &a, &b, &c, &d, &e);
}

/* Builds K_a for every pulse factor a that some Bessel order uses: the
   tables of a unit factor, then every pair's values from them.  Skipped
   (the solver stays matrix-free) when K would take more than half of the
   free device memory. */
static int asm_build(gade_solver *s)
{
    if (!s->rc || s->npairs == 0 || s->asm_ok) return GADE_OK;
    for (int par : s->h_pair_par)
        if (par < 0) return GADE_OK;             /* a pair coupled by both parities: stay matrix-free */
    const size_t WB = (size_t)s->W * s->B, per = (size_t)s->npairs * WB;
    if (WB % 2) return GADE_OK;
    s->lpar[0] = s->lmax > 0 ? 0 : -1;
    s->lpar[1] = s->lmax > 1 ? 1 : -1;
    /* K depends only on the radial tables: one set unless the pulses have their own */
    const int nset = s->g_ext ? s->npulse : 1;
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    const bool mixed = s->prec == GADE_PREC_MIXED;
    const double need = (double)per * (24.0 * nset + (mixed ? 12.0 : 8.0) * s->npulse);
    if (need > 0.5 * (double)fr) return GADE_OK;
    int rc;
    if ((rc = dev_upload(s, &s->d_K, (const double *)nullptr, per * 3 * nset))) return rc;
    if ((rc = dev_upload(s, &s->d_A, (const double *)nullptr, per * s->npulse))) return rc;
    if (mixed) {
        /* chunk-major float copy; padded rows stay zero */
        s->RMp = (s->RM + 3) & ~3;
        s->a32_stride = (size_t)s->nchunk * s->npairs * s->W * s->RMp;
        float *a32 = nullptr;
        if ((rc = dev_upload(s, &a32, (const float *)nullptr, s->a32_stride * s->npulse))) return rc;
        s->d_A32 = a32;
    }
    s->asm_kstride = s->g_ext ? 3 * per : 0;
    if ((rc = dev_upload(s, &s->d_pair_par, s->h_pair_par.data(), s->h_pair_par.size()))) return rc;
    int *d_pr = nullptr, *d_lp = nullptr, *d_ll = nullptr, *d_le = nullptr;
    if ((rc = dev_upload(s, &d_pr, s->h_pair_r.data(), s->h_pair_r.size()))) return rc;
    if ((rc = dev_upload(s, &d_lp, s->h_le_ptr.data(), s->h_le_ptr.size()))) return rc;
    if ((rc = dev_upload(s, &d_ll, s->h_le_l.data(), s->h_le_l.size()))) return rc;
    if ((rc = dev_upload(s, &d_le, s->h_le_e.data(), s->h_le_e.size()))) return rc;
    const int prof = s->profile;
    s->profile = 0;
    for (int ks = 0; ks < nset && !rc; ks++)
    for (int a = 0; a < 6 && !rc; a++) {
        int l0 = -1;
        for (int l = 0; l < s->lmax && l0 < 0; l++)
            if ((l % 2 + 1) % 2 == a % 2) l0 = l;
        if (l0 < 0) continue;
        const int ia = (a - (l0 % 2 + 1) % 2) / 2;
        /* the previous factor's coefficient copy reads the pinned buffer
           when it runs: wait for it before rewriting the buffer */
        if (cudaStreamSynchronize(s->stream) != cudaSuccess) { rc = fail(GADE_ERR_CUDA, "assembled operator: K build failed"); break; }
        /* coefficients of a unit factor a: imaginary part 1 in every order of its parity */
        for (int l = 0; l < s->lmax; l++)
            for (int j = 0; j < 3; j++)
                s->h_coef[l * 3 + j] = make_double2(0.0, ((l % 2 + 1) % 2 == a % 2 && j == ia) ? 1.0 : 0.0);
        if (cudaMemcpyAsync(s->d_coef, s->h_coef, sizeof(double2) * s->lmax * 3, cudaMemcpyHostToDevice,
                            s->stream) != cudaSuccess) { rc = fail(GADE_ERR_CUDA, "assembled operator: coefficient upload failed"); break; }
        {
            /* the unit factor's tables from table set ks (the radial tables of pulse ks) */
            TabP T;
            T.lmax = s->lmax; T.nk = s->nk; T.W = s->W; T.B = s->B; T.kvals = s->d_kvals;
            T.g = (const double *)s->d_g + (size_t)ks * s->gstride;
            T.gt = (const double *)s->d_gt + (size_t)ks * s->gstride;
            T.M = (R4<double>::T *)s->d_M + (size_t)ks * s->mstride;
            T.M32 = nullptr; T.Mdd = nullptr; T.plist = nullptr; T.gstride = s->gstride; T.mstride = s->mstride;
            const int per_l = s->W * s->B;
            k_tables<true, 1><<<dim3((unsigned)((per_l + 255) / 256), s->lmax, 1), 256, 0, s->stream>>>(T, s->d_coef);
            if (cudaGetLastError() != cudaSuccess) { rc = fail(GADE_ERR_CUDA, "assembled operator: table launch failed"); break; }
        }
        dim3 grid((unsigned)((WB + 255) / 256), (unsigned)s->npairs);
        k_build_K<<<grid, 256, 0, s->stream>>>(s->d_K + (size_t)ks * 3 * per,
                                               (const R4<double>::T *)s->d_M + (size_t)ks * s->mstride, s->nk,
                                               (int)WB, a, d_pr, s->d_pair_par, s->d_row_kidx, d_lp, d_ll, d_le,
                                               (const double *)s->d_ang_a0, (const double *)s->d_ang_a0k,
                                               (const double *)s->d_ang_a1, (const double *)s->d_ang_a1k);
        if (cudaGetLastError() != cudaSuccess) { rc = fail(GADE_ERR_CUDA, "assembled operator: K build launch failed"); break; }
    }
    if (!rc && cudaStreamSynchronize(s->stream) != cudaSuccess) rc = fail(GADE_ERR_CUDA, "assembled operator: K build failed");
    s->profile = prof;
    s->has_time = 0;             /* the tables held a unit factor */
    dev_release(s, d_pr); dev_release(s, d_lp); dev_release(s, d_ll); dev_release(s, d_le);
    if (rc) return rc;
    for (int f = 0; f < 2; f++)
        for (int sep = 0; sep < 2; sep++) {
            int n = 0;
            const size_t sm = asm_smem_bytes(s, f ? sizeof(float2) : sizeof(double2));
            cudaError_t e;
            if (f && sep) { s->occ_asm[f][sep] = 1; continue; }   /* no complex64 instance with S x apart */
            if (f) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_apply_asm32, 256, asm32_smem_bytes(s));
            else e = sep ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_apply_asm<double, true>, 256, sm)
                         : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_apply_asm<double, false>, 256, sm);
            if (e != cudaSuccess || n < 1) { cudaGetLastError(); n = 1; }
            s->occ_asm[f][sep] = n > 8 ? 8 : n;
        }
    if ((rc = asm_partitions(s))) return rc;
    /* costs: 2 FMAs per stored value of the pairs' nonzero slots plus the
       diagonal blocks (complex, 4 FMAs); the values stream once per apply */
    s->asm_flops = 2.0 * (2.0 * (double)s->npairs * s->blk_nnz + 4.0 * (double)s->nblk * s->blk_nnz);
    s->asm_bytes = 8.0 * (double)per + 16.0 * (double)s->nk * WB + 4.0 * s->npairs + 48.0 * (double)s->n;
    s->asmb_flops = 2.0 * 3.0 * (double)per;
    s->asmb_bytes = 8.0 * 4.0 * (double)per;
    s->asm_ok = 1;
    return GADE_OK;
}

/* a launch with programmatic stream serialization (see pdl_enter) */
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args)
{
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = GADE_PDL;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

/* this step's assembled couplings from d_coef */
static int launch_assemble(gade_solver *s, cudaStream_t st)
{
    const int WB2 = s->W * s->B / 2;
    const size_t per2 = (size_t)s->npairs * WB2;
    prof_begin(s, st);
    A32Map F = {(float *)s->d_A32, s->d_row_pos, s->B, s->W, s->RMp, s->npairs, s->a32_stride};
    k_assemble<<<dim3((unsigned)((WB2 + 255) / 256), (unsigned)s->npairs, (unsigned)s->nslot), 256, 0, st>>>(
        (double2 *)s->d_A, F, (const double2 *)s->d_K, WB2, s->d_pair_par, s->d_coef,
        make_int2(s->lpar[0], s->lpar[1]), s->d_plist, per2, s->asm_kstride / 2, s->lmax);
    prof_end(s, st, 2);
    CKL();
    s->has_time = 1;
    return GADE_OK;
}

static OpP op_params32(const gade_solver *s);

/* the assembled operator in FP64 (x double2) or complex64 (x float2) */
template <typename R>
static int launch_apply_asm(gade_solver *s, const typename Cx<R>::T *x, int mode, VecP V, RedP red, cudaStream_t st)
{
    const bool f32 = sizeof(R) == 4;
    OpP P = f32 ? op_params32(s) : op_params(s);
    P.A = f32 ? (const void *)s->d_A32 : (const void *)s->d_A;
    P.pair_c = s->d_pair_c;
    P.astride = f32 ? s->a32_stride : (size_t)s->npairs * s->W * s->B;
    const bool sep = mode == AX_RHS || mode == AX_PARTS || mode == AX_MIX;
    if (f32 && sep) return fail(GADE_ERR_ARG, "complex64 assembled apply: mode %d has no float instance", mode);
    /* batches run the plain partition (their pulses fill the SMs) */
    const PartList &pl = (s->asm_part && s->nslot == 1) ? s->part_asm_bal[s->occ_asm[f32][sep]] : s->part_asm[0];
    P.seg_ptr = pl.d_seg_ptr;
    P.pieces = pl.d_pieces;
    dim3 grid(s->nslot, pl.nseg);
    const size_t smem = asm_smem_bytes(s, sizeof(typename Cx<R>::T));
    prof_begin(s, st);
    /* FP64 with programmatic dependent launch; the complex64 inner solve
       measured slower with it (4% per mixed step) and launches plainly */
    if (!f32) {
        if (sep) launch_pdl(k_apply_asm<R, true>, grid, dim3(256), smem, st, P, x, mode, V, red);
        else launch_pdl(k_apply_asm<R, false>, grid, dim3(256), smem, st, P, x, mode, V, red);
    } else {
        /* the values stream through shared memory by cp.async.bulk */
        k_apply_asm32<<<grid, 256, asm32_smem_bytes(s), st>>>(P, (const float2 *)x, mode, V, red, s->RMp, s->npairs,
                                                              s->max_row_pairs);
    }
    prof_end(s, st, f32 ? 0 : 0);
    CKL();
    return GADE_OK;
}

static int launch_apply(gade_solver *s, const double2 *x, int mode, VecP V, int redkind, cudaStream_t st,
                        int pred = PRED_NONE, DevScal *pb = nullptr)
{
    if (s->use_asm) return launch_apply_asm<double>(s, x, mode, V, make_red(s, s->d_sc, redkind, pred, nullptr, pb), st);
    OpP P = op_params(s);
    RedP red = make_red(s, s->d_sc, redkind, pred, nullptr, pb);
    dim3 grid(s->nslot, op_partition(s, P, false, mode));
    int nt;
    size_t smem;
    apply_dims(s, sizeof(double2), &nt, &smem);
    prof_begin(s, st);
    k_apply_launch<double>(s, grid, nt, smem, st, P, x, mode, V, red);
    prof_end(s, st, 0);
    CKL();
    return GADE_OK;
}

static PcT pc_params(const gade_solver *s, const void *FL, const void *FU, int pred)
{
    PcT Q;
    Q.nblk = s->nblk; Q.B = s->B; Q.Bp = s->Bp; Q.nch = s->nch;
    Q.row_kidx = s->d_row_kidx; Q.ord = s->d_ord; Q.FL = FL; Q.FU = FU;
    Q.plist = s->d_plist; Q.vstride = s->n; Q.fstride = s->fstride; Q.pred = pred;
    Q.spin_limit = s->pc_wait ? s->pc_wait : MBAR_SPIN_LIMIT;
    Q.withhold = s->pc_withhold;
    return Q;
}

static int launch_precond(gade_solver *s, int mode, const double2 *in0, const double2 *in1, double2 *io,
                          double2 *out, cudaStream_t st, int pred = PRED_NONE)
{
    PcT Q = pc_params(s, s->d_FL, s->d_FU, pred);
    const size_t smem = pc_smem_bytes(s, sizeof(double2));
    dim3 grid(s->nslot, s->nblk), block(32 * s->pc_nw);
    prof_begin(s, st);
    if (s->pc_nw == 8) {
        if (s->bwp == 16) launch_pdl(k_precond_tma<double, 16, 8>, grid, block, smem, st, Q, mode, in0, in1, io, out, s->d_sc);
        else launch_pdl(k_precond_tma<double, 32, 8>, grid, block, smem, st, Q, mode, in0, in1, io, out, s->d_sc);
    } else {
        if (s->bwp == 16) launch_pdl(k_precond_tma<double, 16, 4>, grid, block, smem, st, Q, mode, in0, in1, io, out, s->d_sc);
        else launch_pdl(k_precond_tma<double, 32, 4>, grid, block, smem, st, Q, mode, in0, in1, io, out, s->d_sc);
    }
    prof_end(s, st, 1);
    CKL();
    return GADE_OK;
}

/* coefficients of pulse k: c_a = SoL * (i h dt_k/2) * f_a, as in tools/solver.c:274 */
static int fill_coef(gade_solver *s, int k, const double *ft)
{
    const double hdt2 = s->h * s->dts[k] / 2;
    double2 *c = s->h_coef + (size_t)k * s->lmax * 3;
    for (int l = 0; l < s->lmax; l++)
        for (int ia = 0; ia < 3; ia++) {
            int a = (l % 2 + 1) % 2 + 2 * ia;
            double fr = ft[2 * a], fi = ft[2 * a + 1];
            /* (SoL * (0 + i hdt2)) * (fr + i fi) */
            double cr = 0.0 * SOL, ci = SOL * hdt2;
            c[l * 3 + ia] = make_double2(cr * fr - ci * fi, cr * fi + ci * fr);
        }
    if (s->rc)
        for (int a = 0; a < 6; a++)
            if (ft[2 * a + 1] != 0.0)
                return fail(GADE_ERR_ARG, "pulse factor f_%d has an imaginary part; the real-coupling tables need real f(t)", a);
    return GADE_OK;
}

/* per-step radial tables of the listed pulses from d_coef (which: 1 FP64, 2
   FP32, 3 both in one pass) */
static int launch_table_kernels(gade_solver *s, int which, cudaStream_t st)
{
    TabP T;
    T.lmax = s->lmax; T.nk = s->nk; T.W = s->W; T.B = s->B;
    T.kvals = s->d_kvals; T.g = s->d_g; T.gt = s->d_gt; T.M = s->d_M; T.M32 = s->d_M32; T.Mdd = s->d_Mdd;
    T.plist = s->d_plist; T.gstride = s->gstride; T.mstride = s->mstride;
    if (!s->d_M32) which &= ~2;
    if (!s->d_Mdd || !s->rc) which &= ~4;
    if (!which) return GADE_OK;
    const int per_l = s->W * s->B, nt = 256;
    dim3 grid((unsigned)((per_l + nt - 1) / nt), s->lmax, s->nslot);
    prof_begin(s, st);
#define KT(OUT_) do { if (s->rc) k_tables<true, OUT_><<<grid, nt, 0, st>>>(T, s->d_coef); \
                      else k_tables<false, OUT_><<<grid, nt, 0, st>>>(T, s->d_coef); } while (0)
    switch (which) {
    case 1: KT(1); break;
    case 2: KT(2); break;
    case 3: KT(3); break;
    case 4: if (s->rc) k_tables<true, 4><<<grid, nt, 0, st>>>(T, s->d_coef); break;
    case 5: if (s->rc) k_tables<true, 5><<<grid, nt, 0, st>>>(T, s->d_coef); break;
    case 6: if (s->rc) k_tables<true, 6><<<grid, nt, 0, st>>>(T, s->d_coef); break;
    default: if (s->rc) k_tables<true, 7><<<grid, nt, 0, st>>>(T, s->d_coef); break;
    }
#undef KT
    prof_end(s, st, 2);
    CKL();
    if (which & 1) s->m64_stale = 0;
    s->has_time = 1;
    return GADE_OK;
}

static int launch_tables(gade_solver *s, const double *ft, int which = 1)
{
    int rc = fill_coef(s, 0, ft);
    if (rc) return rc;
    CK(cudaMemcpyAsync(s->d_coef, s->h_coef, sizeof(double2) * (size_t)s->lmax * 3, cudaMemcpyHostToDevice, s->stream));
    if (s->use_asm && which) return launch_assemble(s, s->stream);   /* FP64 values and their float copy */
    return launch_table_kernels(s, which, s->stream);
}

static int sync_scal(gade_solver *s)
{
    CK(cudaMemcpyAsync(s->h_sc, s->d_sc, sizeof(DevScal), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (s->h_sc->err) {
        unsigned e = s->h_sc->err;
        CK(cudaMemsetAsync(&s->d_sc->err, 0, sizeof(unsigned), s->stream));
        return fail(GADE_ERR_CUDA, "device wait timed out (flags %u): TMA copy did not complete", e);
    }
    return GADE_OK;
}

/* the FP64 radial tables of the last step, where a mixed step with the
   double-float residual pass left them out (from its coefficients, d_coef) */
static int ensure_fp64_tables(gade_solver *s)
{
    if (!s->m64_stale || s->use_asm) return GADE_OK;
    return launch_table_kernels(s, 1, s->stream);
}

extern "C" int gade_solver_set_time(gade_solver *s, const double *ft)
{
    if (!s || !ft) return fail(GADE_ERR_ARG, "gade_solver_set_time: NULL argument");
    CK(cudaSetDevice(s->device));
    int rc = launch_tables(s, ft, 3);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream));
    return GADE_OK;
}

extern "C" int gade_solver_set_x(gade_solver *s, const double *x, int64_t n)
{
    if (!s || !x) return fail(GADE_ERR_ARG, "gade_solver_set_x: NULL argument");
    if (n != s->n) return fail(GADE_ERR_ARG, "gade_solver_set_x: size %lld != %lld", (long long)n, s->n);
    CK(cudaSetDevice(s->device));
    CK(cudaMemcpyAsync(s->x, x, sizeof(double2) * (size_t)n, cudaMemcpyHostToDevice, s->stream));
    /* a new state has no extrapolation history */
    if (s->d_hprev) CK(cudaMemsetAsync(s->d_hprev, 0, sizeof(int), s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return GADE_OK;
}

extern "C" int gade_solver_get_x(gade_solver *s, double *x, int64_t n)
{
    if (!s || !x) return fail(GADE_ERR_ARG, "gade_solver_get_x: NULL argument");
    if (n != s->n) return fail(GADE_ERR_ARG, "gade_solver_get_x: size %lld != %lld", (long long)n, s->n);
    CK(cudaSetDevice(s->device));
    CK(cudaMemcpyAsync(x, s->x, sizeof(double2) * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return GADE_OK;
}

extern "C" int gade_solver_apply(gade_solver *s, const double *x, double *y, double *Sx, double *Hx)
{
    if (!s || !x) return fail(GADE_ERR_ARG, "gade_solver_apply: NULL argument");
    if (!s->has_time) return fail(GADE_ERR_STATE, "gade_solver_apply: call gade_solver_set_time first");
    CK(cudaSetDevice(s->device));
    {
        int rc0 = ensure_fp64_tables(s);
        if (rc0) return rc0;
    }
    const size_t bytes = sizeof(double2) * (size_t)s->n;
    CK(cudaMemcpyAsync(s->tmp0, x, bytes, cudaMemcpyHostToDevice, s->stream));
    VecP V = {};
    int rc;
    if (y) {
        V.out0 = s->tmp1;
        if ((rc = launch_apply(s, s->tmp0, AX_PLAIN, V, RED_NONE, s->stream))) return rc;
        CK(cudaMemcpyAsync(y, s->tmp1, bytes, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    if (Sx || Hx) {
        V.out0 = s->tmp1; V.out1 = s->s;   /* s is scratch here */
        if ((rc = launch_apply(s, s->tmp0, AX_PARTS, V, RED_NONE, s->stream))) return rc;
        if (Sx) CK(cudaMemcpyAsync(Sx, s->tmp1, bytes, cudaMemcpyDeviceToHost, s->stream));
        if (Hx) CK(cudaMemcpyAsync(Hx, s->s, bytes, cudaMemcpyDeviceToHost, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    return GADE_OK;
}

extern "C" int gade_solver_apply_device(gade_solver *s, const void *x_dev, void *y_dev, void *stream)
{
    if (!s || !x_dev || !y_dev) return fail(GADE_ERR_ARG, "gade_solver_apply_device: NULL argument");
    if (!s->has_time) return fail(GADE_ERR_STATE, "gade_solver_apply_device: call gade_solver_set_time first");
    if (s->m64_stale && !s->use_asm) {
        /* refreshed on the solver's stream, which the caller's stream may not follow */
        CK(cudaSetDevice(s->device));
        int rc0 = ensure_fp64_tables(s);
        if (rc0) return rc0;
        CK(cudaStreamSynchronize(s->stream));
    }
    VecP V = {};
    V.out0 = y_dev;
    return launch_apply(s, (const double2 *)x_dev, AX_PLAIN, V, RED_NONE,
                        stream ? (cudaStream_t)stream : s->stream);
}

extern "C" int gade_solver_precond(gade_solver *s, const double *b, double *z)
{
    if (!s || !b || !z) return fail(GADE_ERR_ARG, "gade_solver_precond: NULL argument");
    CK(cudaSetDevice(s->device));
    const size_t bytes = sizeof(double2) * (size_t)s->n;
    CK(cudaMemcpyAsync(s->tmp0, b, bytes, cudaMemcpyHostToDevice, s->stream));
    int rc = launch_precond(s, PC_PLAIN, s->tmp0, nullptr, nullptr, s->tmp1, s->stream);
    if (rc) return rc;
    CK(cudaMemcpyAsync(z, s->tmp1, bytes, cudaMemcpyDeviceToHost, s->stream));
    return sync_scal(s);
}

extern "C" int64_t gade_solver_launch_count(const gade_solver *s) { return s ? s->launches : -1; }

static OpP op_params32(const gade_solver *s)
{
    OpP P = op_params(s);
    P.ang_a0 = s->d_a32[0]; P.ang_a0k = s->d_a32[1]; P.ang_a1 = s->d_a32[2]; P.ang_a1k = s->d_a32[3];
    P.M = s->d_M32; P.S_ell = s->d_S32; P.Hst_ell = s->d_H32; P.D_ell = s->d_D32;
    return P;
}

static int launch_apply32(gade_solver *s, const float2 *x, int mode, VecP V, int redkind, DevScal *sc,
                          int pred = PRED_NONE)
{
    if (s->use_asm) return launch_apply_asm<float>(s, x, mode, V, make_red(s, sc, redkind, pred), s->stream);
    OpP P = op_params32(s);
    RedP red = make_red(s, sc, redkind, pred);
    dim3 grid(s->nslot, op_partition(s, P, true, mode));
    int nt;
    size_t smem;
    apply_dims(s, sizeof(float2), &nt, &smem);
    prof_begin(s, s->stream);
    k_apply_launch<float>(s, grid, nt, smem, s->stream, P, x, mode, V, red);
    prof_end(s, s->stream, 0);
    CKL();
    return GADE_OK;
}

static int launch_precond32(gade_solver *s, int mode, const float2 *in0, const float2 *in1, float2 *io,
                            float2 *out, DevScal *sc, int pred = PRED_NONE)
{
    PcT Q = pc_params(s, s->d_FL32, s->d_FU32, pred);
    /* 4 warps: the complex64 solves are not bound by the FP64 units, and 8
       warps measured slower in the mixed step (0.099 against 0.080 ms per
       step at N = 244,000) */
    const size_t smem = pc_smem_bytes(s, sizeof(float2));
    dim3 grid(s->nslot, s->nblk);
    prof_begin(s, s->stream);
    if (s->bwp == 16) k_precond_tma<float, 16, 4><<<grid, 128, smem, s->stream>>>(Q, mode, in0, in1, io, out, sc);
    else k_precond_tma<float, 32, 4><<<grid, 128, smem, s->stream>>>(Q, mode, in0, in1, io, out, sc);
    prof_end(s, s->stream, 1);
    CKL();
    return GADE_OK;
}

/*
 * Partition of a single pulse's operator work: when one pulse's (chunk, block
 * row) units are too few or too uneven to balance the SMs, either 2-4 CTAs
 * share each unit (order split) or the balanced segments cut the work into
 * one equal share per resident CTA.  The choice is made by timing the
 * operator (FP64, plus two complex64 applies in mixed precision) for every
 * candidate on the zeroed tables, once at creation; a candidate after the
 * plain layout is kept only for a clear gain.
 */
static int choose_split(gade_solver *s)
{
    const long long ctas = (long long)s->nchunk * s->nblk;
    int maxs = (int)((8LL * s->nsm + ctas - 1) / ctas);
    if (maxs > 4) maxs = 4;
    for (int k = 0; k < 5; k++) s->split_ms[k] = 0.f;
    int rc;
    for (int ns = 2; ns <= maxs; ns++)
        if ((rc = part_build_split(s, ns))) return rc;
    if ((rc = part_build_balanced_all(s))) return rc;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_ns = 1;
    double best_gamma = 1.0;
    int best_waves = 1;
    /* candidates in order: plain, order splits, balanced (0) with three
       weights of the gather in its cost model, then with two and three
       segments per resident CTA slot (the block scheduler hands the later
       ones to the CTA slots that free first) */
    const double gammas[5] = {1.0, 0.7, 1.4, 1.0, 1.0};
    const int waves[5] = {1, 1, 1, 2, 3};
    for (int c = 0; c < maxs + 5; c++) {
        const int ns = c < maxs ? c + 1 : 0;
        if (ns == 0) {
            s->bal_gamma = gammas[c - maxs];
            s->bal_waves = waves[c - maxs];
            for (PartList &pl : s->part_bal) part_release(s, pl);
            if ((rc = part_build_balanced_all(s))) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
        }
        s->nsplit = ns;
        for (int rep = 0; rep < 4; rep++) {
            if (rep == 1) CK(cudaEventRecord(e0, s->stream));
            VecP V = {}; V.out0 = s->tmp1; V.in0 = s->r0;
            rc = launch_apply(s, s->x, AX_R0V, V, RED_R0V, s->stream);
            for (int k = 0; !rc && s->prec == GADE_PREC_MIXED && k < 2; k++) {
                VecP V32 = {}; V32.out0 = s->v32; V32.in0 = s->r032;
                rc = launch_apply32(s, s->y32, AX_R0V, V32, RED_R0V, s->d_sc, PRED_NONE);
            }
            if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
        }
        CK(cudaEventRecord(e1, s->stream));
        CK(cudaEventSynchronize(e1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (ns == 0 && s->split_ms[0] > 0.f && ms / 3 >= s->split_ms[0]) continue;   /* keep the best weight's time */
        s->split_ms[ns] = ms / 3;
        if (ms < best * 0.98f || (ns == 0 && best_ns == 0 && ms < best)) {
            best = ms;
            best_ns = ns;
            if (ns == 0) { best_gamma = s->bal_gamma; best_waves = s->bal_waves; }
        }
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    if (s->bal_gamma != best_gamma || s->bal_waves != best_waves) {
        s->bal_gamma = best_gamma;
        s->bal_waves = best_waves;
        for (PartList &pl : s->part_bal) part_release(s, pl);
        if ((rc = part_build_balanced_all(s))) return rc;
    }
    s->nsplit = best_ns;
    return GADE_OK;
}

/* ms per FP64 apply (R0V) of the current operator and partition, plus two
   complex64 applies in mixed precision (as choose_split times them) */
static int time_fp64_apply(gade_solver *s, float *ms)
{
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int rc = GADE_OK;
    for (int rep = 0; rep < 4 && !rc; rep++) {
        if (rep == 1 && cudaEventRecord(e0, s->stream) != cudaSuccess) rc = fail(GADE_ERR_CUDA, "event record failed");
        VecP V = {}; V.out0 = s->tmp1; V.in0 = s->r0;
        if (!rc) rc = launch_apply(s, s->x, AX_R0V, V, RED_R0V, s->stream);
        for (int k = 0; !rc && s->prec == GADE_PREC_MIXED && k < 2; k++) {
            VecP V32 = {}; V32.out0 = s->v32; V32.in0 = s->r032;
            rc = launch_apply32(s, s->y32, AX_R0V, V32, RED_R0V, s->d_sc, PRED_NONE);
        }
    }
    float t = 0;
    if (!rc && (cudaEventRecord(e1, s->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&t, e0, e1) != cudaSuccess))
        rc = fail(GADE_ERR_CUDA, "apply timing failed");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / 3;
    return rc;
}

/*
 * Matrix-free or assembled operator for one pulse with real couplings:
 * the assembled values (K_a) are built, both of their partitions timed, and
 * the assembled operator is kept when its apply is clearly faster than the
 * matrix-free one chosen by choose_split (its per-step assembly replaces the
 * radial tables).
 */
/* ms of the step's tables of the current operator: the matrix-free radial
   tables or the assembly of the coupling values (float copies included in
   mixed precision) */
static int time_step_tables(gade_solver *s, float *ms)
{
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const int which = s->prec == GADE_PREC_MIXED ? 3 : 1;
    int rc = s->use_asm ? launch_assemble(s, s->stream) : launch_table_kernels(s, which, s->stream);
    if (!rc && cudaEventRecord(e0, s->stream) != cudaSuccess) rc = fail(GADE_ERR_CUDA, "event record failed");
    for (int rep = 0; rep < 3 && !rc; rep++)
        rc = s->use_asm ? launch_assemble(s, s->stream) : launch_table_kernels(s, which, s->stream);
    float t = 0;
    if (!rc && (cudaEventRecord(e1, s->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&t, e0, e1) != cudaSuccess))
        rc = fail(GADE_ERR_CUDA, "table timing failed");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / 3;
    s->has_time = 0;
    return rc;
}

/* A step's operator cost: its tables plus three operator applies (the
   right-hand side and one BiCGSTAB iteration; in mixed precision the timed
   apply is the FP64 residual pass plus one inner iteration's two complex64
   applies, so it counts once) */
static float step_cost(const gade_solver *s, float tables_ms, float apply_ms)
{
    return tables_ms + (s->prec == GADE_PREC_MIXED ? 1.0f : 3.0f) * apply_ms;
}

static int choose_operator(gade_solver *s)
{
    s->mf_ms = s->split_ms[s->nsplit >= 1 && s->nsplit <= 4 ? s->nsplit : 0];
    s->asm_ms[0] = s->asm_ms[1] = 0.f;
    int rc = asm_build(s);
    if (rc || !s->asm_ok) return rc;
    float tab_mf = 0.f, tab_asm = 0.f;
    s->use_asm = 0;
    if ((rc = time_step_tables(s, &tab_mf))) return rc;
    s->use_asm = 1;
    for (int part = 0; part < 2 && !rc; part++) {
        s->asm_part = part;
        rc = time_fp64_apply(s, &s->asm_ms[part]);
    }
    if (!rc) rc = time_step_tables(s, &tab_asm);
    if (rc) { s->use_asm = 0; return rc; }
    s->asm_part = s->asm_ms[1] < s->asm_ms[0] ? 1 : 0;
    const float best = s->asm_ms[s->asm_part];
    s->tab_ms[0] = tab_mf;
    s->tab_ms[1] = tab_asm;
    s->use_asm = (s->mf_ms <= 0.f ||
                  step_cost(s, tab_asm, best) < 0.98f * step_cost(s, tab_mf, s->mf_ms)) ? 1 : 0;
    return GADE_OK;
}

extern "C" int gade_solver_set_operator(gade_solver *s, int32_t assembled)
{
    if (!s) return fail(GADE_ERR_ARG, "gade_solver_set_operator: NULL solver");
    if (assembled != 0 && assembled != 1)
        return fail(GADE_ERR_ARG, "gade_solver_set_operator: %d is neither 0 (matrix-free) nor 1 (assembled)", assembled);
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    int rc;
    if (assembled && !s->asm_ok) {
        if ((rc = asm_build(s))) return rc;
        if (!s->asm_ok)
            return fail(GADE_ERR_ARG, "gade_solver_set_operator: the assembled operator needs real couplings, "
                                      "each pair coupled by orders of one parity, and device memory for its values");
        s->asm_part = 1;
    }
    if (s->engine) batch_drop_graphs(s->engine);
    s->use_asm = assembled;
    s->has_time = 0;             /* the next set_time or step fills the chosen operator's tables */
    return GADE_OK;
}

extern "C" int gade_solver_operator(const gade_solver *s, int32_t *assembled, float *ms)
{
    if (!s) return fail(GADE_ERR_ARG, "gade_solver_operator: NULL solver");
    if (assembled) *assembled = s->use_asm;
    if (ms) {
        ms[0] = s->mf_ms; ms[1] = s->asm_ms[0]; ms[2] = s->asm_ms[1];
        ms[3] = s->tab_ms[0]; ms[4] = s->tab_ms[1];
    }
    return GADE_OK;
}

extern "C" int gade_solver_create(const gade_problem *p, double dt, double h, int32_t precision,
                                  int32_t device, gade_solver **out)
{
    if (!p || !out) return fail(GADE_ERR_ARG, "gade_solver_create: NULL argument");
    *out = nullptr;
    if (precision != GADE_PREC_FP64 && precision != GADE_PREC_MIXED)
        return fail(GADE_ERR_ARG, "gade_solver_create: unknown precision %d", precision);
    if (!(dt > 0) || !std::isfinite(dt)) return fail(GADE_ERR_ARG, "gade_solver_create: dt must be finite and > 0");
    int rc = solver_create(p, 1, &dt, nullptr, h, precision, device, 0, out);
    if (rc) return rc;
    if ((rc = choose_split(*out))) { gade_solver_free(*out); *out = nullptr; return rc; }
    if ((rc = choose_operator(*out))) { gade_solver_free(*out); *out = nullptr; return rc; }
    return GADE_OK;
}


extern "C" int gade_solver_step(gade_solver *s, const double *ft, int32_t maxit, double tol,
                                gade_step_stats *stats)
{
    if (!s || !ft) return fail(GADE_ERR_ARG, "gade_solver_step: NULL argument");
    if (maxit < 0) return fail(GADE_ERR_ARG, "gade_solver_step: maxit < 0");
    if (!(tol >= 0) || !std::isfinite(tol)) return fail(GADE_ERR_ARG, "gade_solver_step: tol must be finite and >= 0");
    CK(cudaSetDevice(s->device));
    return solver_engine_step(s, ft, maxit, tol, stats);
}

extern "C" int gade_solver_step_host(gade_solver *s, const double *x_in, const double *ft, int32_t maxit, double tol,
                                     double *x_out, gade_step_stats *stats)
{
    if (!s || !ft) return fail(GADE_ERR_ARG, "gade_solver_step_host: NULL argument");
    if (maxit < 0) return fail(GADE_ERR_ARG, "gade_solver_step_host: maxit < 0");
    if (!(tol >= 0) || !std::isfinite(tol)) return fail(GADE_ERR_ARG, "gade_solver_step_host: tol must be finite and >= 0");
    CK(cudaSetDevice(s->device));
    if (x_in) {
        /* stream-ordered before the step; like gade_solver_set_x, a new state
           has no extrapolation history */
        CK(cudaMemcpyAsync(s->x, x_in, sizeof(double2) * (size_t)s->n, cudaMemcpyHostToDevice, s->stream));
        if (s->d_hprev) CK(cudaMemsetAsync(s->d_hprev, 0, sizeof(int), s->stream));
    }
    return solver_engine_step(s, ft, maxit, tol, stats, x_out);
}

extern "C" int gade_solver_time_apply(gade_solver *s, int32_t reps, double *ms)
{
    if (!s || !ms || reps < 1) return fail(GADE_ERR_ARG, "gade_solver_time_apply: bad argument");
    if (!s->has_time) return fail(GADE_ERR_STATE, "gade_solver_time_apply: call gade_solver_set_time first");
    CK(cudaSetDevice(s->device));
    {
        int rc0 = ensure_fp64_tables(s);
        if (rc0) return rc0;
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    VecP V = {}; V.out0 = s->tmp1;
    int rc;
    if ((rc = launch_apply(s, s->x, AX_PLAIN, V, RED_NONE, s->stream))) return rc;
    CK(cudaEventRecord(e0, s->stream));
    for (int k = 0; k < reps; k++)
        if ((rc = launch_apply(s, s->x, AX_PLAIN, V, RED_NONE, s->stream))) return rc;
    CK(cudaEventRecord(e1, s->stream));
    CK(cudaEventSynchronize(e1));
    float t = 0;
    CK(cudaEventElapsedTime(&t, e0, e1));
    *ms = t / reps;
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    return GADE_OK;
}

extern "C" int gade_solver_time_apply_mixed(gade_solver *s, int32_t reps, double *ms)
{
    if (!s || !ms || reps < 1) return fail(GADE_ERR_ARG, "gade_solver_time_apply_mixed: bad argument");
    if (s->prec != GADE_PREC_MIXED) return fail(GADE_ERR_STATE, "gade_solver_time_apply_mixed: not a mixed-precision solver");
    if (!s->has_time) return fail(GADE_ERR_STATE, "gade_solver_time_apply_mixed: call gade_solver_set_time first");
    CK(cudaSetDevice(s->device));
    int rc;
    /* this step's complex64 operator: the assembly wrote both copies; the
       matrix-free tables are refreshed in both precisions */
    if (!s->use_asm && (rc = launch_table_kernels(s, 3, s->stream))) return rc;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    VecP V = {}; V.out0 = s->v32; V.in0 = s->r032;
    /* the inner solve's apply with its <r0, v> reduction (on the inner record,
       which every refinement sweep re-initialises) */
    if ((rc = launch_apply32(s, s->y32, AX_R0V, V, RED_R0V, s->d_sc2))) return rc;
    CK(cudaEventRecord(e0, s->stream));
    for (int k = 0; k < reps; k++)
        if ((rc = launch_apply32(s, s->y32, AX_R0V, V, RED_R0V, s->d_sc2))) return rc;
    CK(cudaEventRecord(e1, s->stream));
    CK(cudaEventSynchronize(e1));
    float t = 0;
    CK(cudaEventElapsedTime(&t, e0, e1));
    *ms = t / reps;
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    return GADE_OK;
}

extern "C" int gade_solver_time_precond(gade_solver *s, int32_t reps, double *ms)
{
    if (!s || !ms || reps < 1) return fail(GADE_ERR_ARG, "gade_solver_time_precond: bad argument");
    CK(cudaSetDevice(s->device));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    int rc;
    if ((rc = launch_precond(s, PC_PLAIN, s->x, nullptr, nullptr, s->tmp1, s->stream))) return rc;
    CK(cudaEventRecord(e0, s->stream));
    for (int k = 0; k < reps; k++)
        if ((rc = launch_precond(s, PC_PLAIN, s->x, nullptr, nullptr, s->tmp1, s->stream))) return rc;
    CK(cudaEventRecord(e1, s->stream));
    CK(cudaEventSynchronize(e1));
    float t = 0;
    CK(cudaEventElapsedTime(&t, e0, e1));
    *ms = t / reps;
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    return GADE_OK;
}

extern "C" void *gade_solver_stream(const gade_solver *s) { return s ? (void *)s->stream : nullptr; }

extern "C" int gade_solver_profile(gade_solver *s, int32_t enable)
{
    if (!s) return fail(GADE_ERR_ARG, "gade_solver_profile: NULL solver");
    CK(cudaSetDevice(s->device));
    prof_collect(s);
    s->profile = enable ? 1 : 0;
    return GADE_OK;
}

extern "C" int gade_solver_kernel_times(gade_solver *s, gade_kernel_times *out)
{
    if (!s || !out) return fail(GADE_ERR_ARG, "gade_solver_kernel_times: NULL argument");
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    prof_collect(s);
    out->apply_launches = s->prof_n[0]; out->apply_ms = s->prof_ms[0];
    out->precond_launches = s->prof_n[1]; out->precond_ms = s->prof_ms[1];
    out->other_launches = s->prof_n[2]; out->other_ms = s->prof_ms[2];
    for (int k = 0; k < 3; k++) { s->prof_n[k] = 0; s->prof_ms[k] = 0; }
    return GADE_OK;
}

/* 8 independent FMA chains per thread; 2 flops per FMA */
__global__ void k_fp64_peak(double *out, int iters, double m, double c)
{
    double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
    double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
    for (int i = 0; i < iters; i++) {
        a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
        a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
    double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == 1234.5) out[blockIdx.x * blockDim.x + threadIdx.x] = s;   /* keep the chains live */
}

extern "C" int gade_probe_fp64_peak(int32_t device, double *tflops)
{
    if (!tflops) return fail(GADE_ERR_ARG, "gade_probe_fp64_peak: NULL argument");
    CK(cudaSetDevice(device));
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, device));
    const int blocks = prop.multiProcessorCount * 8, threads = 256, iters = 4096;
    double *out = nullptr;
    CK(cudaMalloc(&out, sizeof(double) * blocks * threads));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    k_fp64_peak<<<blocks, threads>>>(out, iters, 0.9999999, 1e-12);   /* warm-up */
    CK(cudaGetLastError());
    float best = 1e30f;
    for (int rep = 0; rep < 5; rep++) {
        CK(cudaEventRecord(e0));
        k_fp64_peak<<<blocks, threads>>>(out, iters, 0.9999999, 1e-12);
        CK(cudaEventRecord(e1));
        CK(cudaEventSynchronize(e1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) best = ms;
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    cudaFree(out);
    const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return GADE_OK;
}

extern "C" int gade_solver_set_split(gade_solver *s, int32_t nsplit)
{
    if (!s) return fail(GADE_ERR_ARG, "gade_solver_set_split: NULL solver");
    if (nsplit < 0 || nsplit > 4) return fail(GADE_ERR_ARG, "gade_solver_set_split: nsplit %d not in 0..4", nsplit);
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    if (s->engine) batch_drop_graphs(s->engine);
    int rc;
    if (nsplit >= 2 && !s->part_split[nsplit].nseg && (rc = part_build_split(s, nsplit))) return rc;
    if (nsplit == 0 && (rc = part_build_balanced_all(s))) return rc;
    s->nsplit = nsplit;
    return GADE_OK;
}

extern "C" int gade_solver_balanced(const gade_solver *s, int32_t *segments, int32_t *pieces, float *ms,
                                    double *gather_weight)
{
    if (!s) return fail(GADE_ERR_ARG, "gade_solver_balanced: NULL solver");
    const PartList &pl = s->part_bal[s->occ[0][0]];
    if (segments) *segments = pl.nseg;
    if (pieces) *pieces = pl.npieces;
    if (ms) *ms = s->split_ms[0];
    if (gather_weight) *gather_weight = s->bal_gamma > 0 ? s->bal_gamma : 1.0;
    return GADE_OK;
}

extern "C" int gade_solver_split(const gade_solver *s, int32_t *nsplit, float *split_ms)
{
    if (!s) return fail(GADE_ERR_ARG, "gade_solver_split: NULL solver");
    if (nsplit) *nsplit = s->nsplit;
    if (split_ms) for (int k = 0; k < 4; k++) split_ms[k] = s->split_ms[k + 1];
    return GADE_OK;
}

extern "C" int gade_solver_flops(const gade_solver *s, double *apply_flops, double *precond_flops)
{
    if (!s) return fail(GADE_ERR_ARG, "gade_solver_flops: NULL solver");
    if (apply_flops) *apply_flops = s->use_asm ? s->asm_flops : s->apply_flops;
    if (precond_flops) *precond_flops = s->precond_flops;
    return GADE_OK;
}

extern "C" int gade_solver_apply_bytes(const gade_solver *s, double *bytes)
{
    if (!s || !bytes) return fail(GADE_ERR_ARG, "gade_solver_apply_bytes: NULL argument");
    *bytes = s->use_asm ? s->asm_bytes : s->apply_bytes;
    return GADE_OK;
}

extern "C" int gade_solver_assembly_cost(const gade_solver *s, double *flops, double *bytes)
{
    if (!s) return fail(GADE_ERR_ARG, "gade_solver_assembly_cost: NULL solver");
    if (flops) *flops = s->use_asm ? s->asmb_flops : 0.0;
    if (bytes) *bytes = s->use_asm ? s->asmb_bytes : 0.0;
    return GADE_OK;
}

/* ------------------------------------------------------------------ */
/* allocation-free operator apply + dot                                */
/* ------------------------------------------------------------------ */
/* Cross-CTA reduction scratch of gade_solver_apply_dot_noalloc: per-CTA
 * partial sums followed by the arrival ticket.  It is a file-scope device
 * array, so the library holds it on every GPU that loads it until exit and
 * the entry point needs no allocation.  All calls share it. */
#define GADE_NOALLOC_MAX_CTAS 16384
static __device__ __align__(256) double g_noalloc_scratch[GADE_NOALLOC_MAX_CTAS * NRED + 32];

#include <mutex>
static std::mutex g_noalloc_mu;
static double *g_noalloc_dev_ptr[256];   /* device address of the array, per device ordinal */

extern "C" int gade_solver_apply_dot_noalloc(gade_solver *s, const void *x_dev, const void *r0_dev, void *y_dev,
                                             void *dot_dev, void *stream)
{
    if (!s || !x_dev || !r0_dev || !y_dev || !dot_dev)
        return fail(GADE_ERR_ARG, "gade_solver_apply_dot_noalloc: NULL argument");
    if (!s->has_time) return fail(GADE_ERR_STATE, "gade_solver_apply_dot_noalloc: call gade_solver_set_time first");
    if (s->m64_stale && !s->use_asm) {
        /* refreshed on the solver's stream, which the caller's stream may not follow */
        CK(cudaSetDevice(s->device));
        int rc0 = ensure_fp64_tables(s);
        if (rc0) return rc0;
        CK(cudaStreamSynchronize(s->stream));
    }
    if (s->device < 0 || s->device >= 256) return fail(GADE_ERR_ARG, "gade_solver_apply_dot_noalloc: device ordinal out of range");
    const long long ncta = (long long)s->nchunk * s->nblk;
    if (ncta > GADE_NOALLOC_MAX_CTAS)
        return fail(GADE_ERR_ARG,
                    "gade_solver_apply_dot_noalloc: problem needs %lld reduction slots, more than the %d of the "
                    "library's fixed scratch array; use the allocating path (gade_solver_step/apply)",
                    ncta, GADE_NOALLOC_MAX_CTAS);
    CK(cudaSetDevice(s->device));
    double *base = nullptr;
    {
        /* once per device, with that device current: the host-side symbol is
           only a stand-in, the kernel needs the device address */
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_dev_ptr[s->device]) {
            void *ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr)
                return fail(GADE_ERR_CUDA, "gade_solver_apply_dot_noalloc: cudaGetSymbolAddress failed: %s",
                            cudaGetErrorString(e));
            g_noalloc_dev_ptr[s->device] = (double *)ptr;
        }
        base = g_noalloc_dev_ptr[s->device];
    }
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    unsigned int *ticket = (unsigned int *)(base + (size_t)GADE_NOALLOC_MAX_CTAS * NRED);
    /* the arrival ticket must start at zero */
    CK(cudaMemsetAsync(ticket, 0, sizeof(unsigned int), st));
    OpP P = op_params(s);        /* one piece per unit: no partial-sum scratch */
    RedP red = make_red(s, s->d_sc, RED_DOT_OUT, PRED_NONE);
    red.part = base; red.ticket = ticket; red.out = (double *)dot_dev;
    VecP V = {};
    V.out0 = y_dev;
    V.in0 = r0_dev;
    if (s->use_asm) {
        /* the assembled operator, one piece per unit */
        P.A = s->d_A;
        P.pair_c = s->d_pair_c;
        P.astride = (size_t)s->npairs * s->W * s->B;
        P.seg_ptr = s->part_asm[0].d_seg_ptr;
        P.pieces = s->part_asm[0].d_pieces;
        k_apply_asm<double, false><<<dim3(1, s->part_asm[0].nseg), 256, asm_smem_bytes(s, sizeof(double2)), st>>>(
            P, (const double2 *)x_dev, AX_R0V, V, red);
        CKL();
        return GADE_OK;
    }
    dim3 grid(1, s->part_split[1].nseg);
    int nt;
    size_t smem;
    apply_dims(s, sizeof(double2), &nt, &smem);
    k_apply_launch<double>(s, grid, nt, smem, st, P, (const double2 *)x_dev, AX_R0V, V, red);
    CKL();
    return GADE_OK;
}

/* ------------------------------------------------------------------ */
/* batched pulses                                                      */
/* ------------------------------------------------------------------ */
/*
 * A batch holds npulse Crank-Nicolson problems on one set of angular tables,
 * h0 and S; each pulse has its own dt, radial tables g and block-LU factors.
 * Every kernel runs over the pulses of the launch list (grid x = pulse slot),
 * and BiCGSTAB's control (convergence, iteration limit, restart test) lives
 * in the reduction epilogues, so a step is a fixed kernel sequence: the
 * tables, the right-hand side and K predicated iterations, captured once as
 * a CUDA graph and replayed.  The host reads the pulse states after each
 * replay and replays the iteration graph (preceded by the predicated restart
 * launch when a pulse asks for one) until no pulse is running.  A pulse
 * whose time grid has ended leaves the launch list (graphs are re-captured),
 * so finished pulses cost nothing.
 */
struct gade_batch {
    gade_solver *s;
    std::vector<int> list;          /* pulses of the current launch list */
    int kiter, kfixed;              /* iterations per captured launch; fixed value or 0 (adaptive) */
    int kwin, kwin_steps;           /* largest iteration count since the last shrink, steps since */
    double tol_c;
    int maxit_c;
    int use_graphs;
    cudaGraphExec_t g_first, g_iter, g_restart;
    long long replays, steps;
    float tune_ms[4];
    int tune_cs[4], ntune;
    double2 *d_corr;                /* [npulse][n] initial-guess corrections (mixed) */
    int use_guess;
    int internal;                   /* the step engine of a gade_solver (one pulse, no launch list) */
    double2 *xout_host;             /* one pulse: host buffer that receives the state with the control read-back */
    long long nodes[3];             /* kernels of each captured graph */
};

static void batch_drop_graphs(gade_batch *b)
{
    if (b->g_first) cudaGraphExecDestroy(b->g_first);
    if (b->g_iter) cudaGraphExecDestroy(b->g_iter);
    if (b->g_restart) cudaGraphExecDestroy(b->g_restart);
    b->g_first = b->g_iter = b->g_restart = nullptr;
}

/* K predicated BiCGSTAB iterations of every listed pulse still running */
static int batch_seq_iters(gade_batch *b, int K, cudaStream_t st)
{
    gade_solver *s = b->s;
    int rc;
    const size_t rsm = sizeof(double) * NRED * s->upd_block;
    for (int it = 0; it < K; it++) {
        if ((rc = launch_precond(s, PC_P, s->r, s->v, s->p, s->y, st, PRED_RUN))) return rc;
        VecP A1 = {}; A1.out0 = s->v; A1.in0 = s->r0;
        if ((rc = launch_apply(s, s->y, AX_R0V, A1, RED_R0V, st, PRED_RUN))) return rc;
        if ((rc = launch_precond(s, PC_S, s->r, s->v, s->s, s->z, st, PRED_RUN))) return rc;
        VecP A2 = {}; A2.out0 = s->t; A2.in0 = s->s;
        if ((rc = launch_apply(s, s->z, AX_TS, A2, RED_TS, st, PRED_RUN))) return rc;
        RedP red = make_red(s, s->d_sc, RED_UPDATE, PRED_RUN);
        launch_pdl(k_update<double>, dim3(s->upd_grid, s->nslot), dim3(s->upd_block), rsm, st,
                   s->n, s->x, (const double2 *)s->y, (const double2 *)s->z, s->r, (const double2 *)s->s,
                   (const double2 *)s->t, (const double2 *)s->r0, red, (const int *)s->d_plist);
        CKL();
    }
    return GADE_OK;
}

/* mixed precision: one refinement sweep of every listed pulse that needs
   one (FP64 residual pass, inner-solve start), K inner complex64 iterations
   of every pulse whose inner solve runs, then the delta update and the
   certification test of every pulse whose inner solve has ended */
/* the residual pass of a mixed step runs in double-float when the solver
   has the double-float tables and the operator is matrix-free */
static bool use_dd(const gade_solver *s) { return s->mix_dd && s->d_Mdd && !s->use_asm; }
static DdVec dd_vecs(const gade_solver *s)
{
    DdVec q = {nullptr, nullptr, nullptr};
    if (use_dd(s)) { q.x = s->xdd; q.d = s->ddd; q.w = s->wdd; }
    return q;
}

/* r = -S delta - H (2 x_n + delta), |b|^2, x_n^H S x_n (AX_MIX) with the
   matrix-free operator in double-float */
static int launch_apply_mix_dd(gade_solver *s, VecP V, cudaStream_t st)
{
    OpP P = op_params(s);
    P.ang_a0 = s->d_ang_dd[0]; P.ang_a0k = s->d_ang_dd[1]; P.ang_a1 = s->d_ang_dd[2]; P.ang_a1k = s->d_ang_dd[3];
    P.M = s->d_Mdd; P.S_ell = s->d_Sdd; P.Hst_ell = s->d_Hdd; P.D_ell = nullptr;
    RedP red = make_red(s, s->d_sc, RED_MIX, PRED_MIX, nullptr, s->d_sc2);
    dim3 grid(s->nslot, op_partition(s, P, false, AX_MIX));
    int nt;
    size_t smem;
    apply_dims(s, sizeof(cdd), &nt, &smem, true);
    V.in0dd = s->xdd; V.in1dd = s->ddd;
    prof_begin(s, st);
    if (s->zskip) k_apply<dd, true, true, true><<<grid, nt, smem, st>>>(P, s->wdd, AX_MIX, V, red);
    else k_apply<dd, true, true, false><<<grid, nt, smem, st>>>(P, s->wdd, AX_MIX, V, red);
    prof_end(s, st, 0);
    CKL();
    return GADE_OK;
}

static int batch_seq_sweep(gade_batch *b, int K, cudaStream_t st)
{
    gade_solver *s = b->s;
    int rc;
    const long long n = s->n;
    const int blk = s->upd_block;
    const dim3 grid(s->upd_grid, s->nslot);
    const size_t rsm = sizeof(double) * NRED * blk;
    VecP R = {};
    R.out0 = s->r; R.in0 = s->x; R.in1 = s->delta64;
    if (use_dd(s)) rc = launch_apply_mix_dd(s, R, st);
    else rc = launch_apply(s, s->tmp0, AX_MIX, R, RED_MIX, st, PRED_MIX, s->d_sc2);
    if (rc) return rc;
    {
        RedP red = make_red(s, s->d_sc2, RED_RHS, PRED_MIX, s->d_sc, nullptr);
        k_inner_init<<<grid, blk, rsm, st>>>(n, s->r, s->e32, s->ri32, s->r032, s->p32, s->v32, red, s->d_plist);
        CKL();
    }
    for (int it = 0; it < K; it++) {
        if ((rc = launch_precond32(s, PC_P, s->ri32, s->v32, s->p32, s->y32, s->d_sc2, PRED_RUN))) return rc;
        VecP A1 = {}; A1.out0 = s->v32; A1.in0 = s->r032;
        if ((rc = launch_apply32(s, s->y32, AX_R0V, A1, RED_R0V, s->d_sc2, PRED_RUN))) return rc;
        if ((rc = launch_precond32(s, PC_S, s->ri32, s->v32, s->s32, s->z32, s->d_sc2, PRED_RUN))) return rc;
        VecP A2 = {}; A2.out0 = s->t32; A2.in0 = s->s32;
        if ((rc = launch_apply32(s, s->z32, AX_TS, A2, RED_TS, s->d_sc2, PRED_RUN))) return rc;
        RedP red = make_red(s, s->d_sc2, RED_UPDATE, PRED_RUN);
        k_update<float><<<grid, blk, rsm, st>>>(n, s->e32, s->y32, s->z32, s->ri32, s->s32, s->t32, s->r032,
                                                red, s->d_plist);
        CKL();
    }
    const BPred fin = {s->d_plist, s->d_sc, s->d_sc2, PRED_FIN};
    k_delta_add<<<grid, blk, 0, st>>>(n, s->delta64, s->e32, s->d32, s->x, s->tmp0, fin, dd_vecs(s));
    CKL();
    k_mixed_ctl<<<dim3(1, s->nslot), 32, 0, st>>>(fin);
    CKL();
    return GADE_OK;
}

static int batch_seq_first(gade_batch *b, cudaStream_t st)
{
    gade_solver *s = b->s;
    int rc;
    if (s->prec == GADE_PREC_MIXED) {
        /* the double-float residual pass needs no FP64 tables: they are
           rebuilt from the step's coefficients by the next FP64 apply */
        if ((rc = s->use_asm ? launch_assemble(s, st) : launch_table_kernels(s, use_dd(s) ? 6 : 3, st))) return rc;
        const BPred all = {s->d_plist, s->d_sc, s->d_sc2, PRED_NONE};
        k_mixed_prep<<<dim3(s->upd_grid, s->nslot), s->upd_block, 0, st>>>(
            s->n, s->x, s->xprev, s->d_hprev, s->delta64, s->d32, s->tmp0, all, b->use_guess ? b->d_corr : nullptr,
            dd_vecs(s));
        CKL();
        return batch_seq_sweep(b, b->kiter, st);
    }
    /* the step's FP64 tables: assembled couplings or the matrix-free radial tables */
    if ((rc = s->use_asm ? launch_assemble(s, st) : launch_table_kernels(s, 1, st))) return rc;
    VecP V = {};
    V.out0 = s->rhs; V.out1 = s->r; V.out2 = s->r0;
    if ((rc = launch_apply(s, s->x, AX_RHS, V, RED_RHS, st, PRED_NONE))) return rc;
    return batch_seq_iters(b, b->kiter, st);
}

static int batch_seq_restart(gade_batch *b, cudaStream_t st)
{
    gade_solver *s = b->s;
    VecP R = {};
    R.in0 = s->rhs; R.out1 = s->r; R.out2 = s->r0;
    return launch_apply(s, s->x, AX_RESTART, R, RED_RESTART, st, PRED_RESTART);
}

/* which: 0 first, 1 iterations, 2 restart */
static int batch_run_seq(gade_batch *b, int which)
{
    cudaStream_t st = b->s->stream;
    switch (which) {
    case 0: return batch_seq_first(b, st);
    case 1: return b->s->prec == GADE_PREC_MIXED ? batch_seq_sweep(b, b->kiter, st) : batch_seq_iters(b, b->kiter, st);
    default: return batch_seq_restart(b, st);
    }
}

static int batch_launch(gade_batch *b, int which)
{
    gade_solver *s = b->s;
    b->replays++;
    if (!b->use_graphs) return batch_run_seq(b, which);
    cudaGraphExec_t *slot = which == 0 ? &b->g_first : which == 1 ? &b->g_iter : &b->g_restart;
    if (!*slot) {
        cudaGraph_t g = nullptr;
        const long long before = s->launches;
        CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        int rc = batch_run_seq(b, which);
        cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
        /* capturing launches nothing: count the kernels at every replay */
        b->nodes[which] = s->launches - before;
        s->launches = before;
        if (rc) { if (g) cudaGraphDestroy(g); return rc; }
        if (ce != cudaSuccess) return fail(GADE_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
        ce = cudaGraphInstantiate(slot, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) { *slot = nullptr; return fail(GADE_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(ce)); }
    }
    CK(cudaGraphLaunch(*slot, s->stream));
    s->launches += b->nodes[which];
    return GADE_OK;
}

static int batch_set_list(gade_batch *b, const std::vector<int> &list)
{
    gade_solver *s = b->s;
    if (list == b->list || b->internal) return GADE_OK;
    CK(cudaMemcpyAsync(s->d_plist, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    b->list = list;
    s->nslot = (int)list.size();
    batch_drop_graphs(b);
    return GADE_OK;
}

/* Candidate row-chunk sizes, each timed on one batched operator apply (the
   step's dominant kernel) over all pulses; the fastest is kept. */
static int batch_autotune(gade_batch *b, const gade_problem *p)
{
    gade_solver *s = b->s;
    const int cand[4] = {16, 32, 48, 64};
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    float best = 1e30f;
    gade_setup *keep = nullptr;
    char err[1024];
    b->ntune = 0;
    const bool mixed = s->prec == GADE_PREC_MIXED;
    for (int c = 0; c < 4; c++) {
        gade_setup *su = nullptr;
        int rc = gade_setup_build(p, s->dts[0], s->h, cand[c], &su, err, sizeof(err));
        if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return fail(rc, "%s", err); }
        if (b->ntune > 0 && su->chunk_splines == b->tune_cs[b->ntune - 1]) { gade_setup_release(su); continue; }
        if (su->chunk_rows_max > 128 || su->chunk_cols_max > 256) { gade_setup_release(su); continue; }
        if ((rc = set_chunking(s, su))) { gade_setup_release(su); cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
        VecP V = {}; V.in0 = s->r0;
        float ms = 0;
        for (int rep = 0; rep < 4; rep++) {
            if (rep == 1) CK(cudaEventRecord(e0, s->stream));
            /* mixed precision: one FP64 residual pass and four complex64 applies,
               about one step's mix */
            V.out0 = s->tmp1; V.in0 = s->r0;
            rc = launch_apply(s, s->y, AX_R0V, V, RED_R0V, s->stream);
            for (int k = 0; mixed && !rc && k < 4; k++) {
                VecP V32 = {}; V32.out0 = s->v32; V32.in0 = s->r032;
                rc = launch_apply32(s, s->y32, AX_R0V, V32, RED_R0V, s->d_sc);
            }
            if (rc) { gade_setup_release(su); cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
        }
        CK(cudaEventRecord(e1, s->stream));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        ms /= 3;
        b->tune_cs[b->ntune] = su->chunk_splines;
        b->tune_ms[b->ntune] = ms;
        b->ntune++;
        if (ms < best) { best = ms; if (keep) gade_setup_release(keep); keep = su; }
        else gade_setup_release(su);
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    if (!keep) return fail(GADE_ERR_ARG, "no row-chunk size fits the operator kernel");
    int rc = set_chunking(s, keep);
    gade_setup_release(keep);
    return rc;
}

/* Matrix-free or assembled operator for a batch: the assembled values of
   every pulse (K shared when the pulses share their radial tables) against
   the matrix-free operator, both timed as one apply of all pulses */
static int batch_choose_operator(gade_batch *b)
{
    gade_solver *s = b->s;
    int rc = asm_build(s);
    if (rc || !s->asm_ok) return rc;
    if ((rc = batch_set_list(b, b->list))) return rc;
    float mf = 0.f, am = 0.f, tmf = 0.f, tam = 0.f;
    s->use_asm = 0;
    if ((rc = time_fp64_apply(s, &mf)) || (rc = time_step_tables(s, &tmf))) return rc;
    s->use_asm = 1;
    s->asm_part = 0;
    if ((rc = time_fp64_apply(s, &am)) || (rc = time_step_tables(s, &tam))) { s->use_asm = 0; return rc; }
    s->mf_ms = mf;
    s->asm_ms[0] = am;
    s->asm_ms[1] = 0.f;
    s->tab_ms[0] = tmf;
    s->tab_ms[1] = tam;
    s->use_asm = step_cost(s, tam, am) < 0.98f * step_cost(s, tmf, mf) ? 1 : 0;
    s->has_time = 0;
    return GADE_OK;
}

extern "C" int gade_batch_operator(const gade_batch *b, int32_t *assembled, float *ms)
{
    if (!b) return fail(GADE_ERR_ARG, "gade_batch_operator: NULL batch");
    return gade_solver_operator(b->s, assembled, ms);
}

extern "C" int gade_batch_set_operator(gade_batch *b, int32_t assembled)
{
    if (!b) return fail(GADE_ERR_ARG, "gade_batch_set_operator: NULL batch");
    int rc = gade_solver_set_operator(b->s, assembled);
    if (rc) return rc;
    batch_drop_graphs(b);
    return GADE_OK;
}

extern "C" int gade_batch_create(const gade_problem *p, int32_t npulse, const double *dt, const double *g,
                                 double h, int32_t precision, int32_t device, const gade_batch_options *opt,
                                 gade_batch **out)
{
    if (!p || !dt || !out) return fail(GADE_ERR_ARG, "gade_batch_create: NULL argument");
    *out = nullptr;
    if (npulse < 1 || npulse > 65535) return fail(GADE_ERR_ARG, "gade_batch_create: npulse %d out of range", npulse);
    if (precision != GADE_PREC_FP64 && precision != GADE_PREC_MIXED)
        return fail(GADE_ERR_ARG, "gade_batch_create: unknown precision %d", precision);
    gade_batch_options o = {0, 0, 1};
    if (opt) o = *opt;
    if (o.chunk_splines < 0 || o.chunk_splines > 64 || o.iters_per_launch < 0 || o.iters_per_launch > 64)
        return fail(GADE_ERR_ARG, "gade_batch_create: option out of range");
    gade_solver *s = nullptr;
    int rc = solver_create(p, npulse, dt, g, h, precision, device, o.chunk_splines, &s);
    if (rc) return rc;
    if (npulse == 1) {
        /* a batch always runs from a launch list, even with one pulse */
        int zero = 0;
        if ((rc = dev_upload(s, &s->d_plist, &zero, 1))) { gade_solver_free(s); return rc; }
    }
    gade_batch *b = new gade_batch();
    b->s = s;
    b->kfixed = o.iters_per_launch;
    b->kiter = o.iters_per_launch > 0 ? o.iters_per_launch : 2;
    b->use_graphs = o.use_graphs != 0;
    b->tol_c = -1; b->maxit_c = -1;
    for (int k = 0; k < npulse; k++) b->list.push_back(k);
    s->nslot = npulse;
    if (o.chunk_splines == 0 && (rc = batch_autotune(b, p))) { gade_batch_free(b); return rc; }
    if ((rc = batch_choose_operator(b))) { gade_batch_free(b); return rc; }
    *out = b;
    return GADE_OK;
}

extern "C" void gade_batch_free(gade_batch *b)
{
    if (!b) return;
    if (b->s) { cudaSetDevice(b->s->device); cudaStreamSynchronize(b->s->stream); }
    batch_drop_graphs(b);
    gade_solver_free(b->s);
    delete b;
}

extern "C" int gade_batch_set_x(gade_batch *b, int32_t pulse, const double *x, int64_t n)
{
    if (!b || !x) return fail(GADE_ERR_ARG, "gade_batch_set_x: NULL argument");
    gade_solver *s = b->s;
    if (pulse < 0 || pulse >= s->npulse) return fail(GADE_ERR_ARG, "gade_batch_set_x: no pulse %d", pulse);
    if (n != s->n) return fail(GADE_ERR_ARG, "gade_batch_set_x: size %lld != %lld", (long long)n, s->n);
    CK(cudaSetDevice(s->device));
    CK(cudaMemcpyAsync(s->x + (size_t)pulse * s->n, x, sizeof(double2) * (size_t)n, cudaMemcpyHostToDevice, s->stream));
    /* a new state has no extrapolation history */
    if (s->d_hprev) CK(cudaMemsetAsync(s->d_hprev + pulse, 0, sizeof(int), s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return GADE_OK;
}

extern "C" int gade_batch_get_x(gade_batch *b, int32_t pulse, double *x, int64_t n)
{
    if (!b || !x) return fail(GADE_ERR_ARG, "gade_batch_get_x: NULL argument");
    gade_solver *s = b->s;
    if (pulse < 0 || pulse >= s->npulse) return fail(GADE_ERR_ARG, "gade_batch_get_x: no pulse %d", pulse);
    if (n != s->n) return fail(GADE_ERR_ARG, "gade_batch_get_x: size %lld != %lld", (long long)n, s->n);
    CK(cudaSetDevice(s->device));
    CK(cudaMemcpyAsync(x, s->x + (size_t)pulse * s->n, sizeof(double2) * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return GADE_OK;
}

/* iterations per captured launch: large enough that most steps need one
   replay (grown at once), shrunk after 8 steps that all needed fewer (every
   predicated-off iteration still launches its kernels) */
#define BATCH_SHRINK_STEPS 8
static void batch_adapt(gade_batch *b, int kmax)
{
    if (b->kfixed) return;
    int want = kmax + 1 > 1 ? kmax + 1 : 1;
    if (want > 64) want = 64;
    if (want > b->kwin) b->kwin = want;
    b->kwin_steps++;
    if (want > b->kiter || (b->kwin_steps >= BATCH_SHRINK_STEPS && b->kwin < b->kiter)) {
        b->kiter = want > b->kiter ? want : b->kwin;
        b->kwin = 0; b->kwin_steps = 0;
        batch_drop_graphs(b);
    } else if (b->kwin_steps >= BATCH_SHRINK_STEPS) {
        b->kwin = 0; b->kwin_steps = 0;
    }
}

/* Mixed-precision step of the listed pulses: the refinement of the
   single-pulse mixed step, with its tests in the reduction epilogues. */
static int clear_workspace(gade_solver *s, int k);

static int batch_step_mixed(gade_batch *b, const std::vector<int> &list, int32_t maxit, double tol,
                            gade_step_stats *stats)
{
    gade_solver *s = b->s;
    int rc;
    const int maxit_in = maxit < 50 ? maxit : 50;
    if (tol != b->tol_c || maxit != b->maxit_c) {
        for (int k = 0; k < s->npulse; k++) {
            DevScal &a = s->h_sc[k], &in = s->h_sc2[k];
            a = DevScal{};
            a.ctl = 1; a.tol2rel = tol * tol; a.maxit = maxit; a.maxit_in = maxit_in;
            in = DevScal{};
            in.ctl = 2; in.maxit = maxit_in; in.state = ST_DONE;
        }
        CK(cudaMemcpyAsync(s->d_sc, s->h_sc, sizeof(DevScal) * s->npulse, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(s->d_sc2, s->h_sc2, sizeof(DevScal) * s->npulse, cudaMemcpyHostToDevice, s->stream));
        b->tol_c = tol; b->maxit_c = maxit;
    }
    CK(cudaMemcpyAsync(s->d_coef, s->h_coef, sizeof(double2) * (size_t)s->npulse * s->lmax * 3,
                       cudaMemcpyHostToDevice, s->stream));
    if ((rc = batch_launch(b, 0))) return rc;
    /* each replay advances every running pulse by a sweep or by inner
       iterations, and both are bounded */
    const long long guard_max = (long long)(MIXED_MAX_SWEEPS + 1) * (maxit_in + 2) + 2;
    int kmax = 0;
    for (long long guard = 0;; guard++) {
        CK(cudaMemcpyAsync(s->h_sc, s->d_sc, sizeof(DevScal) * s->npulse, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaMemcpyAsync(s->h_sc2, s->d_sc2, sizeof(DevScal) * s->npulse, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        int nrun = 0;
        for (int k : list) {
            const DevScal &a = s->h_sc[k], &in = s->h_sc2[k];
            if (a.err | in.err) {
                CK(cudaMemsetAsync(&s->d_sc[k].err, 0, sizeof(unsigned), s->stream));
                CK(cudaMemsetAsync(&s->d_sc2[k].err, 0, sizeof(unsigned), s->stream));
                if ((rc = clear_workspace(s, k))) return rc;
                return fail(GADE_ERR_CUDA, "pulse %d: device wait timed out (flags %u): TMA copy did not complete",
                            k, a.err | in.err);
            }
            if (a.state == ST_BAD)
                return fail(GADE_ERR_NUMERIC, "pulse %d: non-finite right-hand side or refinement residual", k);
            if (a.state == ST_RUN) nrun++;
            if (in.iter > kmax) kmax = in.iter;
        }
        if (!nrun) break;
        if (guard > guard_max) return fail(GADE_ERR_STATE, "gade_batch_step: refinement control did not terminate");
        if ((rc = batch_launch(b, 1))) return rc;
    }
    {
        const BPred done = {s->d_plist, s->d_sc, s->d_sc2, PRED_DONE};
        k_mixed_finish<<<dim3(s->upd_grid, s->nslot), s->upd_block, 0, s->stream>>>(s->n, s->x, s->xprev, s->delta64,
                                                                                   s->d_hprev, done);
        CKL();
    }
    int stalled = -1;
    for (int k : list) {
        const DevScal &a = s->h_sc[k];
        gade_step_stats st = {};
        if (a.state == ST_ZERO) {
            CK(cudaMemsetAsync(s->x + (size_t)k * s->n, 0, sizeof(double2) * (size_t)s->n, s->stream));
            CK(cudaMemsetAsync(s->d_hprev + k, 0, sizeof(int), s->stream));
        } else {
            st.iters = a.inner_total;
            st.inner_iters = a.inner_total;
            st.refinements = a.refinements;
            st.true_residual = sqrt(a.rr / a.rhs_sqnorm);
            st.tol_error = st.true_residual;
            st.snorm = a.snorm;
            st.init_residual = sqrt(a.rr_init / a.rhs_sqnorm);
            if (a.stalled && stalled < 0) stalled = k;
        }
        if (stats) stats[k] = st;
    }
    if (b->xout_host) {
        CK(cudaMemcpyAsync(b->xout_host, s->x, sizeof(double2) * (size_t)s->n, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    if (use_dd(s)) s->m64_stale = 1;
    b->steps++;
    batch_adapt(b, kmax);
    if (stalled >= 0) {
        const DevScal &a = s->h_sc[stalled];
        return fail(GADE_ERR_NUMERIC, "pulse %d: mixed-precision refinement stalled at |r|/|b| = %.3e > tol %.3e after %d sweeps",
                    stalled, sqrt(a.rr / a.rhs_sqnorm), tol, a.sweeps);
    }
    return GADE_OK;
}

static int batch_step_fp64(gade_batch *b, const std::vector<int> &list, int32_t maxit, double tol,
                           gade_step_stats *stats);

/* After a step that ended on a device wait limit the vectors of pulse k are
   partial; BiCGSTAB's p and v, which carry over from one step to the next
   (tools/bicgstab.c:28-31), are cleared as after creation so that the next
   step from a state set by the caller is that of a new solver. */
static int clear_workspace(gade_solver *s, int k)
{
    const size_t off = (size_t)k * s->n, bytes = sizeof(double2) * (size_t)s->n;
    if (s->p) CK(cudaMemsetAsync(s->p + off, 0, bytes, s->stream));
    if (s->v) CK(cudaMemsetAsync(s->v + off, 0, bytes, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return GADE_OK;
}

extern "C" int gade_solver_restart(gade_solver *s, const double *x, int64_t n)
{
    int rc = gade_solver_set_x(s, x, n);
    if (rc) return rc;
    if (s->xprev) CK(cudaMemsetAsync(s->xprev, 0, sizeof(double2) * (size_t)s->n, s->stream));
    return clear_workspace(s, 0);
}

extern "C" int gade_solver_set_wait_limit(gade_solver *s, uint32_t polls)
{
    if (!s) return fail(GADE_ERR_ARG, "gade_solver_set_wait_limit: NULL solver");
    s->pc_wait = polls;
    if (s->engine) batch_drop_graphs(s->engine);   /* the graphs hold the old kernel parameters */
    return GADE_OK;
}

extern "C" int gade_solver_set_precond_warps(gade_solver *s, int32_t warps)
{
    if (!s) return fail(GADE_ERR_ARG, "gade_solver_set_precond_warps: NULL solver");
    if (warps != 4 && warps != 8) return fail(GADE_ERR_ARG, "gade_solver_set_precond_warps: warps must be 4 or 8");
    s->pc_nw = warps;
    if (s->engine) batch_drop_graphs(s->engine);   /* the graphs hold the old launch shape */
    return GADE_OK;
}

extern "C" int gade_solver_inject_wait_timeout(gade_solver *s, int32_t stage)
{
    if (!s) return fail(GADE_ERR_ARG, "gade_solver_inject_wait_timeout: NULL solver");
    if (stage < -1) return fail(GADE_ERR_ARG, "gade_solver_inject_wait_timeout: stage must be >= -1");
    s->pc_withhold = stage;
    if (s->engine) batch_drop_graphs(s->engine);
    return GADE_OK;
}

extern "C" int gade_solver_set_residual_precision(gade_solver *s, int32_t mode)
{
    if (!s || (mode != 0 && mode != 1)) return fail(GADE_ERR_ARG, "gade_solver_set_residual_precision: bad argument");
    if (mode == 1 && !s->d_Mdd)
        return fail(GADE_ERR_ARG, "gade_solver_set_residual_precision: double-float needs a mixed-precision solver "
                                  "with real couplings");
    s->mix_dd = mode;
    if (s->engine) batch_drop_graphs(s->engine);
    return GADE_OK;
}

extern "C" int gade_solver_residual_precision(const gade_solver *s, int32_t *mode, int32_t *in_use)
{
    if (!s) return fail(GADE_ERR_ARG, "gade_solver_residual_precision: NULL solver");
    if (mode) *mode = s->mix_dd;
    if (in_use) *in_use = (s->prec == GADE_PREC_MIXED && use_dd(s)) ? 1 : 0;
    return GADE_OK;
}

extern "C" int gade_batch_set_residual_precision(gade_batch *b, int32_t mode)
{
    if (!b) return fail(GADE_ERR_ARG, "gade_batch_set_residual_precision: NULL batch");
    int rc = gade_solver_set_residual_precision(b->s, mode);
    if (rc) return rc;
    batch_drop_graphs(b);
    return GADE_OK;
}

extern "C" int gade_batch_set_wait_limit(gade_batch *b, uint32_t polls)
{
    if (!b) return fail(GADE_ERR_ARG, "gade_batch_set_wait_limit: NULL batch");
    b->s->pc_wait = polls;
    batch_drop_graphs(b);
    return GADE_OK;
}

extern "C" int gade_batch_step(gade_batch *b, const int32_t *active, const double *ft, int32_t maxit, double tol,
                               gade_step_stats *stats)
{
    if (!b || !ft) return fail(GADE_ERR_ARG, "gade_batch_step: NULL argument");
    if (maxit < 0) return fail(GADE_ERR_ARG, "gade_batch_step: maxit < 0");
    if (!(tol >= 0) || !std::isfinite(tol)) return fail(GADE_ERR_ARG, "gade_batch_step: tol must be finite and >= 0");
    gade_solver *s = b->s;
    CK(cudaSetDevice(s->device));
    std::vector<int> list;
    for (int k = 0; k < s->npulse; k++)
        if (!active || active[k]) list.push_back(k);
    if (stats)
        for (int k = 0; k < s->npulse; k++) stats[k] = gade_step_stats{};
    if (list.empty()) return GADE_OK;
    int rc;
    for (int k : list)
        if ((rc = fill_coef(s, k, ft + 12 * (size_t)k))) {
            char msg[512];
            snprintf(msg, sizeof(msg), "%s", gade_last_error());
            return fail(rc, "pulse %d: %s", k, msg);
        }
    if ((rc = batch_set_list(b, list))) return rc;
    if (s->prec == GADE_PREC_MIXED) return batch_step_mixed(b, list, maxit, tol, stats);
    return batch_step_fp64(b, list, maxit, tol, stats);
}

/* FP64 step of the listed pulses with device-side BiCGSTAB control */
static int batch_step_fp64(gade_batch *b, const std::vector<int> &list, int32_t maxit, double tol,
                           gade_step_stats *stats)
{
    gade_solver *s = b->s;
    int rc;
    if (tol != b->tol_c || maxit != b->maxit_c) {
        /* control values of every pulse (the rest of each record is reset by
           the right-hand-side reduction of the step) */
        for (int k = 0; k < s->npulse; k++) {
            DevScal &d = s->h_sc[k];
            d = DevScal{};
            d.ctl = 1; d.tol2rel = tol * tol; d.maxit = maxit;
        }
        CK(cudaMemcpyAsync(s->d_sc, s->h_sc, sizeof(DevScal) * s->npulse, cudaMemcpyHostToDevice, s->stream));
        b->tol_c = tol; b->maxit_c = maxit;
    }
    CK(cudaMemcpyAsync(s->d_coef, s->h_coef, sizeof(double2) * (size_t)s->npulse * s->lmax * 3,
                       cudaMemcpyHostToDevice, s->stream));
    if ((rc = batch_launch(b, 0))) return rc;
    /* every replay advances each running pulse by at least one iteration, so
       the loop ends within maxit replays */
    int kmax = 0;
    for (long long guard = 0;; guard++) {
        CK(cudaMemcpyAsync(s->h_sc, s->d_sc, sizeof(DevScal) * s->npulse, cudaMemcpyDeviceToHost, s->stream));
        /* the state travels with the control record: final if this read-back ends the step */
        if (b->xout_host)
            CK(cudaMemcpyAsync(b->xout_host, s->x, sizeof(double2) * (size_t)s->n, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        int nrun = 0, nrestart = 0;
        for (int k : list) {
            const DevScal &d = s->h_sc[k];
            if (d.err) {
                CK(cudaMemsetAsync(&s->d_sc[k].err, 0, sizeof(unsigned), s->stream));
                if ((rc = clear_workspace(s, k))) return rc;
                return fail(GADE_ERR_CUDA, "pulse %d: device wait timed out (flags %u): TMA copy did not complete", k, d.err);
            }
            if (d.state == ST_BAD) return fail(GADE_ERR_NUMERIC, "pulse %d: BiCGSTAB residual became non-finite at iteration %d", k, d.iter);
            if (d.state == ST_RUN) nrun++;
            if (d.state == ST_RESTART) nrestart++;
            if (d.iter > kmax) kmax = d.iter;
        }
        if (!nrun && !nrestart) break;
        if (guard > (long long)maxit + 2) return fail(GADE_ERR_STATE, "gade_batch_step: iteration control did not terminate");
        if (nrestart && (rc = batch_launch(b, 2))) return rc;
        if ((rc = batch_launch(b, 1))) return rc;
    }
    for (int k : list) {
        const DevScal &d = s->h_sc[k];
        gade_step_stats st = {};
        if (d.state == ST_ZERO) {
            CK(cudaMemsetAsync(s->x + (size_t)k * s->n, 0, sizeof(double2) * (size_t)s->n, s->stream));
            if (b->xout_host) {
                memset(b->xout_host, 0, sizeof(double2) * (size_t)s->n);
                CK(cudaStreamSynchronize(s->stream));
            }
        } else {
            st.iters = d.iter;
            st.tol_error = sqrt(d.rr / d.rhs_sqnorm);
            st.restarts = d.restarts;
        }
        if (stats) stats[k] = st;
    }
    b->steps++;
    batch_adapt(b, kmax);
    return GADE_OK;
}

extern "C" int gade_batch_get_info(const gade_batch *b, gade_batch_info *info)
{
    if (!b || !info) return fail(GADE_ERR_ARG, "gade_batch_get_info: NULL argument");
    const gade_solver *s = b->s;
    *info = gade_batch_info{};
    info->npulse = s->npulse;
    info->active = (int32_t)b->list.size();
    info->chunk_splines = s->cs;
    info->iters_per_launch = b->kiter;
    info->graph_replays = b->replays;
    info->steps = b->steps;
    info->ntune = b->ntune;
    for (int k = 0; k < b->ntune && k < 4; k++) { info->tune_cs[k] = b->tune_cs[k]; info->tune_ms[k] = b->tune_ms[k]; }
    info->apply_flops = s->apply_flops;
    return GADE_OK;
}

extern "C" void *gade_batch_stream(const gade_batch *b) { return b && b->s ? (void *)b->s->stream : nullptr; }

extern "C" int gade_batch_state_device(gade_batch *b, void **x_dev, int64_t *ld)
{
    if (!b || !x_dev || !ld) return fail(GADE_ERR_ARG, "gade_batch_state_device: NULL argument");
    *x_dev = b->s->x;
    *ld = b->s->n;
    return GADE_OK;
}

extern "C" int gade_batch_guess_buffer(gade_batch *b, void **corr_dev, int64_t *ld)
{
    if (!b || !corr_dev || !ld) return fail(GADE_ERR_ARG, "gade_batch_guess_buffer: NULL argument");
    gade_solver *s = b->s;
    if (s->prec != GADE_PREC_MIXED) return fail(GADE_ERR_STATE, "gade_batch_guess_buffer: only mixed-precision batches take a guess");
    if (!b->d_corr) {
        CK(cudaSetDevice(s->device));
        int rc = dev_upload(s, &b->d_corr, (const double2 *)nullptr, (size_t)s->npulse * s->n);
        if (rc) return rc;
    }
    *corr_dev = b->d_corr;
    *ld = s->n;
    return GADE_OK;
}

extern "C" int gade_batch_use_guess(gade_batch *b, int32_t enable)
{
    if (!b) return fail(GADE_ERR_ARG, "gade_batch_use_guess: NULL batch");
    if (enable && !b->d_corr) return fail(GADE_ERR_STATE, "gade_batch_use_guess: no guess buffer (gade_batch_guess_buffer)");
    if ((enable != 0) != (b->use_guess != 0)) batch_drop_graphs(b);
    b->use_guess = enable != 0;
    return GADE_OK;
}

/*
 * gade_solver_step runs on the batch engine with one pulse: the same kernels
 * in the same order, BiCGSTAB's control (or the mixed-precision refinement's)
 * in the reduction epilogues and the step replayed from captured CUDA graphs,
 * so the host waits once per replay instead of once per iteration.  While
 * event profiling is on the kernels are launched directly (the events of a
 * replayed graph could not be told apart).
 */
static int solver_engine_step(gade_solver *s, const double *ft, int32_t maxit, double tol, gade_step_stats *stats,
                              double *x_out)
{
    if (!s->engine) {
        gade_batch *b = new gade_batch();
        b->s = s;
        b->internal = 1;
        b->kiter = 2;
        b->use_graphs = 1;
        b->tol_c = -1; b->maxit_c = -1;
        b->list.push_back(0);
        s->engine = b;
    }
    gade_batch *b = s->engine;
    const int want_graphs = s->profile ? 0 : 1;
    if (want_graphs != b->use_graphs) { batch_drop_graphs(b); b->use_graphs = want_graphs; }
    int rc = fill_coef(s, 0, ft);
    if (rc) return rc;
    gade_step_stats st = {};
    b->xout_host = (double2 *)x_out;
    rc = s->prec == GADE_PREC_MIXED ? batch_step_mixed(b, b->list, maxit, tol, &st)
                                    : batch_step_fp64(b, b->list, maxit, tol, &st);
    b->xout_host = nullptr;
    if (stats) *stats = st;
    return rc;
}

static void solver_engine_free(gade_solver *s)
{
    if (!s || !s->engine) return;
    batch_drop_graphs(s->engine);
    delete s->engine;
    s->engine = nullptr;
}
