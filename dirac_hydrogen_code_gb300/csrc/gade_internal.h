/*
 * Internal structures shared by the host set-up (C) and the CUDA solver.
 *
 * Terminology follows the reference tools/ solver:
 *   block       one angular state (kappa, mu); the compact block pattern is
 *               H.csr ("Hall", tools/dirac_solver.c:225-226)
 *   blkdim      radial basis size of a block (2*(Nsplines+5))
 *   base pattern the sparsity shared by every radial matrix g, h0, s
 *               (src/dumpBdpCouplings.cpp:239-258)
 *   l           Bessel expansion order, 0..lmax-1
 */
#ifndef GADE_INTERNAL_H
#define GADE_INTERNAL_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { double re, im; } gc64;   /* layout of complex128 */

/* host copy of every solver input, as read from the reference files */
typedef struct gade_problem {
    int lmax, nblk, blkdim, blk_nnz;
    int64_t n;                    /* nblk * blkdim */
    int32_t *hall_Ap, *hall_Ai;   /* compact block pattern (nblk rows) */
    int32_t *perm;                /* compact -> original angular index */
    int *kappa;                   /* kappa of each compact block row */
    int32_t *g_Ap, *g_Ai;         /* base pattern (blkdim rows)       */
    gc64 *g, *gt;                 /* [a][l][q][blk_nnz], a<6, q<4     */
    gc64 *h0;                     /* [4][blk_nnz]                      */
    gc64 *s;                      /* [3][blk_nnz]                      */
    gc64 *H0, *H1;                /* [hall_nnz][lmax] angular couplings */
    gc64 *psi0;                   /* psi0.vec values (n)               */
    int32_t *xperm;               /* psi0.vec permutation (n)          */
    int real_coupling;            /* g, gt real and H0l, H1l imaginary */
    int dkb_zero;                 /* the radial tables vanish where the kinetically balanced
                                     halves of the basis are zero (gade_dkb_zero) */
} gade_problem;

/* device-ready set-up arrays derived from a problem and a time step */
typedef struct gade_setup {
    int nblk, B, lmax, W;         /* W: ELL width of the base pattern     */
    int nk;                       /* number of distinct kappa values      */
    int *kvals;                   /* [nk]                                 */
    int *row_kidx;                /* [nblk] index into kvals              */
    int ell_halves;               /* slots 0..14: columns of the first radial half, 15..29 the second,
                                     slot = half*15 + (column spline - row spline + 7) */
    int32_t *ell_pos;             /* [W][B] CSR position or -1            */
    int32_t *ell_col;             /* [W][B] column or -1                  */
    /* row chunks: every block row is split into the same nchunk row sets */
    int nchunk, chunk_rows_max, chunk_cols_max;
    int chunk_splines;            /* splines (of each half) per row chunk  */
    int32_t *chunk_nrows, *chunk_ncols;    /* [nchunk]                     */
    int32_t *chunk_rows;          /* [nchunk][chunk_rows_max] row (or -1) */
    int32_t *chunk_cols;          /* [nchunk][chunk_cols_max] col (or -1) */
    int32_t *chunk_lcol;          /* [nchunk][W][chunk_rows_max] local col index or -1 */
    /* angular terms: for block row r and order l, the list of coupled
       blocks c with H0l(r,c), H1l(r,c); a0k = H0l*kappa_c, a1k = H1l*kappa_c */
    int32_t *ang_ptr;             /* [nblk*lmax + 1] */
    int32_t *ang_c;
    gc64 *ang_a0, *ang_a0k, *ang_a1, *ang_a1k;
    int32_t *act_ptr;             /* [nblk+1] active (r,l) list         */
    int32_t *act_l;
    int64_t n_ang, n_act;
    /* stationary blocks per kappa, ELL layout [nk][W][B] */
    gc64 *S_ell, *Hst_ell;
    /* preconditioner: exact LU of P^T = (S + i h dt/2 h0)^T per kappa, in
       the banded ordering ord[] (natural index of each ordered row) */
    int32_t *ord;                 /* [B] ordered -> natural                */
    int bw, Bp, nch;              /* bandwidth, padded size (32*nch)       */
    gc64 *Lb;                     /* [nk][bw][Bp]   L(i, i-d), d=1..bw     */
    gc64 *Ub;                     /* [nk][bw][Bp]   U(i, i+d)              */
    gc64 *Linv;                   /* [nk][nch][32][32] (col-major: [j][i]) */
    gc64 *Uinv;                   /* [nk][nch][32][32]                      */
    double dt, h;
} gade_setup;

int gade_problem_read(const char *dir, int lmax, gade_problem **out, char *err, size_t errlen);
void gade_problem_release(gade_problem *p);
int gade_setup_build(const gade_problem *p, double dt, double h, int chunk_splines,
                     gade_setup **out, char *err, size_t errlen);
void gade_setup_release(gade_setup *s);
/* tpos[k]: CSR position of the transpose of base-pattern entry k; nonzero
   when the pattern is not structurally symmetric */
int gade_problem_transpose_map(const gade_problem *p, int32_t *tpos);
/* 1 when the radial tables g (loader layout) have the DKB zero blocks */
int gade_dkb_zero(const gade_problem *p, const gc64 *g);

/* kappa of an angular index, tools/solver_common.c:30-37 */
int gade_ik(int i);

#ifdef __cplusplus
}
#endif
#endif
