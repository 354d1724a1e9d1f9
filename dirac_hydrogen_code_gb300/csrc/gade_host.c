/*
 * Host side of the GB300 Crank-Nicolson step: reading the reference input
 * files and building every set-up array the CUDA solver needs.
 *
 * Reads follow tools/dirac_solver.c:223-388 and tools/csr.c:262-318; the
 * stationary blocks follow tools/solver.c:409-458; the preconditioner
 * replaces the SuperLU ILU of tools/solver.c:460-485 + tools/superlu.c:154-266
 * by an exact LU of each distinct diagonal block of P^T (see gade_setup_build).
 */
#define _GNU_SOURCE
#include "gade_internal.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define SOL 137.035999084

static void seterr(char *err, size_t len, const char *fmt, ...)
{
    if (!err || !len) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, len, fmt, ap);
    va_end(ap);
}

int gade_ik(int i)
{
    int ii = i / 4;
    int abskappa = (int)(0.5 * (sqrt(8.0 * ii + 1.0) - 1.0)) + 1;
    int sgnmod = abskappa * 4 > 4 ? abskappa * 4 : 4;
    double sgnfloor = 2 * abskappa * (abskappa - 1);
    int sgnkappa = ((i - sgnfloor) / sgnmod >= 0.5) - ((i - sgnfloor) / sgnmod < 0.5);
    return abskappa * sgnkappa;
}

/* ------------------------------------------------------------------ */
/* CSR files                                                           */
/* ------------------------------------------------------------------ */
typedef struct {
    int32_t n, nnz;
    int32_t *Ap, *Ai;
    gc64 *Ax;
    int32_t *perm;
    int32_t npart;
    int32_t *dist;
} csr_t;

static void csr_free_(csr_t *m)
{
    free(m->Ap); free(m->Ai); free(m->Ax); free(m->perm); free(m->dist);
    memset(m, 0, sizeof(*m));
}

static int csr_load(const char *dir, const char *name, csr_t *m, char *err, size_t len)
{
    char path[4096];
    memset(m, 0, sizeof(*m));
    snprintf(path, sizeof(path), "%s/%s", dir, name);
    FILE *fd = fopen(path, "rb");
    if (!fd) { seterr(err, len, "cant open %s", path); return 1; }
    int ok = fread(&m->n, 4, 1, fd) == 1 && fread(&m->nnz, 4, 1, fd) == 1 && m->n >= 0 && m->nnz >= 0;
    if (ok) {
        m->Ap = malloc(sizeof(int32_t) * ((size_t)m->n + 1));
        m->Ai = malloc(sizeof(int32_t) * ((size_t)m->nnz + 1));
        m->Ax = malloc(sizeof(gc64) * ((size_t)m->nnz + 1));
        ok = m->Ap && m->Ai && m->Ax &&
             fread(m->Ap, 4, (size_t)m->n + 1, fd) == (size_t)m->n + 1;
    }
    if (ok && m->Ap[m->n] != m->nnz) {
        seterr(err, len, "wrong file format (nnz) in %s: nrows %d nnz %d Ap %d", path, m->n, m->nnz, m->Ap[m->n]);
        fclose(fd); csr_free_(m); return 2;
    }
    ok = ok && fread(m->Ai, 4, (size_t)m->nnz, fd) == (size_t)m->nnz &&
         fread(m->Ax, sizeof(gc64), (size_t)m->nnz, fd) == (size_t)m->nnz;
    if (!ok) { seterr(err, len, "wrong file format in %s", path); fclose(fd); csr_free_(m); return 2; }
    for (int32_t r = 0; r < m->n; r++) {
        if (m->Ap[r] > m->Ap[r + 1]) { seterr(err, len, "wrong file format in %s: Ap not monotone", path); fclose(fd); csr_free_(m); return 2; }
    }
    for (int32_t k = 0; k < m->nnz; k++) {
        if (m->Ai[k] < 0 || m->Ai[k] >= m->n) { seterr(err, len, "wrong file format in %s: column out of range", path); fclose(fd); csr_free_(m); return 2; }
    }
    /* optional permutation + partitioning trailer (H.csr) */
    m->perm = malloc(sizeof(int32_t) * ((size_t)m->n + 1));
    if (m->n > 0 && fread(m->perm, 4, (size_t)m->n, fd) == (size_t)m->n) {
        if (fread(&m->npart, 4, 1, fd) != 1) {
            seterr(err, len, "wrong file format in %s: partitioning info not found", path);
            fclose(fd); csr_free_(m); return 2;
        }
        if (m->npart < 1) { seterr(err, len, "wrong file format in %s: partitioning info inconsistent", path); fclose(fd); csr_free_(m); return 2; }
        m->dist = malloc(sizeof(int32_t) * ((size_t)m->npart + 1));
        if (fread(m->dist, 4, (size_t)m->npart + 1, fd) != (size_t)m->npart + 1) {
            seterr(err, len, "wrong file format in %s: partitioning info inconsistent", path);
            fclose(fd); csr_free_(m); return 2;
        }
    } else {
        free(m->perm); m->perm = NULL;
    }
    fclose(fd);
    return 0;
}

/* position of column col in row r (sorted columns), or -1: csr_get_value */
static int32_t csr_find(const int32_t *Ap, const int32_t *Ai, int32_t r, int32_t col)
{
    int32_t lo = Ap[r], hi = Ap[r + 1] - 1;
    while (lo <= hi) {
        int32_t mid = (lo + hi) / 2;
        if (Ai[mid] == col) return mid;
        if (Ai[mid] < col) lo = mid + 1; else hi = mid - 1;
    }
    /* fall back to a linear scan for unsorted rows */
    for (int32_t k = Ap[r]; k < Ap[r + 1]; k++) if (Ai[k] == col) return k;
    return -1;
}

void gade_problem_release(gade_problem *p)
{
    if (!p) return;
    free(p->hall_Ap); free(p->hall_Ai); free(p->perm); free(p->kappa);
    free(p->g_Ap); free(p->g_Ai); free(p->g); free(p->gt); free(p->h0); free(p->s);
    free(p->H0); free(p->H1); free(p->psi0); free(p->xperm);
    free(p);
}

static int same_pattern(const csr_t *a, const csr_t *b)
{
    return a->n == b->n && a->nnz == b->nnz &&
           !memcmp(a->Ap, b->Ap, sizeof(int32_t) * ((size_t)a->n + 1)) &&
           !memcmp(a->Ai, b->Ai, sizeof(int32_t) * (size_t)a->nnz);
}

int gade_problem_read(const char *dir, int lmax, gade_problem **out, char *err, size_t len)
{
    char name[256];
    int rc = 0;
    *out = NULL;
    if (lmax < 1) { seterr(err, len, "lmax must be >= 1 (got %d)", lmax); return 4; }
    gade_problem *p = calloc(1, sizeof(*p));
    csr_t hall = {0}, g0 = {0}, m = {0};
    csr_t *H = calloc((size_t)2 * lmax, sizeof(csr_t));
    p->lmax = lmax;

    if ((rc = csr_load(dir, "H.csr", &hall, err, len))) goto fail;
    if (!hall.perm) { seterr(err, len, "H.csr has no permutation trailer (run the structure step)"); rc = 2; goto fail; }
    if (hall.npart != 1) { seterr(err, len, "H.csr is partitioned for %d ranks; this solver runs one partition", hall.npart); rc = 2; goto fail; }
    p->nblk = hall.n;
    p->hall_Ap = hall.Ap; p->hall_Ai = hall.Ai; p->perm = hall.perm;
    hall.Ap = hall.Ai = hall.perm = NULL;

    for (int l = 0; l < lmax; l++) {
        snprintf(name, sizeof(name), "H0l%d.csr", l);
        if ((rc = csr_load(dir, name, &H[2 * l], err, len))) goto fail;
        snprintf(name, sizeof(name), "H1l%d.csr", l);
        if ((rc = csr_load(dir, name, &H[2 * l + 1], err, len))) goto fail;
    }
    if ((rc = csr_load(dir, "g0a0l0.csr", &g0, err, len))) goto fail;
    p->blkdim = g0.n; p->blk_nnz = g0.nnz;
    p->n = (int64_t)p->nblk * p->blkdim;
    p->g_Ap = g0.Ap; p->g_Ai = g0.Ai; g0.Ap = g0.Ai = NULL;
    const size_t bn = (size_t)p->blk_nnz;
    p->g = calloc((size_t)6 * lmax * 4 * bn, sizeof(gc64));
    p->gt = calloc((size_t)6 * lmax * 4 * bn, sizeof(gc64));
    if (!p->g || !p->gt) { seterr(err, len, "out of host memory"); rc = 5; goto fail; }
    for (int a = 0; a < 6; a++)
        for (int l = 0; l < lmax; l++)
            for (int q = 0; q < 4; q++) {
                snprintf(name, sizeof(name), "g%da%dl%d.csr", q, a, l);
                if ((rc = csr_load(dir, name, &m, err, len))) goto fail;
                csr_t base = {p->blkdim, p->blk_nnz, p->g_Ap, p->g_Ai};
                if (!same_pattern(&m, &base)) {
                    seterr(err, len, "%s does not share the base pattern of g0a0l0.csr", name);
                    rc = 2; csr_free_(&m); goto fail;
                }
                gc64 *dst = p->g + (((size_t)a * lmax + l) * 4 + q) * bn;
                gc64 *dstt = p->gt + (((size_t)a * lmax + l) * 4 + q) * bn;
                memcpy(dst, m.Ax, bn * sizeof(gc64));
                /* conjugate transpose on the same pattern: csr_conj_transpose */
                for (int32_t r = 0; r < m.n; r++)
                    for (int32_t k = m.Ap[r]; k < m.Ap[r + 1]; k++) {
                        int32_t pos = csr_find(m.Ap, m.Ai, m.Ai[k], r);
                        if (pos < 0) { seterr(err, len, "cant set matrix value: (%d,%d) not present in CSR.", m.Ai[k], r); rc = 2; csr_free_(&m); goto fail; }
                        dstt[pos].re = m.Ax[k].re;
                        dstt[pos].im = -m.Ax[k].im;
                    }
                csr_free_(&m);
            }
    p->h0 = calloc(4 * bn, sizeof(gc64));
    p->s = calloc(3 * bn, sizeof(gc64));
    for (int i = 0; i < 4; i++) {
        snprintf(name, sizeof(name), "h0%d.csr", i);
        if ((rc = csr_load(dir, name, &m, err, len))) goto fail;
        csr_t base = {p->blkdim, p->blk_nnz, p->g_Ap, p->g_Ai};
        if (!same_pattern(&m, &base)) { seterr(err, len, "%s does not share the base pattern", name); rc = 2; csr_free_(&m); goto fail; }
        memcpy(p->h0 + i * bn, m.Ax, bn * sizeof(gc64));
        csr_free_(&m);
    }
    for (int i = 0; i < 3; i++) {
        snprintf(name, sizeof(name), "s%d.csr", i);
        if ((rc = csr_load(dir, name, &m, err, len))) goto fail;
        csr_t base = {p->blkdim, p->blk_nnz, p->g_Ap, p->g_Ai};
        if (!same_pattern(&m, &base)) { seterr(err, len, "%s does not share the base pattern", name); rc = 2; csr_free_(&m); goto fail; }
        memcpy(p->s + i * bn, m.Ax, bn * sizeof(gc64));
        csr_free_(&m);
    }

    /* kappa per compact block, angular couplings per Hall entry
       (tools/gpu_solver.cu:137-188) */
    p->kappa = malloc(sizeof(int) * (size_t)p->nblk);
    const int32_t hnnz = p->hall_Ap[p->nblk];
    p->H0 = calloc((size_t)hnnz * lmax, sizeof(gc64));
    p->H1 = calloc((size_t)hnnz * lmax, sizeof(gc64));
    int nang = H[0].n;
    for (int r = 0; r < p->nblk; r++) {
        if (p->perm[r] < 0 || p->perm[r] >= nang) { seterr(err, len, "H.csr permutation entry %d out of range", p->perm[r]); rc = 2; goto fail; }
        p->kappa[r] = gade_ik(p->perm[r]);
    }
    for (int l = 0; l < 2 * lmax; l++)
        if (H[l].n != nang) { seterr(err, len, "H0l/H1l dimensions differ"); rc = 2; goto fail; }
    for (int r = 0; r < p->nblk; r++)
        for (int32_t cp = p->hall_Ap[r]; cp < p->hall_Ap[r + 1]; cp++) {
            int32_t orow = p->perm[r], ocol = p->perm[p->hall_Ai[cp]];
            for (int l = 0; l < lmax; l++) {
                int32_t k0 = csr_find(H[2 * l].Ap, H[2 * l].Ai, orow, ocol);
                int32_t k1 = csr_find(H[2 * l + 1].Ap, H[2 * l + 1].Ai, orow, ocol);
                if (k0 >= 0) p->H0[(size_t)cp * lmax + l] = H[2 * l].Ax[k0];
                if (k1 >= 0) p->H1[(size_t)cp * lmax + l] = H[2 * l + 1].Ax[k1];
            }
        }

    /* initial state */
    {
        snprintf(name, sizeof(name), "%s/psi0.vec", dir);
        FILE *fd = fopen(name, "rb");
        int32_t n;
        if (!fd) { seterr(err, len, "cant open %s", name); rc = 1; goto fail; }
        if (fread(&n, 4, 1, fd) != 1 || (int64_t)n != p->n) {
            seterr(err, len, "wrong file format in %s (expected %lld entries)", name, (long long)p->n);
            fclose(fd); rc = 2; goto fail;
        }
        p->psi0 = malloc(sizeof(gc64) * (size_t)n);
        p->xperm = malloc(sizeof(int32_t) * (size_t)n);
        if (fread(p->psi0, sizeof(gc64), (size_t)n, fd) != (size_t)n ||
            fread(p->xperm, 4, (size_t)n, fd) != (size_t)n) {
            seterr(err, len, "wrong file format in %s", name); fclose(fd); rc = 2; goto fail;
        }
        fclose(fd);
        for (int32_t i = 0; i < n; i++)
            if (p->xperm[i] < 0 || p->xperm[i] >= n) { seterr(err, len, "psi0.vec permutation out of range"); rc = 2; goto fail; }
    }

    /* real-coupling structure: g real, H0l/H1l purely imaginary */
    {
        int rcpl = 1;
        size_t ng = (size_t)6 * lmax * 4 * bn;
        for (size_t i = 0; i < ng && rcpl; i++) if (p->g[i].im != 0.0) rcpl = 0;
        for (size_t i = 0; i < (size_t)hnnz * lmax && rcpl; i++)
            if (p->H0[i].re != 0.0 || p->H1[i].re != 0.0) rcpl = 0;
        p->real_coupling = rcpl;
        p->dkb_zero = gade_dkb_zero(p, p->g);
    }

    for (int l = 0; l < 2 * lmax; l++) csr_free_(&H[l]);
    free(H); csr_free_(&hall); csr_free_(&g0);
    *out = p;
    return 0;
fail:
    for (int l = 0; l < 2 * lmax; l++) csr_free_(&H[l]);
    free(H); csr_free_(&hall); csr_free_(&g0);
    gade_problem_release(p);
    return rc ? rc : 2;
}

/* ------------------------------------------------------------------ */
/* set-up                                                              */
/* ------------------------------------------------------------------ */
static inline gc64 cmul(gc64 a, gc64 b) { gc64 r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline gc64 cadd(gc64 a, gc64 b) { gc64 r = {a.re + b.re, a.im + b.im}; return r; }
static inline gc64 csub(gc64 a, gc64 b) { gc64 r = {a.re - b.re, a.im - b.im}; return r; }
static inline gc64 cscale(gc64 a, double s) { gc64 r = {a.re * s, a.im * s}; return r; }
static inline gc64 cdiv(gc64 a, gc64 b)
{
    double d = b.re * b.re + b.im * b.im;
    gc64 r = {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
    return r;
}

void gade_setup_release(gade_setup *s)
{
    if (!s) return;
    free(s->kvals); free(s->row_kidx); free(s->ell_pos); free(s->ell_col);
    free(s->chunk_nrows); free(s->chunk_ncols); free(s->chunk_rows); free(s->chunk_cols); free(s->chunk_lcol);
    free(s->ang_ptr); free(s->ang_c); free(s->ang_a0); free(s->ang_a0k); free(s->ang_a1); free(s->ang_a1k);
    free(s->act_ptr); free(s->act_l);
    free(s->S_ell); free(s->Hst_ell); free(s->ord); free(s->Lb); free(s->Ub); free(s->Linv); free(s->Uinv);
    free(s);
}

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/*
 * Exact LU (no pivoting) of one banded block A (ordered, dense band storage
 * band[i*(2bw+1) + (j-i+bw)]).  S is symmetric positive definite and
 * i*h*dt/2*h0 skew-Hermitian, so P = S + i*h*dt/2*h0 has a positive definite
 * Hermitian part and its LU without pivoting exists.
 */
static int band_lu(gc64 *band, int B, int bw)
{
    const int w = 2 * bw + 1;
    for (int k = 0; k < B; k++) {
        gc64 piv = band[(size_t)k * w + bw];
        if (piv.re == 0.0 && piv.im == 0.0) return -1 - k;
        int iend = k + bw < B - 1 ? k + bw : B - 1;
        for (int i = k + 1; i <= iend; i++) {
            gc64 *lik = &band[(size_t)i * w + (k - i + bw)];
            if (lik->re == 0.0 && lik->im == 0.0) continue;
            *lik = cdiv(*lik, piv);
            for (int j = k + 1; j <= iend; j++) {
                gc64 ukj = band[(size_t)k * w + (j - k + bw)];
                gc64 *aij = &band[(size_t)i * w + (j - i + bw)];
                *aij = csub(*aij, cmul(*lik, ukj));
            }
        }
    }
    return 0;
}

/* 1 when the radial tables g ([a][l][q][blk_nnz], the loader's layout)
   vanish where the DKB basis makes them vanish: with P0/Q0 the large and
   Pk/Qk the kinetically balanced parts (Pk zero on the first radial half,
   Qk on the second), g1 = <Pk|Q0> is zero on first-half rows, g2 = <P0|Qk>
   on second-half columns and g3 = <Pk|Qk> outside (second-half rows,
   first-half columns).  The per-step table M1 is then zero on second-half
   columns and M3 on first-half columns, which the operator kernel skips. */
int gade_dkb_zero(const gade_problem *p, const gc64 *g)
{
    const int B = p->blkdim, ns = B / 2;
    if (B % 2) return 0;
    const size_t bn = (size_t)p->blk_nnz;
    for (int a = 0; a < 6; a++)
        for (int l = 0; l < p->lmax; l++)
            for (int q = 1; q < 4; q++) {
                const gc64 *m = g + (((size_t)a * p->lmax + l) * 4 + q) * bn;
                for (int32_t r = 0; r < B; r++)
                    for (int32_t k = p->g_Ap[r]; k < p->g_Ap[r + 1]; k++) {
                        const int c = p->g_Ai[k];
                        const int zero = q == 1 ? r < ns : q == 2 ? c >= ns : !(r >= ns && c < ns);
                        if (zero && (m[k].re != 0.0 || m[k].im != 0.0)) return 0;
                    }
            }
    return 1;
}

int gade_problem_transpose_map(const gade_problem *p, int32_t *tpos)
{
    for (int32_t r = 0; r < p->blkdim; r++)
        for (int32_t k = p->g_Ap[r]; k < p->g_Ap[r + 1]; k++) {
            int32_t pos = csr_find(p->g_Ap, p->g_Ai, p->g_Ai[k], r);
            if (pos < 0) return 1;
            tpos[k] = pos;
        }
    return 0;
}

int gade_setup_build(const gade_problem *p, double dt, double h, int chunk_splines,
                     gade_setup **out, char *err, size_t len)
{
    *out = NULL;
    gade_setup *s = calloc(1, sizeof(*s));
    const int B = p->blkdim, lmax = p->lmax, nblk = p->nblk;
    const int32_t *GAp = p->g_Ap, *GAi = p->g_Ai;
    s->nblk = nblk; s->B = B; s->lmax = lmax; s->dt = dt; s->h = h;

    /* distinct kappa values */
    s->kvals = malloc(sizeof(int) * (size_t)nblk);
    s->row_kidx = malloc(sizeof(int) * (size_t)nblk);
    for (int r = 0; r < nblk; r++) {
        int k = p->kappa[r], found = -1;
        for (int j = 0; j < s->nk; j++) if (s->kvals[j] == k) { found = j; break; }
        if (found < 0) { found = s->nk; s->kvals[s->nk++] = k; }
        s->row_kidx[r] = found;
    }

    /* ELL view of the base pattern.  The DKB basis pairs spline s (first
       radial half) with spline s of the second half; every entry couples
       splines at most 7 apart.  When that holds the slots are laid out by
       column half and spline offset (15 + 15), so slot t of a row always
       means the same relative column and the first 15 slots hold exactly the
       first-half columns.  Otherwise the slots follow CSR order. */
    int W = 0;
    for (int i = 0; i < B; i++) if (GAp[i + 1] - GAp[i] > W) W = GAp[i + 1] - GAp[i];
    int halves = (B % 2 == 0);
    const int ns = B / 2;
    for (int i = 0; i < B && halves; i++)
        for (int32_t k = GAp[i]; k < GAp[i + 1]; k++) {
            const int d = GAi[k] % ns - i % ns;
            if (d < -7 || d > 7) { halves = 0; break; }
        }
    if (halves) W = 30;
    s->W = W;
    s->ell_halves = halves;
    s->ell_pos = malloc(sizeof(int32_t) * (size_t)W * B);
    s->ell_col = malloc(sizeof(int32_t) * (size_t)W * B);
    for (size_t e = 0; e < (size_t)W * B; e++) { s->ell_pos[e] = -1; s->ell_col[e] = -1; }
    for (int i = 0; i < B; i++)
        for (int32_t k = GAp[i]; k < GAp[i + 1]; k++) {
            const int j = halves ? (GAi[k] >= ns ? 15 : 0) + (GAi[k] % ns - i % ns) + 7 : k - GAp[i];
            s->ell_pos[(size_t)j * B + i] = k;
            s->ell_col[(size_t)j * B + i] = GAi[k];
        }

    /* row chunks: spline s together with its partner s+B/2 when B is even */
    {
        int half = (B % 2 == 0) ? B / 2 : B;
        int cs = chunk_splines > 0 ? chunk_splines : 64;
        if (cs > half) cs = half;
        s->chunk_splines = cs;
        int rows_per = (B % 2 == 0) ? 2 * cs : cs;
        s->nchunk = (half + cs - 1) / cs;
        s->chunk_rows_max = rows_per;
        s->chunk_nrows = calloc((size_t)s->nchunk, sizeof(int32_t));
        s->chunk_ncols = calloc((size_t)s->nchunk, sizeof(int32_t));
        s->chunk_rows = malloc(sizeof(int32_t) * (size_t)s->nchunk * rows_per);
        int32_t *tmpcols = malloc(sizeof(int32_t) * (size_t)rows_per * W);
        int32_t **cols = calloc((size_t)s->nchunk, sizeof(int32_t *));
        int maxc = 0;
        for (int q = 0; q < s->nchunk; q++) {
            int n = 0;
            for (int t = 0; t < cs; t++) {
                int sp = q * cs + t;
                if (sp >= half) break;
                s->chunk_rows[(size_t)q * rows_per + n++] = sp;
                if (B % 2 == 0) s->chunk_rows[(size_t)q * rows_per + n++] = sp + half;
            }
            /* order rows increasing so consecutive threads read consecutive table entries */
            qsort(s->chunk_rows + (size_t)q * rows_per, (size_t)n, sizeof(int32_t), cmp_i32);
            for (int t = n; t < rows_per; t++) s->chunk_rows[(size_t)q * rows_per + t] = -1;
            s->chunk_nrows[q] = n;
            int nc = 0;
            for (int t = 0; t < n; t++) {
                int i = s->chunk_rows[(size_t)q * rows_per + t];
                for (int32_t k = GAp[i]; k < GAp[i + 1]; k++) tmpcols[nc++] = GAi[k];
            }
            qsort(tmpcols, (size_t)nc, sizeof(int32_t), cmp_i32);
            int u = 0;
            for (int t = 0; t < nc; t++) if (u == 0 || tmpcols[t] != tmpcols[u - 1]) tmpcols[u++] = tmpcols[t];
            cols[q] = malloc(sizeof(int32_t) * (size_t)(u ? u : 1));
            memcpy(cols[q], tmpcols, sizeof(int32_t) * (size_t)u);
            s->chunk_ncols[q] = u;
            if (u > maxc) maxc = u;
        }
        s->chunk_cols_max = maxc;
        s->chunk_cols = malloc(sizeof(int32_t) * (size_t)s->nchunk * maxc);
        s->chunk_lcol = malloc(sizeof(int32_t) * (size_t)s->nchunk * W * rows_per);
        for (int q = 0; q < s->nchunk; q++) {
            int u = s->chunk_ncols[q];
            for (int t = 0; t < maxc; t++) s->chunk_cols[(size_t)q * maxc + t] = t < u ? cols[q][t] : -1;
            for (int j = 0; j < W; j++)
                for (int t = 0; t < rows_per; t++) {
                    int32_t lc = -1;
                    int i = s->chunk_rows[(size_t)q * rows_per + t];
                    if (i >= 0) {
                        int32_t col = s->ell_col[(size_t)j * B + i];
                        if (col >= 0) {
                            int32_t *hit = bsearch(&col, cols[q], (size_t)u, sizeof(int32_t), cmp_i32);
                            lc = (int32_t)(hit - cols[q]);
                        }
                    }
                    s->chunk_lcol[((size_t)q * W + j) * rows_per + t] = lc;
                }
            free(cols[q]);
        }
        free(cols); free(tmpcols);
    }

    /* angular terms per (r, l) */
    {
        const int32_t *Ap = p->hall_Ap, *Ai = p->hall_Ai;
        s->ang_ptr = calloc((size_t)nblk * lmax + 1, sizeof(int32_t));
        int64_t cnt = 0;
        for (int r = 0; r < nblk; r++)
            for (int l = 0; l < lmax; l++) {
                for (int32_t cp = Ap[r]; cp < Ap[r + 1]; cp++) {
                    gc64 a0 = p->H0[(size_t)cp * lmax + l], a1 = p->H1[(size_t)cp * lmax + l];
                    if (a0.re != 0 || a0.im != 0 || a1.re != 0 || a1.im != 0) cnt++;
                }
                s->ang_ptr[r * lmax + l + 1] = (int32_t)cnt;
            }
        s->n_ang = cnt;
        s->ang_c = malloc(sizeof(int32_t) * (size_t)(cnt + 1));
        s->ang_a0 = malloc(sizeof(gc64) * (size_t)(cnt + 1));
        s->ang_a0k = malloc(sizeof(gc64) * (size_t)(cnt + 1));
        s->ang_a1 = malloc(sizeof(gc64) * (size_t)(cnt + 1));
        s->ang_a1k = malloc(sizeof(gc64) * (size_t)(cnt + 1));
        s->act_ptr = calloc((size_t)nblk + 1, sizeof(int32_t));
        s->act_l = malloc(sizeof(int32_t) * ((size_t)nblk * lmax + 1));
        int64_t e = 0, na = 0;
        for (int r = 0; r < nblk; r++) {
            for (int l = 0; l < lmax; l++) {
                int64_t e0 = e;
                for (int32_t cp = Ap[r]; cp < Ap[r + 1]; cp++) {
                    gc64 a0 = p->H0[(size_t)cp * lmax + l], a1 = p->H1[(size_t)cp * lmax + l];
                    if (a0.re != 0 || a0.im != 0 || a1.re != 0 || a1.im != 0) {
                        int c = Ai[cp];
                        double kc = (double)p->kappa[c];
                        s->ang_c[e] = c;
                        s->ang_a0[e] = a0; s->ang_a0k[e] = cscale(a0, kc);
                        s->ang_a1[e] = a1; s->ang_a1k[e] = cscale(a1, kc);
                        e++;
                    }
                }
                if (e > e0) s->act_l[na++] = l;
            }
            s->act_ptr[r + 1] = (int32_t)na;
        }
        s->n_act = na;
    }

    /* stationary blocks per kappa (tools/solver.c:419-452) */
    const size_t bn = (size_t)p->blk_nnz;
    gc64 *Sk = malloc(sizeof(gc64) * (size_t)s->nk * bn);
    gc64 *Hk = malloc(sizeof(gc64) * (size_t)s->nk * bn);
    {
        gc64 ihdt = {0.0, h * dt / 2};
        for (int kk = 0; kk < s->nk; kk++) {
            double k = (double)s->kvals[kk];
            for (size_t i = 0; i < bn; i++) {
                gc64 sv = cadd(cadd(p->s[i], cscale(p->s[bn + i], k)), cscale(p->s[2 * bn + i], k * k));
                gc64 hv = cadd(cadd(cadd(p->h0[i], cscale(p->h0[bn + i], k)), cscale(p->h0[2 * bn + i], k * k)),
                               cscale(p->h0[3 * bn + i], k * k * k));
                Sk[kk * bn + i] = sv;
                Hk[kk * bn + i] = cmul(ihdt, hv);
            }
        }
        s->S_ell = calloc((size_t)s->nk * W * B, sizeof(gc64));
        s->Hst_ell = calloc((size_t)s->nk * W * B, sizeof(gc64));
        for (int kk = 0; kk < s->nk; kk++)
            for (int j = 0; j < W; j++)
                for (int i = 0; i < B; i++) {
                    int32_t k = s->ell_pos[(size_t)j * B + i];
                    if (k < 0) continue;
                    s->S_ell[((size_t)kk * W + j) * B + i] = Sk[kk * bn + k];
                    s->Hst_ell[((size_t)kk * W + j) * B + i] = Hk[kk * bn + k];
                }
    }

    /* preconditioner ordering: interleave the two radial halves when that
       narrows the band (the DKB blocks are 2x2 banded) */
    {
        s->ord = malloc(sizeof(int32_t) * (size_t)B);
        int32_t *pos = malloc(sizeof(int32_t) * (size_t)B);
        int bw_nat = 0, bw_il = 0;
        for (int i = 0; i < B; i++)
            for (int32_t k = GAp[i]; k < GAp[i + 1]; k++) {
                int d = abs(GAi[k] - i);
                if (d > bw_nat) bw_nat = d;
            }
        if (B % 2 == 0) {
            int half = B / 2;
            for (int i = 0; i < B; i++) pos[i] = i < half ? 2 * i : 2 * (i - half) + 1;
            for (int i = 0; i < B; i++)
                for (int32_t k = GAp[i]; k < GAp[i + 1]; k++) {
                    int d = abs(pos[GAi[k]] - pos[i]);
                    if (d > bw_il) bw_il = d;
                }
        }
        int use_il = (B % 2 == 0) && bw_il < bw_nat;
        for (int i = 0; i < B; i++) {
            int pi = use_il ? pos[i] : i;
            s->ord[pi] = i;
            pos[i] = pi;
        }
        int bw = use_il ? bw_il : bw_nat;
        if (bw < 1) bw = 1;
        s->bw = bw;
        s->nch = (B + 31) / 32;
        s->Bp = 32 * s->nch;
        const int Bp = s->Bp, w = 2 * bw + 1;
        s->Lb = calloc((size_t)s->nk * bw * Bp, sizeof(gc64));
        s->Ub = calloc((size_t)s->nk * bw * Bp, sizeof(gc64));
        s->Linv = calloc((size_t)s->nk * s->nch * 1024, sizeof(gc64));
        s->Uinv = calloc((size_t)s->nk * s->nch * 1024, sizeof(gc64));
        gc64 *band = malloc(sizeof(gc64) * (size_t)B * w);
        gc64 *blk = malloc(sizeof(gc64) * 1024);
        for (int kk = 0; kk < s->nk; kk++) {
            memset(band, 0, sizeof(gc64) * (size_t)B * w);
            /* ordered matrix Q(a,b) = P^T(ord a, ord b) = P(ord b, ord a) */
            for (int i = 0; i < B; i++)
                for (int32_t k = GAp[i]; k < GAp[i + 1]; k++) {
                    int j = GAi[k];
                    gc64 v = cadd(Sk[kk * bn + k], Hk[kk * bn + k]);   /* P(i, j) */
                    int a = pos[j], b = pos[i];                        /* Q(a, b) = P(i, j) with ord a = j, ord b = i */
                    band[(size_t)a * w + (b - a + bw)] = v;
                }
            int lu = band_lu(band, B, bw);
            if (lu) {
                seterr(err, len, "preconditioner block kappa=%d has a zero pivot at row %d", s->kvals[kk], -lu - 1);
                free(band); free(blk); free(pos); free(Sk); free(Hk); gade_setup_release(s);
                return 5;
            }
            for (int d = 1; d <= bw; d++)
                for (int i = 0; i < B; i++) {
                    if (i - d >= 0) s->Lb[((size_t)kk * bw + d - 1) * Bp + i] = band[(size_t)i * w + (-d + bw)];
                    if (i + d < B) s->Ub[((size_t)kk * bw + d - 1) * Bp + i] = band[(size_t)i * w + (d + bw)];
                }
            for (int c = 0; c < s->nch; c++) {
                /* inverse of the unit-lower diagonal block of L, column-major [j][i] */
                gc64 *Li = s->Linv + ((size_t)kk * s->nch + c) * 1024;
                gc64 *Ui = s->Uinv + ((size_t)kk * s->nch + c) * 1024;
                for (int j = 0; j < 32; j++) {          /* column j of the inverse */
                    gc64 x[32];
                    for (int i = 0; i < 32; i++) {
                        gc64 v = {i == j ? 1.0 : 0.0, 0.0};
                        int gi = 32 * c + i;
                        for (int m = j; m < i; m++) {
                            int gm = 32 * c + m;
                            if (gi < B && gm < B && gi - gm <= bw)
                                v = csub(v, cmul(band[(size_t)gi * w + (gm - gi + bw)], x[m]));
                        }
                        x[i] = (i < j) ? (gc64){0, 0} : v;
                    }
                    for (int i = 0; i < 32; i++) Li[(size_t)j * 32 + i] = x[i];
                }
                for (int j = 0; j < 32; j++) {          /* inverse of the upper diagonal block */
                    gc64 x[32];
                    for (int i = 31; i >= 0; i--) {
                        int gi = 32 * c + i;
                        if (gi >= B) { x[i] = (gc64){i == j ? 1.0 : 0.0, 0.0}; continue; }
                        if (i > j) { x[i] = (gc64){0, 0}; continue; }
                        gc64 v = {i == j ? 1.0 : 0.0, 0.0};
                        for (int m = i + 1; m <= j; m++) {
                            int gm = 32 * c + m;
                            if (gm < B && gm - gi <= bw)
                                v = csub(v, cmul(band[(size_t)gi * w + (gm - gi + bw)], x[m]));
                        }
                        x[i] = cdiv(v, band[(size_t)gi * w + bw]);
                    }
                    for (int i = 0; i < 32; i++) Ui[(size_t)j * 32 + i] = x[i];
                }
            }
        }
        free(band); free(blk); free(pos);
    }
    free(Sk); free(Hk);
    *out = s;
    return 0;
}
