/*
 * Link-time hooks for the pinned reference oracle (oracle/build_ref.py):
 *  - --wrap=bicgstab: optionally overrides the hard-coded tolerance and
 *    iteration cap (tools/dirac_solver.c:506-507; env GADE_REF_TOL,
 *    GADE_REF_MAXIT), records iterations and tolerance of every step
 *    (GADE_REF_LOG: step, iterations, tolerance, BiCGSTAB microseconds and
 *    the wall clock at its end, whose differences time whole steps), writes
 *    the state after every step (GADE_REF_XOUT; the
 *    reference itself writes only every 2000 steps), keeps a copy of the
 *    state every k steps in <GADE_REF_XOUT>.<step> (GADE_REF_XSNAP_EVERY=k)
 *    and can stop after a number of steps (GADE_REF_MAXSTEPS).
 *  - --wrap=calloc: pads allocations; the reference indexes
 *    itersarr/tolsarr/timearr[iter] one or two past their calloc'd length
 *    (tools/dirac_solver.c:498-500, 575-577).
 * Oracle build only.
 */
#include <stdio.h>
#include <stdlib.h>
#include <sys/time.h>

#include "bicgstab.h"

void __real_bicgstab(spmv_fun spmv, const void *mat, const cdouble_t *rhs, cdouble_t *x, int nrow, int ncol,
                     int local_col_beg, precond_fun psolve, const void *precond, solver_workspace_t *wsp,
                     int *iters, double *tol_error);

void __wrap_bicgstab(spmv_fun spmv, const void *mat, const cdouble_t *rhs, cdouble_t *x, int nrow, int ncol,
                     int local_col_beg, precond_fun psolve, const void *precond, solver_workspace_t *wsp,
                     int *iters, double *tol_error)
{
    static int step = 0;
    const char *e;
    if ((e = getenv("GADE_REF_TOL"))) *tol_error = atof(e);
    if ((e = getenv("GADE_REF_MAXIT"))) *iters = atoi(e);
    struct timeval t0, t1;
    gettimeofday(&t0, NULL);
    __real_bicgstab(spmv, mat, rhs, x, nrow, ncol, local_col_beg, psolve, precond, wsp, iters, tol_error);
    gettimeofday(&t1, NULL);
    step++;
    if ((e = getenv("GADE_REF_LOG"))) {
        FILE *f = fopen(e, step == 1 ? "w" : "a");
        if (f) {
            fprintf(f, "%d %d %.17e %ld %ld\n", step, *iters, *tol_error,
                    (long)((t1.tv_sec - t0.tv_sec) * 1000000L + (t1.tv_usec - t0.tv_usec)),
                    (long)(t1.tv_sec * 1000000L + t1.tv_usec));
            fclose(f);
        }
    }
    if ((e = getenv("GADE_REF_XOUT"))) {
        FILE *f = fopen(e, "wb");
        if (f) {
            fwrite(x + local_col_beg, sizeof(cdouble_t), (size_t)nrow, f);
            fclose(f);
        }
        const char *every = getenv("GADE_REF_XSNAP_EVERY");
        if (every && atoi(every) > 0 && step % atoi(every) == 0) {
            char path[4096];
            snprintf(path, sizeof path, "%s.%d", e, step);
            if ((f = fopen(path, "wb"))) {
                fwrite(x + local_col_beg, sizeof(cdouble_t), (size_t)nrow, f);
                fclose(f);
            }
        }
    }
    if ((e = getenv("GADE_REF_MAXSTEPS")) && step >= atoi(e)) exit(0);
}

void *__real_calloc(size_t n, size_t size);
void *__wrap_calloc(size_t n, size_t size) { return __real_calloc(n + 16, size); }
