/*
 * dirac_solver — drop-in replacement of the reference tools/dirac_solver
 * (tools/dirac_solver.c:170-642) running the Crank-Nicolson time loop on one
 * GB300 through libgade_gb300.
 *
 * Same command line (-t maxtime -l lmax -i E0 -o omega -c cycles
 * -n Ntime [-s start_iter] [-v]), same input files in the working directory
 * (H.csr, H0l<l>.csr, H1l<l>.csr, g<q>a<a>l<l>.csr, h0<n>.csr, s<n>.csr,
 * psi0.vec) and same outputs (x<iter>.out every 2000 steps, runstats.txt,
 * the stdout lines).  Backward-compatible additions (long options):
 *   --tol X          BiCGSTAB relative tolerance (default 1e-16, as the reference)
 *   --maxit N        BiCGSTAB iteration cap (default 500, as the reference)
 *   --final-dump     also write x<last>.out and runstats.txt after the last step
 *   --restart FILE   start from an x<iter>.out file instead of psi0.vec
 *   --precision P    fp64 (default) or mixed (complex64 inner solves)
 *   --device N       CUDA device ordinal (default 0)
 *   --stats FILE     per-step JSON lines: iter, time, iters, tol_error, us
 *   --dir DIR        directory holding the input files (default ".")
 */
#define _GNU_SOURCE
#include <getopt.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include "gade.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static double now_us(void)
{
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return tv.tv_sec * 1e6 + tv.tv_usec;
}

/* beoyndDipolePulse_axialPart, tools/solver_common.c:53-65 */
static void pulse(double E0, double omega, double T, double t, double *ft)
{
    const double phi = -M_PI / 2;
    memset(ft, 0, sizeof(double) * 12);
    ft[0] = -E0 / (4 * omega) * cos(phi + t * (2 * M_PI / T + omega));
    ft[2] = -E0 / (4 * omega) * sin(phi + t * (2 * M_PI / T + omega));
    ft[4] = -E0 / (4 * omega) * cos(-phi + t * (2 * M_PI / T - omega));
    ft[6] = E0 / (4 * omega) * sin(-phi + t * (2 * M_PI / T - omega));
    ft[8] = E0 / (2 * omega) * cos(phi + t * omega);
    ft[10] = E0 / (2 * omega) * sin(phi + t * omega);
}

static int write_output(const char *dir, int iter, const double *x, const int32_t *xperm, int64_t n,
                        const int *itersarr, const double *tolsarr, const long *timearr, int niter)
{
    char fname[4096];
    double *xorig = malloc(sizeof(double) * 2 * (size_t)n);
    if (!xorig) return 1;
    for (int64_t i = 0; i < n; i++) {
        xorig[2 * (size_t)xperm[i]] = x[2 * i];
        xorig[2 * (size_t)xperm[i] + 1] = x[2 * i + 1];
    }
    snprintf(fname, sizeof(fname), "%s/x%d.out", dir, iter);
    printf("saving output file x%d.out\n", iter);
    FILE *fd = fopen(fname, "w+");
    if (!fd) { free(xorig); fprintf(stderr, "cant open %s\n", fname); return 1; }
    int nrows = (int)n, ncols = 1;
    fwrite(&nrows, sizeof(int), 1, fd);
    fwrite(&ncols, sizeof(int), 1, fd);
    fwrite(xorig, sizeof(double) * 2, (size_t)n, fd);
    fclose(fd);
    free(xorig);
    snprintf(fname, sizeof(fname), "%s/runstats.txt", dir);
    FILE *fs = fopen(fname, "w+");
    if (!fs) return 1;
    for (int i = 0; i < niter; i++) fprintf(fs, "%d, %e, %ld\n", itersarr[i], tolsarr[i], timearr[i]);
    fclose(fs);
    return 0;
}

static int read_restart(const char *fname, double *x, const int32_t *xperm, int64_t n)
{
    FILE *fd = fopen(fname, "rb");
    if (!fd) { fprintf(stderr, "cant open %s\n", fname); return 1; }
    int nrows, ncols;
    if (fread(&nrows, 4, 1, fd) != 1 || fread(&ncols, 4, 1, fd) != 1 || (int64_t)nrows * ncols != n) {
        fprintf(stderr, "wrong file format in %s\n", fname); fclose(fd); return 1;
    }
    double *xorig = malloc(sizeof(double) * 2 * (size_t)n);
    if (fread(xorig, sizeof(double) * 2, (size_t)n, fd) != (size_t)n) {
        fprintf(stderr, "wrong file format in %s\n", fname); fclose(fd); free(xorig); return 1;
    }
    fclose(fd);
    for (int64_t i = 0; i < n; i++) {
        x[2 * i] = xorig[2 * (size_t)xperm[i]];
        x[2 * i + 1] = xorig[2 * (size_t)xperm[i] + 1];
    }
    free(xorig);
    return 0;
}

#define DIE(...) do { fprintf(stderr, __VA_ARGS__); fprintf(stderr, "\n"); exit(1); } while (0)

int main(int argc, char *argv[])
{
    int opt, lmax = 0, iter = 1, comm_info = 0, final_dump = 0, device = 0, maxit = 500;
    double intensity = 0, omega = 0, cycles = 0, maxtime = 0, time = 0, iterations = 0, tol = 1e-16;
    const char *restart = NULL, *stats_path = NULL, *dir = ".";
    int precision = GADE_PREC_FP64;

    if (argc < 5) {
        fprintf(stderr, "Usage: %s -l time -l lmax -i intensity -o omega -c cycles\n", argv[0]);
        exit(EXIT_FAILURE);
    }
    static struct option longopts[] = {
        {"tol", required_argument, 0, 1}, {"maxit", required_argument, 0, 2},
        {"final-dump", no_argument, 0, 3}, {"restart", required_argument, 0, 4},
        {"precision", required_argument, 0, 5}, {"device", required_argument, 0, 6},
        {"stats", required_argument, 0, 7}, {"dir", required_argument, 0, 8}, {0, 0, 0, 0}};
    while ((opt = getopt_long(argc, argv, "t:l:i:o:c:n:v:s:", longopts, NULL)) != -1) {
        switch (opt) {
        case 't': maxtime = atof(optarg); break;
        case 'l': lmax = atoi(optarg); break;
        case 'i': intensity = atof(optarg); break;
        case 'o': omega = atof(optarg); break;
        case 'c': cycles = atof(optarg); break;
        case 'n': iterations = atof(optarg); break;
        case 'v': comm_info = 1; break;
        case 's':
            printf("%s", optarg);
            fflush(stdout);
            printf("%d\n", atoi(optarg));
            fflush(stdout);
            iter = atoi(optarg);
            break;
        case 1: tol = atof(optarg); break;
        case 2: maxit = atoi(optarg); break;
        case 3: final_dump = 1; break;
        case 4: restart = optarg; break;
        case 5:
            if (!strcmp(optarg, "fp64")) precision = GADE_PREC_FP64;
            else if (!strcmp(optarg, "mixed")) precision = GADE_PREC_MIXED;
            else DIE("unknown precision %s (fp64|mixed)", optarg);
            break;
        case 6: device = atoi(optarg); break;
        case 7: stats_path = optarg; break;
        case 8: dir = optarg; break;
        default:
            fprintf(stderr, "Usage: %s [-lioc]\n", argv[0]);
            exit(EXIT_FAILURE);
        }
    }
    double dt = maxtime / iterations;
    double h = 1;
    const double T = cycles * 2 * M_PI / omega;   /* beyondDipolePulse_init */

    printf("Parameters:\n");
    printf(" - time       %f\n", maxtime);
    printf(" - lmax       %d\n", lmax);
    printf(" - intensity  %lf\n", intensity);
    printf(" - omega      %lf\n", omega);
    printf(" - cycles     %lf\n", cycles);
    printf(" - iterations %lf\n", iterations);
    printf(" - dt         %.15lf\n", dt);
    printf(" - h          %lf\n", h);
    if (comm_info) {
        printf("single partition: no inter-rank communication\n");
        return 0;
    }

    gade_problem *prob = NULL;
    if (gade_problem_load(dir, lmax, &prob)) DIE("%s", gade_last_error());
    gade_problem_info info;
    gade_problem_get_info(prob, &info);
    printf("0: All matrices read correctly. System info:\n");
    printf(" - H dim:         %d x %d\n", info.nblk, info.nblk);
    printf(" - Hall dim:      %d x %d\n", info.nblk, info.nblk);
    printf(" - Hall nnz:      %lld\n", (long long)info.hall_nnz);
    printf(" - Hfull_blk dim: %d x %d\n", info.nblk, info.nblk);
    printf(" - Hfull dim:     %lld x %lld\n", (long long)info.n, (long long)info.n);
    printf(" - Hfull nnz:     %lld\n", (long long)info.nnz_full);
    fflush(stdout);

    const int64_t n = info.n;
    double *x = malloc(sizeof(double) * 2 * (size_t)n);
    int32_t *xperm = malloc(sizeof(int32_t) * (size_t)n);
    gade_problem_get_psi0(prob, x, xperm);
    if (restart && read_restart(restart, x, xperm, n)) exit(1);

    gade_solver *solver = NULL;
    double t0 = now_us();
    if (gade_solver_create(prob, dt, h, precision, device, &solver)) DIE("%s", gade_last_error());
    if (gade_solver_set_x(solver, x, n)) DIE("%s", gade_last_error());
    printf("GPU solver set up in %.3f s (matrix-free operator, block-LU preconditioner)\n", (now_us() - t0) * 1e-6);

    /* the reference indexes these arrays with iter = 1..Ntime(+1): pad */
    int nslots = (int)iterations + 4;
    int *itersarr = calloc((size_t)nslots, sizeof(int));
    double *tolsarr = calloc((size_t)nslots, sizeof(double));
    long *timearr = calloc((size_t)nslots, sizeof(long));
    FILE *fstats = stats_path ? fopen(stats_path, "w") : NULL;

    time = dt * (iter - 1);
    double big0 = now_us();
    int last_iter = iter - 1;
    while (time <= maxtime) {
        double ft[12];
        gade_step_stats st;
        time = time + dt;
        pulse(intensity, omega, T, time, ft);
        if (iter % 10 == 0) {
            printf("iteration %d simulation time %lf\n", iter, time);
            fflush(stdout);
        }
        double s0 = now_us();
        if (gade_solver_step(solver, ft, maxit, tol, &st)) DIE("step %d: %s", iter, gade_last_error());
        long bicgtime = (long)(now_us() - s0);
        if (iter >= 0 && iter < nslots) {
            itersarr[iter] = st.iters;
            tolsarr[iter] = st.tol_error;
            timearr[iter] = bicgtime;
        }
        if (fstats)
            fprintf(fstats, "{\"iter\": %d, \"time\": %.17g, \"iters\": %d, \"tol_error\": %.6e, \"us\": %ld}\n",
                    iter, time, st.iters, st.tol_error, bicgtime);
        if (iter % 2000 == 0) {
            if (gade_solver_get_x(solver, x, n)) DIE("%s", gade_last_error());
            if (write_output(dir, iter, x, xperm, n, itersarr, tolsarr, timearr, (int)iterations)) DIE("cannot write output");
        }
        last_iter = iter;
        iter++;
    }
    double total = now_us() - big0;
    if (final_dump && last_iter % 2000 != 0) {
        if (gade_solver_get_x(solver, x, n)) DIE("%s", gade_last_error());
        if (write_output(dir, last_iter, x, xperm, n, itersarr, tolsarr, timearr, (int)iterations)) DIE("cannot write output");
    }
    printf("Total runtime: ");
    printf("time:\t\t%li.%.6lis\n", (long)total / 1000000, (long)total % 1000000);
    if (fstats) fclose(fstats);
    gade_solver_free(solver);
    gade_problem_free(prob);
    free(x); free(xperm); free(itersarr); free(tolsarr); free(timearr);
    return 0;
}
