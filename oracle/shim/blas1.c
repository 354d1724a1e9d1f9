/* The four Fortran-ABI BLAS1 routines tools/bicgstab.c calls (zdotc_, zaxpy_,
 * zscal_, zaxpby_), in plain C with the reference BLAS loop order.
 * Oracle build only. */
#include <complex.h>

double complex zdotc_(const int *n, const double complex *x, const int *incx, const double complex *y, const int *incy)
{
    double complex s = 0;
    for (int i = 0; i < *n; i++) s += conj(x[i * *incx]) * y[i * *incy];
    return s;
}

void zaxpy_(const int *n, const double complex *a, const double complex *x, const int *incx, double complex *y, const int *incy)
{
    for (int i = 0; i < *n; i++) y[i * *incy] += *a * x[i * *incx];
}

void zscal_(const int *n, const double complex *a, double complex *x, const int *incx)
{
    for (int i = 0; i < *n; i++) x[i * *incx] *= *a;
}

void zaxpby_(const int *n, const double complex *a, const double complex *x, const int *incx,
             const double complex *b, double complex *y, const int *incy)
{
    for (int i = 0; i < *n; i++) y[i * *incy] = *a * x[i * *incx] + *b * y[i * *incy];
}
