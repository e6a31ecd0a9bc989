/*
 * Level-1 BLAS prototypes in the Fortran pointer-argument convention that
 * MATLAB's blas.h exposes (every argument by pointer, ptrdiff_t sizes).
 * The implementations in blas_shim.c are this project's; see that file for
 * the summation order they fix.
 *
 * Test infrastructure only: nothing in the product links this.
 */
#pragma once

#include <stddef.h>

void  sswap(const ptrdiff_t *n, float *x, const ptrdiff_t *incx, float *y, const ptrdiff_t *incy);
void  dswap(const ptrdiff_t *n, double *x, const ptrdiff_t *incx, double *y, const ptrdiff_t *incy);
void  sscal(const ptrdiff_t *n, const float *a, float *x, const ptrdiff_t *incx);
void  dscal(const ptrdiff_t *n, const double *a, double *x, const ptrdiff_t *incx);
void  scopy(const ptrdiff_t *n, const float *x, const ptrdiff_t *incx, float *y, const ptrdiff_t *incy);
void  dcopy(const ptrdiff_t *n, const double *x, const ptrdiff_t *incx, double *y, const ptrdiff_t *incy);
void  saxpy(const ptrdiff_t *n, const float *a, const float *x, const ptrdiff_t *incx, float *y, const ptrdiff_t *incy);
void  daxpy(const ptrdiff_t *n, const double *a, const double *x, const ptrdiff_t *incx, double *y, const ptrdiff_t *incy);
float sdot(const ptrdiff_t *n, const float *x, const ptrdiff_t *incx, const float *y, const ptrdiff_t *incy);
double ddot(const ptrdiff_t *n, const double *x, const ptrdiff_t *incx, const double *y, const ptrdiff_t *incy);
float snrm2(const ptrdiff_t *n, const float *x, const ptrdiff_t *incx);
double dnrm2(const ptrdiff_t *n, const double *x, const ptrdiff_t *incx);
float sasum(const ptrdiff_t *n, const float *x, const ptrdiff_t *incx);
double dasum(const ptrdiff_t *n, const double *x, const ptrdiff_t *incx);
