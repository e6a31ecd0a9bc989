/*
 * Level-1 BLAS for the oracle build of QSM.m's MEX sources.
 *
 * MATLAB links these MEX files against -lmwblas (MKL), whose summation order
 * is unpublished, so the reference's PCG inner products cannot be pinned to
 * MATLAB bit-for-bit.  This shim fixes ONE documented order instead, the
 * "lane order" that the GPU library's reductions also use:
 *
 *   lanes:  QSM_RED_LANES = 2^18 partial sums; element i goes to lane
 *           i mod 2^18, and each lane accumulates its elements in increasing
 *           i, starting from +0.0 (acc = acc + x[i]*y[i], no fused multiply-add);
 *   blocks: lanes are grouped in 1024 blocks of 256; each block is reduced by
 *           halving: for s = 128, 64, ..., 1: a[t] = a[t] + a[t+s] (t < s);
 *   final:  the 1024 block sums are reduced by the same halving.
 *
 * nrm2 is sqrt(dot(x, x)) in that order (no scaling pass); asum likewise sums
 * |x[i]|.  axpy/scal/copy/swap are element-wise and order-free.
 *
 * Test infrastructure only: nothing in the product links this.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "blas.h"

#define RED_LANES (1u << 18)
#define RED_BLOCK 256u
#define RED_NBLK (RED_LANES / RED_BLOCK)

static void halve_d(double *a, size_t n)
{
    for (size_t s = n >> 1; s > 0; s >>= 1)
        for (size_t t = 0; t < s; ++t)
            a[t] = a[t] + a[t + s];
}

static void halve_f(float *a, size_t n)
{
    for (size_t s = n >> 1; s > 0; s >>= 1)
        for (size_t t = 0; t < s; ++t)
            a[t] = a[t] + a[t + s];
}

/* mode 0: sum x*y, 1: sum x*x, 2: sum |x| */
static double lane_sum_d(size_t n, const double *x, const double *y, int mode)
{
    double *lane = (double *)calloc(RED_LANES, sizeof(double));
    double blk[RED_NBLK];
    for (size_t i = 0; i < n; ++i) {
        double v = mode == 0 ? x[i] * y[i] : mode == 1 ? x[i] * x[i] : fabs(x[i]);
        size_t t = i & (RED_LANES - 1);
        lane[t] = lane[t] + v;
    }
    for (size_t b = 0; b < RED_NBLK; ++b) {
        halve_d(lane + b * RED_BLOCK, RED_BLOCK);
        blk[b] = lane[b * RED_BLOCK];
    }
    halve_d(blk, RED_NBLK);
    free(lane);
    return blk[0];
}

static float lane_sum_f(size_t n, const float *x, const float *y, int mode)
{
    float *lane = (float *)calloc(RED_LANES, sizeof(float));
    float blk[RED_NBLK];
    for (size_t i = 0; i < n; ++i) {
        float v = mode == 0 ? x[i] * y[i] : mode == 1 ? x[i] * x[i] : fabsf(x[i]);
        size_t t = i & (RED_LANES - 1);
        lane[t] = lane[t] + v;
    }
    for (size_t b = 0; b < RED_NBLK; ++b) {
        halve_f(lane + b * RED_BLOCK, RED_BLOCK);
        blk[b] = lane[b * RED_BLOCK];
    }
    halve_f(blk, RED_NBLK);
    free(lane);
    return blk[0];
}

/* Only unit strides occur in QSM.m (mx_blas.c passes incx = incy = 1). */

void sswap(const ptrdiff_t *n, float *x, const ptrdiff_t *incx, float *y, const ptrdiff_t *incy)
{
    (void)incx; (void)incy;
    for (ptrdiff_t i = 0; i < *n; ++i) { float t = x[i]; x[i] = y[i]; y[i] = t; }
}

void dswap(const ptrdiff_t *n, double *x, const ptrdiff_t *incx, double *y, const ptrdiff_t *incy)
{
    (void)incx; (void)incy;
    for (ptrdiff_t i = 0; i < *n; ++i) { double t = x[i]; x[i] = y[i]; y[i] = t; }
}

void sscal(const ptrdiff_t *n, const float *a, float *x, const ptrdiff_t *incx)
{
    (void)incx;
    for (ptrdiff_t i = 0; i < *n; ++i) x[i] = *a * x[i];
}

void dscal(const ptrdiff_t *n, const double *a, double *x, const ptrdiff_t *incx)
{
    (void)incx;
    for (ptrdiff_t i = 0; i < *n; ++i) x[i] = *a * x[i];
}

void scopy(const ptrdiff_t *n, const float *x, const ptrdiff_t *incx, float *y, const ptrdiff_t *incy)
{
    (void)incx; (void)incy;
    memcpy(y, x, (size_t)*n * sizeof(float));
}

void dcopy(const ptrdiff_t *n, const double *x, const ptrdiff_t *incx, double *y, const ptrdiff_t *incy)
{
    (void)incx; (void)incy;
    memcpy(y, x, (size_t)*n * sizeof(double));
}

void saxpy(const ptrdiff_t *n, const float *a, const float *x, const ptrdiff_t *incx, float *y, const ptrdiff_t *incy)
{
    (void)incx; (void)incy;
    for (ptrdiff_t i = 0; i < *n; ++i) y[i] = y[i] + *a * x[i];
}

void daxpy(const ptrdiff_t *n, const double *a, const double *x, const ptrdiff_t *incx, double *y, const ptrdiff_t *incy)
{
    (void)incx; (void)incy;
    for (ptrdiff_t i = 0; i < *n; ++i) y[i] = y[i] + *a * x[i];
}

float sdot(const ptrdiff_t *n, const float *x, const ptrdiff_t *incx, const float *y, const ptrdiff_t *incy)
{
    (void)incx; (void)incy;
    return lane_sum_f((size_t)*n, x, y, 0);
}

double ddot(const ptrdiff_t *n, const double *x, const ptrdiff_t *incx, const double *y, const ptrdiff_t *incy)
{
    (void)incx; (void)incy;
    return lane_sum_d((size_t)*n, x, y, 0);
}

float snrm2(const ptrdiff_t *n, const float *x, const ptrdiff_t *incx)
{
    (void)incx;
    return sqrtf(lane_sum_f((size_t)*n, x, x, 1));
}

double dnrm2(const ptrdiff_t *n, const double *x, const ptrdiff_t *incx)
{
    (void)incx;
    return sqrt(lane_sum_d((size_t)*n, x, x, 1));
}

float sasum(const ptrdiff_t *n, const float *x, const ptrdiff_t *incx)
{
    (void)incx;
    return lane_sum_f((size_t)*n, x, x, 2);
}

double dasum(const ptrdiff_t *n, const double *x, const ptrdiff_t *incx)
{
    (void)incx;
    return lane_sum_d((size_t)*n, x, x, 2);
}
