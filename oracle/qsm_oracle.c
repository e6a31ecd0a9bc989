/*
 * qsm_oracle.c -- CPU oracle for the QSM.m hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a C restatement, in this project's own
 * code, of the algorithms in QSM.m's C-MEX sources (src/inversion/mex,
 * src/utils/fd/mex, src/unwrap/mex, src/utils/poisson_solver/mex).  It is
 * what tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * compare and time the GPU library against; the library itself never links
 * or calls it.
 *
 * Parity pin: every routine is checked bit-for-bit against the reference's
 * own sources compiled by oracle/ref/Makefile (the shared objects in oracle/_ref, driven by
 * oracle/refmex.py) through the committed golden fixtures in tests/golden/.
 *
 * Inner products and norms that the reference leaves to MATLAB's BLAS (and
 * the TGV/TV convergence monitors, an OpenMP reduction there) use the
 * "lane order" documented in oracle/ref/mexshim/blas_shim.c, which the GPU
 * library's reductions also follow, so multigrid-PCG iterates are
 * reproducible bit-for-bit between this oracle and the GPU.
 *
 * Built with -std=c11 -O2 -ffp-contract=off -fopenmp (no fused multiply-add,
 * as in the reference build).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define RED_LANES ((size_t)1 << 18)
#define RED_BLOCK ((size_t)256)
#define RED_NBLK (RED_LANES / RED_BLOCK)

/* ---------------- lane-order reductions ---------------- */

static void halve(double *a, size_t n)
{
    for (size_t s = n >> 1; s > 0; s >>= 1)
        for (size_t t = 0; t < s; ++t) a[t] = a[t] + a[t + s];
}

static void halvef(float *a, size_t n)
{
    for (size_t s = n >> 1; s > 0; s >>= 1)
        for (size_t t = 0; t < s; ++t) a[t] = a[t] + a[t + s];
}

static double finish(double *lane)
{
    double blk[RED_NBLK];
    for (size_t b = 0; b < RED_NBLK; ++b) {
        halve(lane + b * RED_BLOCK, RED_BLOCK);
        blk[b] = lane[b * RED_BLOCK];
    }
    halve(blk, RED_NBLK);
    return blk[0];
}

static float finishf(float *lane)
{
    float blk[RED_NBLK];
    for (size_t b = 0; b < RED_NBLK; ++b) {
        halvef(lane + b * RED_BLOCK, RED_BLOCK);
        blk[b] = lane[b * RED_BLOCK];
    }
    halvef(blk, RED_NBLK);
    return blk[0];
}

/* dot(x, y) in lane order; FP32 inputs accumulate in FP32 (like sdot) and
 * the result is widened, as mx_dot does (mx_blas.c:108-131). */
double orc_lane_dot(const void *x, const void *y, size_t n, int is_float)
{
    if (is_float) {
        float *lane = (float *)calloc(RED_LANES, sizeof(float));
        const float *a = (const float *)x, *b = (const float *)y;
        #pragma omp parallel for schedule(static)
        for (size_t t = 0; t < RED_LANES; ++t)
            for (size_t i = t; i < n; i += RED_LANES) lane[t] = lane[t] + a[i] * b[i];
        float r = finishf(lane);
        free(lane);
        return (double)r;
    }
    double *lane = (double *)calloc(RED_LANES, sizeof(double));
    const double *a = (const double *)x, *b = (const double *)y;
    #pragma omp parallel for schedule(static)
    for (size_t t = 0; t < RED_LANES; ++t)
        for (size_t i = t; i < n; i += RED_LANES) lane[t] = lane[t] + a[i] * b[i];
    double r = finish(lane);
    free(lane);
    return r;
}

double orc_lane_nrm2(const void *x, size_t n, int is_float)
{
    if (is_float) return (double)sqrtf((float)orc_lane_dot(x, x, n, 1));
    return sqrt(orc_lane_dot(x, x, n, 0));
}

/* The four FP64 sums of convergence_check{d,f} (pd_tgv_mex.c:981-1045):
 * s = {sum chi^2, sum eta^2, sum (chi-chi0)^2, sum (eta-eta0)^2}. */
void orc_lane_sum4(double *s, size_t n, const void *chi, const void *chi0,
                   const void *eta, const void *eta0, int is_float)
{
    double *lane = (double *)calloc(4 * RED_LANES, sizeof(double));
    #pragma omp parallel for schedule(static)
    for (size_t t = 0; t < RED_LANES; ++t) {
        double a = 0.0, b = 0.0, c = 0.0, d = 0.0;
        for (size_t i = t; i < n; i += RED_LANES) {
            if (is_float) {
                const float x = ((const float *)chi)[i], x0 = ((const float *)chi0)[i];
                const float e = ((const float *)eta)[i], e0 = ((const float *)eta0)[i];
                a = a + (double)x * (double)x;
                b = b + (double)e * (double)e;
                c = c + (double)(x - x0) * ((double)x - (double)x0);
                d = d + (double)(e - e0) * ((double)e - (double)e0);
            } else {
                const double x = ((const double *)chi)[i], x0 = ((const double *)chi0)[i];
                const double e = ((const double *)eta)[i], e0 = ((const double *)eta0)[i];
                a = a + x * x;
                b = b + e * e;
                c = c + (x - x0) * (x - x0);
                d = d + (e - e0) * (e - e0);
            }
        }
        lane[t] = a;
        lane[RED_LANES + t] = b;
        lane[2 * RED_LANES + t] = c;
        lane[3 * RED_LANES + t] = d;
    }
    for (int q = 0; q < 4; ++q) s[q] = finish(lane + (size_t)q * RED_LANES);
    free(lane);
}

/* element-wise BLAS-1 in the semantics of sscal/dscal and saxpy/daxpy */
void orc_scal(void *x, double a, size_t n, int is_float)
{
    if (is_float) {
        const float af = (float)a;
        float *v = (float *)x;
        for (size_t i = 0; i < n; ++i) v[i] = af * v[i];
    } else {
        double *v = (double *)x;
        for (size_t i = 0; i < n; ++i) v[i] = a * v[i];
    }
}

void orc_axpy(void *y, double a, const void *x, size_t n, int is_float)
{
    if (is_float) {
        const float af = (float)a;
        float *v = (float *)y;
        const float *u = (const float *)x;
        for (size_t i = 0; i < n; ++i) v[i] = v[i] + af * u[i];
    } else {
        double *v = (double *)y;
        const double *u = (const double *)x;
        for (size_t i = 0; i < n; ++i) v[i] = v[i] + a * u[i];
    }
}

/* ---------------- integer mask work (bit-exact) ---------------- */

/* init_bitmask (pd_tgv_mex.c:1050-1121 / pd_tv_mex.c:800-871): the only
 * output used later is mi[l] = 1 iff all six face neighbours of l lie in
 * the grid and in m (m[l] itself is not required).  The per-axis bit word
 * mb is never read afterwards and is not formed. */
void orc_interior_mask(uint8_t *mi, const uint8_t *m, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                mi[l] = (uint8_t)((i > 0 && m[l - 1]) && (i + 1 < nx && m[l + 1]) &&
                                  (j > 0 && m[l - nx]) && (j + 1 < ny && m[l + nx]) &&
                                  (k > 0 && m[l - nxny]) && (k + 1 < nz && m[l + nxny]));
            }
}

/* coarsen_grid_mex.c:52-125: coarse interior voxel (i2,j2,k2) is in G2 iff
 * the fine voxel (2i2-1, 2j2-1, 2k2-1) and its +1 neighbours in x, y, z (the
 * 2x2x2 block) are in G, where a +1 neighbour on the last interior fine
 * index or beyond (i >= nx-2) counts as present. */
void orc_coarsen_grid(uint8_t *G2, const uint8_t *G, const size_t *sz2, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const size_t nx2 = sz2[0], ny2 = sz2[1], nz2 = sz2[2], nxny2 = nx2 * ny2;
    memset(G2, 0, nxny2 * nz2);
    for (size_t k2 = 1; k2 + 1 < nz2; ++k2)
        for (size_t j2 = 1; j2 + 1 < ny2; ++j2)
            for (size_t i2 = 1; i2 + 1 < nx2; ++i2) {
                const size_t i = 2 * i2 - 1, j = 2 * j2 - 1, k = 2 * k2 - 1;
                const size_t l = i + nx * j + nxny * k;
                const int bi = !(i < nx - 2), bj = !(j < ny - 2), bk = !(k < nz - 2);
                G2[i2 + nx2 * j2 + nxny2 * k2] = (uint8_t)(G[l] &&
                    (bi || G[l + 1]) && (bj || G[l + nx]) && (bk || G[l + nxny]) &&
                    (bi || bj || G[l + 1 + nx]) && (bi || bk || G[l + 1 + nxny]) &&
                    (bj || bk || G[l + nx + nxny]) && (bi || bj || bk || G[l + 1 + nx + nxny]));
            }
}

/* boundary_mask_mex.c:46-132.  b = G on the outermost interior shell and on
 * every 2x2x2 block (anchored at odd interior indices) that is not wholly in
 * G; B = 1 where G and b holds at the voxel or a face neighbour.  B is only
 * written where G (the rest keeps the caller's contents). */
void orc_boundary_mask(uint8_t *B, const uint8_t *G, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    if (nx < 3 || ny < 3 || nz < 3) return;
    uint8_t *b = (uint8_t *)calloc(nxny * nz, 1);
    for (size_t k = 1; k + 1 < nz; ++k)
        for (size_t j = 1; j + 1 < ny; ++j)
            for (size_t i = 1; i + 1 < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (i == 1 || j == 1 || k == 1 || i == nx - 2 || j == ny - 2 || k == nz - 2) b[l] = G[l];
            }
    for (size_t k = 1; k + 1 < nz; k += 2)
        for (size_t j = 1; j + 1 < ny; j += 2)
            for (size_t i = 1; i + 1 < nx; i += 2) {
                size_t l = i + nx * j + nxny * k;
                const size_t o[8] = {0, 1, nx, nxny, 1 + nx, 1 + nxny, nx + nxny, 1 + nx + nxny};
                int full = 1;
                for (int q = 0; q < 8; ++q) full = full && G[l + o[q]];
                if (!full)
                    for (int q = 0; q < 8; ++q) b[l + o[q]] = G[l + o[q]];
            }
    for (size_t k = 1; k + 1 < nz; ++k)
        for (size_t j = 1; j + 1 < ny; ++j)
            for (size_t i = 1; i + 1 < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (G[l])
                    B[l] = (uint8_t)(b[l - nxny] || b[l - nx] || b[l - 1] || b[l] || b[l + 1] || b[l + nx] || b[l + nxny]);
            }
    free(b);
}

/* boundary_mask_l1_mex.c:49-117: band of L1 width l1 inside G. */
void orc_boundary_mask_l1(uint8_t *B, const uint8_t *G, const size_t *sz, uint8_t l1)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    uint8_t *GL = (uint8_t *)calloc(nxny * nz + 1, 1);
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (i == 0 || j == 0 || k == 0 || i == nx - 1 || j == ny - 1 || k == nz - 1)
                    B[l] = GL[l] = G[l];
                else
                    B[l] = GL[l] = (uint8_t)(G[l] && !(G[l - 1] && G[l + 1] && G[l - nx] && G[l + nx] && G[l - nxny] && G[l + nxny]));
            }
    for (size_t L1 = 1; L1 < l1; ++L1)
        for (size_t k = L1; k + L1 < nz; ++k)
            for (size_t j = L1; j + L1 < ny; ++j)
                for (size_t i = L1; i + L1 < nx; ++i) {
                    size_t l = i + nx * j + nxny * k;
                    if (G[l] && !GL[l] &&
                        (GL[l - 1] == L1 || GL[l + 1] == L1 || GL[l - nx] == L1 || GL[l + nx] == L1 ||
                         GL[l - nxny] == L1 || GL[l + nxny] == L1)) {
                        B[l] = 1;
                        GL[l] = (uint8_t)(L1 + 1);
                    }
                }
    free(GL);
}

void orc_pad_u8(uint8_t *xp, const uint8_t *x, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxp = nx + 2, nxnyp = (nx + 2) * (ny + 2);
    memset(xp, 0, (nx + 2) * (ny + 2) * (nz + 2));
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            memcpy(xp + 1 + nxp * (j + 1) + nxnyp * (k + 1), x + nx * j + nx * ny * k, nx);
}

/* ---------------- typed bodies ---------------- */

#define T double
#define SFX _d
#define SQRT sqrt
#define FMOD fmod
#include "qsm_oracle_body.h"
#undef T
#undef SFX
#undef SQRT
#undef FMOD

#define T float
#define SFX _f
#define SQRT sqrtf
#define FMOD fmodf
#include "qsm_oracle_body.h"
#undef T
#undef SFX
#undef SQRT
#undef FMOD
