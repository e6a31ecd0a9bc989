/*
 * Type-generic body of the CPU oracle; included twice by qsm_oracle.c, once
 * with T=double (suffix _d) and once with T=float (suffix _f).
 *
 * TEST INFRASTRUCTURE ONLY (see qsm_oracle.c).  Each routine restates, in this
 * project's own code, the arithmetic of one QSM.m C-MEX loop nest: the same
 * per-voxel expression with the same association order and the same
 * double->float constant casts, so results agree bit-for-bit with the
 * reference built from its sources (checked against oracle/_ref and the
 * golden fixtures).  Loop structure is free: every routine here is a
 * per-voxel rule, which is also how the GPU kernels are written.
 *
 * Layout: column-major, x fastest, l = i + nx*j + nx*ny*k; vector fields are
 * component-major (p1, p2, p3 at offsets 0, N, 2N); masks are uint8.
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

/* ------------------------------------------------------------------ */
/* Finite-difference operators (src/utils/fd/mex, src/inversion/mex,   */
/* src/unwrap/mex).  dims: sz[0..2] = nx, ny, nz.                      */
/* ------------------------------------------------------------------ */

/* gradf_mex.c:149-245: forward differences, one-sided backward on the far
 * face (the far corner's copies at :238-242 equal that rule). */
void FN(orc_gradf)(T *dx, T *dy, T *dz, const T *u, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(1.0 / h[0]), hy = (T)(1.0 / h[1]), hz = (T)(1.0 / h[2]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                dx[l] = i + 1 < nx ? hx * (u[l + 1] - u[l]) : hx * (u[l] - u[l - 1]);
                dy[l] = j + 1 < ny ? hy * (u[l + nx] - u[l]) : hy * (u[l] - u[l - nx]);
                dz[l] = k + 1 < nz ? hz * (u[l + nxny] - u[l]) : hz * (u[l] - u[l - nxny]);
            }
}

/* gradb_mex.c:142-229: backward differences, one-sided forward on the near face. */
void FN(orc_gradb)(T *dx, T *dy, T *dz, const T *u, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(1.0 / h[0]), hy = (T)(1.0 / h[1]), hz = (T)(1.0 / h[2]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                dx[l] = i > 0 ? hx * (u[l] - u[l - 1]) : hx * (u[l + 1] - u[l]);
                dy[l] = j > 0 ? hy * (u[l] - u[l - nx]) : hy * (u[l + nx] - u[l]);
                dz[l] = k > 0 ? hz * (u[l] - u[l - nxny]) : hz * (u[l + nxny] - u[l]);
            }
}

/* gradc_mex.c:309-563: central differences, one-sided on both faces.  The
 * "i = nx-1, k = 0" loop there (:396, float :138) steps j by 1 instead of nx,
 * so on the k = 0 plane every linear index l in [2nx-1, nx*ny-2] ends up with
 * dx = backward, dy = central, dz = forward; that overwrite is reproduced. */
void FN(orc_gradc)(T *dx, T *dy, T *dz, const T *u, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(1.0 / h[0]), hy = (T)(1.0 / h[1]), hz = (T)(1.0 / h[2]);
    const T hx2 = (T)(0.5 / h[0]), hy2 = (T)(0.5 / h[1]), hz2 = (T)(0.5 / h[2]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (k == 0 && l >= 2 * nx - 1 && l + 2 <= nxny) {
                    dx[l] = hx * (u[l] - u[l - 1]);
                    dy[l] = hy2 * (u[l + nx] - u[l - nx]);
                    dz[l] = hz * (u[l + nxny] - u[l]);
                    continue;
                }
                dx[l] = i == 0 ? hx * (u[l + 1] - u[l]) : i + 1 == nx ? hx * (u[l] - u[l - 1]) : hx2 * (u[l + 1] - u[l - 1]);
                dy[l] = j == 0 ? hy * (u[l + nx] - u[l]) : j + 1 == ny ? hy * (u[l] - u[l - nx]) : hy2 * (u[l + nx] - u[l - nx]);
                dz[l] = k == 0 ? hz * (u[l + nxny] - u[l]) : k + 1 == nz ? hz * (u[l] - u[l - nxny]) : hz2 * (u[l + nxny] - u[l - nxny]);
            }
}

/* gradfm_mex.c:105-154: masked forward gradient, written only where G. */
void FN(orc_gradfm)(T *dx, T *dy, T *dz, const T *u, const uint8_t *G, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(1.0 / h[0]), hy = (T)(1.0 / h[1]), hz = (T)(1.0 / h[2]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (!G[l]) continue;
                dx[l] = (i + 1 < nx && G[l + 1]) ? hx * (u[l + 1] - u[l]) : (i > 0 && G[l - 1]) ? hx * (u[l] - u[l - 1]) : (T)0;
                dy[l] = (j + 1 < ny && G[l + nx]) ? hy * (u[l + nx] - u[l]) : (j > 0 && G[l - nx]) ? hy * (u[l] - u[l - nx]) : (T)0;
                dz[l] = (k + 1 < nz && G[l + nxny]) ? hz * (u[l + nxny] - u[l]) : (k > 0 && G[l - nxny]) ? hz * (u[l] - u[l - nxny]) : (T)0;
            }
}

/* gradbm_mex.c:106-154: masked backward gradient. */
void FN(orc_gradbm)(T *dx, T *dy, T *dz, const T *u, const uint8_t *G, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(1.0 / h[0]), hy = (T)(1.0 / h[1]), hz = (T)(1.0 / h[2]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (!G[l]) continue;
                dx[l] = (i > 0 && G[l - 1]) ? hx * (u[l] - u[l - 1]) : (i + 1 < nx && G[l + 1]) ? hx * (u[l + 1] - u[l]) : (T)0;
                dy[l] = (j > 0 && G[l - nx]) ? hy * (u[l] - u[l - nx]) : (j + 1 < ny && G[l + nx]) ? hy * (u[l + nx] - u[l]) : (T)0;
                dz[l] = (k > 0 && G[l - nxny]) ? hz * (u[l] - u[l - nxny]) : (k + 1 < nz && G[l + nxny]) ? hz * (u[l + nxny] - u[l]) : (T)0;
            }
}

/* gradcm_mex.c:122-186: masked central gradient. */
void FN(orc_gradcm)(T *dx, T *dy, T *dz, const T *u, const uint8_t *G, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(1.0 / h[0]), hy = (T)(1.0 / h[1]), hz = (T)(1.0 / h[2]);
    const T hx2 = (T)(0.5 / h[0]), hy2 = (T)(0.5 / h[1]), hz2 = (T)(0.5 / h[2]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (!G[l]) continue;
                int xf = i + 1 < nx && G[l + 1], xb = i > 0 && G[l - 1];
                int yf = j + 1 < ny && G[l + nx], yb = j > 0 && G[l - nx];
                int zf = k + 1 < nz && G[l + nxny], zb = k > 0 && G[l - nxny];
                dx[l] = (xf && xb) ? hx2 * (u[l + 1] - u[l - 1]) : xf ? hx * (u[l + 1] - u[l]) : xb ? hx * (u[l] - u[l - 1]) : (T)0;
                dy[l] = (yf && yb) ? hy2 * (u[l + nx] - u[l - nx]) : yf ? hy * (u[l + nx] - u[l]) : yb ? hy * (u[l] - u[l - nx]) : (T)0;
                dz[l] = (zf && zb) ? hz2 * (u[l + nxny] - u[l - nxny]) : zf ? hz * (u[l + nxny] - u[l]) : zb ? hz * (u[l] - u[l - nxny]) : (T)0;
            }
}

/* gradf_adj_mex.c:153-249: du = (-1/h)-weighted backward divergence with a
 * one-sided forward difference on the near face; (x + y) + z order. */
void FN(orc_gradf_adj)(T *du, const T *x, const T *y, const T *z, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(-1.0 / h[0]), hy = (T)(-1.0 / h[1]), hz = (T)(-1.0 / h[2]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                T a = i > 0 ? x[l] - x[l - 1] : x[l + 1] - x[l];
                T b = j > 0 ? y[l] - y[l - nx] : y[l + nx] - y[l];
                T c = k > 0 ? z[l] - z[l - nxny] : z[l + nxny] - z[l];
                du[l] = hx * a + hy * b + hz * c;
            }
}

/* gradb_adj_mex.c:159-261: forward divergence, one-sided backward on the far face. */
void FN(orc_gradb_adj)(T *du, const T *x, const T *y, const T *z, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(-1.0 / h[0]), hy = (T)(-1.0 / h[1]), hz = (T)(-1.0 / h[2]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                T a = i + 1 < nx ? x[l + 1] - x[l] : x[l] - x[l - 1];
                T b = j + 1 < ny ? y[l + nx] - y[l] : y[l] - y[l - nx];
                T c = k + 1 < nz ? z[l + nxny] - z[l] : z[l] - z[l - nxny];
                du[l] = hx * a + hy * b + hz * c;
            }
}

/* gradfm_adj_mex.c:110-162: per axis backward if the -1 neighbour is in G,
 * else forward, else 0; summed (dx + dy) + dz; written only where G. */
void FN(orc_gradfm_adj)(T *du, const T *x, const T *y, const T *z, const uint8_t *G, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(-1.0 / h[0]), hy = (T)(-1.0 / h[1]), hz = (T)(-1.0 / h[2]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (!G[l]) continue;
                T c = (k > 0 && G[l - nxny]) ? hz * (z[l] - z[l - nxny]) : (k + 1 < nz && G[l + nxny]) ? hz * (z[l + nxny] - z[l]) : (T)0;
                T b = (j > 0 && G[l - nx]) ? hy * (y[l] - y[l - nx]) : (j + 1 < ny && G[l + nx]) ? hy * (y[l + nx] - y[l]) : (T)0;
                T a = (i > 0 && G[l - 1]) ? hx * (x[l] - x[l - 1]) : (i + 1 < nx && G[l + 1]) ? hx * (x[l + 1] - x[l]) : (T)0;
                du[l] = a + b + c;
            }
}

/* gradbm_adj_mex.c:110-162: forward if the +1 neighbour is in G, else backward. */
void FN(orc_gradbm_adj)(T *du, const T *x, const T *y, const T *z, const uint8_t *G, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(-1.0 / h[0]), hy = (T)(-1.0 / h[1]), hz = (T)(-1.0 / h[2]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (!G[l]) continue;
                T a = (i + 1 < nx && G[l + 1]) ? hx * (x[l + 1] - x[l]) : (i > 0 && G[l - 1]) ? hx * (x[l] - x[l - 1]) : (T)0;
                T b = (j + 1 < ny && G[l + nx]) ? hy * (y[l + nx] - y[l]) : (j > 0 && G[l - nx]) ? hy * (y[l] - y[l - nx]) : (T)0;
                T c = (k + 1 < nz && G[l + nxny]) ? hz * (z[l + nxny] - z[l]) : (k > 0 && G[l - nxny]) ? hz * (z[l] - z[l - nxny]) : (T)0;
                du[l] = a + b + c;
            }
}

/* gradfp_mex.c:147-242: periodic forward gradient (wraps at the far face). */
void FN(orc_gradfp)(T *dx, T *dy, T *dz, const T *u, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const size_t NX = nx - 1, NY = nx * (ny - 1), NZ = nxny * (nz - 1);
    const T hx = (T)(1.0 / h[0]), hy = (T)(1.0 / h[1]), hz = (T)(1.0 / h[2]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                dx[l] = hx * ((i + 1 < nx ? u[l + 1] : u[l - NX]) - u[l]);
                dy[l] = hy * ((j + 1 < ny ? u[l + nx] : u[l - NY]) - u[l]);
                dz[l] = hz * ((k + 1 < nz ? u[l + nxny] : u[l - NZ]) - u[l]);
            }
}

/* gradfp_adj_mex.c:156-257: exact transpose of gradfp.  The reference sums
 * the three axis terms in a region-dependent order: (x + y) + z on k = 0,
 * (z + x) + y for k > 0, j = 0, and (z + y) + x for k > 0, j > 0. */
void FN(orc_gradfp_adj)(T *du, const T *x, const T *y, const T *z, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const size_t NX = nx - 1, NY = nx * (ny - 1), NZ = nxny * (nz - 1);
    const T hx = (T)(-1.0 / h[0]), hy = (T)(-1.0 / h[1]), hz = (T)(-1.0 / h[2]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                T a = hx * (x[l] - (i > 0 ? x[l - 1] : x[l + NX]));
                T b = hy * (y[l] - (j > 0 ? y[l - nx] : y[l + NY]));
                T c = hz * (z[l] - (k > 0 ? z[l - nxny] : z[l + NZ]));
                du[l] = k == 0 ? (a + b) + c : j == 0 ? (c + a) + b : (c + b) + a;
            }
}

/* lap1_mex.c:136-205 with stencils :263-315.  Per axis the stencil is chosen
 * from 2*G[+1] + G[-1] in the interior, and is forced forward on the near
 * face / backward on the far face; a one-sided stencil uses 4, 3 or 2 points
 * by the availability of the farther neighbours. */
static inline T FN(lap_axis)(const T *u, const uint8_t *G, size_t l, size_t a, size_t n, size_t i, int sel)
{
    /* i: position along the axis in units of a; n: extent in units of a */
    switch (sel) {
    case 3: return u[l - a] - (T)2 * u[l] + u[l + a];
    case 2:
        if (i + 3 < n && G[l + 2 * a] && G[l + 3 * a])
            return (T)2 * u[l] - (T)5 * u[l + a] + (T)4 * u[l + 2 * a] - u[l + 3 * a];
        if (i + 2 < n && G[l + 2 * a])
            return u[l] - (T)2 * u[l + a] + u[l + 2 * a];
        return u[l + a] - u[l];
    case 1:
        if (i >= 3 && G[l - 3 * a] && G[l - 2 * a])
            return -u[l - 3 * a] + (T)4 * u[l - 2 * a] - (T)5 * u[l - a] + (T)2 * u[l];
        if (i >= 2 && G[l - 2 * a])
            return u[l - 2 * a] - (T)2 * u[l - a] + u[l];
        return u[l - a] - u[l];
    default: return (T)0;
    }
}

static inline int FN(lap_sel)(const uint8_t *G, size_t l, size_t a, size_t i, size_t n)
{
    if (i >= 1 && i + 1 < n)
        return 2 * G[l + a] + G[l - a];
    return (i == 0) * 2 + (i + 1 == n);
}

void FN(orc_lap1)(T *du, const T *u, const uint8_t *G, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(1.0 / (h[0] * h[0])), hy = (T)(1.0 / (h[1] * h[1])), hz = (T)(1.0 / (h[2] * h[2]));
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            for (size_t i = 0; i < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (!G[l]) continue;
                T d = hx * FN(lap_axis)(u, G, l, 1, nx, i, FN(lap_sel)(G, l, 1, i, nx));
                d = d + hy * FN(lap_axis)(u, G, l, nx, ny, j, FN(lap_sel)(G, l, nx, j, ny));
                d = d + hz * FN(lap_axis)(u, G, l, nxny, nz, k, FN(lap_sel)(G, l, nxny, k, nz));
                du[l] = d;
            }
}

/* lapw_mex.c:54-187: Laplacian of a wrapped phase on the interior; each
 * one-sided difference is wrapped into [-pi, pi] only when it lies outside. */
static inline T FN(wrap_pi)(T x)
{
    const T pi = (T)3.14159265358979323846;
    const T tau = (T)(2 * 3.14159265358979323846);
    if (!(x < -pi || x > pi)) return x;
    x = x + pi;
    return x < (T)0 ? FMOD(x, tau) + pi : FMOD(x, tau) - pi;
}

void FN(orc_lapw)(T *du, const T *u, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(1.0 / (h[0] * h[0])), hy = (T)(1.0 / (h[1] * h[1])), hz = (T)(1.0 / (h[2] * h[2]));
    #pragma omp parallel for schedule(static)
    for (size_t k = 1; k < nz - 1; ++k)
        for (size_t j = 1; j + 1 < ny; ++j)
            for (size_t i = 1; i + 1 < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                T d = hx * (FN(wrap_pi)(u[l + 1] - u[l]) - FN(wrap_pi)(u[l] - u[l - 1]));
                d = d + hy * (FN(wrap_pi)(u[l + nx] - u[l]) - FN(wrap_pi)(u[l] - u[l - nx]));
                d = d + hz * (FN(wrap_pi)(u[l + nxny] - u[l]) - FN(wrap_pi)(u[l] - u[l - nxny]));
                du[l] = d;
            }
}

/* ------------------------------------------------------------------ */
/* Primal-dual TGV / TV (src/inversion/mex/pd_tgv_mex.c, pd_tv_mex.c)  */
/* ------------------------------------------------------------------ */

/* Step sizes of mx_pdd/mx_pdf (pd_tgv_mex.c:272-278, pd_tv_mex.c:255-261):
 * TV uses the same K^2 including the wave-operator norm. */
static void FN(pd_steps)(const double *h, double *tau, double *sigma)
{
    double gnrm = 4.0 * (1.0 / (h[0] * h[0]) + 1.0 / (h[1] * h[1]) + 1.0 / (h[2] * h[2]));
    double wnrm = 6.0 * (1.0 / (h[0] * h[0]) + 1.0 / (h[1] * h[1]) + 2.0 / (h[2] * h[2])) / 3.0;
    double K2 = gnrm * gnrm + wnrm * wnrm;
    *tau = 1 / sqrt(K2);
    *sigma = 1 / (*tau * K2);
}

/* pd_tgv_mex.c:332-646 (update_dual{f,d}) over voxels with mi != 0. */
static void FN(tgv_dual)(T *nu, T *p, T *q, const T *chi_, const T *eta_, const T *w_,
                         const T *f, const uint8_t *mi, double alpha0, double alpha1,
                         double sigma, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny, N = nxny * nz;
    const T hx = (T)(sigma / h[0]), hy = (T)(sigma / h[1]), hz = (T)(sigma / h[2]);
    const T hx2 = (T)(0.5 * sigma / h[0]), hy2 = (T)(0.5 * sigma / h[1]), hz2 = (T)(0.5 * sigma / h[2]);
    const T lhx = (T)(sigma / (h[0] * h[0])), lhy = (T)(sigma / (h[1] * h[1])), lhz = (T)(sigma / (h[2] * h[2]));
    const T lhh = (T)-2 * (lhx + lhy + lhz);
    const T whx = (T)(-sigma / (3.0 * h[0] * h[0])), why = (T)(-sigma / (3.0 * h[1] * h[1]));
    const T whz = (T)(sigma * 2.0 / (3.0 * h[2] * h[2]));
    const T whh = (T)-2 * (whx + why + whz);
    const T alp0 = (T)alpha0, alp1 = (T)alpha1;
    const T alp02 = (T)(alpha0 * alpha0), alp12 = (T)(alpha1 * alpha1);
    const T sg = (T)sigma;
    T *p1 = p, *p2 = p + N, *p3 = p + 2 * N;
    T *q1 = q, *q2 = q + N, *q3 = q + 2 * N, *q4 = q + 3 * N, *q5 = q + 4 * N, *q6 = q + 5 * N;
    const T *w1 = w_, *w2 = w_ + N, *w3 = w_ + 2 * N;
    #pragma omp parallel for schedule(static)
    for (size_t k = 1; k < nz - 1; ++k)
        for (size_t j = 1; j + 1 < ny; ++j)
            for (size_t i = 1; i + 1 < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (!mi[l]) continue;
                const T c0 = chi_[l];
                T lap = lhh * eta_[l] + lhx * (eta_[l - 1] + eta_[l + 1]) + lhy * (eta_[l - nx] + eta_[l + nx]) + lhz * (eta_[l - nxny] + eta_[l + nxny]);
                T wav = whh * c0 + whx * (chi_[l - 1] + chi_[l + 1]) + why * (chi_[l - nx] + chi_[l + nx]) + whz * (chi_[l - nxny] + chi_[l + nxny]);
                nu[l] = nu[l] + ((lap - wav) + f[l]);

                T a1 = p1[l] + hx * (chi_[l + 1] - c0) - sg * w1[l];
                T a2 = p2[l] + hy * (chi_[l + nx] - c0) - sg * w2[l];
                T a3 = p3[l] + hz * (chi_[l + nxny] - c0) - sg * w3[l];
                T s = a1 * a1 + a2 * a2 + a3 * a3;
                if (s > alp12) {
                    s = alp1 / SQRT(s);
                    a1 = a1 * s; a2 = a2 * s; a3 = a3 * s;
                }
                p1[l] = a1; p2[l] = a2; p3[l] = a3;

                const T v1 = w1[l], v2 = w2[l], v3 = w3[l];
                T b1 = q1[l] + hx * (w1[l + 1] - v1);
                T b2 = q2[l] + hx2 * (w2[l + 1] - v2) + hy2 * (w1[l + nx] - v1);
                T b3 = q3[l] + hx2 * (w3[l + 1] - v3) + hz2 * (w1[l + nxny] - v1);
                T b4 = q4[l] + hy * (w2[l + nx] - v2);
                T b5 = q5[l] + hy2 * (w3[l + nx] - v3) + hz2 * (w2[l + nxny] - v2);
                T b6 = q6[l] + hz * (w3[l + nxny] - v3);
                s = b1 * b1 + b4 * b4 + b6 * b6 + (T)2 * (b2 * b2 + b3 * b3 + b5 * b5);
                if (s > alp02) {
                    s = alp0 / SQRT(s);
                    b1 = b1 * s; b2 = b2 * s; b3 = b3 * s; b4 = b4 * s; b5 = b5 * s; b6 = b6 * s;
                }
                q1[l] = b1; q2[l] = b2; q3[l] = b3; q4[l] = b4; q5[l] = b5; q6[l] = b6;
            }
}

/* pd_tgv_mex.c:659-977 (update_primal{f,d}) over voxels with m != 0,
 * including the single-h w update and 1/(1+tau) of the reference. */
static void FN(tgv_primal)(T *chi, T *eta, T *w, T *chi_, T *eta_, T *w_,
                           const T *nu, const T *p, const T *q, const uint8_t *m,
                           double tau, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny, N = nxny * nz;
    const T hx = (T)(tau / h[0]), hy = (T)(tau / h[1]), hz = (T)(tau / h[2]);
    const T lhx = (T)(tau / (h[0] * h[0])), lhy = (T)(tau / (h[1] * h[1])), lhz = (T)(tau / (h[2] * h[2]));
    const T lhh = (T)-2 * (lhx + lhy + lhz);
    const T whx = (T)(-tau / (3.0 * h[0] * h[0])), why = (T)(-tau / (3.0 * h[1] * h[1]));
    const T whz = (T)(tau * 2.0 / (3.0 * h[2] * h[2]));
    const T whh = (T)-2 * (whx + why + whz);
    const T tt = (T)tau;
    const T tau1 = (T)(1.0 / (1.0 + tau));
    const T *p1 = p, *p2 = p + N, *p3 = p + 2 * N;
    const T *q1 = q, *q2 = q + N, *q3 = q + 2 * N, *q4 = q + 3 * N, *q5 = q + 4 * N, *q6 = q + 5 * N;
    T *w1 = w, *w2 = w + N, *w3 = w + 2 * N;
    T *w1_ = w_, *w2_ = w_ + N, *w3_ = w_ + 2 * N;
    #pragma omp parallel for schedule(static)
    for (size_t k = 1; k < nz - 1; ++k)
        for (size_t j = 1; j + 1 < ny; ++j)
            for (size_t i = 1; i + 1 < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (!m[l]) continue;
                const T en = eta[l], cn = chi[l], w1n = w1[l], w2n = w2[l], w3n = w3[l];
                const T x = nu[l - 1] + nu[l + 1];
                const T y = nu[l - nx] + nu[l + nx];
                const T z = nu[l - nxny] + nu[l + nxny];
                const T e1 = tau1 * (en - lhh * nu[l] - lhx * x - lhy * y - lhz * z);
                const T c1 = cn + (hx * (p1[l] - p1[l - 1]) + hy * (p2[l] - p2[l - nx]) + hz * (p3[l] - p3[l - nxny]) +
                                   (whh * nu[l] + whx * x + why * y + whz * z));
                const T u1 = w1n + (tt * p1[l] + hx * (q1[l] - q1[l - 1] + q2[l] - q2[l - nx] + q3[l] - q3[l - nxny]));
                const T u2 = w2n + (tt * p2[l] + hy * (q2[l] - q2[l - 1] + q4[l] - q4[l - nx] + q5[l] - q5[l - nxny]));
                const T u3 = w3n + (tt * p3[l] + hz * (q3[l] - q3[l - 1] + q5[l] - q5[l - nx] + q6[l] - q6[l - nxny]));
                eta[l] = e1; chi[l] = c1; w1[l] = u1; w2[l] = u2; w3[l] = u3;
                /* extragradient, THETA = 1 (pd_tgv_mex.c:13-14, :961-970) */
                eta_[l] = e1 + (T)1 * (e1 - en);
                chi_[l] = c1 + (T)1 * (c1 - cn);
                w1_[l] = u1 + (T)1 * (u1 - w1n);
                w2_[l] = u2 + (T)1 * (u2 - w2n);
                w3_[l] = u3 + (T)1 * (u3 - w3n);
            }
}

/* pd_tv_mex.c:314-513 (update_dual{f,d}). */
static void FN(tv_dual)(T *nu, T *p, const T *chi_, const T *eta_, const T *f, const uint8_t *mi,
                        double lam, double sigma, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny, N = nxny * nz;
    const T hx = (T)(sigma / h[0]), hy = (T)(sigma / h[1]), hz = (T)(sigma / h[2]);
    const T lhx = (T)(sigma / (h[0] * h[0])), lhy = (T)(sigma / (h[1] * h[1])), lhz = (T)(sigma / (h[2] * h[2]));
    const T lhh = (T)-2 * (lhx + lhy + lhz);
    const T whx = (T)(-sigma / (3.0 * h[0] * h[0])), why = (T)(-sigma / (3.0 * h[1] * h[1]));
    const T whz = (T)(sigma * 2.0 / (3.0 * h[2] * h[2]));
    const T whh = (T)-2 * (whx + why + whz);
    const T lm = (T)lam, lm2 = (T)(lam * lam);
    T *p1 = p, *p2 = p + N, *p3 = p + 2 * N;
    #pragma omp parallel for schedule(static)
    for (size_t k = 1; k < nz - 1; ++k)
        for (size_t j = 1; j + 1 < ny; ++j)
            for (size_t i = 1; i + 1 < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (!mi[l]) continue;
                const T c0 = chi_[l];
                T lap = lhh * eta_[l] + lhx * (eta_[l - 1] + eta_[l + 1]) + lhy * (eta_[l - nx] + eta_[l + nx]) + lhz * (eta_[l - nxny] + eta_[l + nxny]);
                T wav = whh * c0 + whx * (chi_[l - 1] + chi_[l + 1]) + why * (chi_[l - nx] + chi_[l + nx]) + whz * (chi_[l - nxny] + chi_[l + nxny]);
                nu[l] = nu[l] + ((lap - wav) + f[l]);
                T a1 = p1[l] + hx * (chi_[l + 1] - c0);
                T a2 = p2[l] + hy * (chi_[l + nx] - c0);
                T a3 = p3[l] + hz * (chi_[l + nxny] - c0);
                T s = a1 * a1 + a2 * a2 + a3 * a3;
                if (s > lm2) {
                    s = lm / SQRT(s);
                    a1 = a1 * s; a2 = a2 * s; a3 = a3 * s;
                }
                p1[l] = a1; p2[l] = a2; p3[l] = a3;
            }
}

/* pd_tv_mex.c:524-727 (update_primal{f,d}). */
static void FN(tv_primal)(T *chi, T *eta, T *chi_, T *eta_, const T *nu, const T *p, const uint8_t *m,
                          double tau, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny, N = nxny * nz;
    const T hx = (T)(tau / h[0]), hy = (T)(tau / h[1]), hz = (T)(tau / h[2]);
    const T lhx = (T)(tau / (h[0] * h[0])), lhy = (T)(tau / (h[1] * h[1])), lhz = (T)(tau / (h[2] * h[2]));
    const T lhh = (T)-2 * (lhx + lhy + lhz);
    const T whx = (T)(-tau / (3.0 * h[0] * h[0])), why = (T)(-tau / (3.0 * h[1] * h[1]));
    const T whz = (T)(tau * 2.0 / (3.0 * h[2] * h[2]));
    const T whh = (T)-2 * (whx + why + whz);
    const T tau1 = (T)(1.0 / (1.0 + tau));
    const T *p1 = p, *p2 = p + N, *p3 = p + 2 * N;
    #pragma omp parallel for schedule(static)
    for (size_t k = 1; k < nz - 1; ++k)
        for (size_t j = 1; j + 1 < ny; ++j)
            for (size_t i = 1; i + 1 < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (!m[l]) continue;
                const T en = eta[l], cn = chi[l];
                const T x = nu[l - 1] + nu[l + 1];
                const T y = nu[l - nx] + nu[l + nx];
                const T z = nu[l - nxny] + nu[l + nxny];
                const T e1 = tau1 * (en - lhh * nu[l] - lhx * x - lhy * y - lhz * z);
                const T c1 = cn + (hx * (p1[l] - p1[l - 1]) + hy * (p2[l] - p2[l - nx]) + hz * (p3[l] - p3[l - nxny]) +
                                   (whh * nu[l] + whx * x + why * y + whz * z));
                eta[l] = e1; chi[l] = c1;
                eta_[l] = e1 + (T)1 * (e1 - en);
                chi_[l] = c1 + (T)1 * (c1 - cn);
            }
}

/* convergence_check{d,f} (pd_tgv_mex.c:981-1045): FP64 sums of chi^2,
 * eta^2, (chi-chi0)^2, (eta-eta0)^2.  The FP32 variant squares a float
 * difference cast to double times an exact double difference (:1032-1035).
 * Sums use the lane order shared with the GPU library. */
static uint8_t FN(pd_check)(double *nr1, double *nr2, const T *chi, const T *chi0,
                            const T *eta, const T *eta0, double tol, size_t N)
{
    double s[4];
    orc_lane_sum4(s, N, (const void *)chi, (const void *)chi0, (const void *)eta, (const void *)eta0, sizeof(T) == 4);
    double n1 = sqrt(s[2] / s[0]);
    double n2 = sqrt(s[3] / s[1]);
    *nr1 = n1;
    *nr2 = n2;
    return (uint8_t)((n1 < tol) && (n2 < 2.0 * tol));
}

/* mexFunction + mx_pdd/mx_pdf of pd_tgv_mex.c:105-323.  d2f is copied (the
 * reference duplicates it, :1150), chi is returned; *iters receives the
 * number of iterations run. */
int FN(orc_pd_tgv)(T *chi_out, const T *d2f, const uint8_t *mask, const double *h,
                   double lam, double alpha, double tol, uint32_t maxiter, const size_t *sz,
                   uint32_t *iters, double *monitors)
{
    const size_t N = sz[0] * sz[1] * sz[2];
    T *buf = (T *)calloc(23 * N + 1, sizeof(T));
    uint8_t *mi = (uint8_t *)calloc(N + 1, 1);
    if (!buf || !mi) { free(buf); free(mi); return -1; }
    T *chi = buf, *eta = buf + N, *w = buf + 2 * N, *chi_ = buf + 5 * N, *eta_ = buf + 6 * N, *w_ = buf + 7 * N;
    T *nu = buf + 10 * N, *p = buf + 11 * N, *q = buf + 14 * N, *f = buf + 20 * N, *chi0 = buf + 21 * N, *eta0 = buf + 22 * N;
    orc_interior_mask(mi, mask, sz);
    double tau, sigma;
    FN(pd_steps)(h, &tau, &sigma);
    const double alpha1 = lam, alpha0 = alpha * lam;
    const T sg = (T)sigma;
    for (size_t l = 0; l < N; ++l) f[l] = sg * d2f[l];
    double nr1 = 1.0, nr2 = 1.0;
    uint32_t it = 0;
    for (uint32_t i = 0; i < maxiter; ++i) {
        const int chk = ((i + 1) % 10) == 0;
        if (chk) { memcpy(chi0, chi, N * sizeof(T)); memcpy(eta0, eta, N * sizeof(T)); }
        FN(tgv_dual)(nu, p, q, chi_, eta_, w_, f, mi, alpha0, alpha1, sigma, h, sz);
        FN(tgv_primal)(chi, eta, w, chi_, eta_, w_, nu, p, q, mask, tau, h, sz);
        it = i + 1;
        if (chk && FN(pd_check)(&nr1, &nr2, chi, chi0, eta, eta0, tol, N)) break;
    }
    memcpy(chi_out, chi, N * sizeof(T));
    if (iters) *iters = it;
    if (monitors) { monitors[0] = nr1; monitors[1] = nr2; }
    free(buf); free(mi);
    return 0;
}

/* mexFunction + mx_pdd/mx_pdf of pd_tv_mex.c:101-306. */
int FN(orc_pd_tv)(T *chi_out, const T *d2f, const uint8_t *mask, const double *h,
                  double lam, double tol, uint32_t maxiter, const size_t *sz,
                  uint32_t *iters, double *monitors)
{
    const size_t N = sz[0] * sz[1] * sz[2];
    T *buf = (T *)calloc(11 * N + 1, sizeof(T));
    uint8_t *mi = (uint8_t *)calloc(N + 1, 1);
    if (!buf || !mi) { free(buf); free(mi); return -1; }
    T *chi = buf, *eta = buf + N, *chi_ = buf + 2 * N, *eta_ = buf + 3 * N, *nu = buf + 4 * N;
    T *p = buf + 5 * N, *f = buf + 8 * N, *chi0 = buf + 9 * N, *eta0 = buf + 10 * N;
    orc_interior_mask(mi, mask, sz);
    double tau, sigma;
    FN(pd_steps)(h, &tau, &sigma);
    const T sg = (T)sigma;
    for (size_t l = 0; l < N; ++l) f[l] = sg * d2f[l];
    double nr1 = 1.0, nr2 = 1.0;
    uint32_t it = 0;
    for (uint32_t i = 0; i < maxiter; ++i) {
        const int chk = ((i + 1) % 10) == 0;
        if (chk) { memcpy(chi0, chi, N * sizeof(T)); memcpy(eta0, eta, N * sizeof(T)); }
        FN(tv_dual)(nu, p, chi_, eta_, f, mi, lam, sigma, h, sz);
        FN(tv_primal)(chi, eta, chi_, eta_, nu, p, mask, tau, h, sz);
        it = i + 1;
        if (chk && FN(pd_check)(&nr1, &nr2, chi, chi0, eta, eta0, tol, N)) break;
    }
    memcpy(chi_out, chi, N * sizeof(T));
    if (iters) *iters = it;
    if (monitors) { monitors[0] = nr1; monitors[1] = nr2; }
    free(buf); free(mi);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Multigrid pieces (src/utils/poisson_solver/mex)                      */
/* ------------------------------------------------------------------ */

/* gauss_seidel_mex.c:78-311 with GAUSS_SEIDEL_RED_BLACK.  Per sweep, two
 * colour passes over the interior; within a pass no voxel reads another of
 * the same pass, so the order inside a pass is free.  Forward: pass 0 =
 * (i+j+k) even, pass 1 = (i+j+k) odd except i = 1.  Reverse: pass 0 =
 * (i+j+k) = nx+1 (mod 2), pass 1 = (i+j+k) = nx (mod 2) except i = nx-2. */
void FN(orc_gauss_seidel)(T *v, const T *f, const uint8_t *G, const double *h, const size_t *sz,
                          int32_t iter, int rev)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(1.0 / (h[0] * h[0])), hy = (T)(1.0 / (h[1] * h[1])), hz = (T)(1.0 / (h[2] * h[2]));
    const T hh = (T)(1.0 / (2.0 * (double)(hx + hy + hz)));
    if (nx < 3 || ny < 3 || nz < 3) return;
    const size_t par0 = rev ? (nx + 1) & 1 : 0;
    const size_t skip_i = rev ? nx - 2 : 1;
    while (iter-- > 0) {
        for (int s = 0; s < 2; ++s) {
            const size_t par = s == 0 ? par0 : par0 ^ 1;
            #pragma omp parallel for schedule(static)
            for (size_t k = 1; k < nz - 1; ++k)
                for (size_t j = 1; j < ny - 1; ++j) {
                    size_t i0 = 1 + ((1 + j + k + par) & 1);
                    for (size_t i = i0; i < nx - 1; i += 2) {
                        if (s == 1 && i == skip_i) continue;
                        size_t l = i + nx * j + nxny * k;
                        if (!G[l]) continue;
                        v[l] = hh * (f[l] + (hx * (v[l - 1] + v[l + 1]) + hy * (v[l - nx] + v[l + nx]) + hz * (v[l - nxny] + v[l + nxny])));
                    }
                }
        }
    }
}

/* residual_mex.c:82-165: r = f + Delta_h x on the interior of G. */
void FN(orc_residual)(T *r, const T *f, const T *x, const uint8_t *G, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(1.0 / (h[0] * h[0])), hy = (T)(1.0 / (h[1] * h[1])), hz = (T)(1.0 / (h[2] * h[2]));
    const T hh = (T)(-2.0 * (hx + hy + hz));
    #pragma omp parallel for schedule(static)
    for (size_t k = 1; k < nz - 1; ++k)
        for (size_t j = 1; j + 1 < ny; ++j)
            for (size_t i = 1; i + 1 < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (!G[l]) continue;
                r[l] = f[l] + (hh * x[l] + hx * (x[l - 1] + x[l + 1]) + hy * (x[l - nx] + x[l + nx]) + hz * (x[l - nxny] + x[l + nxny]));
            }
}

/* lapmg_mex.c:73-154: du = Delta_h u on the interior of G. */
void FN(orc_lapmg)(T *du, const T *u, const uint8_t *G, const double *h, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxny = nx * ny;
    const T hx = (T)(1.0 / (h[0] * h[0])), hy = (T)(1.0 / (h[1] * h[1])), hz = (T)(1.0 / (h[2] * h[2]));
    const T hh = (T)(-2.0 * (hx + hy + hz));
    #pragma omp parallel for schedule(static)
    for (size_t k = 1; k < nz - 1; ++k)
        for (size_t j = 1; j + 1 < ny; ++j)
            for (size_t i = 1; i + 1 < nx; ++i) {
                size_t l = i + nx * j + nxny * k;
                if (!G[l]) continue;
                du[l] = hh * u[l] + hx * (u[l - 1] + u[l + 1]) + hy * (u[l - nx] + u[l + nx]) + hz * (u[l - nxny] + u[l + nxny]);
            }
}

/* restrict_mex.c:72-332: 27-point full weighting onto the coarse interior,
 * coarse (i2,j2,k2) centred on fine (2i2-1, 2j2-1, 2k2-1).  The corner,
 * edge and face groups are summed in the reference's fixed order
 * (:292-326) and combined as ((c*A + e*B) + f*C) + x/8; zero where !G2. */
void FN(orc_restrict)(T *x2, const T *x, const uint8_t *G2, const size_t *sz2, const size_t *sz)
{
    const size_t nx = sz[0], nxny = sz[0] * sz[1];
    const size_t nx2 = sz2[0], ny2 = sz2[1], nz2 = sz2[2], nxny2 = nx2 * ny2;
    #pragma omp parallel for schedule(static)
    for (size_t k2 = 1; k2 < nz2 - 1; ++k2)
        for (size_t j2 = 1; j2 + 1 < ny2; ++j2)
            for (size_t i2 = 1; i2 + 1 < nx2; ++i2) {
                size_t l2 = i2 + nx2 * j2 + nxny2 * k2;
                size_t l = (2 * i2 - 1) + nx * (2 * j2 - 1) + nxny * (2 * k2 - 1);
                if (!G2[l2]) { x2[l2] = (T)0; continue; }
#define X(a, b, c) x[l + (a) + (b) * nx + (c) * nxny]
                T A = X(-1, -1, -1) + X(1, -1, -1) + X(-1, 1, -1) + X(1, 1, -1) + X(-1, -1, 1) + X(1, -1, 1) + X(-1, 1, 1) + X(1, 1, 1);
                T B = X(0, -1, -1) + X(-1, 0, -1) + X(1, 0, -1) + X(0, 1, -1) + X(1, -1, 0) + X(-1, -1, 0) + X(-1, 1, 0) +
                      X(1, 1, 0) + X(0, -1, 1) + X(-1, 0, 1) + X(1, 0, 1) + X(0, 1, 1);
                T C = X(0, 0, -1) + X(0, -1, 0) + X(-1, 0, 0) + X(1, 0, 0) + X(0, 1, 0) + X(0, 0, 1);
#undef X
                x2[l2] = (T)0.015625 * A + (T)0.03125 * B + (T)0.0625 * C + (T)0.125 * x[l];
            }
}

/* prolong_mex.c / correct_mex.c:73-304: trilinear interpolation of the
 * coarse interior onto fine voxels (2i2-1 + a, 2j2-1 + b, 2k2-1 + c), a,b,c
 * in {0,1}; the neighbour sums keep the reference's order.  add = 0
 * overwrites (prolong), add = 1 adds (correct); either way the value is
 * 0 where !G. */
void FN(orc_prolong_correct)(T *x, const T *x2, const uint8_t *G, const size_t *sz, const size_t *sz2, int add)
{
    const size_t nx = sz[0], nxny = sz[0] * sz[1];
    const size_t nx2 = sz2[0], ny2 = sz2[1], nz2 = sz2[2], nxny2 = nx2 * ny2;
    #pragma omp parallel for schedule(static)
    for (size_t k2 = 1; k2 < nz2 - 1; ++k2)
        for (size_t j2 = 1; j2 + 1 < ny2; ++j2)
            for (size_t i2 = 1; i2 + 1 < nx2; ++i2) {
                size_t l2 = i2 + nx2 * j2 + nxny2 * k2;
                size_t l = (2 * i2 - 1) + nx * (2 * j2 - 1) + nxny * (2 * k2 - 1);
                for (int c = 0; c < 2; ++c)
                    for (int b = 0; b < 2; ++b)
                        for (int a = 0; a < 2; ++a) {
                            size_t lf = l + a + nx * b + nxny * c;
                            T val = (T)0;
                            if (G[lf]) {
                                const T c0 = x2[l2];
                                const size_t ox = 1, oy = nx2, oz = nxny2;
                                switch (a + 2 * b + 4 * c) {
                                case 0: val = c0; break;
                                case 1: val = (T)0.5 * (c0 + x2[l2 + ox]); break;
                                case 2: val = (T)0.5 * (c0 + x2[l2 + oy]); break;
                                case 4: val = (T)0.5 * (c0 + x2[l2 + oz]); break;
                                case 3: val = (T)0.25 * (c0 + x2[l2 + ox] + x2[l2 + oy] + x2[l2 + ox + oy]); break;
                                case 5: val = (T)0.25 * (c0 + x2[l2 + ox] + x2[l2 + oz] + x2[l2 + ox + oz]); break;
                                case 6: val = (T)0.25 * (c0 + x2[l2 + oy] + x2[l2 + oz] + x2[l2 + oy + oz]); break;
                                default:
                                    val = (T)0.125 * (c0 + x2[l2 + ox] + x2[l2 + oy] + x2[l2 + oz] + x2[l2 + ox + oy] +
                                                      x2[l2 + ox + oz] + x2[l2 + oy + oz] + x2[l2 + ox + oy + oz]);
                                }
                            }
                            x[lf] = add ? x[lf] + val : val;
                        }
            }
}

/* pairwise masked squared norm, norm2_mex.c:83-131 (blocks of <= 128). */
static T FN(norm22)(const T *x, const uint8_t *G, size_t n)
{
    if (n <= 128) {
        T s = G[0] ? x[0] * x[0] : (T)0;
        for (size_t i = 1; i < n; ++i)
            if (G[i]) s += x[i] * x[i];
        return s;
    }
    size_t m = n >> 1;
    return FN(norm22)(x, G, m) + FN(norm22)(x + m, G + m, n - m);
}

T FN(orc_norm2)(const T *x, const uint8_t *G, size_t n)
{
    return SQRT(FN(norm22)(x, G, n));
}

/* pad / unpad by one voxel (mx_util.c:8-133). */
void FN(orc_pad)(T *xp, const T *x, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxp = nx + 2, nxnyp = (nx + 2) * (ny + 2);
    memset(xp, 0, (nx + 2) * (ny + 2) * (nz + 2) * sizeof(T));
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            memcpy(xp + 1 + nxp * (j + 1) + nxnyp * (k + 1), x + nx * j + nx * ny * k, nx * sizeof(T));
}

void FN(orc_unpad)(T *x, const T *xp, const size_t *sz)
{
    const size_t nx = sz[0], ny = sz[1], nz = sz[2], nxp = nx + 2, nxnyp = (nx + 2) * (ny + 2);
    for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
            memcpy(x + nx * j + nx * ny * k, xp + 1 + nxp * (j + 1) + nxnyp * (k + 1), nx * sizeof(T));
}

/* ---- multigrid hierarchy and drivers (mgpcg_mex.c, mg_mex.c, fmg_mex.c) ---- */

typedef struct {
    size_t sz[3], n;
    T *v, *f, *r;
    uint8_t *G, *B;
    double h[3];
} FN(Level);

static double FN(nrm2)(const T *x, size_t n)
{
    return orc_lane_nrm2(x, n, sizeof(T) == 4);
}

/* mx_init (mgpcg_mex.c:282-332; fmg_mex.c:162-212 also restricts f down). */
static int FN(mg_init)(FN(Level) *L, int nl, const T *v0, const T *f, const uint8_t *mask,
                       const double *h, const size_t *sz, int fmg)
{
    memset(L, 0, sizeof(FN(Level)) * (size_t)nl);
    for (int i = 0; i < nl; ++i) {
        if (i == 0) {
            L[0].sz[0] = sz[0] + 2; L[0].sz[1] = sz[1] + 2; L[0].sz[2] = sz[2] + 2;
            memcpy(L[0].h, h, sizeof(L[0].h));
        } else {
            for (int d = 0; d < 3; ++d) {
                L[i].sz[d] = ((L[i - 1].sz[d] - 2 + 1) >> 1) + 2;
                L[i].h[d] = L[i - 1].h[d] * 2.0;
            }
        }
        L[i].n = L[i].sz[0] * L[i].sz[1] * L[i].sz[2];
        L[i].v = (T *)calloc(L[i].n, sizeof(T));
        L[i].f = (T *)calloc(L[i].n, sizeof(T));
        L[i].r = (T *)calloc(L[i].n, sizeof(T));
        L[i].G = (uint8_t *)calloc(L[i].n, 1);
        L[i].B = (uint8_t *)calloc(L[i].n, 1);
        if (!L[i].v || !L[i].f || !L[i].r || !L[i].G || !L[i].B) return -1;
        if (i == 0) {
            if (v0) FN(orc_pad)(L[0].v, v0, sz);
            FN(orc_pad)(L[0].f, f, sz);
            orc_pad_u8(L[0].G, mask, sz);
        } else {
            orc_coarsen_grid(L[i].G, L[i - 1].G, L[i].sz, L[i - 1].sz);
            if (fmg) FN(orc_restrict)(L[i].f, L[i - 1].f, L[i].G, L[i].sz, L[i - 1].sz);
        }
        orc_boundary_mask(L[i].B, L[i].G, L[i].sz);
    }
    return 0;
}

static void FN(mg_free)(FN(Level) *L, int nl)
{
    for (int i = 0; i < nl; ++i) {
        free(L[i].v); free(L[i].f); free(L[i].r); free(L[i].G); free(L[i].B);
    }
}

/* mx_cycle (mgpcg_mex.c:242-279, identical in mg_mex.c / fmg_mex.c). */
static void FN(mg_cycle)(FN(Level) *L, int l, int nl, int mu, int pre, int post, int nb)
{
    if (l < nl - 1) {
        const int32_t bs = (1 << l) * nb;
        FN(orc_gauss_seidel)(L[l].v, L[l].f, L[l].G, L[l].h, L[l].sz, pre, 1);
        FN(orc_gauss_seidel)(L[l].v, L[l].f, L[l].B, L[l].h, L[l].sz, bs, 1);
        FN(orc_residual)(L[l].r, L[l].f, L[l].v, L[l].G, L[l].h, L[l].sz);
        FN(orc_restrict)(L[l + 1].f, L[l].r, L[l + 1].G, L[l + 1].sz, L[l].sz);
        memset(L[l + 1].v, 0, L[l + 1].n * sizeof(T));
        for (int i = 0; i < mu; ++i) {
            FN(mg_cycle)(L, l + 1, nl, mu, pre, post, nb);
            if (l + 1 == nl - 1) break;
        }
        FN(orc_prolong_correct)(L[l].v, L[l + 1].v, L[l].G, L[l].sz, L[l + 1].sz, 1);
        FN(orc_gauss_seidel)(L[l].v, L[l].f, L[l].B, L[l].h, L[l].sz, bs, 0);
        FN(orc_gauss_seidel)(L[l].v, L[l].f, L[l].G, L[l].h, L[l].sz, post, 0);
    } else {
        const double tol = sizeof(T) == 4 ? 1e-4 : 1e-8;
        const double reltol = tol * FN(nrm2)(L[l].f, L[l].n);
        for (int i = 0; i < 1024; ++i) {
            FN(orc_gauss_seidel)(L[l].v, L[l].f, L[l].G, L[l].h, L[l].sz, 128, 1);
            FN(orc_gauss_seidel)(L[l].v, L[l].f, L[l].G, L[l].h, L[l].sz, 128, 0);
            FN(orc_residual)(L[l].r, L[l].f, L[l].v, L[l].G, L[l].h, L[l].sz);
            if (FN(nrm2)(L[l].r, L[l].n) < reltol) break;
        }
    }
}

/* mx_mg (mgpcg_mex.c:219-239, mg_mex.c:94-114). */
static void FN(mg_run)(FN(Level) *L, int nl, double tol, int maxit, int mu, int pre, int post, int nb)
{
    if (tol > 0.0) {
        const double reltol = tol * FN(nrm2)(L[0].f, L[0].n);
        for (int i = 0; i < maxit; ++i) {
            FN(orc_residual)(L[0].r, L[0].f, L[0].v, L[0].G, L[0].h, L[0].sz);
            if (FN(nrm2)(L[0].r, L[0].n) < reltol) break;
            FN(mg_cycle)(L, 0, nl, mu, pre, post, nb);
        }
    } else {
        for (int i = 0; i < maxit; ++i) FN(mg_cycle)(L, 0, nl, mu, pre, post, nb);
    }
}

/* mexFunction + mx_pcg of mgpcg_mex.c:73-216.  resnorm (length maxitcg,
 * may be NULL) receives the residual history the reference allocates but
 * never returns. */
int FN(orc_mgpcg)(T *v_out, const T *v0, const T *f, const uint8_t *mask, const double *h, const size_t *sz,
                  double tolcg, int32_t maxitcg, double tolmg, int32_t maxitmg, int32_t mu,
                  int32_t npre, int32_t npost, int32_t nb, int32_t nl, int32_t *iters, double *resnorm)
{
    if (nl > 16 || nl < 1) return -2;
    FN(Level) L[16];
    if (FN(mg_init)(L, nl, v0, f, mask, h, sz, 0)) { FN(mg_free)(L, nl); return -1; }
    const size_t n = L[0].n;
    T *x = (T *)malloc(n * sizeof(T));
    T *pp = (T *)calloc(n, sizeof(T));
    memcpy(x, L[0].v, n * sizeof(T));
    T *r = L[0].f, *q = L[0].v;
    double rho = 1.0, prevrho, res = FN(nrm2)(r, n);
    const double reltol = tolcg * res;
    memset(q, 0, n * sizeof(T));
    FN(orc_lapmg)(q, x, L[0].G, L[0].h, L[0].sz);
    orc_scal(q, -1.0, n, sizeof(T) == 4);
    orc_axpy(r, -1.0, q, n, sizeof(T) == 4);
    res = FN(nrm2)(r, n);
    int32_t it = 0;
    for (int32_t i = 0; i < maxitcg; ++i) {
        if (res <= reltol) break;
        prevrho = rho;
        memset(q, 0, n * sizeof(T));
        FN(mg_run)(L, nl, tolmg, maxitmg, mu, npre, npost, nb);
        rho = orc_lane_dot(r, q, n, sizeof(T) == 4);
        double beta = rho / prevrho;
        orc_scal(pp, beta, n, sizeof(T) == 4);
        orc_axpy(pp, 1.0, q, n, sizeof(T) == 4);
        FN(orc_lapmg)(q, pp, L[0].G, L[0].h, L[0].sz);
        orc_scal(q, -1.0, n, sizeof(T) == 4);
        double a = rho / orc_lane_dot(pp, q, n, sizeof(T) == 4);
        orc_axpy(x, a, pp, n, sizeof(T) == 4);
        orc_axpy(r, -a, q, n, sizeof(T) == 4);
        res = FN(nrm2)(r, n);
        if (resnorm) resnorm[i] = res;
        it += 1;
    }
    FN(orc_unpad)(v_out, x, sz);
    if (iters) *iters = it;
    free(x); free(pp);
    FN(mg_free)(L, nl);
    return 0;
}

/* mexFunction of mg_mex.c:55-91. */
int FN(orc_mg)(T *v_out, const T *v0, const T *f, const uint8_t *mask, const double *h, const size_t *sz,
               double tol, int32_t maxit, int32_t mu, int32_t npre, int32_t npost, int32_t nb, int32_t nl)
{
    if (nl > 16 || nl < 1) return -2;
    FN(Level) L[16];
    if (FN(mg_init)(L, nl, v0, f, mask, h, sz, 0)) { FN(mg_free)(L, nl); return -1; }
    FN(mg_run)(L, nl, tol, maxit, mu, npre, npost, nb);
    FN(orc_unpad)(v_out, L[0].v, sz);
    FN(mg_free)(L, nl);
    return 0;
}

/* mx_fmg of fmg_mex.c:93-119. */
static void FN(fmg_run)(FN(Level) *L, int l, int nl, double tol, int maxit, int mu, int pre, int post, int nb)
{
    if (l < nl - 1) {
        FN(fmg_run)(L, l + 1, nl, tol, maxit, mu, pre, post, nb);
        FN(orc_prolong_correct)(L[l].v, L[l + 1].v, L[l].G, L[l].sz, L[l + 1].sz, 0);
    }
    if (l == 0 && tol > 0.0) {
        const double reltol = tol * FN(nrm2)(L[0].f, L[0].n);
        for (int i = 0; i < 1000 * maxit; ++i) {
            FN(orc_residual)(L[0].r, L[0].f, L[0].v, L[0].G, L[0].h, L[0].sz);
            if (FN(nrm2)(L[0].r, L[0].n) < reltol) break;
            FN(mg_cycle)(L, l, nl, mu, pre, post, nb);
        }
    } else {
        for (int i = 0; i < maxit; ++i) FN(mg_cycle)(L, l, nl, mu, pre, post, nb);
    }
}

/* mexFunction of fmg_mex.c:54-90. */
int FN(orc_fmg)(T *v_out, const T *f, const uint8_t *mask, const double *h, const size_t *sz,
                double tol, int32_t maxit, int32_t mu, int32_t npre, int32_t npost, int32_t nb, int32_t nl)
{
    if (nl > 16 || nl < 1) return -2;
    FN(Level) L[16];
    if (FN(mg_init)(L, nl, NULL, f, mask, h, sz, 1)) { FN(mg_free)(L, nl); return -1; }
    FN(fmg_run)(L, 0, nl, tol, maxit, mu, npre, npost, nb);
    FN(orc_unpad)(v_out, L[0].v, sz);
    FN(mg_free)(L, nl);
    return 0;
}

#undef FN
#undef CAT
#undef CAT_
