/*
 * Thin C-MEX shims over the GB300 library: one MEX gateway per QSM.m hot-path
 * gateway, with the same name, usage string, argument order and in-place
 * semantics, forwarding mxGetData() pointers to the C ABI (include/qsm_gpu.h).
 * Host arrays are copied to the GPU and back inside each call.
 *
 * Build one gateway per define, e.g. from MATLAB:
 *   mex -DQSM_MEX_PD_TGV -I<repo>/include qsm_mex.c -L<repo>/qsm.m_gb300 -lqsm_gb300 -output pd_tgv_mex
 * Gateways: QSM_MEX_PD_TGV, QSM_MEX_PD_TV, QSM_MEX_GRADF, QSM_MEX_GRADB, QSM_MEX_GRADC,
 * QSM_MEX_GRADFM, QSM_MEX_GRADBM, QSM_MEX_GRADCM, QSM_MEX_GRADF_ADJ, QSM_MEX_GRADB_ADJ,
 * QSM_MEX_GRADFM_ADJ, QSM_MEX_GRADBM_ADJ, QSM_MEX_GRADFP, QSM_MEX_GRADFP_ADJ,
 * QSM_MEX_LAP1, QSM_MEX_LAPW, QSM_MEX_MGPCG, QSM_MEX_MG, QSM_MEX_FMG, and the multigrid
 * pieces QSM_MEX_GAUSS_SEIDEL, QSM_MEX_RESIDUAL, QSM_MEX_LAPMG, QSM_MEX_RESTRICT,
 * QSM_MEX_PROLONG, QSM_MEX_CORRECT, QSM_MEX_COARSEN_GRID, QSM_MEX_BOUNDARY_MASK,
 * QSM_MEX_BOUNDARY_MASK_L1, QSM_MEX_NORM2 (output names: the lower-case gateway + "_mex").
 *
 * Whole MATLAB functions (same name, arguments, defaults and outputs; placed ahead
 * of the .m files on the path they take over the call):
 *   -DQSM_MEX_SSTGV -output sstgv, QSM_MEX_LBV (lbv), QSM_MEX_UNWRAP_LAPLACIAN
 *   (unwrapLaplacian), QSM_MEX_SHARP (sharp), QSM_MEX_VSHARP (vsharp), QSM_MEX_RESHARP
 *   (resharp), QSM_MEX_ISMV (ismv), QSM_MEX_PDF (pdf).
 * Arrays may be 4-D (echoes last); masks may be logical, uint8, single or double
 * (non-zero is inside).  lbv's mgopts is [] or the vector [maxit npre npost nboundary]
 * in place of the struct.
 */
#include <stdint.h>
#include "mex.h"
#include "qsm_gpu.h"

static qsm_ctx *g_ctx = NULL;

static inline void ctx_release(void)
{
    if (g_ctx) qsm_ctx_destroy(g_ctx);
    g_ctx = NULL;
}

static inline qsm_ctx *ctx_get(void)
{
    if (!g_ctx) {
        if (qsm_ctx_create(0, &g_ctx) != QSM_OK) mexErrMsgTxt("qsm: no usable CUDA device");
        mexAtExit(ctx_release);
    }
    return g_ctx;
}

static inline void check(qsm_status st)
{
    if (st != QSM_OK) mexErrMsgTxt(qsm_last_error(g_ctx));
}

static inline qsm_dtype dtype_of(const mxArray *a) { return mxIsSingle(a) ? QSM_F32 : QSM_F64; }

static inline void dims_of(const mxArray *a, size_t d[3])
{
    const mwSize nd = mxGetNumberOfDimensions(a);
    const mwSize *s = mxGetDimensions(a);
    d[0] = s[0];
    d[1] = nd > 1 ? s[1] : 1;
    d[2] = nd > 2 ? s[2] : 1;
}

/* for the whole-function gateways: optional arguments, 4-D sizes, masks */
static inline int given(int nrhs, const mxArray *prhs[], int i)
{
    return i < nrhs && mxGetNumberOfElements(prhs[i]) > 0;
}

static inline double elem(const mxArray *a, size_t i)
{
    switch (mxGetClassID(a)) {
    case mxDOUBLE_CLASS: return ((const double *)mxGetData(a))[i];
    case mxSINGLE_CLASS: return ((const float *)mxGetData(a))[i];
    case mxLOGICAL_CLASS:
    case mxUINT8_CLASS: return ((const uint8_t *)mxGetData(a))[i];
    default: mexErrMsgTxt("qsm: numeric argument expected"); return 0.0;
    }
}

static inline double opt(int nrhs, const mxArray *prhs[], int i, double def)
{
    return given(nrhs, prhs, i) ? elem(prhs[i], 0) : def;
}

static inline void dims4_of(const mxArray *a, size_t d[4])
{
    const mwSize nd = mxGetNumberOfDimensions(a);
    const mwSize *s = mxGetDimensions(a);
    d[0] = s[0];
    d[1] = nd > 1 ? s[1] : 1;
    d[2] = nd > 2 ? s[2] : 1;
    d[3] = 1;
    for (mwSize k = 3; k < nd; ++k) d[3] *= s[k];
}

/* vsz (or bdir): a scalar is repeated, else three entries */
static inline void vec3_of(const mxArray *a, double v[3])
{
    const size_t n = mxGetNumberOfElements(a);
    if (n != 1 && n != 3) mexErrMsgTxt("qsm: vsz and bdir need 1 or 3 entries");
    for (int k = 0; k < 3; ++k) v[k] = elem(a, n == 1 ? 0 : (size_t)k);
}

/* uint8 0/1 view of a mask; a converted copy goes to *tmp (destroy it after the call) */
static inline const uint8_t *mask_of(const mxArray *a, mxArray **tmp)
{
    *tmp = NULL;
    if (mxGetClassID(a) == mxLOGICAL_CLASS || mxGetClassID(a) == mxUINT8_CLASS)
        return (const uint8_t *)mxGetData(a);
    *tmp = mxCreateNumericArray(mxGetNumberOfDimensions(a), mxGetDimensions(a), mxUINT8_CLASS, mxREAL);
    uint8_t *m = (uint8_t *)mxGetData(*tmp);
    const size_t n = mxGetNumberOfElements(a);
    for (size_t i = 0; i < n; ++i) m[i] = elem(a, i) != 0.0;
    return m;
}

/* an output with the size and class of a */
static inline mxArray *like(const mxArray *a)
{
    return mxCreateNumericArray(mxGetNumberOfDimensions(a), mxGetDimensions(a), mxGetClassID(a), mxREAL);
}

/* a logical output with the size of the mask a */
static inline mxArray *mask_like(const mxArray *a)
{
    return mxCreateLogicalArray(mxGetNumberOfDimensions(a), mxGetDimensions(a));
}

static inline void ret_one(int nlhs, mxArray *plhs[])
{
    if (nlhs == 1) plhs[0] = mxCreateDoubleScalar(1.0);
}

#if defined(QSM_MEX_PD_TGV) || defined(QSM_MEX_PD_TV)
/* chi = pd_tgv_mex(d2f, mask, vsz, lam, alpha, tol, maxiter, verbose)  (pd_tgv_mex.c:104-135)
 * chi = pd_tv_mex(d2f, mask, vsz, lam, tol, maxiter, verbose)          (pd_tv_mex.c:100-130) */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
#ifdef QSM_MEX_PD_TGV
    if ((nrhs != 8) || (nlhs > 1))
        mexErrMsgTxt("Usage: chi = pd_tgv_mex(d2f, mask, vsz, lam, alpha, tol, maxiter, verbose);");
    const int o = 0;
#else
    if ((nrhs != 7) || (nlhs > 1))
        mexErrMsgTxt("Usage: chi = pd_tv_mex(d2f, mask, vsz, lam, tol, maxiter, verbose);");
    const int o = -1;
#endif
    size_t d[3];
    dims_of(prhs[0], d);
    plhs[0] = mxCreateNumericArray(mxGetNumberOfDimensions(prhs[0]), mxGetDimensions(prhs[0]),
                                   mxGetClassID(prhs[0]), mxREAL);
    qsm_ctx *ctx = ctx_get();
    const double *h = (const double *)mxGetData(prhs[2]);
    const double lam = mxGetScalar(prhs[3]);
    const double tol = mxGetScalar(prhs[5 + o]);
    const uint32_t maxiter = (uint32_t)mxGetScalar(prhs[6 + o]);
    const uint32_t verbose = (uint32_t)mxGetScalar(prhs[7 + o]);
#ifdef QSM_MEX_PD_TGV
    check(qsm_pd_tgv(ctx, dtype_of(prhs[0]), d, mxGetData(prhs[0]), (const uint8_t *)mxGetData(prhs[1]), h, lam,
                     mxGetScalar(prhs[4]), tol, maxiter, verbose, mxGetData(plhs[0]), NULL));
#else
    check(qsm_pd_tv(ctx, dtype_of(prhs[0]), d, mxGetData(prhs[0]), (const uint8_t *)mxGetData(prhs[1]), h, lam,
                    tol, maxiter, verbose, mxGetData(plhs[0]), NULL));
#endif
}

#elif defined(QSM_MEX_GRADF) || defined(QSM_MEX_GRADB) || defined(QSM_MEX_GRADC) || defined(QSM_MEX_GRADFP)
/* grad{f,b,c}_mex(dx, dy, dz, u, h), gradfp_mex(dx, dy, dz, u, h): written in place */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 5) || (nlhs > 1)) {
#if defined(QSM_MEX_GRADF)
        mexErrMsgTxt("Usage: gradf_mex(dx, dy, dz, u, h);");
#elif defined(QSM_MEX_GRADB)
        mexErrMsgTxt("Usage: gradb_mex(dx, dy, dz, u, h);");
#elif defined(QSM_MEX_GRADC)
        mexErrMsgTxt("Usage: gradc_mex(dx, dy, dz, u, h);");
#else
        mexErrMsgTxt("Usage: gradfp_mex(dx, dy, dz, u, h);");
#endif
    }
    size_t d[3];
    dims_of(prhs[0], d);
    qsm_ctx *ctx = ctx_get();
    void *dx = mxGetData(prhs[0]), *dy = mxGetData(prhs[1]), *dz = mxGetData(prhs[2]);
    const void *u = mxGetData(prhs[3]);
    const double *h = (const double *)mxGetData(prhs[4]);
#if defined(QSM_MEX_GRADF)
    check(qsm_gradf(ctx, dtype_of(prhs[0]), d, dx, dy, dz, u, h));
#elif defined(QSM_MEX_GRADB)
    check(qsm_gradb(ctx, dtype_of(prhs[0]), d, dx, dy, dz, u, h));
#elif defined(QSM_MEX_GRADC)
    check(qsm_gradc(ctx, dtype_of(prhs[0]), d, dx, dy, dz, u, h));
#else
    check(qsm_gradfp(ctx, dtype_of(prhs[0]), d, dx, dy, dz, u, h));
#endif
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_GRADFM) || defined(QSM_MEX_GRADBM) || defined(QSM_MEX_GRADCM)
/* grad{f,b,c}m_mex(dx, dy, dz, u, G, h): written in place where G */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 6) || (nlhs > 1)) {
#if defined(QSM_MEX_GRADFM)
        mexErrMsgTxt("Usage: gradfm_mex(dx, dy, dz, u, G, h);");
#elif defined(QSM_MEX_GRADBM)
        mexErrMsgTxt("Usage: gradbm_mex(dx, dy, dz, u, G, h);");
#else
        mexErrMsgTxt("Usage: gradcm_mex(dx, dy, dz, u, G, h);");
#endif
    }
    size_t d[3];
    dims_of(prhs[0], d);
    qsm_ctx *ctx = ctx_get();
    void *dx = mxGetData(prhs[0]), *dy = mxGetData(prhs[1]), *dz = mxGetData(prhs[2]);
    const void *u = mxGetData(prhs[3]);
    const uint8_t *G = (const uint8_t *)mxGetData(prhs[4]);
    const double *h = (const double *)mxGetData(prhs[5]);
#if defined(QSM_MEX_GRADFM)
    check(qsm_gradfm(ctx, dtype_of(prhs[0]), d, dx, dy, dz, u, G, h));
#elif defined(QSM_MEX_GRADBM)
    check(qsm_gradbm(ctx, dtype_of(prhs[0]), d, dx, dy, dz, u, G, h));
#else
    check(qsm_gradcm(ctx, dtype_of(prhs[0]), d, dx, dy, dz, u, G, h));
#endif
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_GRADF_ADJ) || defined(QSM_MEX_GRADB_ADJ) || defined(QSM_MEX_GRADFP_ADJ)
/* grad{f,b}_adj_mex(du, x, y, z, h), gradfp_adj_mex(du, x, y, z, h): written in place */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 5) || (nlhs > 1)) {
#if defined(QSM_MEX_GRADF_ADJ)
        mexErrMsgTxt("Usage: gradf_adj_mex(du, x, y, z, h);");
#elif defined(QSM_MEX_GRADB_ADJ)
        mexErrMsgTxt("Usage: gradb_adj_mex(du, x, y, z, h);");
#else
        mexErrMsgTxt("Usage: gradfp_adj_mex(du, x, y, z, h);");
#endif
    }
    size_t d[3];
    dims_of(prhs[0], d);
    qsm_ctx *ctx = ctx_get();
    void *du = mxGetData(prhs[0]);
    const void *x = mxGetData(prhs[1]), *y = mxGetData(prhs[2]), *z = mxGetData(prhs[3]);
    const double *h = (const double *)mxGetData(prhs[4]);
#if defined(QSM_MEX_GRADF_ADJ)
    check(qsm_gradf_adj(ctx, dtype_of(prhs[0]), d, du, x, y, z, h));
#elif defined(QSM_MEX_GRADB_ADJ)
    check(qsm_gradb_adj(ctx, dtype_of(prhs[0]), d, du, x, y, z, h));
#else
    check(qsm_gradfp_adj(ctx, dtype_of(prhs[0]), d, du, x, y, z, h));
#endif
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_GRADFM_ADJ) || defined(QSM_MEX_GRADBM_ADJ)
/* grad{f,b}m_adj_mex(du, x, y, z, G, h): written in place where G */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 6) || (nlhs > 1)) {
#if defined(QSM_MEX_GRADFM_ADJ)
        mexErrMsgTxt("Usage: gradfm_adj_mex(du, x, y, z, G, h);");
#else
        mexErrMsgTxt("Usage: gradbm_adj_mex(du, x, y, z, G, h);");
#endif
    }
    size_t d[3];
    dims_of(prhs[0], d);
    qsm_ctx *ctx = ctx_get();
    void *du = mxGetData(prhs[0]);
    const void *x = mxGetData(prhs[1]), *y = mxGetData(prhs[2]), *z = mxGetData(prhs[3]);
    const uint8_t *G = (const uint8_t *)mxGetData(prhs[4]);
    const double *h = (const double *)mxGetData(prhs[5]);
#if defined(QSM_MEX_GRADFM_ADJ)
    check(qsm_gradfm_adj(ctx, dtype_of(prhs[0]), d, du, x, y, z, G, h));
#else
    check(qsm_gradbm_adj(ctx, dtype_of(prhs[0]), d, du, x, y, z, G, h));
#endif
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_LAP1)
/* lap1_mex(d2u, u, G, h) (usage string "lap_mex", lap1_mex.c:33) */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 4) || (nlhs > 1)) mexErrMsgTxt("Usage: lap_mex(d2u, u, G, h);");
    size_t d[3];
    dims_of(prhs[0], d);
    check(qsm_lap1(ctx_get(), dtype_of(prhs[0]), d, mxGetData(prhs[0]), mxGetData(prhs[1]),
                   (const uint8_t *)mxGetData(prhs[2]), (const double *)mxGetData(prhs[3])));
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_LAPW)
/* lapw_mex(d2u, u, h) (lapw_mex.c:21-51) */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 3) || (nlhs > 1)) mexErrMsgTxt("Usage: lapw_mex(d2u, u, h);");
    size_t d[3];
    dims_of(prhs[0], d);
    check(qsm_lapw(ctx_get(), dtype_of(prhs[0]), d, mxGetData(prhs[0]), mxGetData(prhs[1]),
                   (const double *)mxGetData(prhs[2])));
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_GAUSS_SEIDEL)
/* gauss_seidel_mex(v, f, G, h, iter, reverse) (gauss_seidel_mex.c:19-58): v in place */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 6) || (nlhs > 1)) mexErrMsgTxt("Usage: gauss_seidel_mex(v, f, G, h, iter, reverse);");
    size_t d[3];
    dims_of(prhs[0], d);
    check(qsm_gauss_seidel(ctx_get(), dtype_of(prhs[0]), d, mxGetData(prhs[0]), mxGetData(prhs[1]),
                           (const uint8_t *)mxGetData(prhs[2]), (const double *)mxGetData(prhs[3]),
                           (int32_t)mxGetScalar(prhs[4]), (int32_t)(uint8_t)mxGetScalar(prhs[5])));
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_RESIDUAL)
/* residual_mex(r, f, x, G, h) (residual_mex.c:17-49): r in place */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 5) || (nlhs > 1)) mexErrMsgTxt("Usage: residual_mex(r, f, x, G, h);");
    size_t d[3];
    dims_of(prhs[0], d);
    check(qsm_residual(ctx_get(), dtype_of(prhs[0]), d, mxGetData(prhs[0]), mxGetData(prhs[1]),
                       mxGetData(prhs[2]), (const uint8_t *)mxGetData(prhs[3]), (const double *)mxGetData(prhs[4])));
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_LAPMG)
/* lapmg_mex(d2u, u, G, h) (lapmg_mex.c:17-45): d2u in place */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 4) || (nlhs > 1)) mexErrMsgTxt("Usage: lapmg_mex(d2u, u, G, h);");
    size_t d[3];
    dims_of(prhs[0], d);
    check(qsm_lapmg(ctx_get(), dtype_of(prhs[0]), d, mxGetData(prhs[0]), mxGetData(prhs[1]),
                    (const uint8_t *)mxGetData(prhs[2]), (const double *)mxGetData(prhs[3])));
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_RESTRICT)
/* restrict_mex(x2, x, G2) (restrict_mex.c:17-45): x2 in place */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 3) || (nlhs > 1)) mexErrMsgTxt("Usage: restrict_mex(x2, x, G2);");
    size_t d2[3], d[3];
    dims_of(prhs[0], d2);
    dims_of(prhs[1], d);
    check(qsm_restrict(ctx_get(), dtype_of(prhs[0]), d2, mxGetData(prhs[0]), d, mxGetData(prhs[1]),
                       (const uint8_t *)mxGetData(prhs[2])));
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_PROLONG) || defined(QSM_MEX_CORRECT)
/* prolong_mex(x, x2, G) (prolong_mex.c:17-45), correct_mex(x, x2, G) (correct_mex.c:17-45): x in place */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
#ifdef QSM_MEX_PROLONG
    if ((nrhs != 3) || (nlhs > 1)) mexErrMsgTxt("Usage: prolong_mex(x, x2, G);");
#else
    if ((nrhs != 3) || (nlhs > 1)) mexErrMsgTxt("Usage: correct_mex(x, x2, G);");
#endif
    size_t d[3], d2[3];
    dims_of(prhs[0], d);
    dims_of(prhs[1], d2);
#ifdef QSM_MEX_PROLONG
    check(qsm_prolong(ctx_get(), dtype_of(prhs[0]), d, mxGetData(prhs[0]), d2, mxGetData(prhs[1]),
                      (const uint8_t *)mxGetData(prhs[2])));
#else
    check(qsm_correct(ctx_get(), dtype_of(prhs[0]), d, mxGetData(prhs[0]), d2, mxGetData(prhs[1]),
                      (const uint8_t *)mxGetData(prhs[2])));
#endif
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_COARSEN_GRID)
/* coarsen_grid_mex(G2, G) (coarsen_grid_mex.c:12-33): G2 in place */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 2) || (nlhs > 1)) mexErrMsgTxt("Usage: coarsen_grid_mex(G2, G);");
    size_t d2[3], d[3];
    dims_of(prhs[0], d2);
    dims_of(prhs[1], d);
    check(qsm_coarsen_grid(ctx_get(), d2, (uint8_t *)mxGetData(prhs[0]), d, (const uint8_t *)mxGetData(prhs[1])));
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_BOUNDARY_MASK) || defined(QSM_MEX_BOUNDARY_MASK_L1)
/* boundary_mask_mex(B, G) (boundary_mask_mex.c:11-29), boundary_mask_l1_mex(B, G, l1)
 * (boundary_mask_l1_mex.c:12-32, usage string "boundary_mask_mex"; erodeMask.m:37 calls it): B in place */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    size_t d[3];
#ifdef QSM_MEX_BOUNDARY_MASK
    if ((nrhs != 2) || (nlhs > 1)) mexErrMsgTxt("Usage: boundary_mask_mex(B, G);");
    dims_of(prhs[0], d);
    check(qsm_boundary_mask(ctx_get(), d, (uint8_t *)mxGetData(prhs[0]), (const uint8_t *)mxGetData(prhs[1])));
#else
    if ((nrhs != 3) || (nlhs > 1)) mexErrMsgTxt("Usage: boundary_mask_mex(B, G, l1);");
    dims_of(prhs[0], d);
    check(qsm_boundary_mask_l1(ctx_get(), d, (uint8_t *)mxGetData(prhs[0]), (const uint8_t *)mxGetData(prhs[1]),
                               (uint8_t)mxGetScalar(prhs[2])));
#endif
    ret_one(nlhs, plhs);
}

#elif defined(QSM_MEX_NORM2)
/* p = norm2_mex(x, G) (norm2_mex.c:21-51): a scalar of the class of x */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 2) || (nlhs > 1)) mexErrMsgTxt("Usage: p = norm2_mex(x, G);");
    if (!mxIsSingle(prhs[0]) && !mxIsDouble(prhs[0])) mexErrMsgTxt("x must be single or double");
    double p = 0.0;
    check(qsm_norm2(ctx_get(), dtype_of(prhs[0]), mxGetNumberOfElements(prhs[0]), mxGetData(prhs[0]),
                    (const uint8_t *)mxGetData(prhs[1]), &p));
    const mwSize one[1] = {1};
    plhs[0] = mxCreateNumericArray(1, one, mxGetClassID(prhs[0]), mxREAL);
    if (mxIsSingle(prhs[0])) *(float *)mxGetData(plhs[0]) = (float)p;
    else *(double *)mxGetData(plhs[0]) = p;
}

#elif defined(QSM_MEX_MGPCG)
/* v = mgpcg_mex(v, f, mask, vsz, tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nboundary, nlevels, verbose) */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 14) || (nlhs > 1))
        mexErrMsgTxt("Usage: v = mgpcg_mex(v, f, mask, vsz, tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nboundary, nlevels, verbose)");
    size_t d[3];
    dims_of(prhs[1], d);
    plhs[0] = mxCreateNumericArray(mxGetNumberOfDimensions(prhs[1]), mxGetDimensions(prhs[1]),
                                   mxGetClassID(prhs[1]), mxREAL);
    check(qsm_mgpcg(ctx_get(), dtype_of(prhs[1]), d, mxGetData(prhs[0]), mxGetData(prhs[1]),
                    (const uint8_t *)mxGetData(prhs[2]), (const double *)mxGetData(prhs[3]), mxGetScalar(prhs[4]),
                    (int32_t)mxGetScalar(prhs[5]), mxGetScalar(prhs[6]), (int32_t)mxGetScalar(prhs[7]),
                    (int32_t)mxGetScalar(prhs[8]), (int32_t)mxGetScalar(prhs[9]), (int32_t)mxGetScalar(prhs[10]),
                    (int32_t)mxGetScalar(prhs[11]), (int32_t)mxGetScalar(prhs[12]), (int32_t)mxGetScalar(prhs[13]),
                    mxGetData(plhs[0]), NULL));
}

#elif defined(QSM_MEX_MG)
/* v = mg_mex(v, f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels) */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 11) || (nlhs > 1))
        mexErrMsgTxt("Usage: v = mg_mex(v, f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels)");
    size_t d[3];
    dims_of(prhs[1], d);
    plhs[0] = mxCreateNumericArray(mxGetNumberOfDimensions(prhs[1]), mxGetDimensions(prhs[1]),
                                   mxGetClassID(prhs[1]), mxREAL);
    check(qsm_mg(ctx_get(), dtype_of(prhs[1]), d, mxGetData(prhs[0]), mxGetData(prhs[1]),
                 (const uint8_t *)mxGetData(prhs[2]), (const double *)mxGetData(prhs[3]), mxGetScalar(prhs[4]),
                 (int32_t)mxGetScalar(prhs[5]), (int32_t)mxGetScalar(prhs[6]), (int32_t)mxGetScalar(prhs[7]),
                 (int32_t)mxGetScalar(prhs[8]), (int32_t)mxGetScalar(prhs[9]), (int32_t)mxGetScalar(prhs[10]),
                 mxGetData(plhs[0]), NULL));
}

#elif defined(QSM_MEX_FMG)
/* v = fmg_mex(f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels) */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if ((nrhs != 10) || (nlhs > 1))
        mexErrMsgTxt("Usage: v = fmg_mex(f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels)");
    size_t d[3];
    dims_of(prhs[0], d);
    plhs[0] = mxCreateNumericArray(mxGetNumberOfDimensions(prhs[0]), mxGetDimensions(prhs[0]),
                                   mxGetClassID(prhs[0]), mxREAL);
    check(qsm_fmg(ctx_get(), dtype_of(prhs[0]), d, mxGetData(prhs[0]), (const uint8_t *)mxGetData(prhs[1]),
                  (const double *)mxGetData(prhs[2]), mxGetScalar(prhs[3]), (int32_t)mxGetScalar(prhs[4]),
                  (int32_t)mxGetScalar(prhs[5]), (int32_t)mxGetScalar(prhs[6]), (int32_t)mxGetScalar(prhs[7]),
                  (int32_t)mxGetScalar(prhs[8]), (int32_t)mxGetScalar(prhs[9]), mxGetData(plhs[0]), NULL));
}

#elif defined(QSM_MEX_SSTGV)
/* x = sstgv(phas, mask, vsz, lambda, alpha, tol, maxit, verbose)  (src/inversion/sstgv.m:1-46);
 * single input runs the fused FP32 path (echoes batched, bit-identical to the plain FP32
 * solve), double input the plain FP64 path */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if (nrhs < 3 || nrhs > 8 || nlhs > 1)
        mexErrMsgTxt("Usage: x = sstgv(phas, mask, vsz, [lambda], [alpha], [tol], [maxit], [verbose]);");
    size_t d[4];
    double h[3];
    mxArray *tm;
    dims4_of(prhs[0], d);
    vec3_of(prhs[2], h);
    const uint8_t *m = mask_of(prhs[1], &tm);
    plhs[0] = like(prhs[0]);
    const qsm_status st = qsm_sstgv(ctx_get(), dtype_of(prhs[0]), d, mxGetData(prhs[0]), m, h,
                                    opt(nrhs, prhs, 3, 1e-4), opt(nrhs, prhs, 4, 3.0), opt(nrhs, prhs, 5, 3e-4),
                                    (uint32_t)opt(nrhs, prhs, 6, 5000.0), (uint32_t)opt(nrhs, prhs, 7, 1.0),
                                    mxIsSingle(prhs[0]) ? 1 : 0, mxGetData(plhs[0]), NULL);
    if (tm) mxDestroyArray(tm);
    check(st);
}

#elif defined(QSM_MEX_LBV)
/* fl = lbv(f, mask, vsz, tol, maxit, mgopts, verbose)  (src/bgremove/lbv.m:1-59) */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if (nrhs < 3 || nrhs > 7 || nlhs > 1)
        mexErrMsgTxt("Usage: fl = lbv(f, mask, vsz, [tol], [maxit], [mgopts], [verbose]);");
    size_t d[4];
    double h[3], mg[4] = {2, 2, 2, 2};
    mxArray *tm;
    dims4_of(prhs[0], d);
    vec3_of(prhs[2], h);
    if (given(nrhs, prhs, 5)) {
        if (mxGetNumberOfElements(prhs[5]) != 4) mexErrMsgTxt("lbv: mgopts is [maxit npre npost nboundary]");
        for (int k = 0; k < 4; ++k) mg[k] = elem(prhs[5], (size_t)k);
    }
    const uint8_t *m = mask_of(prhs[1], &tm);
    plhs[0] = like(prhs[0]);
    const qsm_status st =
        qsm_lbv(ctx_get(), dtype_of(prhs[0]), d, mxGetData(prhs[0]), m, h, opt(nrhs, prhs, 3, 1e-8),
                (int32_t)opt(nrhs, prhs, 4, 0.0), (int32_t)mg[0], (int32_t)mg[1], (int32_t)mg[2], (int32_t)mg[3],
                (int32_t)opt(nrhs, prhs, 6, 0.0), 0, mxGetData(plhs[0]), NULL);
    if (tm) mxDestroyArray(tm);
    check(st);
}

#elif defined(QSM_MEX_UNWRAP_LAPLACIAN)
/* [uphas, d2phas] = unwrapLaplacian(phas, mask, vsz)  (src/unwrap/unwrapLaplacian.m:1-42) */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if (nrhs != 3 || nlhs > 2) mexErrMsgTxt("Usage: [uphas, d2phas] = unwrapLaplacian(phas, mask, vsz);");
    size_t d[4];
    double h[3];
    mxArray *tm;
    dims4_of(prhs[0], d);
    vec3_of(prhs[2], h);
    const uint8_t *m = mask_of(prhs[1], &tm);
    plhs[0] = like(prhs[0]);
    mxArray *d2 = like(prhs[0]);
    const qsm_status st = qsm_unwrap_laplacian(ctx_get(), dtype_of(prhs[0]), d, mxGetData(prhs[0]), m, h, 0,
                                               mxGetData(plhs[0]), mxGetData(d2));
    if (tm) mxDestroyArray(tm);
    if (nlhs > 1) plhs[1] = d2;
    else mxDestroyArray(d2);
    check(st);
}

#elif defined(QSM_MEX_SHARP) || defined(QSM_MEX_VSHARP) || defined(QSM_MEX_RESHARP) || defined(QSM_MEX_ISMV)
/* [fl, mask] = sharp(f, mask, vsz, r, thr)                  (src/bgremove/sharp.m:1-34)
 * [fl, mask] = vsharp(f, mask, vsz, rs, thr)                (src/bgremove/vsharp.m:1-33)
 * [fl, mask] = resharp(f, mask, vsz, r, lambda, tol, maxit) (src/bgremove/resharp.m:1-39)
 * [fl, mask] = ismv(f, mask, vsz, r, tol, maxit, verbose)   (src/bgremove/ismv.m:1-39) */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
#if defined(QSM_MEX_SHARP)
    if (nrhs < 3 || nrhs > 5 || nlhs > 2) mexErrMsgTxt("Usage: [fl, mask] = sharp(f, mask, vsz, [r], [thr]);");
#elif defined(QSM_MEX_VSHARP)
    if (nrhs < 3 || nrhs > 5 || nlhs > 2) mexErrMsgTxt("Usage: [fl, mask] = vsharp(f, mask, vsz, [rs], [thr]);");
#elif defined(QSM_MEX_RESHARP)
    if (nrhs < 3 || nrhs > 7 || nlhs > 2)
        mexErrMsgTxt("Usage: [fl, mask] = resharp(f, mask, vsz, [r], [lambda], [tol], [maxit]);");
#else
    if (nrhs < 3 || nrhs > 7 || nlhs > 2)
        mexErrMsgTxt("Usage: [fl, mask] = ismv(f, mask, vsz, [r], [tol], [maxit], [verbose]);");
#endif
    size_t d[4];
    double h[3];
    mxArray *tm;
    dims4_of(prhs[0], d);
    vec3_of(prhs[2], h);
    const uint8_t *m = mask_of(prhs[1], &tm);
    plhs[0] = like(prhs[0]);
    mxArray *mo = mask_like(prhs[1]);
    qsm_ctx *ctx = ctx_get();
    const qsm_dtype dt = dtype_of(prhs[0]);
    qsm_status st;
#if defined(QSM_MEX_SHARP)
    st = qsm_sharp(ctx, dt, d, mxGetData(prhs[0]), m, h, opt(nrhs, prhs, 3, 9.0), opt(nrhs, prhs, 4, 0.05),
                   mxGetData(plhs[0]), (uint8_t *)mxGetData(mo));
#elif defined(QSM_MEX_VSHARP)
    double rs[64];
    int32_t nr = 0;
    if (given(nrhs, prhs, 3)) {
        const size_t n = mxGetNumberOfElements(prhs[3]);
        if (n > 64) mexErrMsgTxt("vsharp: at most 64 radii");
        for (size_t k = 0; k < n; ++k) rs[k] = elem(prhs[3], k);
        nr = (int32_t)n;
    }
    st = qsm_vsharp(ctx, dt, d, mxGetData(prhs[0]), m, h, nr ? rs : NULL, nr, opt(nrhs, prhs, 4, 0.05),
                    mxGetData(plhs[0]), (uint8_t *)mxGetData(mo));
#elif defined(QSM_MEX_RESHARP)
    st = qsm_resharp(ctx, dt, d, mxGetData(prhs[0]), m, h, opt(nrhs, prhs, 3, 3.0), opt(nrhs, prhs, 4, 1e-2),
                     opt(nrhs, prhs, 5, -1.0), (int32_t)opt(nrhs, prhs, 6, 0.0), 0, mxGetData(plhs[0]),
                     (uint8_t *)mxGetData(mo), NULL);
#else
    st = qsm_ismv(ctx, dt, d, mxGetData(prhs[0]), m, h, opt(nrhs, prhs, 3, 3.0), opt(nrhs, prhs, 4, -1.0),
                  (int32_t)opt(nrhs, prhs, 5, 500.0), (int32_t)opt(nrhs, prhs, 6, 0.0), mxGetData(plhs[0]),
                  (uint8_t *)mxGetData(mo), NULL);
#endif
    if (tm) mxDestroyArray(tm);
    if (nlhs > 1) plhs[1] = mo;
    else mxDestroyArray(mo);
    check(st);
}

#elif defined(QSM_MEX_PDF)
/* fl = pdf(f, mask, vsz, w, bdir, lambda, tol, maxit, verbose)  (src/bgremove/pdf.m:1-52);
 * w is converted to the class of f */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if (nrhs < 3 || nrhs > 9 || nlhs > 1)
        mexErrMsgTxt("Usage: fl = pdf(f, mask, vsz, [w], [bdir], [lambda], [tol], [maxit], [verbose]);");
    size_t d[4];
    double h[3], b[3] = {0.0, 0.0, 1.0};
    mxArray *tm, *tw = NULL;
    dims4_of(prhs[0], d);
    vec3_of(prhs[2], h);
    if (given(nrhs, prhs, 4)) vec3_of(prhs[4], b);
    const void *w = NULL;
    if (given(nrhs, prhs, 3)) {
        if (mxGetNumberOfElements(prhs[3]) != d[0] * d[1] * d[2]) mexErrMsgTxt("pdf: w must have the mask's size");
        if (mxGetClassID(prhs[3]) == mxGetClassID(prhs[0])) {
            w = mxGetData(prhs[3]);
        } else {
            tw = mxCreateNumericArray(mxGetNumberOfDimensions(prhs[3]), mxGetDimensions(prhs[3]),
                                      mxGetClassID(prhs[0]), mxREAL);
            const size_t n = mxGetNumberOfElements(prhs[3]);
            for (size_t i = 0; i < n; ++i) {
                if (mxIsSingle(prhs[0])) ((float *)mxGetData(tw))[i] = (float)elem(prhs[3], i);
                else ((double *)mxGetData(tw))[i] = elem(prhs[3], i);
            }
            w = mxGetData(tw);
        }
    }
    const uint8_t *m = mask_of(prhs[1], &tm);
    plhs[0] = like(prhs[0]);
    const qsm_status st = qsm_pdf(ctx_get(), dtype_of(prhs[0]), d, mxGetData(prhs[0]), m, w, h, b,
                                  opt(nrhs, prhs, 5, 0.0), opt(nrhs, prhs, 6, 1e-5), (int32_t)opt(nrhs, prhs, 7, 0.0),
                                  (int32_t)opt(nrhs, prhs, 8, 0.0), mxGetData(plhs[0]), NULL);
    if (tm) mxDestroyArray(tm);
    if (tw) mxDestroyArray(tw);
    check(st);
}

#else
#error "define one QSM_MEX_<gateway>"
#endif
