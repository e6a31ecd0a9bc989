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
 * QSM_MEX_LAP1, QSM_MEX_LAPW, QSM_MEX_MGPCG, QSM_MEX_MG, QSM_MEX_FMG.
 */
#include <stdint.h>
#include "mex.h"
#include "qsm_gpu.h"

static qsm_ctx *g_ctx = NULL;

static void ctx_release(void)
{
    if (g_ctx) qsm_ctx_destroy(g_ctx);
    g_ctx = NULL;
}

static qsm_ctx *ctx_get(void)
{
    if (!g_ctx) {
        if (qsm_ctx_create(0, &g_ctx) != QSM_OK) mexErrMsgTxt("qsm: no usable CUDA device");
        mexAtExit(ctx_release);
    }
    return g_ctx;
}

static void check(qsm_status st)
{
    if (st != QSM_OK) mexErrMsgTxt(qsm_last_error(g_ctx));
}

static qsm_dtype dtype_of(const mxArray *a) { return mxIsSingle(a) ? QSM_F32 : QSM_F64; }

static void dims_of(const mxArray *a, size_t d[3])
{
    const mwSize nd = mxGetNumberOfDimensions(a);
    const mwSize *s = mxGetDimensions(a);
    d[0] = s[0];
    d[1] = nd > 1 ? s[1] : 1;
    d[2] = nd > 2 ? s[2] : 1;
}

static void ret_one(int nlhs, mxArray *plhs[])
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

#else
#error "define one QSM_MEX_<gateway>"
#endif
