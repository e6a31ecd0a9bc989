// Shared declarations of the primal-dual solvers (pd.cu plain path,
// pd_fused.cu mixed-precision fused path).
#pragma once

#include "common.cuh"

namespace qsm {

// Device-side control block of one solve.
struct PdCtl {
    double n1, n2;         // monitors of the last check
    uint32_t done;         // set when the stopping test passed
    uint32_t iters;        // iteration count at which it passed
    uint32_t checks;       // checks performed
    uint32_t nonfinite;    // a monitor was NaN/Inf
    uint32_t stalled;      // a bounded wait on a TMA load gave up (QSM_ERR_TIMEOUT)
};

// Device pointers of the plain path's state (component-major fields).
template <typename T>
struct PdState {
    T *chi, *eta, *w, *chi_, *eta_, *w_;   // primal + extragradient copies
    T *nu, *p, *q;                          // dual
    T *f, *chi0, *eta0;                     // scaled data, monitor snapshots
    uint8_t *m, *mi;                        // mask, interior mask
};

// Dual-update constants (pd_tgv_mex.c:366-387 / :527-548).
template <typename T>
struct DualC {
    T hx, hy, hz, hx2, hy2, hz2, lhx, lhy, lhz, lhh, whx, why, whz, whh, alp0, alp1, alp02, alp12, sg;
};

// Primal-update constants (pd_tgv_mex.c:693-708 / :857-872).
template <typename T>
struct PrimalC {
    T hx, hy, hz, lhx, lhy, lhz, lhh, whx, why, whz, whh, tt, tau1;
};

void pd_steps(const double *h, double *tau, double *sigma);
template <typename T> DualC<T> make_dual_c(double sigma, const double *h, double alpha0, double alpha1);
template <typename T> PrimalC<T> make_primal_c(double tau, const double *h);

qsm_status launch_masks(qsm_ctx *ctx, uint8_t *m, uint8_t *mi, const uint8_t *mask, const Dims &d);
template <typename T, typename S> qsm_status launch_scale(qsm_ctx *ctx, T *f, const S *d2f, double sigma, size_t n);
template <typename T, typename S> qsm_status launch_convert(qsm_ctx *ctx, T *o, const S *a, size_t n);
template <typename T>
qsm_status launch_pd_check(qsm_ctx *ctx, const T *chi, const T *chi0, const T *eta, const T *eta0, size_t n,
                           PdCtl *ctl, double tol, uint32_t it);
// Stopping test of convergence_check (pd_tgv_mex.c:1006-1010) on the four
// sums s = {sum chi^2, sum eta^2, sum dchi^2, sum deta^2}.
__device__ __forceinline__ void pd_finish(PdCtl *ctl, const double *s, double tol, uint32_t it)
{
    const double n1 = sqrt(s[2] / s[0]);
    const double n2 = sqrt(s[3] / s[1]);
    ctl->n1 = n1;
    ctl->n2 = n2;
    ctl->checks += 1;
    if (!isfinite(n1) || !isfinite(n2)) ctl->nonfinite = 1;
    if ((n1 < tol) && (n2 < 2.0 * tol)) {
        ctl->done = 1;
        ctl->iters = it;
    }
}

// Per-voxel monitor terms of convergence_check{d,f} (pd_tgv_mex.c:997-1000,
// :1032-1035): the FP32 variant multiplies a float difference (widened) by
// the exact double difference.
__device__ __forceinline__ void mon_terms(double x, double x0, double e, double e0, double &a, double &b,
                                          double &c, double &dd)
{
    a = x * x; b = e * e; c = (x - x0) * (x - x0); dd = (e - e0) * (e - e0);
}
__device__ __forceinline__ void mon_terms(float x, float x0, float e, float e0, double &a, double &b,
                                          double &c, double &dd)
{
    a = (double)x * (double)x;
    b = (double)e * (double)e;
    c = (double)(x - x0) * ((double)x - (double)x0);
    dd = (double)(e - e0) * ((double)e - (double)e0);
}

// Mixed-precision fused solve (pd_fused.cu).  d2f/chi are device arrays of
// `dt`; mask is a device uint8 array.
qsm_status pd_fused(qsm_ctx *ctx, bool tgv, const Dims &d, qsm_dtype dt, const void *d2f, const uint8_t *mask,
                    const double *h, double lam, double alpha, double tol, uint32_t maxiter, uint32_t verbose,
                    void *chi, qsm_pd_info *info);

}  // namespace qsm
