// Primal-dual TGV / TV inversion, plain path: one kernel per loop nest of
// the reference solver (dual update, primal update + extragradient, the
// every-10th-iteration monitor copy and check), evaluated in the caller's
// precision without fused multiply-add.  Bit-identical to the reference
// mx_pdd / mx_pdf in FP64 and FP32.  The mixed-precision fused path is in
// pd_fused.cu; both share the control block and monitor reduction here.
#include <math.h>

#include "common.cuh"
#include "pd.cuh"

namespace qsm {

// ---------------------------------------------------------------------------
// constants (computed on the host in FP64, then cast, as the reference does)
// ---------------------------------------------------------------------------

void pd_steps(const double *h, double *tau, double *sigma)
{
    // pd_tgv_mex.c:272-278 (pd_tv_mex.c:255-261 uses the same K^2)
    double gnrm = 4.0 * (1.0 / (h[0] * h[0]) + 1.0 / (h[1] * h[1]) + 1.0 / (h[2] * h[2]));
    double wnrm = 6.0 * (1.0 / (h[0] * h[0]) + 1.0 / (h[1] * h[1]) + 2.0 / (h[2] * h[2])) / 3.0;
    double K2 = gnrm * gnrm + wnrm * wnrm;
    *tau = 1 / sqrt(K2);
    *sigma = 1 / (*tau * K2);
}

template <typename T>
DualC<T> make_dual_c(double sigma, const double *h, double alpha0, double alpha1)
{
    // pd_tgv_mex.c:527-548 (double) / :366-387 (float casts)
    DualC<T> c;
    c.hx = (T)(sigma / h[0]); c.hy = (T)(sigma / h[1]); c.hz = (T)(sigma / h[2]);
    c.hx2 = (T)(0.5 * sigma / h[0]); c.hy2 = (T)(0.5 * sigma / h[1]); c.hz2 = (T)(0.5 * sigma / h[2]);
    c.lhx = (T)(sigma / (h[0] * h[0])); c.lhy = (T)(sigma / (h[1] * h[1])); c.lhz = (T)(sigma / (h[2] * h[2]));
    c.lhh = (T)-2 * (c.lhx + c.lhy + c.lhz);
    c.whx = (T)(-sigma / (3.0 * h[0] * h[0])); c.why = (T)(-sigma / (3.0 * h[1] * h[1]));
    c.whz = (T)(sigma * 2.0 / (3.0 * h[2] * h[2]));
    c.whh = (T)-2 * (c.whx + c.why + c.whz);
    c.alp0 = (T)alpha0; c.alp1 = (T)alpha1;
    c.alp02 = (T)(alpha0 * alpha0); c.alp12 = (T)(alpha1 * alpha1);
    c.sg = (T)sigma;
    return c;
}

template <typename T>
PrimalC<T> make_primal_c(double tau, const double *h)
{
    // pd_tgv_mex.c:857-872 / :693-708
    PrimalC<T> c;
    c.hx = (T)(tau / h[0]); c.hy = (T)(tau / h[1]); c.hz = (T)(tau / h[2]);
    c.lhx = (T)(tau / (h[0] * h[0])); c.lhy = (T)(tau / (h[1] * h[1])); c.lhz = (T)(tau / (h[2] * h[2]));
    c.lhh = (T)-2 * (c.lhx + c.lhy + c.lhz);
    c.whx = (T)(-tau / (3.0 * h[0] * h[0])); c.why = (T)(-tau / (3.0 * h[1] * h[1]));
    c.whz = (T)(tau * 2.0 / (3.0 * h[2] * h[2]));
    c.whh = (T)-2 * (c.whx + c.why + c.whz);
    c.tt = (T)tau;
    c.tau1 = (T)(1.0 / (1.0 + tau));
    return c;
}

template DualC<float> make_dual_c<float>(double, const double *, double, double);
template DualC<double> make_dual_c<double>(double, const double *, double, double);
template PrimalC<float> make_primal_c<float>(double, const double *);
template PrimalC<double> make_primal_c<double>(double, const double *);

// ---------------------------------------------------------------------------
// setup kernels
// ---------------------------------------------------------------------------

// init_bitmask (pd_tgv_mex.c:1050-1121): mi = all six neighbours in grid & m.
__global__ void interior_mask_k(uint8_t *mi, const uint8_t *__restrict__ m, Dims d)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t j = (size_t)blockIdx.y * blockDim.y + threadIdx.y;
    const size_t k = (size_t)blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= d.nx || j >= d.ny || k >= d.nz) return;
    const size_t nx = d.nx, nxny = d.nxny(), l = i + nx * j + nxny * k;
    mi[l] = (uint8_t)((i > 0 && m[l - 1]) && (i + 1 < d.nx && m[l + 1]) && (j > 0 && m[l - nx]) &&
                      (j + 1 < d.ny && m[l + nx]) && (k > 0 && m[l - nxny]) && (k + 1 < d.nz && m[l + nxny]));
}

// masks normalised to 0/1 (MATLAB logical)
__global__ void mask01_k(uint8_t *o, const uint8_t *__restrict__ m, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        o[l] = m[l] != 0;
}

// f = (T)sigma * d2f (mx_pdd :280-283, mx_pdf :186-189), with an optional
// input conversion (F64 input into an FP32 solve).
template <typename T, typename S>
__global__ void scale_k(T *f, const S *__restrict__ d2f, T s, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        f[l] = s * (T)d2f[l];
}

template <typename T, typename S>
__global__ void convert_k(T *o, const S *__restrict__ a, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        o[l] = (T)a[l];
}

template <typename T, typename S>
qsm_status launch_scale(qsm_ctx *ctx, T *f, const S *d2f, double sigma, size_t n)
{
    scale_k<T, S><<<2048, 256, 0, ctx->stream>>>(f, d2f, (T)sigma, n);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

template <typename T, typename S>
qsm_status launch_convert(qsm_ctx *ctx, T *o, const S *a, size_t n)
{
    convert_k<T, S><<<2048, 256, 0, ctx->stream>>>(o, a, n);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

template qsm_status launch_scale<float, float>(qsm_ctx *, float *, const float *, double, size_t);
template qsm_status launch_scale<float, double>(qsm_ctx *, float *, const double *, double, size_t);
template qsm_status launch_scale<double, double>(qsm_ctx *, double *, const double *, double, size_t);
template qsm_status launch_convert<double, float>(qsm_ctx *, double *, const float *, size_t);

qsm_status launch_masks(qsm_ctx *ctx, uint8_t *m, uint8_t *mi, const uint8_t *mask, const Dims &d)
{
    mask01_k<<<2048, 256, 0, ctx->stream>>>(m, mask, d.n());
    interior_mask_k<<<vox_grid(d), vox_block(), 0, ctx->stream>>>(mi, m, d);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// ---------------------------------------------------------------------------
// plain-path iteration kernels (one thread per interior voxel)
// ---------------------------------------------------------------------------

#define INTERIOR_PROLOGUE                                                     \
    const size_t i = 1 + (size_t)blockIdx.x * blockDim.x + threadIdx.x;       \
    const size_t j = 1 + (size_t)blockIdx.y * blockDim.y + threadIdx.y;       \
    const size_t k = 1 + (size_t)blockIdx.z * blockDim.z + threadIdx.z;       \
    if (i + 1 >= d.nx || j + 1 >= d.ny || k + 1 >= d.nz) return;             \
    const size_t nx = d.nx, nxny = d.nxny(), N = d.n();                      \
    const size_t l = i + nx * j + nxny * k;                                   \
    (void)N;

static inline dim3 interior_grid(const Dims &d)
{
    Dims e{d.nx > 2 ? d.nx - 2 : 0, d.ny > 2 ? d.ny - 2 : 0, d.nz > 2 ? d.nz - 2 : 0};
    return vox_grid(e);
}

// update_dual{d,f} of pd_tgv_mex.c:332-646.
template <typename T>
__global__ void tgv_dual_k(PdState<T> s, DualC<T> c, Dims d, const PdCtl *ctl)
{
    if (ctl->done) return;
    INTERIOR_PROLOGUE
    if (!s.mi[l]) return;
    const T *chi_ = s.chi_, *eta_ = s.eta_;
    const T *w1 = s.w_, *w2 = s.w_ + N, *w3 = s.w_ + 2 * N;
    T *p1 = s.p, *p2 = s.p + N, *p3 = s.p + 2 * N;
    T *q1 = s.q, *q2 = s.q + N, *q3 = s.q + 2 * N, *q4 = s.q + 3 * N, *q5 = s.q + 4 * N, *q6 = s.q + 5 * N;
    const T c0 = chi_[l];
    const T lap = c.lhh * eta_[l] + c.lhx * (eta_[l - 1] + eta_[l + 1]) + c.lhy * (eta_[l - nx] + eta_[l + nx]) +
                  c.lhz * (eta_[l - nxny] + eta_[l + nxny]);
    const T wav = c.whh * c0 + c.whx * (chi_[l - 1] + chi_[l + 1]) + c.why * (chi_[l - nx] + chi_[l + nx]) +
                  c.whz * (chi_[l - nxny] + chi_[l + nxny]);
    s.nu[l] = s.nu[l] + ((lap - wav) + s.f[l]);

    T a1 = p1[l] + c.hx * (chi_[l + 1] - c0) - c.sg * w1[l];
    T a2 = p2[l] + c.hy * (chi_[l + nx] - c0) - c.sg * w2[l];
    T a3 = p3[l] + c.hz * (chi_[l + nxny] - c0) - c.sg * w3[l];
    T x = a1 * a1 + a2 * a2 + a3 * a3;
    if (x > c.alp12) {
        x = c.alp1 / sqrt(x);
        a1 = a1 * x; a2 = a2 * x; a3 = a3 * x;
    }
    p1[l] = a1; p2[l] = a2; p3[l] = a3;

    const T v1 = w1[l], v2 = w2[l], v3 = w3[l];
    T b1 = q1[l] + c.hx * (w1[l + 1] - v1);
    T b2 = q2[l] + c.hx2 * (w2[l + 1] - v2) + c.hy2 * (w1[l + nx] - v1);
    T b3 = q3[l] + c.hx2 * (w3[l + 1] - v3) + c.hz2 * (w1[l + nxny] - v1);
    T b4 = q4[l] + c.hy * (w2[l + nx] - v2);
    T b5 = q5[l] + c.hy2 * (w3[l + nx] - v3) + c.hz2 * (w2[l + nxny] - v2);
    T b6 = q6[l] + c.hz * (w3[l + nxny] - v3);
    x = b1 * b1 + b4 * b4 + b6 * b6 + (T)2 * (b2 * b2 + b3 * b3 + b5 * b5);
    if (x > c.alp02) {
        x = c.alp0 / sqrt(x);
        b1 = b1 * x; b2 = b2 * x; b3 = b3 * x; b4 = b4 * x; b5 = b5 * x; b6 = b6 * x;
    }
    q1[l] = b1; q2[l] = b2; q3[l] = b3; q4[l] = b4; q5[l] = b5; q6[l] = b6;
}

// update_primal{d,f} of pd_tgv_mex.c:659-977 (THETA = 1 extragradient).
template <typename T>
__global__ void tgv_primal_k(PdState<T> s, PrimalC<T> c, Dims d, const PdCtl *ctl)
{
    if (ctl->done) return;
    INTERIOR_PROLOGUE
    if (!s.m[l]) return;
    const T *nu = s.nu;
    const T *p1 = s.p, *p2 = s.p + N, *p3 = s.p + 2 * N;
    const T *q1 = s.q, *q2 = s.q + N, *q3 = s.q + 2 * N, *q4 = s.q + 3 * N, *q5 = s.q + 4 * N, *q6 = s.q + 5 * N;
    T *w1 = s.w, *w2 = s.w + N, *w3 = s.w + 2 * N;
    const T en = s.eta[l], cn = s.chi[l], w1n = w1[l], w2n = w2[l], w3n = w3[l];
    const T x = nu[l - 1] + nu[l + 1];
    const T y = nu[l - nx] + nu[l + nx];
    const T z = nu[l - nxny] + nu[l + nxny];
    const T e1 = c.tau1 * (en - c.lhh * nu[l] - c.lhx * x - c.lhy * y - c.lhz * z);
    const T c1 = cn + (c.hx * (p1[l] - p1[l - 1]) + c.hy * (p2[l] - p2[l - nx]) + c.hz * (p3[l] - p3[l - nxny]) +
                       (c.whh * nu[l] + c.whx * x + c.why * y + c.whz * z));
    const T u1 = w1n + (c.tt * p1[l] + c.hx * (q1[l] - q1[l - 1] + q2[l] - q2[l - nx] + q3[l] - q3[l - nxny]));
    const T u2 = w2n + (c.tt * p2[l] + c.hy * (q2[l] - q2[l - 1] + q4[l] - q4[l - nx] + q5[l] - q5[l - nxny]));
    const T u3 = w3n + (c.tt * p3[l] + c.hz * (q3[l] - q3[l - 1] + q5[l] - q5[l - nx] + q6[l] - q6[l - nxny]));
    s.eta[l] = e1; s.chi[l] = c1; w1[l] = u1; w2[l] = u2; w3[l] = u3;
    s.eta_[l] = e1 + (T)1 * (e1 - en);
    s.chi_[l] = c1 + (T)1 * (c1 - cn);
    s.w_[l] = u1 + (T)1 * (u1 - w1n);
    s.w_[l + N] = u2 + (T)1 * (u2 - w2n);
    s.w_[l + 2 * N] = u3 + (T)1 * (u3 - w3n);
}

// update_dual{d,f} of pd_tv_mex.c:314-513.
template <typename T>
__global__ void tv_dual_k(PdState<T> s, DualC<T> c, Dims d, const PdCtl *ctl)
{
    if (ctl->done) return;
    INTERIOR_PROLOGUE
    if (!s.mi[l]) return;
    const T *chi_ = s.chi_, *eta_ = s.eta_;
    T *p1 = s.p, *p2 = s.p + N, *p3 = s.p + 2 * N;
    const T c0 = chi_[l];
    const T lap = c.lhh * eta_[l] + c.lhx * (eta_[l - 1] + eta_[l + 1]) + c.lhy * (eta_[l - nx] + eta_[l + nx]) +
                  c.lhz * (eta_[l - nxny] + eta_[l + nxny]);
    const T wav = c.whh * c0 + c.whx * (chi_[l - 1] + chi_[l + 1]) + c.why * (chi_[l - nx] + chi_[l + nx]) +
                  c.whz * (chi_[l - nxny] + chi_[l + nxny]);
    s.nu[l] = s.nu[l] + ((lap - wav) + s.f[l]);
    T a1 = p1[l] + c.hx * (chi_[l + 1] - c0);
    T a2 = p2[l] + c.hy * (chi_[l + nx] - c0);
    T a3 = p3[l] + c.hz * (chi_[l + nxny] - c0);
    T x = a1 * a1 + a2 * a2 + a3 * a3;
    if (x > c.alp12) {
        x = c.alp1 / sqrt(x);
        a1 = a1 * x; a2 = a2 * x; a3 = a3 * x;
    }
    p1[l] = a1; p2[l] = a2; p3[l] = a3;
}

// update_primal{d,f} of pd_tv_mex.c:524-727.
template <typename T>
__global__ void tv_primal_k(PdState<T> s, PrimalC<T> c, Dims d, const PdCtl *ctl)
{
    if (ctl->done) return;
    INTERIOR_PROLOGUE
    if (!s.m[l]) return;
    const T *nu = s.nu;
    const T *p1 = s.p, *p2 = s.p + N, *p3 = s.p + 2 * N;
    const T en = s.eta[l], cn = s.chi[l];
    const T x = nu[l - 1] + nu[l + 1];
    const T y = nu[l - nx] + nu[l + nx];
    const T z = nu[l - nxny] + nu[l + nxny];
    const T e1 = c.tau1 * (en - c.lhh * nu[l] - c.lhx * x - c.lhy * y - c.lhz * z);
    const T c1 = cn + (c.hx * (p1[l] - p1[l - 1]) + c.hy * (p2[l] - p2[l - nx]) + c.hz * (p3[l] - p3[l - nxny]) +
                       (c.whh * nu[l] + c.whx * x + c.why * y + c.whz * z));
    s.eta[l] = e1; s.chi[l] = c1;
    s.eta_[l] = e1 + (T)1 * (e1 - en);
    s.chi_[l] = c1 + (T)1 * (c1 - cn);
}

// ---------------------------------------------------------------------------
// convergence check: FP64 lane-order sums of convergence_check{d,f}
// (pd_tgv_mex.c:981-1045), then the stopping test of :1010.
// ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(RED_BLOCK) pd_check_k(const T *__restrict__ chi, const T *__restrict__ chi0,
                                                        const T *__restrict__ eta, const T *__restrict__ eta0, size_t n,
                                                        double *part, unsigned int *count, PdCtl *ctl, double tol,
                                                        uint32_t it)
{
    __shared__ double sm[RED_BLOCK];
    __shared__ bool last;
    __shared__ double res[4];
    if (ctl->done) return;
    const int tid = threadIdx.x;
    const size_t t = (size_t)blockIdx.x * RED_BLOCK + tid;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (size_t i = t; i < n; i += RED_LANES) {
        double a, b, c, dd;
        mon_terms(chi[i], chi0[i], eta[i], eta0[i], a, b, c, dd);
        acc[0] = acc[0] + a; acc[1] = acc[1] + b; acc[2] = acc[2] + c; acc[3] = acc[3] + dd;
    }
    for (int q = 0; q < 4; ++q) {
        sm[tid] = acc[q];
        __syncthreads();
        for (int s = RED_BLOCK / 2; s > 0; s >>= 1) {
            if (tid < s) sm[tid] = sm[tid] + sm[tid + s];
            __syncthreads();
        }
        if (tid == 0) part[q * RED_NBLK + blockIdx.x] = sm[0];
        __syncthreads();
    }
    if (tid == 0) {
        __threadfence();
        last = atomicAdd(count, 1u) == RED_NBLK - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int q = 0; q < 4; ++q) {
        const double *pp = part + q * RED_NBLK;
        double a = __ldcg(pp + tid), b = __ldcg(pp + tid + 256), c = __ldcg(pp + tid + 512), e = __ldcg(pp + tid + 768);
        double v = (a + c) + (b + e);
        sm[tid] = v;
        __syncthreads();
        for (int s = RED_BLOCK / 2; s > 0; s >>= 1) {
            if (tid < s) sm[tid] = sm[tid] + sm[tid + s];
            __syncthreads();
        }
        if (tid == 0) res[q] = sm[0];
        __syncthreads();
    }
    if (tid == 0) {
        pd_finish(ctl, res, tol, it);
        *count = 0;
    }
}

template <typename T>
qsm_status launch_pd_check(qsm_ctx *ctx, const T *chi, const T *chi0, const T *eta, const T *eta0, size_t n,
                           PdCtl *ctl, double tol, uint32_t it)
{
    pd_check_k<T><<<RED_NBLK, RED_BLOCK, 0, ctx->stream>>>(chi, chi0, eta, eta0, n, ctx->red_partial,
                                                           ctx->red_count, ctl, tol, it);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

template qsm_status launch_pd_check<float>(qsm_ctx *, const float *, const float *, const float *, const float *,
                                           size_t, PdCtl *, double, uint32_t);
template qsm_status launch_pd_check<double>(qsm_ctx *, const double *, const double *, const double *,
                                            const double *, size_t, PdCtl *, double, uint32_t);

// ---------------------------------------------------------------------------
// plain-path driver
// ---------------------------------------------------------------------------

template <typename T>
static qsm_status pd_plain(qsm_ctx *ctx, bool tgv, const Dims &d, const void *d2f_dev, const uint8_t *mask_dev,
                           const double *h, double lam, double alpha, double tol, uint32_t maxiter,
                           uint32_t verbose, T *chi_out, qsm_pd_info *info)
{
    Range nvtx_range("pd_plain");
    const size_t N = d.n();
    const int narr = tgv ? 23 : 11;
    void *blk = nullptr;
    QSM_TRY(dalloc(ctx, &blk, (size_t)narr * N * sizeof(T) + 2 * N + sizeof(PdCtl) + 256));
    QSM_CUDA(cudaMemsetAsync(blk, 0, (size_t)narr * N * sizeof(T) + 2 * N + sizeof(PdCtl) + 256, ctx->stream));
    T *b = (T *)blk;
    PdState<T> s;
    memset(&s, 0, sizeof s);
    if (tgv) {
        s.chi = b; s.eta = b + N; s.w = b + 2 * N; s.chi_ = b + 5 * N; s.eta_ = b + 6 * N; s.w_ = b + 7 * N;
        s.nu = b + 10 * N; s.p = b + 11 * N; s.q = b + 14 * N; s.f = b + 20 * N; s.chi0 = b + 21 * N; s.eta0 = b + 22 * N;
    } else {
        s.chi = b; s.eta = b + N; s.chi_ = b + 2 * N; s.eta_ = b + 3 * N; s.nu = b + 4 * N; s.p = b + 5 * N;
        s.f = b + 8 * N; s.chi0 = b + 9 * N; s.eta0 = b + 10 * N;
    }
    uint8_t *mb = (uint8_t *)(b + (size_t)narr * N);
    s.m = mb;
    s.mi = mb + N;
    PdCtl *ctl = (PdCtl *)(((uintptr_t)(mb + 2 * N) + 255) & ~(uintptr_t)255);

    double tau, sigma;
    pd_steps(h, &tau, &sigma);
    const double alpha1 = lam, alpha0 = alpha * lam;
    QSM_TRY(launch_masks(ctx, s.m, s.mi, mask_dev, d));
    QSM_TRY((launch_scale<T, T>(ctx, s.f, (const T *)d2f_dev, sigma, N)));
    const DualC<T> dc = tgv ? make_dual_c<T>(sigma, h, alpha0, alpha1) : make_dual_c<T>(sigma, h, 0.0, lam);
    const PrimalC<T> pc = make_primal_c<T>(tau, h);
    const dim3 g = interior_grid(d), bl = vox_block();
    const bool empty = g.x == 0 || g.y == 0 || g.z == 0;

    cudaEvent_t e0, e1;
    QSM_CUDA(cudaEventCreate(&e0));
    QSM_CUDA(cudaEventCreate(&e1));
    QSM_CUDA(cudaEventRecord(e0, ctx->stream));
    const uint32_t pmod = maxiter ? maxiter / (verbose > 4 ? (verbose < maxiter ? verbose : maxiter) : (4 < maxiter ? 4 : maxiter)) : 1;
    if (verbose) printf("Iter\t\t||delta chi||\t||delta eta||\n");
    uint32_t enq = 0;
    PdCtl hctl;
    memset(&hctl, 0, sizeof hctl);
    for (uint32_t it = 0; it < maxiter; ++it) {
        const bool chk = ((it + 1) % 10) == 0;
        if (chk) {
            QSM_CUDA(cudaMemcpyAsync(s.chi0, s.chi, N * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
            QSM_CUDA(cudaMemcpyAsync(s.eta0, s.eta, N * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
        }
        if (!empty) {
            if (tgv) {
                tgv_dual_k<T><<<g, bl, 0, ctx->stream>>>(s, dc, d, ctl);
                tgv_primal_k<T><<<g, bl, 0, ctx->stream>>>(s, pc, d, ctl);
            } else {
                tv_dual_k<T><<<g, bl, 0, ctx->stream>>>(s, dc, d, ctl);
                tv_primal_k<T><<<g, bl, 0, ctx->stream>>>(s, pc, d, ctl);
            }
            QSM_CUDA(cudaGetLastError());
        }
        if (chk) QSM_TRY(launch_pd_check<T>(ctx, s.chi, s.chi0, s.eta, s.eta0, N, ctl, tol, it + 1));
        enq = it + 1;
        const bool print = verbose && (it == 0 || it == maxiter - 1 || ((it + 1) % pmod) == 0);
        if (print || (chk && ((it + 1) % 100) == 0)) {
            QSM_CUDA(cudaMemcpyAsync(&hctl, ctl, sizeof(PdCtl), cudaMemcpyDeviceToHost, ctx->stream));
            QSM_CUDA(cudaStreamSynchronize(ctx->stream));
            if (print || hctl.done)
                if (verbose) printf("%5d/%d\t%.3e\t%.3e\n", hctl.done ? hctl.iters : it + 1, maxiter,
                                    hctl.checks ? hctl.n1 : 1.0, hctl.checks ? hctl.n2 : 1.0);
            if (hctl.done) break;
        }
    }
    QSM_CUDA(cudaEventRecord(e1, ctx->stream));
    QSM_CUDA(cudaMemcpyAsync(&hctl, ctl, sizeof(PdCtl), cudaMemcpyDeviceToHost, ctx->stream));
    QSM_CUDA(cudaMemcpyAsync(chi_out, s.chi, N * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (info) {
        info->iters = hctl.done ? hctl.iters : enq;
        info->monitor_chi = hctl.checks ? hctl.n1 : 1.0;
        info->monitor_eta = hctl.checks ? hctl.n2 : 1.0;
        info->seconds = ms * 1e-3;
        info->active_voxels = (uint64_t)(d.nx > 2 ? d.nx - 2 : 0) * (d.ny > 2 ? d.ny - 2 : 0) * (d.nz > 2 ? d.nz - 2 : 0);
        info->tile[0] = info->tile[1] = info->tile[2] = 0;
    }
    QSM_TRY(dfree(ctx, blk));
    return QSM_OK;
}

// Common entry: validation and staging.  fused selects pd_fused.cu.
qsm_status pd_entry(qsm_ctx *ctx, bool tgv, bool fused, qsm_dtype dt, const size_t *dims, const void *d2f,
                    const uint8_t *mask, const double *vsz, double lam, double alpha, double tol,
                    uint32_t maxiter, uint32_t verbose, void *chi, qsm_pd_info *info)
{
    if (!ctx || !dims || !d2f || !mask || !vsz || !chi) return QSM_ERR_ARG;
    if (dt != QSM_F32 && dt != QSM_F64) return QSM_ERR_DTYPE;
    if (dims[0] == 0 || dims[1] == 0 || dims[2] == 0) {
        set_error(ctx, "empty volume");
        return QSM_ERR_DIMS;
    }
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    const size_t es = dt == QSM_F32 ? 4 : 8;
    Staged sf, sm, sc;
    QSM_TRY(stage_in(ctx, sf, d2f, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sm, mask, d.n(), true));
    QSM_TRY(stage_in(ctx, sc, chi, d.n() * es, false));
    qsm_status st;
    if (fused)
        st = pd_fused(ctx, tgv, d, dt, sf.dev, (const uint8_t *)sm.dev, vsz, lam, alpha, tol, maxiter, verbose, sc.dev, info);
    else if (dt == QSM_F32)
        st = pd_plain<float>(ctx, tgv, d, sf.dev, (const uint8_t *)sm.dev, vsz, lam, alpha, tol, maxiter, verbose,
                             (float *)sc.dev, info);
    else
        st = pd_plain<double>(ctx, tgv, d, sf.dev, (const uint8_t *)sm.dev, vsz, lam, alpha, tol, maxiter, verbose,
                              (double *)sc.dev, info);
    QSM_TRY(stage_out(ctx, sf, false));
    QSM_TRY(stage_out(ctx, sm, false));
    QSM_TRY(stage_out(ctx, sc, st == QSM_OK));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return st;
}

}  // namespace qsm

using namespace qsm;

extern "C" {

qsm_status qsm_pd_tgv(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], const void *d2f, const uint8_t *mask,
                      const double vsz[3], double lam, double alpha, double tol, uint32_t maxiter, uint32_t verbose,
                      void *chi, qsm_pd_info *info)
{
    return pd_entry(ctx, true, false, dt, dims, d2f, mask, vsz, lam, alpha, tol, maxiter, verbose, chi, info);
}

qsm_status qsm_pd_tv(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], const void *d2f, const uint8_t *mask,
                     const double vsz[3], double lam, double tol, uint32_t maxiter, uint32_t verbose, void *chi,
                     qsm_pd_info *info)
{
    return pd_entry(ctx, false, false, dt, dims, d2f, mask, vsz, lam, 0.0, tol, maxiter, verbose, chi, info);
}

qsm_status qsm_pd_tgv_fused(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], const void *d2f, const uint8_t *mask,
                            const double vsz[3], double lam, double alpha, double tol, uint32_t maxiter,
                            uint32_t verbose, void *chi, qsm_pd_info *info)
{
    return pd_entry(ctx, true, true, dt, dims, d2f, mask, vsz, lam, alpha, tol, maxiter, verbose, chi, info);
}

qsm_status qsm_pd_tv_fused(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], const void *d2f, const uint8_t *mask,
                           const double vsz[3], double lam, double tol, uint32_t maxiter, uint32_t verbose,
                           void *chi, qsm_pd_info *info)
{
    return pd_entry(ctx, false, true, dt, dims, d2f, mask, vsz, lam, 0.0, tol, maxiter, verbose, chi, info);
}

}  // extern "C"
