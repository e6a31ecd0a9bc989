// Finite-difference operators: gradients (forward / backward / central,
// plain and masked, periodic), their adjoints, the masked Laplacian with
// one-sided boundary stencils and the Laplacian of a wrapped phase.
//
// One thread per voxel.  Every kernel evaluates the per-voxel rule of the
// reference loop nest it replaces with the same expression and association
// order; the file is compiled without fused multiply-add, so results are
// bit-identical to the reference C in FP32 and FP64.  These are single
// sweeps bounded by HBM bandwidth: each reads its inputs once (neighbour
// re-reads hit L1/L2) and writes each output once.
#include "common.cuh"

namespace qsm {

#define VOXEL_PROLOGUE                                                        \
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;           \
    const size_t j = (size_t)blockIdx.y * blockDim.y + threadIdx.y;           \
    const size_t k = (size_t)blockIdx.z * blockDim.z + threadIdx.z;           \
    if (i >= d.nx || j >= d.ny || k >= d.nz) return;                          \
    const size_t nx = d.nx, ny = d.ny, nz = d.nz, nxny = nx * ny;             \
    const size_t l = i + nx * j + nxny * k;                                   \
    (void)ny; (void)nz;

template <typename T> struct H3 { T x, y, z; };

// ---- gradients ----------------------------------------------------------

// gradf_mex.c:149-245
template <typename T>
__global__ void gradf_k(T *dx, T *dy, T *dz, const T *__restrict__ u, H3<T> h, Dims d)
{
    VOXEL_PROLOGUE
    dx[l] = i + 1 < nx ? h.x * (u[l + 1] - u[l]) : h.x * (u[l] - u[l - 1]);
    dy[l] = j + 1 < ny ? h.y * (u[l + nx] - u[l]) : h.y * (u[l] - u[l - nx]);
    dz[l] = k + 1 < nz ? h.z * (u[l + nxny] - u[l]) : h.z * (u[l] - u[l - nxny]);
}

// gradb_mex.c:142-229
template <typename T>
__global__ void gradb_k(T *dx, T *dy, T *dz, const T *__restrict__ u, H3<T> h, Dims d)
{
    VOXEL_PROLOGUE
    dx[l] = i > 0 ? h.x * (u[l] - u[l - 1]) : h.x * (u[l + 1] - u[l]);
    dy[l] = j > 0 ? h.y * (u[l] - u[l - nx]) : h.y * (u[l + nx] - u[l]);
    dz[l] = k > 0 ? h.z * (u[l] - u[l - nxny]) : h.z * (u[l + nxny] - u[l]);
}

// gradc_mex.c:309-563, including the k = 0 plane overwrite of its
// "i = nx-1, k = 0" loop (:396, j stepping by 1): every linear index
// l in [2nx-1, nx*ny-2] of that plane gets (backward, central, forward).
template <typename T>
__global__ void gradc_k(T *dx, T *dy, T *dz, const T *__restrict__ u, H3<T> h, H3<T> h2, Dims d)
{
    VOXEL_PROLOGUE
    if (k == 0 && l >= 2 * nx - 1 && l + 2 <= nxny) {
        dx[l] = h.x * (u[l] - u[l - 1]);
        dy[l] = h2.y * (u[l + nx] - u[l - nx]);
        dz[l] = h.z * (u[l + nxny] - u[l]);
        return;
    }
    dx[l] = i == 0 ? h.x * (u[l + 1] - u[l]) : i + 1 == nx ? h.x * (u[l] - u[l - 1]) : h2.x * (u[l + 1] - u[l - 1]);
    dy[l] = j == 0 ? h.y * (u[l + nx] - u[l]) : j + 1 == ny ? h.y * (u[l] - u[l - nx]) : h2.y * (u[l + nx] - u[l - nx]);
    dz[l] = k == 0 ? h.z * (u[l + nxny] - u[l]) : k + 1 == nz ? h.z * (u[l] - u[l - nxny]) : h2.z * (u[l + nxny] - u[l - nxny]);
}

// gradfm_mex.c:105-154
template <typename T>
__global__ void gradfm_k(T *dx, T *dy, T *dz, const T *__restrict__ u, const uint8_t *__restrict__ G, H3<T> h, Dims d)
{
    VOXEL_PROLOGUE
    if (!G[l]) return;
    dx[l] = (i + 1 < nx && G[l + 1]) ? h.x * (u[l + 1] - u[l]) : (i > 0 && G[l - 1]) ? h.x * (u[l] - u[l - 1]) : (T)0;
    dy[l] = (j + 1 < ny && G[l + nx]) ? h.y * (u[l + nx] - u[l]) : (j > 0 && G[l - nx]) ? h.y * (u[l] - u[l - nx]) : (T)0;
    dz[l] = (k + 1 < nz && G[l + nxny]) ? h.z * (u[l + nxny] - u[l]) : (k > 0 && G[l - nxny]) ? h.z * (u[l] - u[l - nxny]) : (T)0;
}

// gradbm_mex.c:106-154
template <typename T>
__global__ void gradbm_k(T *dx, T *dy, T *dz, const T *__restrict__ u, const uint8_t *__restrict__ G, H3<T> h, Dims d)
{
    VOXEL_PROLOGUE
    if (!G[l]) return;
    dx[l] = (i > 0 && G[l - 1]) ? h.x * (u[l] - u[l - 1]) : (i + 1 < nx && G[l + 1]) ? h.x * (u[l + 1] - u[l]) : (T)0;
    dy[l] = (j > 0 && G[l - nx]) ? h.y * (u[l] - u[l - nx]) : (j + 1 < ny && G[l + nx]) ? h.y * (u[l + nx] - u[l]) : (T)0;
    dz[l] = (k > 0 && G[l - nxny]) ? h.z * (u[l] - u[l - nxny]) : (k + 1 < nz && G[l + nxny]) ? h.z * (u[l + nxny] - u[l]) : (T)0;
}

// gradcm_mex.c:122-186
template <typename T>
__global__ void gradcm_k(T *dx, T *dy, T *dz, const T *__restrict__ u, const uint8_t *__restrict__ G, H3<T> h, H3<T> h2, Dims d)
{
    VOXEL_PROLOGUE
    if (!G[l]) return;
    const bool xf = i + 1 < nx && G[l + 1], xb = i > 0 && G[l - 1];
    const bool yf = j + 1 < ny && G[l + nx], yb = j > 0 && G[l - nx];
    const bool zf = k + 1 < nz && G[l + nxny], zb = k > 0 && G[l - nxny];
    dx[l] = (xf && xb) ? h2.x * (u[l + 1] - u[l - 1]) : xf ? h.x * (u[l + 1] - u[l]) : xb ? h.x * (u[l] - u[l - 1]) : (T)0;
    dy[l] = (yf && yb) ? h2.y * (u[l + nx] - u[l - nx]) : yf ? h.y * (u[l + nx] - u[l]) : yb ? h.y * (u[l] - u[l - nx]) : (T)0;
    dz[l] = (zf && zb) ? h2.z * (u[l + nxny] - u[l - nxny]) : zf ? h.z * (u[l + nxny] - u[l]) : zb ? h.z * (u[l] - u[l - nxny]) : (T)0;
}

// gradfp_mex.c:147-242 (periodic)
template <typename T>
__global__ void gradfp_k(T *dx, T *dy, T *dz, const T *__restrict__ u, H3<T> h, Dims d)
{
    VOXEL_PROLOGUE
    const size_t NX = nx - 1, NY = nx * (ny - 1), NZ = nxny * (nz - 1);
    dx[l] = h.x * ((i + 1 < nx ? u[l + 1] : u[l - NX]) - u[l]);
    dy[l] = h.y * ((j + 1 < ny ? u[l + nx] : u[l - NY]) - u[l]);
    dz[l] = h.z * ((k + 1 < nz ? u[l + nxny] : u[l - NZ]) - u[l]);
}

// ---- adjoints -------------------------------------------------------------

// gradf_adj_mex.c:153-249 (h holds -1/h)
template <typename T>
__global__ void gradf_adj_k(T *du, const T *__restrict__ x, const T *__restrict__ y, const T *__restrict__ z, H3<T> h, Dims d)
{
    VOXEL_PROLOGUE
    const T a = i > 0 ? x[l] - x[l - 1] : x[l + 1] - x[l];
    const T b = j > 0 ? y[l] - y[l - nx] : y[l + nx] - y[l];
    const T c = k > 0 ? z[l] - z[l - nxny] : z[l + nxny] - z[l];
    du[l] = h.x * a + h.y * b + h.z * c;
}

// gradb_adj_mex.c:159-261
template <typename T>
__global__ void gradb_adj_k(T *du, const T *__restrict__ x, const T *__restrict__ y, const T *__restrict__ z, H3<T> h, Dims d)
{
    VOXEL_PROLOGUE
    const T a = i + 1 < nx ? x[l + 1] - x[l] : x[l] - x[l - 1];
    const T b = j + 1 < ny ? y[l + nx] - y[l] : y[l] - y[l - nx];
    const T c = k + 1 < nz ? z[l + nxny] - z[l] : z[l] - z[l - nxny];
    du[l] = h.x * a + h.y * b + h.z * c;
}

// gradfm_adj_mex.c:110-162
template <typename T>
__global__ void gradfm_adj_k(T *du, const T *__restrict__ x, const T *__restrict__ y, const T *__restrict__ z,
                             const uint8_t *__restrict__ G, H3<T> h, Dims d)
{
    VOXEL_PROLOGUE
    if (!G[l]) return;
    const T c = (k > 0 && G[l - nxny]) ? h.z * (z[l] - z[l - nxny]) : (k + 1 < nz && G[l + nxny]) ? h.z * (z[l + nxny] - z[l]) : (T)0;
    const T b = (j > 0 && G[l - nx]) ? h.y * (y[l] - y[l - nx]) : (j + 1 < ny && G[l + nx]) ? h.y * (y[l + nx] - y[l]) : (T)0;
    const T a = (i > 0 && G[l - 1]) ? h.x * (x[l] - x[l - 1]) : (i + 1 < nx && G[l + 1]) ? h.x * (x[l + 1] - x[l]) : (T)0;
    du[l] = a + b + c;
}

// gradbm_adj_mex.c:110-162
template <typename T>
__global__ void gradbm_adj_k(T *du, const T *__restrict__ x, const T *__restrict__ y, const T *__restrict__ z,
                             const uint8_t *__restrict__ G, H3<T> h, Dims d)
{
    VOXEL_PROLOGUE
    if (!G[l]) return;
    const T a = (i + 1 < nx && G[l + 1]) ? h.x * (x[l + 1] - x[l]) : (i > 0 && G[l - 1]) ? h.x * (x[l] - x[l - 1]) : (T)0;
    const T b = (j + 1 < ny && G[l + nx]) ? h.y * (y[l + nx] - y[l]) : (j > 0 && G[l - nx]) ? h.y * (y[l] - y[l - nx]) : (T)0;
    const T c = (k + 1 < nz && G[l + nxny]) ? h.z * (z[l + nxny] - z[l]) : (k > 0 && G[l - nxny]) ? h.z * (z[l] - z[l - nxny]) : (T)0;
    du[l] = a + b + c;
}

// gradfp_adj_mex.c:156-257: axis terms summed (x+y)+z on k = 0,
// (z+x)+y for k > 0, j = 0 and (z+y)+x for k > 0, j > 0.
template <typename T>
__global__ void gradfp_adj_k(T *du, const T *__restrict__ x, const T *__restrict__ y, const T *__restrict__ z, H3<T> h, Dims d)
{
    VOXEL_PROLOGUE
    const size_t NX = nx - 1, NY = nx * (ny - 1), NZ = nxny * (nz - 1);
    const T a = h.x * (x[l] - (i > 0 ? x[l - 1] : x[l + NX]));
    const T b = h.y * (y[l] - (j > 0 ? y[l - nx] : y[l + NY]));
    const T c = h.z * (z[l] - (k > 0 ? z[l - nxny] : z[l + NZ]));
    du[l] = k == 0 ? (a + b) + c : j == 0 ? (c + a) + b : (c + b) + a;
}

// ---- Laplacians -----------------------------------------------------------

// lap1_mex.c:208-315: one axis of the masked Laplacian.  sel = 3 central,
// 2 forward (4/3/2-point by availability), 1 backward, 0 none.
template <typename T>
__device__ __forceinline__ T lap_axis(const T *__restrict__ u, const uint8_t *__restrict__ G, size_t l, size_t a,
                                      size_t n, size_t i, int sel)
{
    switch (sel) {
    case 3: return u[l - a] - (T)2 * u[l] + u[l + a];
    case 2:
        if (i + 3 < n && G[l + 2 * a] && G[l + 3 * a])
            return (T)2 * u[l] - (T)5 * u[l + a] + (T)4 * u[l + 2 * a] - u[l + 3 * a];
        if (i + 2 < n && G[l + 2 * a]) return u[l] - (T)2 * u[l + a] + u[l + 2 * a];
        return u[l + a] - u[l];
    case 1:
        if (i >= 3 && G[l - 3 * a] && G[l - 2 * a])
            return -u[l - 3 * a] + (T)4 * u[l - 2 * a] - (T)5 * u[l - a] + (T)2 * u[l];
        if (i >= 2 && G[l - 2 * a]) return u[l - 2 * a] - (T)2 * u[l - a] + u[l];
        return u[l - a] - u[l];
    default: return (T)0;
    }
}

// lap1_mex.c:170-200: interior selector 2*G[+1] + G[-1]; faces forced.
__device__ __forceinline__ int lap_sel(const uint8_t *__restrict__ G, size_t l, size_t a, size_t i, size_t n)
{
    if (i >= 1 && i + 1 < n) return 2 * G[l + a] + G[l - a];
    return (i == 0) * 2 + (i + 1 == n);
}

// lap1_mex.c:136-205
template <typename T>
__global__ void lap1_k(T *du, const T *__restrict__ u, const uint8_t *__restrict__ G, H3<T> h, Dims d)
{
    VOXEL_PROLOGUE
    if (!G[l]) return;
    T v = h.x * lap_axis(u, G, l, 1, nx, i, lap_sel(G, l, 1, i, nx));
    v = v + h.y * lap_axis(u, G, l, nx, ny, j, lap_sel(G, l, nx, j, ny));
    v = v + h.z * lap_axis(u, G, l, nxny, nz, k, lap_sel(G, l, nxny, k, nz));
    du[l] = v;
}

// lapw_mex.c:10-11, :170-187: wrap into [-pi, pi] only when outside.
template <typename T>
__device__ __forceinline__ T wrap_pi(T x)
{
    const T pi = (T)3.14159265358979323846;
    const T tau = (T)(2 * 3.14159265358979323846);
    if (!(x < -pi || x > pi)) return x;
    x = x + pi;
    return x < (T)0 ? fmod(x, tau) + pi : fmod(x, tau) - pi;
}

// lapw_mex.c:54-167 (interior only)
template <typename T>
__global__ void lapw_k(T *du, const T *__restrict__ u, H3<T> h, Dims d)
{
    VOXEL_PROLOGUE
    if (i == 0 || j == 0 || k == 0 || i + 1 >= nx || j + 1 >= ny || k + 1 >= nz) return;
    T v = h.x * (wrap_pi(u[l + 1] - u[l]) - wrap_pi(u[l] - u[l - 1]));
    v = v + h.y * (wrap_pi(u[l + nx] - u[l]) - wrap_pi(u[l] - u[l - nx]));
    v = v + h.z * (wrap_pi(u[l + nxny] - u[l]) - wrap_pi(u[l] - u[l - nxny]));
    du[l] = v;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

template <typename T> static H3<T> inv_h(const double *h, double s)
{
    return H3<T>{(T)(s / h[0]), (T)(s / h[1]), (T)(s / h[2])};
}
template <typename T> static H3<T> inv_h2(const double *h)
{
    return H3<T>{(T)(1.0 / (h[0] * h[0])), (T)(1.0 / (h[1] * h[1])), (T)(1.0 / (h[2] * h[2]))};
}

enum FdOp {
    OP_GRADF, OP_GRADB, OP_GRADC, OP_GRADFM, OP_GRADBM, OP_GRADCM, OP_GRADFP,
    OP_GRADF_ADJ, OP_GRADB_ADJ, OP_GRADFM_ADJ, OP_GRADBM_ADJ, OP_GRADFP_ADJ,
    OP_LAP1, OP_LAPW
};

template <typename T>
static qsm_status launch_fd(qsm_ctx *ctx, FdOp op, const Dims &d, void **a, const uint8_t *G, const double *h)
{
    const dim3 g = vox_grid(d), b = vox_block();
    cudaStream_t s = ctx->stream;
    T *o0 = (T *)a[0], *o1 = (T *)a[1], *o2 = (T *)a[2];
    const T *i0 = (const T *)a[3], *i1 = (const T *)a[1], *i2 = (const T *)a[2];
    switch (op) {
    case OP_GRADF: gradf_k<T><<<g, b, 0, s>>>(o0, o1, o2, i0, inv_h<T>(h, 1.0), d); break;
    case OP_GRADB: gradb_k<T><<<g, b, 0, s>>>(o0, o1, o2, i0, inv_h<T>(h, 1.0), d); break;
    case OP_GRADC: gradc_k<T><<<g, b, 0, s>>>(o0, o1, o2, i0, inv_h<T>(h, 1.0), inv_h<T>(h, 0.5), d); break;
    case OP_GRADFM: gradfm_k<T><<<g, b, 0, s>>>(o0, o1, o2, i0, G, inv_h<T>(h, 1.0), d); break;
    case OP_GRADBM: gradbm_k<T><<<g, b, 0, s>>>(o0, o1, o2, i0, G, inv_h<T>(h, 1.0), d); break;
    case OP_GRADCM: gradcm_k<T><<<g, b, 0, s>>>(o0, o1, o2, i0, G, inv_h<T>(h, 1.0), inv_h<T>(h, 0.5), d); break;
    case OP_GRADFP: gradfp_k<T><<<g, b, 0, s>>>(o0, o1, o2, i0, inv_h<T>(h, 1.0), d); break;
    // adjoints: a = {du, x, y, z}
    case OP_GRADF_ADJ: gradf_adj_k<T><<<g, b, 0, s>>>(o0, (const T *)a[1], (const T *)a[2], (const T *)a[3], inv_h<T>(h, -1.0), d); break;
    case OP_GRADB_ADJ: gradb_adj_k<T><<<g, b, 0, s>>>(o0, (const T *)a[1], (const T *)a[2], (const T *)a[3], inv_h<T>(h, -1.0), d); break;
    case OP_GRADFM_ADJ: gradfm_adj_k<T><<<g, b, 0, s>>>(o0, (const T *)a[1], (const T *)a[2], (const T *)a[3], G, inv_h<T>(h, -1.0), d); break;
    case OP_GRADBM_ADJ: gradbm_adj_k<T><<<g, b, 0, s>>>(o0, (const T *)a[1], (const T *)a[2], (const T *)a[3], G, inv_h<T>(h, -1.0), d); break;
    case OP_GRADFP_ADJ: gradfp_adj_k<T><<<g, b, 0, s>>>(o0, (const T *)a[1], (const T *)a[2], (const T *)a[3], inv_h<T>(h, -1.0), d); break;
    // Laplacians: a = {d2u, u}
    case OP_LAP1: lap1_k<T><<<g, b, 0, s>>>(o0, (const T *)a[1], G, inv_h2<T>(h), d); break;
    case OP_LAPW: lapw_k<T><<<g, b, 0, s>>>(o0, (const T *)a[1], inv_h2<T>(h), d); break;
    }
    (void)i1; (void)i2;
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// Stages `narr` arrays (the first `nout` are written), the optional mask,
// launches, copies outputs back and waits.
static qsm_status run_fd(qsm_ctx *ctx, qsm_dtype dt, const size_t *dims, FdOp op, int narr, int nout,
                         void **arrs, const uint8_t *G, bool need_G, const double *vsz, size_t min_dim)
{
    if (!ctx || !dims || !vsz) return QSM_ERR_ARG;
    if (dt != QSM_F32 && dt != QSM_F64) return QSM_ERR_DTYPE;
    for (int q = 0; q < narr; ++q)
        if (!arrs[q]) return QSM_ERR_ARG;
    if (need_G && !G) return QSM_ERR_ARG;
    for (int q = 0; q < 3; ++q)
        if (dims[q] < min_dim) {
            set_error(ctx, "every dimension must be >= %zu", min_dim);
            return QSM_ERR_DIMS;
        }
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    const size_t es = dt == QSM_F32 ? 4 : 8;
    Staged st[5];
    void *dev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    for (int q = 0; q < narr; ++q) {
        // outputs are in-place: masked operators leave untouched voxels as
        // the caller had them, so outputs are copied in as well
        QSM_TRY(stage_in(ctx, st[q], arrs[q], d.n() * es, true));
        dev[q] = st[q].dev;
    }
    Staged sg;
    const uint8_t *gdev = nullptr;
    if (need_G) {
        QSM_TRY(stage_in(ctx, sg, G, d.n(), true));
        gdev = (const uint8_t *)sg.dev;
    }
    qsm_status s = dt == QSM_F32 ? launch_fd<float>(ctx, op, d, dev, gdev, vsz)
                                 : launch_fd<double>(ctx, op, d, dev, gdev, vsz);
    for (int q = 0; q < narr; ++q) QSM_TRY(stage_out(ctx, st[q], q < nout));
    if (need_G) QSM_TRY(stage_out(ctx, sg, false));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return s;
}

}  // namespace qsm

using namespace qsm;

extern "C" {

#define GRAD_API(name, OP, masked, mind)                                                               \
    qsm_status qsm_##name(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], void *dx, void *dy,       \
                          void *dz, const void *u, const double vsz[3])                               \
    {                                                                                                  \
        void *a[4] = {dx, dy, dz, const_cast<void *>(u)};                                              \
        return run_fd(ctx, dt, dims, OP, 4, 3, a, nullptr, false, vsz, mind);                          \
    }

GRAD_API(gradf, OP_GRADF, 0, 2)
GRAD_API(gradb, OP_GRADB, 0, 2)
GRAD_API(gradc, OP_GRADC, 0, 2)
GRAD_API(gradfp, OP_GRADFP, 0, 1)

#define GRADM_API(name, OP)                                                                            \
    qsm_status qsm_##name(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], void *dx, void *dy,       \
                          void *dz, const void *u, const uint8_t *G, const double vsz[3])             \
    {                                                                                                  \
        void *a[4] = {dx, dy, dz, const_cast<void *>(u)};                                              \
        return run_fd(ctx, dt, dims, OP, 4, 3, a, G, true, vsz, 1);                                    \
    }

GRADM_API(gradfm, OP_GRADFM)
GRADM_API(gradbm, OP_GRADBM)
GRADM_API(gradcm, OP_GRADCM)

#define ADJ_API(name, OP, mind)                                                                        \
    qsm_status qsm_##name(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], void *du, const void *x,  \
                          const void *y, const void *z, const double vsz[3])                          \
    {                                                                                                  \
        void *a[4] = {du, const_cast<void *>(x), const_cast<void *>(y), const_cast<void *>(z)};        \
        return run_fd(ctx, dt, dims, OP, 4, 1, a, nullptr, false, vsz, mind);                          \
    }

ADJ_API(gradf_adj, OP_GRADF_ADJ, 2)
ADJ_API(gradb_adj, OP_GRADB_ADJ, 2)
ADJ_API(gradfp_adj, OP_GRADFP_ADJ, 1)

#define ADJM_API(name, OP)                                                                             \
    qsm_status qsm_##name(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], void *du, const void *x,  \
                          const void *y, const void *z, const uint8_t *G, const double vsz[3])        \
    {                                                                                                  \
        void *a[4] = {du, const_cast<void *>(x), const_cast<void *>(y), const_cast<void *>(z)};        \
        return run_fd(ctx, dt, dims, OP, 4, 1, a, G, true, vsz, 1);                                    \
    }

ADJM_API(gradfm_adj, OP_GRADFM_ADJ)
ADJM_API(gradbm_adj, OP_GRADBM_ADJ)

qsm_status qsm_lap1(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], void *d2u, const void *u, const uint8_t *G,
                    const double vsz[3])
{
    void *a[2] = {d2u, const_cast<void *>(u)};
    return run_fd(ctx, dt, dims, OP_LAP1, 2, 1, a, G, true, vsz, 2);
}

qsm_status qsm_lapw(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], void *d2u, const void *u, const double vsz[3])
{
    void *a[2] = {d2u, const_cast<void *>(u)};
    return run_fd(ctx, dt, dims, OP_LAPW, 2, 1, a, nullptr, false, vsz, 1);
}

}  // extern "C"
