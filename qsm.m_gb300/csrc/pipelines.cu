// MATLAB-level pipelines of QSM.m on the device: the mask bounding-box crop,
// the echo loop and the MEX calls of
//   sstgv.m:1-71            x = sstgv(phas, mask, vsz, lambda, alpha, tol, maxit, verbose)
//   lbv.m:1-113             fl = lbv(f, mask, vsz, tol, maxit, mgopts, verbose)
//   unwrapLaplacian.m:1-87  [uphas, d2phas] = unwrapLaplacian(phas, mask, vsz)
// composed from this library's gateways (lapw, lap1, pd_tgv/pd_tv, mgpcg)
// with device arrays, so nothing returns to the host between steps.  The
// crop box is cropIndices(mask) (src/utils/cropIndices.m) grown by 2 (sstgv)
// or 1 (lbv, unwrapLaplacian) voxels and clamped to the volume; outputs are
// zero outside it, as the wrappers' zeros(size(...)) + indexed assignment.
// Multi-echo inputs are [nx, ny, nz, ne] with echo t at offset t*nx*ny*nz;
// sstgv with the fused path advances all echoes together in one batch.
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace qsm {

// bounding box of the mask: min/max of x, y, z over voxels with mask != 0
__global__ void bbox_k(unsigned *bb, const uint8_t *__restrict__ m, Dims d)
{
    __shared__ unsigned s[6][256];
    unsigned lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0, 0, 0};
    const size_t N = d.n();
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < N; l += (size_t)gridDim.x * blockDim.x) {
        if (!m[l]) continue;
        const unsigned c[3] = {(unsigned)(l % d.nx), (unsigned)((l / d.nx) % d.ny), (unsigned)(l / d.nxny())};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = min(lo[a], c[a]);
            hi[a] = max(hi[a], c[a]);
        }
    }
    const int t = threadIdx.x;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        s[a][t] = lo[a];
        s[3 + a][t] = hi[a];
    }
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (t < st)
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                s[a][t] = min(s[a][t], s[a][t + st]);
                s[3 + a][t] = max(s[3 + a][t], s[3 + a][t + st]);
            }
        __syncthreads();
    }
    if (t == 0)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            atomicMin(bb + a, s[a][0]);
            atomicMax(bb + 3 + a, s[3 + a][0]);
        }
}

struct Box {
    size_t x0, y0, z0;  // first voxel of the crop (0-based)
    Dims c;             // cropped size
};

// o (cropped) = a (full) on the box
template <typename T>
__global__ void crop_k(T *o, const T *__restrict__ a, Dims d, Box b)
{
    const size_t n = b.c.n();
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
        const size_t i = l % b.c.nx, j = (l / b.c.nx) % b.c.ny, k = l / b.c.nxny();
        o[l] = a[(b.x0 + i) + d.nx * ((b.y0 + j) + d.ny * (b.z0 + k))];
    }
}

// full = 0 outside the box, cropped values inside
template <typename T>
__global__ void scatter_k(T *full, const T *__restrict__ c, Dims d, Box b)
{
    const size_t N = d.n();
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < N; l += (size_t)gridDim.x * blockDim.x) {
        const size_t i = l % d.nx, j = (l / d.nx) % d.ny, k = l / d.nxny();
        const bool in = i >= b.x0 && i < b.x0 + b.c.nx && j >= b.y0 && j < b.y0 + b.c.ny && k >= b.z0 && k < b.z0 + b.c.nz;
        full[l] = in ? c[(i - b.x0) + b.c.nx * ((j - b.y0) + b.c.ny * (k - b.z0))] : (T)0;
    }
}

// o = -a (sstgv.m:79-87, lbv.m:112), or o = -(m .* a) (unwrapLaplacian.m:86)
template <typename T>
__global__ void neg_k(T *o, const T *__restrict__ a, const uint8_t *__restrict__ m, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        o[l] = m ? -((T)(m[l] ? 1 : 0) * a[l]) : -a[l];
}

static unsigned grid_for(size_t n) { return (unsigned)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 8 * 152)); }

// cropIndices(mask): the first and last index of each axis that holds a mask
// voxel (src/utils/cropIndices.m); QSM_ERR_ARG for an empty mask
qsm_status mask_bbox(qsm_ctx *ctx, const uint8_t *mask_dev, const Dims &d, size_t lo[3], size_t hi[3])
{
    unsigned *bb = nullptr;
    QSM_TRY(dalloc(ctx, (void **)&bb, 6 * sizeof(unsigned)));
    const unsigned init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0, 0, 0};
    QSM_CUDA(cudaMemcpyAsync(bb, init, sizeof init, cudaMemcpyHostToDevice, ctx->stream));
    bbox_k<<<grid_for(d.n()), 256, 0, ctx->stream>>>(bb, mask_dev, d);
    QSM_CUDA(cudaGetLastError());
    unsigned h[6];
    QSM_CUDA(cudaMemcpyAsync(h, bb, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    QSM_TRY(dfree(ctx, bb));
    if (h[0] > h[3]) {
        set_error(ctx, "the mask is empty (cropIndices finds no voxel)");
        return QSM_ERR_ARG;
    }
    for (int a = 0; a < 3; ++a) {
        lo[a] = h[a];
        hi[a] = h[3 + a];
    }
    return QSM_OK;
}

// cropIndices(mask) grown by `pad` and clamped (sstgv.m:57-63, lbv.m:86-92)
static qsm_status crop_box(qsm_ctx *ctx, const uint8_t *mask_dev, const Dims &d, int pad, Box *b)
{
    size_t h[3], g[3];
    QSM_TRY(mask_bbox(ctx, mask_dev, d, h, g));
    const size_t n[3] = {d.nx, d.ny, d.nz};
    size_t lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = h[a] >= (size_t)pad ? h[a] - pad : 0;
        hi[a] = std::min<size_t>(n[a] - 1, g[a] + pad);
    }
    b->x0 = lo[0];
    b->y0 = lo[1];
    b->z0 = lo[2];
    b->c = Dims{hi[0] - lo[0] + 1, hi[1] - lo[1] + 1, hi[2] - lo[2] + 1};
    return QSM_OK;
}

template <typename T>
static void crop(qsm_ctx *ctx, T *o, const T *a, const Dims &d, const Box &b)
{
    crop_k<T><<<grid_for(b.c.n()), 256, 0, ctx->stream>>>(o, a, d, b);
}

template <typename T>
static void scatter(qsm_ctx *ctx, T *full, const T *c, const Dims &d, const Box &b)
{
    scatter_k<T><<<grid_for(d.n()), 256, 0, ctx->stream>>>(full, c, d, b);
}

}  // namespace qsm

using namespace qsm;

namespace {

Dims dims3(const size_t *dims) { return Dims{dims[0], dims[1], dims[2]}; }

// mgpcg.m:33-35: nlevels = max(1, floor(log2(min(size(f)))) - 3)
int32_t default_levels(const Dims &c)
{
    const size_t m = std::min(c.nx, std::min(c.ny, c.nz));
    return std::max(1, (int)std::floor(std::log2((double)m)) - 3);
}

qsm_status launch_check(qsm_ctx *ctx, const char *what)
{
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return QSM_OK;
    set_error(ctx, "%s: %s", what, cudaGetErrorString(e));
    return QSM_ERR_CUDA;
}

template <typename T>
qsm_status run_sstgv(qsm_ctx *ctx, const Dims &d, size_t ne, const T *phas, const uint8_t *mask,
                     const double *vsz, double lambda, double alpha, double tol, uint32_t maxit, uint32_t verbose,
                     bool fused, T *x, qsm_pd_info *info)
{
    const qsm_dtype dt = sizeof(T) == 4 ? QSM_F32 : QSM_F64;
    Box b;
    QSM_TRY(crop_box(ctx, mask, d, 2, &b));
    const size_t N = d.n(), n = b.c.n();
    const size_t cd[3] = {b.c.nx, b.c.ny, b.c.nz};
    // cropped mask; per echo: cropped phase, -d2u, chi
    void *blk = nullptr;
    const size_t vb = (n * sizeof(T) + 255) & ~(size_t)255, mb = (n + 255) & ~(size_t)255;
    QSM_TRY(dalloc(ctx, &blk, mb + 3 * ne * vb));
    uint8_t *m = (uint8_t *)blk;
    T *u = (T *)((char *)blk + mb), *f = (T *)((char *)u + ne * vb), *chi = (T *)((char *)f + ne * vb);
    auto ech = [&](T *base, size_t t) { return (T *)((char *)base + t * vb); };
    qsm_status st = QSM_OK;
    crop<uint8_t>(ctx, m, mask, d, b);
    for (size_t t = 0; t < ne && st == QSM_OK; ++t) {
        crop<T>(ctx, ech(u, t), phas + t * N, d, b);
        if (cudaMemsetAsync(ech(f, t), 0, n * sizeof(T), ctx->stream) != cudaSuccess) st = launch_check(ctx, "sstgv");
        if (st == QSM_OK) st = qsm_lapw(ctx, dt, cd, ech(f, t), ech(u, t), vsz);  // d2u = lapw(u, h)
        if (st == QSM_OK) {
            neg_k<T><<<grid_for(n), 256, 0, ctx->stream>>>(ech(f, t), ech(f, t), nullptr, n);
            st = launch_check(ctx, "sstgv");
        }
    }
    const bool tgv = alpha > 2.220446049250313e-16;  // sstgv.m:83 (alpha > eps)
    if (st == QSM_OK && fused && ne > 1) {
        std::vector<size_t> dims(3 * ne);
        std::vector<const void *> fs(ne);
        std::vector<const uint8_t *> ms(ne, m);
        std::vector<void *> xs(ne);
        for (size_t t = 0; t < ne; ++t) {
            for (int a = 0; a < 3; ++a) dims[3 * t + a] = cd[a];
            fs[t] = ech(f, t);
            xs[t] = ech(chi, t);
        }
        st = tgv ? qsm_pd_tgv_batch(ctx, dt, (uint32_t)ne, dims.data(), fs.data(), ms.data(), vsz, lambda, alpha, tol,
                                    maxit, xs.data(), info)
                 : qsm_pd_tv_batch(ctx, dt, (uint32_t)ne, dims.data(), fs.data(), ms.data(), vsz, lambda, tol, maxit,
                                   xs.data(), info);
    } else {
        for (size_t t = 0; t < ne && st == QSM_OK; ++t) {
            qsm_pd_info *it = info ? info + t : nullptr;
            if (tgv)
                st = fused ? qsm_pd_tgv_fused(ctx, dt, cd, ech(f, t), m, vsz, lambda, alpha, tol, maxit, verbose,
                                              ech(chi, t), it)
                           : qsm_pd_tgv(ctx, dt, cd, ech(f, t), m, vsz, lambda, alpha, tol, maxit, verbose, ech(chi, t), it);
            else
                st = fused ? qsm_pd_tv_fused(ctx, dt, cd, ech(f, t), m, vsz, lambda, tol, maxit, verbose, ech(chi, t), it)
                           : qsm_pd_tv(ctx, dt, cd, ech(f, t), m, vsz, lambda, tol, maxit, verbose, ech(chi, t), it);
        }
    }
    for (size_t t = 0; t < ne && st == QSM_OK; ++t) scatter<T>(ctx, x + t * N, ech(chi, t), d, b);
    if (st == QSM_OK) st = launch_check(ctx, "sstgv");
    qsm_status s2 = dfree(ctx, blk);
    return st != QSM_OK ? st : s2;
}

// lbv_ (lbv.m:108-113) and unwrap_ (unwrapLaplacian.m:79-87) share: a
// Laplacian of the cropped input, its negation, mgpcg with LBV's options.
template <typename T>
qsm_status run_poisson(qsm_ctx *ctx, bool unwrap, const Dims &d, size_t ne, const T *in, const uint8_t *mask,
                       const double *vsz, double tol, int32_t maxit, int32_t mg_maxit, int32_t npre, int32_t npost,
                       int32_t nb, int32_t verbose, bool mixed, T *out, T *d2out, qsm_mg_info *info)
{
    const qsm_dtype dt = sizeof(T) == 4 ? QSM_F32 : QSM_F64;
    Box b;
    QSM_TRY(crop_box(ctx, mask, d, 1, &b));
    const size_t N = d.n(), n = b.c.n();
    const size_t cd[3] = {b.c.nx, b.c.ny, b.c.nz};
    void *blk = nullptr;
    const size_t vb = (n * sizeof(T) + 255) & ~(size_t)255, mb = (n + 255) & ~(size_t)255;
    QSM_TRY(dalloc(ctx, &blk, mb + 4 * vb));
    uint8_t *m = (uint8_t *)blk;
    T *u = (T *)((char *)blk + mb), *d2u = (T *)((char *)u + vb), *f = (T *)((char *)d2u + vb),
      *v = (T *)((char *)f + vb);
    const int32_t nl = default_levels(b.c);
    // unwrapLaplacian.m:84: maxitcg = ceil(sqrt(numel(m))) of the cropped mask
    const int32_t mx = unwrap ? (int32_t)std::ceil(std::sqrt((double)n)) : maxit;
    qsm_status st = QSM_OK;
    crop<uint8_t>(ctx, m, mask, d, b);
    for (size_t t = 0; t < ne && st == QSM_OK; ++t) {
        crop<T>(ctx, u, in + t * N, d, b);
        if (cudaMemsetAsync(d2u, 0, n * sizeof(T), ctx->stream) != cudaSuccess) st = launch_check(ctx, "poisson");
        if (st == QSM_OK)
            st = unwrap ? qsm_lapw(ctx, dt, cd, d2u, u, vsz)       // d2u = lapw(u, h)
                        : qsm_lap1(ctx, dt, cd, d2u, u, m, vsz);   // d2u = lap(u, m, h)
        if (st != QSM_OK) break;
        neg_k<T><<<grid_for(n), 256, 0, ctx->stream>>>(f, d2u, unwrap ? m : nullptr, n);
        st = launch_check(ctx, unwrap ? "unwrapLaplacian" : "lbv");
        if (st == QSM_OK && cudaMemsetAsync(v, 0, n * sizeof(T), ctx->stream) != cudaSuccess)
            st = launch_check(ctx, "poisson");
        if (st != QSM_OK) break;
        qsm_mg_info *it = info ? info + t : nullptr;
        double *hist = it ? it->resnorm_hist : nullptr;
        if (it) it->resnorm_hist = nullptr;
        if (mixed && dt == QSM_F64)
            st = qsm_mgpcg_mixed(ctx, cd, (const double *)v, (const double *)f, m, vsz, tol, mx, -1.0, mg_maxit, 1,
                                 npre, npost, nb, nl, verbose, (double *)v, it);
        else
            st = qsm_mgpcg(ctx, dt, cd, v, f, m, vsz, tol, mx, -1.0, mg_maxit, 1, npre, npost, nb, nl, verbose, v, it);
        if (it) it->resnorm_hist = hist;
        if (st != QSM_OK) break;
        scatter<T>(ctx, out + t * N, v, d, b);
        if (d2out) scatter<T>(ctx, d2out + t * N, d2u, d, b);
    }
    if (st == QSM_OK) st = launch_check(ctx, unwrap ? "unwrapLaplacian" : "lbv");
    qsm_status s2 = dfree(ctx, blk);
    return st != QSM_OK ? st : s2;
}

bool check_dims4(const size_t *dims) { return dims && dims[0] && dims[1] && dims[2] && dims[3]; }

struct Io {
    Staged in{}, mask{}, out{}, out2{};
    void release(qsm_ctx *ctx)
    {
        stage_out(ctx, in, false);
        stage_out(ctx, mask, false);
        stage_out(ctx, out, false);
        stage_out(ctx, out2, false);
    }
};

}  // namespace

extern "C" {

qsm_status qsm_sstgv(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[4], const void *phas, const uint8_t *mask,
                     const double vsz[3], double lambda, double alpha, double tol, uint32_t maxit, uint32_t verbose,
                     int32_t fused, void *x, qsm_pd_info *info)
{
    Range nvtx_range("sstgv");
    if (!ctx || !phas || !mask || !vsz || !x) return QSM_ERR_ARG;
    if (dt != QSM_F32 && dt != QSM_F64) return QSM_ERR_DTYPE;
    if (!check_dims4(dims)) return QSM_ERR_DIMS;
    cudaSetDevice(ctx->device);
    const Dims d = dims3(dims);
    const size_t ne = dims[3], es = dt == QSM_F32 ? 4 : 8;
    Io io;
    QSM_TRY(stage_in(ctx, io.in, phas, ne * d.n() * es, true));
    QSM_TRY(stage_in(ctx, io.mask, mask, d.n(), true));
    QSM_TRY(stage_in(ctx, io.out, x, ne * d.n() * es, false));
    qsm_status st = dt == QSM_F32
                        ? run_sstgv<float>(ctx, d, ne, (const float *)io.in.dev, (const uint8_t *)io.mask.dev, vsz,
                                           lambda, alpha, tol, maxit, verbose, fused != 0, (float *)io.out.dev, info)
                        : run_sstgv<double>(ctx, d, ne, (const double *)io.in.dev, (const uint8_t *)io.mask.dev, vsz,
                                            lambda, alpha, tol, maxit, verbose, fused != 0, (double *)io.out.dev, info);
    if (st != QSM_OK) {
        io.release(ctx);
        return st;
    }
    stage_out(ctx, io.in, false);
    stage_out(ctx, io.mask, false);
    QSM_TRY(stage_out(ctx, io.out, true));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return QSM_OK;
}

static qsm_status poisson_entry(qsm_ctx *ctx, bool unwrap, qsm_dtype dt, const size_t dims[4], const void *in,
                                const uint8_t *mask, const double vsz[3], double tol, int32_t maxit, int32_t mg_maxit,
                                int32_t npre, int32_t npost, int32_t nb, int32_t verbose, int32_t mixed, void *out,
                                void *d2out, qsm_mg_info *info)
{
    if (!ctx || !in || !mask || !vsz || !out) return QSM_ERR_ARG;
    if (dt != QSM_F32 && dt != QSM_F64) return QSM_ERR_DTYPE;
    if (!check_dims4(dims)) return QSM_ERR_DIMS;
    cudaSetDevice(ctx->device);
    const Dims d = dims3(dims);
    const size_t ne = dims[3], es = dt == QSM_F32 ? 4 : 8;
    Io io;
    QSM_TRY(stage_in(ctx, io.in, in, ne * d.n() * es, true));
    QSM_TRY(stage_in(ctx, io.mask, mask, d.n(), true));
    QSM_TRY(stage_in(ctx, io.out, out, ne * d.n() * es, false));
    if (d2out) QSM_TRY(stage_in(ctx, io.out2, d2out, ne * d.n() * es, false));
    qsm_status st =
        dt == QSM_F32
            ? run_poisson<float>(ctx, unwrap, d, ne, (const float *)io.in.dev, (const uint8_t *)io.mask.dev, vsz, tol,
                                 maxit, mg_maxit, npre, npost, nb, verbose, false, (float *)io.out.dev,
                                 d2out ? (float *)io.out2.dev : nullptr, info)
            : run_poisson<double>(ctx, unwrap, d, ne, (const double *)io.in.dev, (const uint8_t *)io.mask.dev, vsz,
                                  tol, maxit, mg_maxit, npre, npost, nb, verbose, mixed != 0, (double *)io.out.dev,
                                  d2out ? (double *)io.out2.dev : nullptr, info);
    if (st != QSM_OK) {
        io.release(ctx);
        return st;
    }
    stage_out(ctx, io.in, false);
    stage_out(ctx, io.mask, false);
    QSM_TRY(stage_out(ctx, io.out, true));
    if (d2out) QSM_TRY(stage_out(ctx, io.out2, true));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return QSM_OK;
}

qsm_status qsm_lbv(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[4], const void *f, const uint8_t *mask,
                   const double vsz[3], double tol, int32_t maxit, int32_t mg_maxit, int32_t npre, int32_t npost,
                   int32_t nboundary, int32_t verbose, int32_t mixed, void *fl, qsm_mg_info *info)
{
    Range nvtx_range("lbv");
    if (dims && maxit <= 0)  // lbv.m:60: ceil(sqrt(numel(mask))) of the full mask
        maxit = (int32_t)std::ceil(std::sqrt((double)dims[0] * (double)dims[1] * (double)dims[2]));
    return poisson_entry(ctx, false, dt, dims, f, mask, vsz, tol, maxit, mg_maxit, npre, npost, nboundary, verbose,
                         mixed, fl, nullptr, info);
}

qsm_status qsm_unwrap_laplacian(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[4], const void *phas,
                                const uint8_t *mask, const double vsz[3], int32_t mixed, void *uphas, void *d2phas)
{
    // unwrapLaplacian.m:81-86: tolcg 1e-8, mg maxit 2, npre = npost = 2, nboundary 2
    return poisson_entry(ctx, true, dt, dims, phas, mask, vsz, 1e-8, 0, 2, 2, 2, 2, 0, mixed, uphas, d2phas, nullptr);
}

}  // extern "C"
