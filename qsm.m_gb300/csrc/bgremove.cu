// FFT background-field removal of QSM.m on the GPU:
//   sharp.m:1-84    [fl, mask] = sharp(f, mask, vsz, r, thr)
//   vsharp.m:1-153  [fl, mask] = vsharp(f, mask, vsz, rs, thr)
//   ismv.m:1-112    [fl, mask] = ismv(f, mask, vsz, r, tol, maxit, verbose)
//   pdf.m:1-86      fl = pdf(f, mask, vsz, w, bdir, lambda, tol, maxit, verbose): LSMR
//                   (Fong & Saunders 2011) on the dipole projection, full grid
//   resharp.m:1-88  [fl, mask] = resharp(f, mask, vsz, r, lambda, tol, maxit), its
//                   Tikhonov system solved by conjugate gradients squared (CGS,
//                   Sonneveld 1989, without preconditioner, x0 = 0, stopping when
//                   the recursively updated residual is <= tol * ||b||)
// Each crops f and the mask to cropIndices(mask), zero-pads them to a
// 7-smooth size (padfastfft.m with nextfastfft, third_party/nextfastfft.m),
// and works with spherical-mean-value (SMV) kernels (smvKernel.m): the kernel
// is written on the device directly in ifftshifted order, its spectrum taken
// with one cuFFT R2C (it is real and even, so its transform is real), and
// every convolution is an R2C, one pointwise kernel, a C2R.  Eroded masks
// are real(ifft3(H .* fft3(single(mask)))) > 0.999 in FP32, as the MATLAB
// code evaluates them (single mask, so single FFTs); the field arithmetic is
// in the class of f.  Reductions (iSMV residuals) accumulate in FP64 in a
// fixed order.
#include <cufft.h>
#include <float.h>
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace qsm {

qsm_status mask_bbox(qsm_ctx *ctx, const uint8_t *mask, const Dims &d, size_t lo[3], size_t hi[3]);  // pipelines.cu

namespace {

template <typename T> struct Cx;
template <> struct Cx<double> { using type = cufftDoubleComplex; };
template <> struct Cx<float> { using type = cufftComplex; };

constexpr int BG_BLOCK = 256;
constexpr int BG_GRID = 4 * 152;

unsigned grid_for(size_t n) { return (unsigned)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 8 * 152)); }

// smallest m >= n whose prime factors are all <= 7 (nextfastfft.m)
size_t next_fast(size_t n)
{
    for (size_t m = std::max<size_t>(n, 1);; ++m) {
        size_t k = m;
        for (size_t p : {2, 3, 5, 7})
            while (k % p == 0) k /= p;
        if (k == 1) return m;
    }
}

// padded grid of padfastfft(u(ix,iy,iz), pad) and the crop it holds
struct Grid {
    Dims full{};          // input volume
    size_t c0[3] = {};    // crop origin in the input (cropIndices)
    size_t sz[3] = {};    // crop size
    size_t pre[3] = {};   // zeros before the crop in the padded grid
    Dims p{};             // padded size
    size_t nh = 0;        // half-spectrum points (px/2+1) * py * pz
};

// padfastfft.m 'both': total = nextfastfft(sz + 2 pad) - sz, split in halves,
// an odd total puts the extra voxel before the data when sz is odd, after
// it when sz is even
void pad_sizes(Grid &g, size_t pad)
{
    size_t ps[3];
    for (int a = 0; a < 3; ++a) {
        const size_t tot = pad ? next_fast(g.sz[a] + 2 * pad) - g.sz[a] : 0;
        const size_t half = tot / 2, odd = tot & 1, oddpre = odd & (g.sz[a] & 1);
        g.pre[a] = half + oddpre;
        ps[a] = g.sz[a] + tot;
    }
    g.p = Dims{ps[0], ps[1], ps[2]};
    g.nh = (ps[0] / 2 + 1) * ps[1] * ps[2];
}

// padded p = the crop of a (zeros around it)
template <typename S, typename T>
__global__ void pad_k(T *p, const S *__restrict__ a, Dims d, Dims pd, size_t c0x, size_t c0y, size_t c0z, size_t sx,
                      size_t sy, size_t sz, size_t px0, size_t py0, size_t pz0)
{
    const size_t N = pd.n();
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < N; l += (size_t)gridDim.x * blockDim.x) {
        const size_t i = l % pd.nx, j = (l / pd.nx) % pd.ny, k = l / pd.nxny();
        T v = (T)0;
        if (i >= px0 && i < px0 + sx && j >= py0 && j < py0 + sy && k >= pz0 && k < pz0 + sz)
            v = (T)a[(c0x + i - px0) + d.nx * ((c0y + j - py0) + d.ny * (c0z + k - pz0))];
        p[l] = v;
    }
}

// full = 0 outside the crop, the padded grid's crop inside (unpadfastfft + fl(ix,iy,iz) = ...)
template <typename T>
__global__ void unpad_k(T *full, const T *__restrict__ p, Dims d, Dims pd, size_t c0x, size_t c0y, size_t c0z,
                        size_t sx, size_t sy, size_t sz, size_t px0, size_t py0, size_t pz0)
{
    const size_t N = d.n();
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < N; l += (size_t)gridDim.x * blockDim.x) {
        const size_t i = l % d.nx, j = (l / d.nx) % d.ny, k = l / d.nxny();
        T v = (T)0;
        if (i >= c0x && i < c0x + sx && j >= c0y && j < c0y + sy && k >= c0z && k < c0z + sz)
            v = p[(px0 + i - c0x) + pd.nx * ((py0 + j - c0y) + pd.ny * (pz0 + k - c0z))];
        full[l] = v;
    }
}

// smvKernel(size, r, vsz) / its sum, in ifftshifted order: index i on an
// axis of n points is the offset i (i <= high) or i - n, high = floor(n/2) -
// (n even); inside when (y^2 + x^2) + z^2 <= r^2 (smvKernel.m:29-35)
__device__ __forceinline__ double shift_coord(size_t i, size_t n, double h)
{
    const size_t high = n / 2 - ((n & 1) ? 0 : 1);
    return (i <= high ? (double)i : (double)i - (double)n) * h;
}

template <typename T>
__global__ void smv_k(T *h, Dims pd, double hx, double hy, double hz, double r2, double inv_count)
{
    const size_t N = pd.n();
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < N; l += (size_t)gridDim.x * blockDim.x) {
        const double x = shift_coord(l % pd.nx, pd.nx, hx), y = shift_coord((l / pd.nx) % pd.ny, pd.ny, hy),
                     z = shift_coord(l / pd.nxny(), pd.nz, hz);
        h[l] = (y * y + x * x + z * z <= r2) ? (T)inv_count : (T)0;
    }
}

// number of grid points inside the sphere (the kernel's sum)
size_t smv_count(const Dims &pd, const double *h, double r)
{
    const size_t n[3] = {pd.nx, pd.ny, pd.nz};
    long lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        const long low = (long)(n[a] / 2), high = low - ((n[a] & 1) ? 0 : 1);
        const long R = (long)std::floor(r / h[a]) + 1;
        lo[a] = -std::min(low, R);
        hi[a] = std::min(high, R);
    }
    size_t c = 0;
    for (long k = lo[2]; k <= hi[2]; ++k)
        for (long j = lo[1]; j <= hi[1]; ++j)
            for (long i = lo[0]; i <= hi[0]; ++i) {
                const double x = (double)i * h[0], y = (double)j * h[1], z = (double)k * h[2];
                if (y * y + x * x + z * z <= r * r) ++c;
            }
    return c;
}

template <typename T>
__global__ void real_part_k(T *H, float *H32, const typename Cx<T>::type *__restrict__ c, size_t nh)
{
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nh; q += (size_t)gridDim.x * blockDim.x) {
        const T v = c[q].x;
        H[q] = v;
        H32[q] = (float)v;
    }
}

// M *= H (single)
__global__ void mul_f32_k(cufftComplex *M, const float *__restrict__ H, size_t nh)
{
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nh; q += (size_t)gridDim.x * blockDim.x) {
        const float h = H[q];
        M[q].x = h * M[q].x;
        M[q].y = h * M[q].y;
    }
}

// eroded mask: real(ifft3(...)) > 0.999, the single value compared as a double
__global__ void thresh_k(uint8_t *m, const float *__restrict__ c, float invn, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        m[l] = (double)(c[l] * invn) > 0.999 ? 1 : 0;
}

// F *= (1 - H)  (sharp.m:62-66: h = 1 - h; h .* fft3(f)), or F *= H when one_minus is false
template <typename T>
__global__ void mul_h_k(typename Cx<T>::type *F, const T *__restrict__ H, size_t nh, bool one_minus)
{
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nh; q += (size_t)gridDim.x * blockDim.x) {
        const T h = one_minus ? (T)1 - H[q] : H[q];
        F[q].x = h * F[q].x;
        F[q].y = h * F[q].y;
    }
}

// G = (1 - H) .* F, F kept (vsharp.m:122: hf = ifft3(h .* F))
template <typename T>
__global__ void mul_1mh_to_k(typename Cx<T>::type *G, const typename Cx<T>::type *__restrict__ F,
                             const T *__restrict__ H, size_t nh)
{
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nh; q += (size_t)gridDim.x * blockDim.x) {
        const T h = (T)1 - H[q];
        typename Cx<T>::type o;
        o.x = h * F[q].x;
        o.y = h * F[q].y;
        G[q] = o;
    }
}

// deconvolution by (1 - H) with truncation: f = fft3(f) ./ h; f(abs(h) < thr) = 0 (sharp.m:69-70)
template <typename T>
__global__ void deconv_k(typename Cx<T>::type *F, const T *__restrict__ H, T thr, size_t nh)
{
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nh; q += (size_t)gridDim.x * blockDim.x) {
        const T h = (T)1 - H[q];
        if (fabs(h) < thr) {
            F[q].x = (T)0;
            F[q].y = (T)0;
        } else {
            F[q].x = F[q].x / h;
            F[q].y = F[q].y / h;
        }
    }
}

// ih = 1 ./ (1 - H); ih(abs(1 - H) < thr) = 0 (vsharp.m:100-101), applied to F
template <typename T>
__global__ void mul_inv_k(typename Cx<T>::type *F, const T *__restrict__ H, T thr, size_t nh)
{
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nh; q += (size_t)gridDim.x * blockDim.x) {
        const T h = (T)1 - H[q];
        const T ih = fabs(h) < thr ? (T)0 : (T)1 / h;
        F[q].x = ih * F[q].x;
        F[q].y = ih * F[q].y;
    }
}

// g = m .* (ifft value): the C2R output times 1/N, times the mask
template <typename T>
__global__ void mask_scale_k(T *g, const uint8_t *__restrict__ m, T invn, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        g[l] = (T)(m[l] ? 1 : 0) * (g[l] * invn);
}

// acc += (mk - mprev) .* (ifft value)  (vsharp.m:124, :143)
template <typename T>
__global__ void vsharp_acc_k(T *acc, const T *__restrict__ g, const uint8_t *__restrict__ mk,
                             const uint8_t *__restrict__ mprev, T invn, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        acc[l] = acc[l] + ((T)(mk[l] ? 1 : 0) - (T)(mprev[l] ? 1 : 0)) * (g[l] * invn);
}

template <int NS>
__device__ __forceinline__ void block_sums(double *part, double (&acc)[NS])
{
    __shared__ double red[NS][BG_BLOCK];
    const int t = threadIdx.x;
#pragma unroll
    for (int q = 0; q < NS; ++q) red[q][t] = acc[q];
    __syncthreads();
    for (int s = BG_BLOCK / 2; s > 0; s >>= 1) {
        if (t < s)
#pragma unroll
            for (int q = 0; q < NS; ++q) red[q][t] += red[q][t + s];
        __syncthreads();
    }
    if (t == 0)
#pragma unroll
        for (int q = 0; q < NS; ++q) part[q * gridDim.x + blockIdx.x] = red[q][0];
}

// the block partials summed in a fixed order: thread t adds partials t, t + 256,
// ... in turn, then a shared-memory tree (one block of BG_BLOCK threads)
__global__ void __launch_bounds__(BG_BLOCK) fold_k(double *out, const double *__restrict__ part, int nblk)
{
    __shared__ double red[BG_BLOCK];
    const int t = threadIdx.x;
    double s = 0.0;
    for (int b = t; b < nblk; b += BG_BLOCK) s += part[b];
    red[t] = s;
    __syncthreads();
    for (int h = BG_BLOCK / 2; h > 0; h >>= 1) {
        if (t < h) red[t] += red[t + h];
        __syncthreads();
    }
    if (t == 0) *out = red[0];
}

// iSMV set-up (ismv.m:68-73): bc = (mask1 - m) .* f; sum (m .* f)^2
template <typename T>
__global__ void __launch_bounds__(BG_BLOCK)
ismv_init_k(T *bc, const T *__restrict__ f, const uint8_t *__restrict__ m1, const uint8_t *__restrict__ m, size_t n,
            double *part)
{
    PartialSum<T> ps;
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
        const T v = f[l];
        bc[l] = ((T)(m1[l] ? 1 : 0) - (T)(m[l] ? 1 : 0)) * v;
        const T w = (T)(m[l] ? 1 : 0) * v;
        ps.add(w * w);
    }
    double acc[1] = {ps.get()};
    block_sums<1>(part, acc);
}

// one iSMV step (ismv.m:97-99): f = bc + m .* real(ifft3(h .* fft3(f))); sum (f0 - f)^2
template <typename T>
__global__ void __launch_bounds__(BG_BLOCK)
ismv_step_k(T *f, const T *__restrict__ g, const T *__restrict__ bc, const uint8_t *__restrict__ m, T invn, size_t n,
            double *part)
{
    PartialSum<T> ps;
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
        const T fn = bc[l] + (T)(m[l] ? 1 : 0) * (g[l] * invn);
        const T dlt = f[l] - fn;
        ps.add(dlt * dlt);
        f[l] = fn;
    }
    double acc[1] = {ps.get()};
    block_sums<1>(part, acc);
}

// fl_ = m .* (ft - fb)  (ismv.m:76)
template <typename T>
__global__ void ismv_out_k(T *o, const T *__restrict__ ft, const T *__restrict__ fb, const uint8_t *__restrict__ m,
                           size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        o[l] = (T)(m[l] ? 1 : 0) * (ft[l] - fb[l]);
}

// out = mask1 .* (ifft value) + lambda .* v  (resharp.m:64-68, the operator A)
template <typename T>
__global__ void resharp_op_k(T *out, const T *__restrict__ v, const uint8_t *__restrict__ m, T invn, T lam, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        out[l] = (T)(m[l] ? 1 : 0) * (out[l] * invn) + lam * v[l];
}

// sum x .* y in FP64, fixed order (block partials, then fold_k)
template <typename T>
__global__ void __launch_bounds__(BG_BLOCK)
dot_k(const T *__restrict__ x, const T *__restrict__ y, size_t n, double *part)
{
    PartialSum<T> ps;
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        ps.add(x[l] * y[l]);
    double acc[1] = {ps.get()};
    block_sums<1>(part, acc);
}

// CGS direction updates: u = r + beta q; p = u + beta (q + beta p)
template <typename T>
__global__ void cgs_dir_k(T *u, T *p, const T *__restrict__ r, const T *__restrict__ q, T beta, size_t n, bool first)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
        if (first) {
            u[l] = r[l];
            p[l] = r[l];
        } else {
            const T un = r[l] + beta * q[l];
            u[l] = un;
            p[l] = un + beta * (q[l] + beta * p[l]);
        }
    }
}

// q = u - alpha vh; uh = u + q; x = x + alpha uh
template <typename T>
__global__ void cgs_q_k(T *q, T *uh, T *x, const T *__restrict__ u, const T *__restrict__ vh, T alpha, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
        const T qn = u[l] - alpha * vh[l];
        const T un = u[l] + qn;
        q[l] = qn;
        uh[l] = un;
        x[l] = x[l] + alpha * un;
    }
}

// r = r - alpha w; sum r^2
template <typename T>
__global__ void __launch_bounds__(BG_BLOCK)
cgs_r_k(T *r, const T *__restrict__ w, T alpha, size_t n, double *part)
{
    PartialSum<T> ps;
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
        const T rn = r[l] - alpha * w[l];
        r[l] = rn;
        ps.add(rn * rn);
    }
    double acc[1] = {ps.get()};
    block_sums<1>(part, acc);
}

const char *fft_str(cufftResult r)
{
    switch (r) {
    case CUFFT_ALLOC_FAILED: return "CUFFT_ALLOC_FAILED";
    case CUFFT_INVALID_VALUE: return "CUFFT_INVALID_VALUE";
    case CUFFT_INVALID_SIZE: return "CUFFT_INVALID_SIZE";
    case CUFFT_EXEC_FAILED: return "CUFFT_EXEC_FAILED";
    default: return "cuFFT error";
    }
}

#define BG_FFT(call)                                                                          \
    do {                                                                                      \
        cufftResult r_ = (call);                                                              \
        if (r_ != CUFFT_SUCCESS) {                                                            \
            set_error(ctx, "%s:%d %s: %s", __FILE__, __LINE__, #call, fft_str(r_));           \
            return r_ == CUFFT_ALLOC_FAILED ? QSM_ERR_NOMEM : QSM_ERR_CUDA;                  \
        }                                                                                     \
    } while (0)

// R2C / C2R plans of one padded grid, in T and in FP32 (eroded masks)
template <typename T>
struct Plans {
    cufftHandle f = 0, i = 0, f32 = 0, i32 = 0;
    bool hf = false, hi = false, hf32 = false, hi32 = false;
    void destroy()
    {
        if (hf) cufftDestroy(f);
        if (hi) cufftDestroy(i);
        if (hf32) cufftDestroy(f32);
        if (hi32) cufftDestroy(i32);
        hf = hi = hf32 = hi32 = false;
    }
    qsm_status make(qsm_ctx *ctx, const Dims &p)
    {
        const int nx = (int)p.nx, ny = (int)p.ny, nz = (int)p.nz;
        const bool dbl = sizeof(T) == 8;
        BG_FFT(cufftPlan3d(&f, nz, ny, nx, dbl ? CUFFT_D2Z : CUFFT_R2C));
        hf = true;
        BG_FFT(cufftPlan3d(&i, nz, ny, nx, dbl ? CUFFT_Z2D : CUFFT_C2R));
        hi = true;
        BG_FFT(cufftSetStream(f, ctx->stream));
        BG_FFT(cufftSetStream(i, ctx->stream));
        if (dbl) {
            BG_FFT(cufftPlan3d(&f32, nz, ny, nx, CUFFT_R2C));
            hf32 = true;
            BG_FFT(cufftPlan3d(&i32, nz, ny, nx, CUFFT_C2R));
            hi32 = true;
            BG_FFT(cufftSetStream(f32, ctx->stream));
            BG_FFT(cufftSetStream(i32, ctx->stream));
        }
        return QSM_OK;
    }
    qsm_status fwd(qsm_ctx *ctx, T *in, typename Cx<T>::type *out)
    {
        if (sizeof(T) == 8) BG_FFT(cufftExecD2Z(f, (cufftDoubleReal *)in, (cufftDoubleComplex *)out));
        else BG_FFT(cufftExecR2C(f, (cufftReal *)in, (cufftComplex *)out));
        return QSM_OK;
    }
    qsm_status inv(qsm_ctx *ctx, typename Cx<T>::type *in, T *out)
    {
        if (sizeof(T) == 8) BG_FFT(cufftExecZ2D(i, (cufftDoubleComplex *)in, (cufftDoubleReal *)out));
        else BG_FFT(cufftExecC2R(i, (cufftComplex *)in, (cufftReal *)out));
        return QSM_OK;
    }
    qsm_status fwd32(qsm_ctx *ctx, float *in, cufftComplex *out)
    {
        BG_FFT(cufftExecR2C(sizeof(T) == 8 ? f32 : f, in, out));
        return QSM_OK;
    }
    qsm_status inv32(qsm_ctx *ctx, cufftComplex *in, float *out)
    {
        BG_FFT(cufftExecC2R(sizeof(T) == 8 ? i32 : i, in, out));
        return QSM_OK;
    }
};

// Device work space of one call on one padded grid.
template <typename T>
struct Work {
    using C = typename Cx<T>::type;
    void *blk = nullptr;
    T *a = nullptr, *b = nullptr, *c = nullptr, *e = nullptr;  // real padded arrays (e: kernel/erosion scratch)
    C *F = nullptr, *G = nullptr;                              // half spectra in T (G: scratch)
    T *H = nullptr, *H1 = nullptr;                             // SMV spectra (real half spectrum)
    float *H32 = nullptr, *mf = nullptr;                       // FP32 spectrum; the padded mask as float
    cufftComplex *M = nullptr;                                 // FP32 half spectrum
    uint8_t *m1 = nullptr, *mk = nullptr, *mp = nullptr, *mr = nullptr;  // padded mask, eroded masks
    double *part = nullptr, *sum = nullptr;
    qsm_status alloc(qsm_ctx *ctx, const Grid &g)
    {
        auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
        const size_t N = g.p.n(), nh = g.nh;
        const size_t rb = al(N * sizeof(T)), cb = al(nh * sizeof(C)), hb = al(nh * sizeof(T)), fb = al(N * 4),
                     h32 = al(nh * 4), m32 = al(nh * sizeof(cufftComplex)), mb = al(N);
        const size_t bytes = 4 * rb + 2 * cb + 2 * hb + h32 + fb + m32 + 4 * mb + (BG_GRID + 64) * sizeof(double);
        QSM_TRY(dalloc(ctx, &blk, bytes));
        char *p = (char *)blk;
        a = (T *)p; p += rb;
        b = (T *)p; p += rb;
        c = (T *)p; p += rb;
        e = (T *)p; p += rb;
        F = (C *)p; p += cb;
        G = (C *)p; p += cb;
        H = (T *)p; p += hb;
        H1 = (T *)p; p += hb;
        H32 = (float *)p; p += h32;
        mf = (float *)p; p += fb;
        M = (cufftComplex *)p; p += m32;
        m1 = (uint8_t *)p; p += mb;
        mk = (uint8_t *)p; p += mb;
        mp = (uint8_t *)p; p += mb;
        mr = (uint8_t *)p; p += mb;
        part = (double *)p;
        sum = part + BG_GRID;
        return QSM_OK;
    }
    void release(qsm_ctx *ctx)
    {
        if (blk) dfree(ctx, blk);
        blk = nullptr;
    }
};

template <typename S, typename T>
void pad(qsm_ctx *ctx, T *p, const S *a, const Grid &g)
{
    pad_k<S, T><<<grid_for(g.p.n()), 256, 0, ctx->stream>>>(p, a, g.full, g.p, g.c0[0], g.c0[1], g.c0[2], g.sz[0],
                                                          g.sz[1], g.sz[2], g.pre[0], g.pre[1], g.pre[2]);
}

template <typename T>
void unpad(qsm_ctx *ctx, T *full, const T *p, const Grid &g)
{
    unpad_k<T><<<grid_for(g.full.n()), 256, 0, ctx->stream>>>(full, p, g.full, g.p, g.c0[0], g.c0[1], g.c0[2],
                                                            g.sz[0], g.sz[1], g.sz[2], g.pre[0], g.pre[1], g.pre[2]);
}

qsm_status launched(qsm_ctx *ctx)
{
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// H = real(fft3(ifftshift(smvKernel(size, r, vsz)))) in T and FP32 (scratch: e, G)
template <typename T>
qsm_status smv_spectrum(qsm_ctx *ctx, Plans<T> &pl, Work<T> &w, const Grid &g, const double *h, double r)
{
    const size_t cnt = smv_count(g.p, h, r);
    if (cnt == 0) {
        set_error(ctx, "SMV radius %g holds no voxel", r);
        return QSM_ERR_ARG;
    }
    smv_k<T><<<grid_for(g.p.n()), 256, 0, ctx->stream>>>(w.e, g.p, h[0], h[1], h[2], r * r, 1.0 / (double)cnt);
    QSM_TRY(launched(ctx));
    QSM_TRY(pl.fwd(ctx, w.e, w.G));
    real_part_k<T><<<grid_for(g.nh), 256, 0, ctx->stream>>>(w.H, w.H32, w.G, g.nh);
    return launched(ctx);
}

// out = real(ifft3(H .* fft3(single(mask1)))) > 0.999 (single FFTs)
template <typename T>
qsm_status erode(qsm_ctx *ctx, Plans<T> &pl, Work<T> &w, const Grid &g, uint8_t *out)
{
    QSM_TRY(pl.fwd32(ctx, w.mf, w.M));
    mul_f32_k<<<grid_for(g.nh), 256, 0, ctx->stream>>>(w.M, w.H32, g.nh);
    QSM_TRY(launched(ctx));
    float *tmp = (float *)w.e;  // scratch (T >= 4 bytes per element)
    QSM_TRY(pl.inv32(ctx, w.M, tmp));
    thresh_k<<<grid_for(g.p.n()), 256, 0, ctx->stream>>>(out, tmp, 1.0f / (float)g.p.n(), g.p.n());
    return launched(ctx);
}

// crop box (cropIndices) and padded grid
qsm_status make_grid(qsm_ctx *ctx, const uint8_t *mask, const Dims &d, size_t pad, Grid *g)
{
    size_t lo[3], hi[3];
    QSM_TRY(mask_bbox(ctx, mask, d, lo, hi));
    g->full = d;
    for (int a = 0; a < 3; ++a) {
        g->c0[a] = lo[a];
        g->sz[a] = hi[a] - lo[a] + 1;
    }
    pad_sizes(*g, pad);
    if (g->p.nx > 0x7fffffff || g->p.ny > 0x7fffffff || g->p.nz > 0x7fffffff) return QSM_ERR_DIMS;
    return QSM_OK;
}

enum Method { SHARP, VSHARP, ISMV, RESHARP };

template <typename T>
qsm_status run(qsm_ctx *ctx, Method meth, const Dims &d, size_t ne, const T *f, const uint8_t *mask, const double *h,
               const std::vector<double> &radii, double thr, double tol, int32_t maxit, int32_t verbose, T *fl,
               uint8_t *mask_out, int32_t *iters)
{
    const double rmax = *std::max_element(radii.begin(), radii.end());
    const double hmin = std::min(h[0], std::min(h[1], h[2]));
    Grid g;
    QSM_TRY(make_grid(ctx, mask, d, (size_t)std::ceil(rmax / hmin), &g));
    const size_t N = g.p.n(), nh = g.nh, Nf = d.n();
    const T invn = (T)(1.0 / (double)N);
    Plans<T> pl;
    Work<T> w;
    qsm_status st = pl.make(ctx, g.p);
    if (st == QSM_OK) st = w.alloc(ctx, g);
    if (st != QSM_OK) {
        pl.destroy();
        w.release(ctx);
        return st;
    }
    const unsigned gn = grid_for(N), gh = grid_for(nh);
    T *kv = nullptr;  // RESHARP's eight Krylov vectors
    if (meth == RESHARP && (st = dalloc(ctx, (void **)&kv, 8 * N * sizeof(T))) != QSM_OK) {
        pl.destroy();
        w.release(ctx);
        return st;
    }
    auto body = [&]() -> qsm_status {
        pad<uint8_t, uint8_t>(ctx, w.m1, mask, g);
        pad<uint8_t, float>(ctx, w.mf, mask, g);
        QSM_TRY(launched(ctx));
        if (meth != VSHARP) {  // one radius
            QSM_TRY(smv_spectrum<T>(ctx, pl, w, g, h, radii[0]));
            QSM_TRY(erode<T>(ctx, pl, w, g, w.mk));  // mask1 (sharp.m:58) / m (ismv.m:65)
        }
        const uint8_t *mask_ret = w.mk;
        for (size_t t = 0; t < ne; ++t) {
            const T *ft = f + t * Nf;
            T *out = fl + t * Nf;
            if (meth == SHARP) {
                // f = maskn .* real(ifft3((1 - H) .* fft3(f)))  (sharp.m:62-67)
                pad<T, T>(ctx, w.a, ft, g);
                QSM_TRY(launched(ctx));
                QSM_TRY(pl.fwd(ctx, w.a, w.F));
                mul_h_k<T><<<gh, 256, 0, ctx->stream>>>(w.F, w.H, nh, true);
                QSM_TRY(pl.inv(ctx, w.F, w.b));
                mask_scale_k<T><<<gn, 256, 0, ctx->stream>>>(w.b, w.mk, invn, N);
                // f = maskn .* real(ifft3(fft3(f) ./ (1 - H), truncated at thr))  (:69-71)
                QSM_TRY(pl.fwd(ctx, w.b, w.F));
                deconv_k<T><<<gh, 256, 0, ctx->stream>>>(w.F, w.H, (T)thr, nh);
                QSM_TRY(pl.inv(ctx, w.F, w.b));
                mask_scale_k<T><<<gn, 256, 0, ctx->stream>>>(w.b, w.mk, invn, N);
                QSM_TRY(launched(ctx));
                unpad<T>(ctx, out, w.b, g);
            } else if (meth == VSHARP) {
                // f = sum_k (m_k - m_(k-1)) .* real(ifft3((1 - H_k) .* F)), radii descending
                // (vsharp.m:84-146), then maskn .* real(ifft3(ih .* fft3(f)))  (:149)
                pad<T, T>(ctx, w.c, ft, g);
                QSM_TRY(launched(ctx));
                QSM_TRY(pl.fwd(ctx, w.c, w.F));
                QSM_CUDA(cudaMemsetAsync(w.a, 0, N * sizeof(T), ctx->stream));
                QSM_CUDA(cudaMemsetAsync(w.mp, 0, N, ctx->stream));
                // the returned mask is vsharp.m's last `mask1`: the second smallest
                // radius for an even count of radii, the smallest for an odd count
                const size_t nr = radii.size(), kret = (nr % 2 == 0) ? nr - 2 : nr - 1;
                uint8_t *mk = w.mk, *mp = w.mp;
                for (size_t k = 0; k < nr; ++k) {
                    QSM_TRY(smv_spectrum<T>(ctx, pl, w, g, h, radii[k]));
                    QSM_TRY(erode<T>(ctx, pl, w, g, mk));
                    if (k == 0) QSM_CUDA(cudaMemcpyAsync(w.H1, w.H, nh * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
                    if (k == kret) QSM_CUDA(cudaMemcpyAsync(w.mr, mk, N, cudaMemcpyDeviceToDevice, ctx->stream));
                    mul_1mh_to_k<T><<<gh, 256, 0, ctx->stream>>>(w.G, w.F, w.H, nh);
                    QSM_TRY(pl.inv(ctx, w.G, w.b));
                    vsharp_acc_k<T><<<gn, 256, 0, ctx->stream>>>(w.a, w.b, mk, mp, invn, N);
                    QSM_TRY(launched(ctx));
                    std::swap(mk, mp);  // this radius's mask becomes the previous one
                }
                const uint8_t *mlast = mp;
                QSM_TRY(pl.fwd(ctx, w.a, w.G));
                mul_inv_k<T><<<gh, 256, 0, ctx->stream>>>(w.G, w.H1, (T)thr, nh);
                QSM_TRY(pl.inv(ctx, w.G, w.b));
                mask_scale_k<T><<<gn, 256, 0, ctx->stream>>>(w.b, mlast, invn, N);
                QSM_TRY(launched(ctx));
                unpad<T>(ctx, out, w.b, g);
                mask_ret = w.mr;
            } else if (meth == RESHARP) {
                // RESHARP (resharp.m:62-80): b = mask1 .* real(ifft3((1 - H) .* fft3(f))),
                // x = cgs(A, b, tol, maxit), fl = mask1 .* x
                const T lam = (T)thr;
                T *x = kv, *r = kv + N, *rt = kv + 2 * N, *u = kv + 3 * N, *pp = kv + 4 * N, *q = kv + 5 * N,
                  *vh = kv + 6 * N, *uh = kv + 7 * N;
                auto apply = [&](const T *in, T *outv) -> qsm_status {
                    QSM_CUDA(cudaMemcpyAsync(w.e, in, N * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
                    QSM_TRY(pl.fwd(ctx, w.e, w.F));
                    mul_h_k<T><<<gh, 256, 0, ctx->stream>>>(w.F, w.H, nh, true);
                    QSM_TRY(pl.inv(ctx, w.F, outv));
                    resharp_op_k<T><<<gn, 256, 0, ctx->stream>>>(outv, in, w.mk, invn, lam, N);
                    return launched(ctx);
                };
                auto dot = [&](const T *a_, const T *b_, double *out_) -> qsm_status {
                    dot_k<T><<<BG_GRID, BG_BLOCK, 0, ctx->stream>>>(a_, b_, N, w.part);
                    fold_k<<<1, BG_BLOCK, 0, ctx->stream>>>(w.sum, w.part, BG_GRID);
                    QSM_TRY(launched(ctx));
                    QSM_CUDA(cudaMemcpyAsync(out_, w.sum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
                    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
                    return QSM_OK;
                };
                pad<T, T>(ctx, w.c, ft, g);
                QSM_TRY(launched(ctx));
                QSM_TRY(pl.fwd(ctx, w.c, w.F));
                mul_h_k<T><<<gh, 256, 0, ctx->stream>>>(w.F, w.H, nh, true);
                QSM_TRY(pl.inv(ctx, w.F, w.b));
                mask_scale_k<T><<<gn, 256, 0, ctx->stream>>>(w.b, w.mk, invn, N);  // b
                QSM_TRY(launched(ctx));
                QSM_CUDA(cudaMemsetAsync(x, 0, N * sizeof(T), ctx->stream));
                QSM_CUDA(cudaMemcpyAsync(r, w.b, N * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
                QSM_CUDA(cudaMemcpyAsync(rt, w.b, N * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
                double nb2 = 0.0, rho = 0.0, rho1 = 1.0, sv = 0.0, rr = 0.0;
                QSM_TRY(dot(w.b, w.b, &nb2));
                const double nb = std::sqrt(nb2);
                int32_t it = 0;
                if (nb > 0.0) {
                    for (int32_t ii = 1; ii <= maxit; ++ii) {
                        QSM_TRY(dot(rt, r, &rho));
                        if (rho == 0.0) break;  // breakdown
                        const T beta = (T)(rho / rho1);
                        cgs_dir_k<T><<<gn, 256, 0, ctx->stream>>>(u, pp, r, q, beta, N, ii == 1);
                        QSM_TRY(launched(ctx));
                        QSM_TRY(apply(pp, vh));
                        QSM_TRY(dot(rt, vh, &sv));
                        if (sv == 0.0) break;
                        const T alpha = (T)(rho / sv);
                        cgs_q_k<T><<<gn, 256, 0, ctx->stream>>>(q, uh, x, u, vh, alpha, N);
                        QSM_TRY(launched(ctx));
                        QSM_TRY(apply(uh, vh));  // vh reused for A uh
                        cgs_r_k<T><<<BG_GRID, BG_BLOCK, 0, ctx->stream>>>(r, vh, alpha, N, w.part);
                        fold_k<<<1, BG_BLOCK, 0, ctx->stream>>>(w.sum, w.part, BG_GRID);
                        QSM_TRY(launched(ctx));
                        QSM_CUDA(cudaMemcpyAsync(&rr, w.sum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
                        QSM_CUDA(cudaStreamSynchronize(ctx->stream));
                        rho1 = rho;
                        it = ii;
                        if (verbose) printf("%5d/%d\t%1.3e\n", ii, maxit, std::sqrt(rr) / nb);
                        if (std::sqrt(rr) <= tol * nb) break;
                    }
                }
                if (iters) iters[t] = it;
                QSM_CUDA(cudaMemcpyAsync(w.b, x, N * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
                mask_scale_k<T><<<gn, 256, 0, ctx->stream>>>(w.b, w.mk, (T)1, N);
                QSM_TRY(launched(ctx));
                unpad<T>(ctx, out, w.b, g);
            } else {
                // iSMV (ismv.m:67-107): fb from f by f = bc + m .* real(ifft3(H .* fft3(f)))
                // until ||f0 - f|| <= tol ||m .* f||; fl = m .* (f - fb)
                pad<T, T>(ctx, w.c, ft, g);
                QSM_TRY(launched(ctx));
                ismv_init_k<T><<<BG_GRID, BG_BLOCK, 0, ctx->stream>>>(w.b, w.c, w.m1, w.mk, N, w.part);
                fold_k<<<1, BG_BLOCK, 0, ctx->stream>>>(w.sum, w.part, BG_GRID);
                QSM_TRY(launched(ctx));
                double r2 = 0.0;
                QSM_CUDA(cudaMemcpyAsync(&r2, w.sum, sizeof r2, cudaMemcpyDeviceToHost, ctx->stream));
                QSM_CUDA(cudaMemcpyAsync(w.a, w.c, N * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
                QSM_CUDA(cudaStreamSynchronize(ctx->stream));
                double res = std::sqrt(r2);
                const double reltol = res * tol;
                if (verbose) printf("iter%6s\tresidual\n", "");
                int32_t it = 0;
                for (int32_t ii = 1; ii <= maxit; ++ii) {
                    if (res <= reltol) break;
                    QSM_TRY(pl.fwd(ctx, w.a, w.F));
                    mul_h_k<T><<<gh, 256, 0, ctx->stream>>>(w.F, w.H, nh, false);
                    QSM_TRY(pl.inv(ctx, w.F, w.e));
                    ismv_step_k<T><<<BG_GRID, BG_BLOCK, 0, ctx->stream>>>(w.a, w.e, w.b, w.mk, invn, N, w.part);
                    fold_k<<<1, BG_BLOCK, 0, ctx->stream>>>(w.sum, w.part, BG_GRID);
                    QSM_TRY(launched(ctx));
                    QSM_CUDA(cudaMemcpyAsync(&r2, w.sum, sizeof r2, cudaMemcpyDeviceToHost, ctx->stream));
                    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
                    res = std::sqrt(r2);
                    it = ii;
                    if (verbose) printf("%5d/%d\t%1.3e\n", ii, maxit, res);
                }
                if (verbose) printf("\n");
                if (iters) iters[t] = it;
                ismv_out_k<T><<<gn, 256, 0, ctx->stream>>>(w.b, w.c, w.a, w.mk, N);
                QSM_TRY(launched(ctx));
                unpad<T>(ctx, out, w.b, g);
            }
            QSM_TRY(launched(ctx));
        }
        if (mask_out) {
            unpad<uint8_t>(ctx, mask_out, mask_ret, g);
            QSM_TRY(launched(ctx));
        }
        return QSM_OK;
    };
    st = body();
    cudaStreamSynchronize(ctx->stream);
    if (kv) dfree(ctx, kv);
    pl.destroy();
    w.release(ctx);
    return st;
}

// ---------------------------------------------------------------------------
// PDF (pdf.m:1-86): projection onto dipole fields by LSMR
// ---------------------------------------------------------------------------

// image-space unit dipole (dipoleKernel.m:44-51, 'i') in psf2otf's order
// (centre at index 0): D = (3 (b.r)^2 - |r|^2) / (4 pi |r|^5), D(0) = 0
template <typename T>
__global__ void dipole_i_k(T *D, Dims pd, double hx, double hy, double hz, double bx, double by, double bz)
{
    const size_t N = pd.n();
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < N; l += (size_t)gridDim.x * blockDim.x) {
        const double x = shift_coord(l % pd.nx, pd.nx, hx), y = shift_coord((l / pd.nx) % pd.ny, pd.ny, hy),
                     z = shift_coord(l / pd.nxny(), pd.nz, hz);
        const double rz = bx * x + by * y + bz * z;
        const double r2 = x * x + y * y + z * z;
        const double den = 4.0 * 3.14159265358979323846 * sqrt(r2 * r2 * r2 * r2 * r2);
        D[l] = den == 0.0 ? (T)0 : (T)((3.0 * (rz * rz) - r2) / den);
    }
}

// max |Im D| and max |D| over the half spectrum (the same maxima as over the full
// spectrum of a real kernel); non-negative doubles order like their bit patterns
template <typename T>
__global__ void otf_max_k(unsigned long long *mx, const typename Cx<T>::type *__restrict__ D, size_t nh)
{
    double mi = 0.0, ma = 0.0;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nh; q += (size_t)gridDim.x * blockDim.x) {
        mi = fmax(mi, fabs((double)D[q].y));
        ma = fmax(ma, (double)hypot(D[q].x, D[q].y));
    }
    atomicMax(mx, (unsigned long long)__double_as_longlong(mi));
    atomicMax(mx + 1, (unsigned long long)__double_as_longlong(ma));
}

template <typename T>
__global__ void drop_imag_k(typename Cx<T>::type *D, size_t nh)
{
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nh; q += (size_t)gridDim.x * blockDim.x)
        D[q].y = (T)0;
}

// F .*= D (or conj(D))
template <typename T>
__global__ void mul_c_k(typename Cx<T>::type *F, const typename Cx<T>::type *__restrict__ D, size_t nh, bool conj)
{
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nh; q += (size_t)gridDim.x * blockDim.x) {
        const T dr = D[q].x, di = conj ? -D[q].y : D[q].y;
        const T fr = F[q].x, fi = F[q].y;
        F[q].x = dr * fr - di * fi;
        F[q].y = dr * fi + di * fr;
    }
}

// t = w .* v with w = m (weights) or ~m
template <typename T>
__global__ void weight_k(T *t, const T *__restrict__ v, const T *__restrict__ m, bool notm, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        t[l] = (notm ? (T)(m[l] == (T)0 ? 1 : 0) : m[l]) * v[l];
}

// y = w .* (C2R value / N) - a .* y, sum y^2  (the Golub-Kahan step u = A v - alpha u)
template <typename T>
__global__ void __launch_bounds__(BG_BLOCK)
gk_step_k(T *y, const T *__restrict__ g, const T *__restrict__ m, bool notm, T invn, T a, size_t n, double *part)
{
    PartialSum<T> ps;
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
        const T w = notm ? (T)(m[l] == (T)0 ? 1 : 0) : m[l];
        const T v = w * (g[l] * invn) - a * y[l];
        y[l] = v;
        ps.add(v * v);
    }
    double acc[1] = {ps.get()};
    block_sums<1>(part, acc);
}

template <typename T>
__global__ void scale_k(T *y, T s, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        y[l] = s * y[l];
}

// LSMR updates: hbar = h - c1 hbar; x = x + c2 hbar; h = v - c3 h; sum x^2
template <typename T>
__global__ void __launch_bounds__(BG_BLOCK)
lsmr_upd_k(T *hbar, T *x, T *h, const T *__restrict__ v, T c1, T c2, T c3, size_t n, double *part)
{
    PartialSum<T> ps;
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
        const T hb = h[l] - c1 * hbar[l];
        const T xn = x[l] + c2 * hb;
        hbar[l] = hb;
        x[l] = xn;
        h[l] = v[l] - c3 * h[l];
        ps.add(xn * xn);
    }
    double acc[1] = {ps.get()};
    block_sums<1>(part, acc);
}

// fl = logical(m) .* (f - real(ifft3(D .* fft3(~m .* xb))))  (pdf.m:79-80)
template <typename T>
__global__ void pdf_out_k(T *o, const T *__restrict__ f, const T *__restrict__ g, const T *__restrict__ m, T invn,
                          size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        o[l] = (T)(m[l] != (T)0 ? 1 : 0) * (f[l] - g[l] * invn);
}

template <typename T>
qsm_status run_pdf(qsm_ctx *ctx, const Dims &d, size_t ne, const T *f, const uint8_t *mask, const T *wgt,
                   const double *vsz, const double *bdir, double lambda, double tol, int32_t maxit, int32_t verbose,
                   T *fl, int32_t *iters)
{
    using C = typename Cx<T>::type;
    const size_t N = d.n(), nh = (d.nx / 2 + 1) * d.ny * d.nz;
    const T invn = (T)(1.0 / (double)N);
    const unsigned gn = grid_for(N), gh = grid_for(nh);
    Plans<T> pl;
    QSM_TRY(pl.make(ctx, d));
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t rb = al(N * sizeof(T)), cb = al(nh * sizeof(C));
    void *blk = nullptr;
    qsm_status st = dalloc(ctx, &blk, 8 * rb + 2 * cb + (BG_GRID + 64) * sizeof(double));
    if (st != QSM_OK) {
        pl.destroy();
        return st;
    }
    char *p = (char *)blk;
    T *m = (T *)p, *u = (T *)(p + rb), *v = (T *)(p + 2 * rb), *h = (T *)(p + 3 * rb), *hb = (T *)(p + 4 * rb),
      *x = (T *)(p + 5 * rb), *t1 = (T *)(p + 6 * rb), *t2 = (T *)(p + 7 * rb);
    C *Dh = (C *)(p + 8 * rb), *F = (C *)(p + 8 * rb + cb);
    double *part = (double *)(p + 8 * rb + 2 * cb), *sum = part + BG_GRID;
    auto red = [&](double *out_) -> qsm_status {
        fold_k<<<1, BG_BLOCK, 0, ctx->stream>>>(sum, part, BG_GRID);
        QSM_TRY(launched(ctx));
        QSM_CUDA(cudaMemcpyAsync(out_, sum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        QSM_CUDA(cudaStreamSynchronize(ctx->stream));
        return QSM_OK;
    };
    // y = op(in) - a y and ||y||^2: op = m .* ifft(D .* fft(~m .* in)) (forward) or
    // ~m .* ifft(conj(D) .* fft(m .* in)) (transpose), pdf.m:63-72
    auto gk = [&](T *y, const T *in, bool transpose, T a, double *n2) -> qsm_status {
        weight_k<T><<<gn, 256, 0, ctx->stream>>>(t1, in, m, !transpose, N);
        QSM_TRY(launched(ctx));
        QSM_TRY(pl.fwd(ctx, t1, F));
        mul_c_k<T><<<gh, 256, 0, ctx->stream>>>(F, Dh, nh, transpose);
        QSM_TRY(pl.inv(ctx, F, t2));
        gk_step_k<T><<<BG_GRID, BG_BLOCK, 0, ctx->stream>>>(y, t2, m, transpose, invn, a, N, part);
        return red(n2);
    };
    auto body = [&]() -> qsm_status {
        // D = psf2otf(dipoleKernel(size(mask), vsz, bdir, 'i', class(f))): the kernel in
        // double, rounded to T, transformed in T; psf2otf returns the real part when the
        // imaginary part is roundoff, max|Im D| / max|D| <= N log2(N) eps(T)
        const double bn = std::sqrt(bdir[0] * bdir[0] + bdir[1] * bdir[1] + bdir[2] * bdir[2]);
        const double b0 = bn == 1.0 ? bdir[0] : bdir[0] / bn, b1 = bn == 1.0 ? bdir[1] : bdir[1] / bn,
                     b2 = bn == 1.0 ? bdir[2] : bdir[2] / bn;
        dipole_i_k<T><<<gn, 256, 0, ctx->stream>>>(t1, d, vsz[0], vsz[1], vsz[2], b0, b1, b2);
        QSM_TRY(launched(ctx));
        QSM_TRY(pl.fwd(ctx, t1, Dh));
        unsigned long long *mx = (unsigned long long *)sum;
        QSM_CUDA(cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned long long), ctx->stream));
        otf_max_k<T><<<gh, 256, 0, ctx->stream>>>(mx, Dh, nh);
        QSM_TRY(launched(ctx));
        double mxh[2];
        QSM_CUDA(cudaMemcpyAsync(mxh, mx, sizeof(mxh), cudaMemcpyDeviceToHost, ctx->stream));
        QSM_CUDA(cudaStreamSynchronize(ctx->stream));
        const double eps_t = sizeof(T) == 4 ? (double)FLT_EPSILON : DBL_EPSILON;
        if (mxh[0] / mxh[1] <= (double)N * std::log2((double)N) * eps_t) {
            drop_imag_k<T><<<gh, 256, 0, ctx->stream>>>(Dh, nh);
            QSM_TRY(launched(ctx));
        }
        // m = mask .* w, with w = mask when w is empty or all zero (pdf.m:50-52, 61)
        pad_k<uint8_t, T><<<gn, 256, 0, ctx->stream>>>(m, mask, d, d, 0, 0, 0, d.nx, d.ny, d.nz, 0, 0, 0);
        QSM_TRY(launched(ctx));
        if (wgt) {
            double ww;
            dot_k<T><<<BG_GRID, BG_BLOCK, 0, ctx->stream>>>(wgt, wgt, N, part);
            QSM_TRY(red(&ww));
            if (!(ww == 0.0)) {
                weight_k<T><<<gn, 256, 0, ctx->stream>>>(t1, wgt, m, false, N);
                QSM_TRY(launched(ctx));
                QSM_CUDA(cudaMemcpyAsync(m, t1, N * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
            }
        }
        const double conlim = 1e8, ctol = 1.0 / conlim;
        for (size_t e = 0; e < ne; ++e) {
            const T *fe = f + e * N;
            // LSMR (Fong & Saunders 2011) on min ||A x - b||^2 + lambda^2 ||x||^2, b = m .* f,
            // atol = btol = tol, conlim 1e8, no local reorthogonalisation
            weight_k<T><<<gn, 256, 0, ctx->stream>>>(u, fe, m, false, N);
            dot_k<T><<<BG_GRID, BG_BLOCK, 0, ctx->stream>>>(u, u, N, part);
            double bb, aa, xx;
            QSM_TRY(red(&bb));
            double beta = std::sqrt(bb);
            if (beta > 0.0) scale_k<T><<<gn, 256, 0, ctx->stream>>>(u, (T)(1.0 / beta), N);
            QSM_CUDA(cudaMemsetAsync(v, 0, N * sizeof(T), ctx->stream));
            QSM_CUDA(cudaMemsetAsync(x, 0, N * sizeof(T), ctx->stream));
            QSM_TRY(gk(v, u, true, (T)0, &aa));  // v = A' u
            double alpha = std::sqrt(aa);
            if (alpha > 0.0) scale_k<T><<<gn, 256, 0, ctx->stream>>>(v, (T)(1.0 / alpha), N);
            int32_t itn = 0;
            if (alpha * beta != 0.0) {  // else x = 0 is the exact solution
                QSM_CUDA(cudaMemcpyAsync(h, v, N * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
                QSM_CUDA(cudaMemsetAsync(hb, 0, N * sizeof(T), ctx->stream));
                double zetabar = alpha * beta, alphabar = alpha, rho = 1, rhobar = 1, cbar = 1, sbar = 0;
                double betadd = beta, betad = 0, rhodold = 1, tautildeold = 0, thetatilde = 0, zeta = 0, dd = 0;
                double normA2 = alpha * alpha, maxrbar = 0, minrbar = 1e100;
                const double normb = beta;
                if (verbose) printf("   itn       norm r    norm A'r\n");
                while (itn < maxit) {
                    ++itn;
                    // bidiagonalization: beta u = A v - alpha u; alpha v = A' u - beta v
                    double b2, a2;
                    QSM_TRY(gk(u, v, false, (T)alpha, &b2));
                    beta = std::sqrt(b2);
                    if (beta > 0.0) {
                        scale_k<T><<<gn, 256, 0, ctx->stream>>>(u, (T)(1.0 / beta), N);
                        QSM_TRY(gk(v, u, true, (T)beta, &a2));
                        alpha = std::sqrt(a2);
                        if (alpha > 0.0) scale_k<T><<<gn, 256, 0, ctx->stream>>>(v, (T)(1.0 / alpha), N);
                    }
                    // rotation eliminating the damping term
                    const double alphahat = std::hypot(alphabar, lambda);
                    const double chat = alphabar / alphahat, shat = lambda / alphahat;
                    // plane rotations Q_i and Qbar_i
                    const double rhoold = rho;
                    rho = std::hypot(alphahat, beta);
                    const double c = alphahat / rho, s_ = beta / rho;
                    const double thetanew = s_ * alpha;
                    alphabar = c * alpha;
                    const double rhobarold = rhobar, zetaold = zeta, thetabar = sbar * rho, rhotemp = cbar * rho;
                    rhobar = std::hypot(cbar * rho, thetanew);
                    cbar = cbar * rho / rhobar;
                    sbar = thetanew / rhobar;
                    zeta = cbar * zetabar;
                    zetabar = -sbar * zetabar;
                    // hbar, x, h
                    lsmr_upd_k<T><<<BG_GRID, BG_BLOCK, 0, ctx->stream>>>(
                        hb, x, h, v, (T)(thetabar * rho / (rhoold * rhobarold)), (T)(zeta / (rho * rhobar)),
                        (T)(thetanew / rho), N, part);
                    QSM_TRY(red(&xx));
                    // ||r||
                    const double betaacute = chat * betadd, betacheck = -shat * betadd;
                    const double betahat = c * betaacute;
                    betadd = -s_ * betaacute;
                    const double thetatildeold = thetatilde;
                    const double rhotildeold = std::hypot(rhodold, thetabar);
                    const double ctildeold = rhodold / rhotildeold, stildeold = thetabar / rhotildeold;
                    thetatilde = stildeold * rhobar;
                    rhodold = ctildeold * rhobar;
                    betad = -stildeold * betad + ctildeold * betahat;
                    tautildeold = (zetaold - thetatildeold * tautildeold) / rhotildeold;
                    const double taud = (zeta - thetatilde * tautildeold) / rhodold;
                    dd = dd + betacheck * betacheck;
                    const double normr = std::sqrt(dd + (betad - taud) * (betad - taud) + betadd * betadd);
                    // ||A||, cond(A)
                    normA2 = normA2 + beta * beta;
                    const double normA = std::sqrt(normA2);
                    normA2 = normA2 + alpha * alpha;
                    maxrbar = std::max(maxrbar, rhobarold);
                    if (itn > 1) minrbar = std::min(minrbar, rhobarold);
                    const double condA = std::max(maxrbar, rhotemp) / std::min(minrbar, rhotemp);
                    // stopping rules
                    const double normAr = std::fabs(zetabar), normx = std::sqrt(xx);
                    const double test1 = normr / normb, test2 = normAr / (normA * normr), test3 = 1.0 / condA;
                    const double t1_ = test1 / (1.0 + normA * normx / normb);
                    const double rtol = tol + tol * normA * normx / normb;
                    if (verbose) printf("%6d %10.3e %10.3e\n", itn, normr, normAr);
                    if (itn >= maxit || 1.0 + test3 <= 1.0 || 1.0 + test2 <= 1.0 || 1.0 + t1_ <= 1.0 ||
                        test3 <= ctol || test2 <= tol || test1 <= rtol)
                        break;
                }
            }
            if (iters) iters[e] = itn;
            // fl = logical(m) .* (f - real(ifft3(D .* fft3(~m .* xb))))
            weight_k<T><<<gn, 256, 0, ctx->stream>>>(t1, x, m, true, N);
            QSM_TRY(launched(ctx));
            QSM_TRY(pl.fwd(ctx, t1, F));
            mul_c_k<T><<<gh, 256, 0, ctx->stream>>>(F, Dh, nh, false);
            QSM_TRY(pl.inv(ctx, F, t2));
            pdf_out_k<T><<<gn, 256, 0, ctx->stream>>>(fl + e * N, fe, t2, m, invn, N);
            QSM_TRY(launched(ctx));
        }
        return QSM_OK;
    };
    st = body();
    cudaStreamSynchronize(ctx->stream);
    pl.destroy();
    dfree(ctx, blk);
    return st;
}

qsm_status entry(qsm_ctx *ctx, Method meth, qsm_dtype dt, const size_t dims[4], const void *f, const uint8_t *mask,
                 const double *vsz, const std::vector<double> &radii, double thr, double tol, int32_t maxit,
                 int32_t verbose, void *fl, uint8_t *mask_out, int32_t *iters)
{
    if (!ctx || !dims || !f || !mask || !vsz || !fl) return QSM_ERR_ARG;
    if (dt != QSM_F32 && dt != QSM_F64) return QSM_ERR_DTYPE;
    if (!dims[0] || !dims[1] || !dims[2] || !dims[3]) return QSM_ERR_DIMS;
    for (double r : radii)
        if (!(r > 0.0)) return QSM_ERR_ARG;
    if (!(vsz[0] > 0.0 && vsz[1] > 0.0 && vsz[2] > 0.0)) return QSM_ERR_ARG;
    cudaSetDevice(ctx->device);
    const Dims d{dims[0], dims[1], dims[2]};
    const size_t ne = dims[3], es = dt == QSM_F32 ? 4 : 8;
    Staged sf, sm, so, smo;
    QSM_TRY(stage_in(ctx, sf, f, ne * d.n() * es, true));
    QSM_TRY(stage_in(ctx, sm, mask, d.n(), true));
    QSM_TRY(stage_in(ctx, so, fl, ne * d.n() * es, false));
    if (mask_out) QSM_TRY(stage_in(ctx, smo, mask_out, d.n(), false));
    qsm_status st =
        dt == QSM_F32
            ? run<float>(ctx, meth, d, ne, (const float *)sf.dev, (const uint8_t *)sm.dev, vsz, radii, thr, tol, maxit,
                         verbose, (float *)so.dev, mask_out ? (uint8_t *)smo.dev : nullptr, iters)
            : run<double>(ctx, meth, d, ne, (const double *)sf.dev, (const uint8_t *)sm.dev, vsz, radii, thr, tol,
                          maxit, verbose, (double *)so.dev, mask_out ? (uint8_t *)smo.dev : nullptr, iters);
    stage_out(ctx, sf, false);
    stage_out(ctx, sm, false);
    if (st != QSM_OK) {
        stage_out(ctx, so, false);
        if (mask_out) stage_out(ctx, smo, false);
        return st;
    }
    QSM_TRY(stage_out(ctx, so, true));
    if (mask_out) QSM_TRY(stage_out(ctx, smo, true));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return QSM_OK;
}

}  // namespace
}  // namespace qsm

using namespace qsm;

extern "C" {

qsm_status qsm_sharp(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[4], const void *f, const uint8_t *mask,
                     const double vsz[3], double r, double thr, void *fl, uint8_t *mask_out)
{
    return entry(ctx, SHARP, dt, dims, f, mask, vsz, {r}, thr, 0.0, 0, 0, fl, mask_out, nullptr);
}

qsm_status qsm_vsharp(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[4], const void *f, const uint8_t *mask,
                      const double vsz[3], const double *radii, int32_t nradii, double thr, void *fl,
                      uint8_t *mask_out)
{
    Range nvtx_range("vsharp");
    if (!vsz) return QSM_ERR_ARG;
    std::vector<double> rs;
    if (nradii > 0) {
        if (!radii) return QSM_ERR_ARG;
        rs.assign(radii, radii + nradii);
    } else {
        // vsharp.m:49: rs = 9 : -2*max(vsz) : 2*max(vsz)
        const double hmax = std::max(vsz[0], std::max(vsz[1], vsz[2]));
        for (int k = 0;; ++k) {
            const double r = 9.0 + k * (-2.0 * hmax);
            if (r < 2.0 * hmax) break;
            rs.push_back(r);
        }
    }
    std::sort(rs.begin(), rs.end(), [](double x, double y) { return x > y; });
    if (rs.size() < 2) {
        if (ctx) set_error(ctx, "vsharp needs at least two radii (vsharp.m reads ih from the first pair)");
        return QSM_ERR_ARG;
    }
    return entry(ctx, VSHARP, dt, dims, f, mask, vsz, rs, thr, 0.0, 0, 0, fl, mask_out, nullptr);
}

qsm_status qsm_resharp(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[4], const void *f, const uint8_t *mask,
                       const double vsz[3], double r, double lambda, double tol, int32_t maxit, int32_t verbose,
                       void *fl, uint8_t *mask_out, int32_t *iters)
{
    if (tol < 0.0) tol = dt == QSM_F32 ? 3.4526698300124393e-04 : 1.4901161193847656e-08;  // sqrt(eps(class))
    if (dims && maxit <= 0)  // resharp.m:42: ceil(sqrt(numel(mask)))
        maxit = (int32_t)std::ceil(std::sqrt((double)dims[0] * (double)dims[1] * (double)dims[2]));
    return entry(ctx, RESHARP, dt, dims, f, mask, vsz, {r}, lambda, tol, maxit, verbose, fl, mask_out, iters);
}

qsm_status qsm_ismv(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[4], const void *f, const uint8_t *mask,
                    const double vsz[3], double r, double tol, int32_t maxit, int32_t verbose, void *fl,
                    uint8_t *mask_out, int32_t *iters)
{
    if (tol < 0.0) tol = dt == QSM_F32 ? 3.4526698300124393e-04 : 1.4901161193847656e-08;  // sqrt(eps(class))
    if (maxit < 0) return QSM_ERR_ARG;
    return entry(ctx, ISMV, dt, dims, f, mask, vsz, {r}, 0.0, tol, maxit, verbose, fl, mask_out, iters);
}

qsm_status qsm_pdf(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[4], const void *f, const uint8_t *mask,
                   const void *w, const double vsz[3], const double bdir[3], double lambda, double tol,
                   int32_t maxit, int32_t verbose, void *fl, int32_t *iters)
{
    Range nvtx_range("pdf");
    if (!ctx || !dims || !f || !mask || !vsz || !bdir || !fl) return QSM_ERR_ARG;
    if (dt != QSM_F32 && dt != QSM_F64) return QSM_ERR_DTYPE;
    if (!dims[0] || !dims[1] || !dims[2] || !dims[3]) return QSM_ERR_DIMS;
    if (dims[0] > 0x7fffffff || dims[1] > 0x7fffffff || dims[2] > 0x7fffffff) return QSM_ERR_DIMS;
    if (bdir[0] == 0.0 && bdir[1] == 0.0 && bdir[2] == 0.0) return QSM_ERR_ARG;
    if (!(vsz[0] > 0.0 && vsz[1] > 0.0 && vsz[2] > 0.0)) return QSM_ERR_ARG;
    cudaSetDevice(ctx->device);
    const Dims d{dims[0], dims[1], dims[2]};
    if (maxit <= 0) maxit = (int32_t)std::ceil(std::sqrt((double)d.n()));  // pdf.m:47
    if (tol < 0.0) tol = 1e-5;                                              // pdf.m:48
    const size_t ne = dims[3], es = dt == QSM_F32 ? 4 : 8;
    Staged sf, sm, sw, so;
    QSM_TRY(stage_in(ctx, sf, f, ne * d.n() * es, true));
    QSM_TRY(stage_in(ctx, sm, mask, d.n(), true));
    if (w) QSM_TRY(stage_in(ctx, sw, w, d.n() * es, true));
    QSM_TRY(stage_in(ctx, so, fl, ne * d.n() * es, false));
    qsm_status st =
        dt == QSM_F32
            ? run_pdf<float>(ctx, d, ne, (const float *)sf.dev, (const uint8_t *)sm.dev,
                             w ? (const float *)sw.dev : nullptr, vsz, bdir, lambda, tol, maxit, verbose,
                             (float *)so.dev, iters)
            : run_pdf<double>(ctx, d, ne, (const double *)sf.dev, (const uint8_t *)sm.dev,
                              w ? (const double *)sw.dev : nullptr, vsz, bdir, lambda, tol, maxit, verbose,
                              (double *)so.dev, iters);
    stage_out(ctx, sf, false);
    stage_out(ctx, sm, false);
    if (w) stage_out(ctx, sw, false);
    if (st != QSM_OK) {
        stage_out(ctx, so, false);
        return st;
    }
    QSM_TRY(stage_out(ctx, so, true));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return QSM_OK;
}

}  // extern "C"
