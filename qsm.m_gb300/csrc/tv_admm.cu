// FFT total-variation inversion (ADMM) of src/inversion/tv.m:101-277 on the
// GPU: the data term's solve u = real(ifft3(iA .* (F + fft3(r)))) runs as a
// cuFFT R2C, one fused pointwise k-space kernel, and a cuFFT C2R; the
// gradient, shrinkage, multiplier update and residual norms are fused
// stencil kernels.  tv.m's stopping test and rho update (:226-268) run on the
// device (tv_ctl_k, FP64, the host's arithmetic), so iterations are queued
// without a host round trip; the host reads the control state every eighth
// iteration.
//
// k-space terms come from per-axis tables and one stored half-spectrum array:
//   D(k) = 1/3 - (k.b)^2/|k|^2, D(0) = 0, k_a = fftfreq(n_a, h_a)
//        (dipoleKernel.m:56-65, ifftshifted so DC is first), stored once per
//        solve in the working precision;
//   L(k) = sum_a (2/h_a^2)(1 - cos(2 pi i_a/n_a)), the symbol of the negated
//        7-point Laplacian (laplaceKernel.m, tv.m:140-142): separable, so three
//        1-D tables of FP64 terms;
//   iA   = 1/(mu D^2 + rho L), 0 where not finite (tv.m:144-145), formed in
//        the k-space kernel, so a rho update costs nothing.
// No trigonometry and one division per point per iteration: FP64 arithmetic
// runs at a small fraction of the FP32 rate on this GPU.  u = real(ifft3(X))
// equals the C2R of the Hermitian part of X; the stored half spectrum
// therefore carries, on planes where index negation is not frequency
// negation (even-size Nyquist planes) and B0 is oblique, the average of the
// multipliers at k and at the negated index.
//
// FP64 (the MATLAB default class) or FP32 arithmetic by dtype; every
// reduction accumulates in FP64 with a fixed order (block partials folded
// in block order), so results are run-to-run deterministic.
#include <cufft.h>
#include <math.h>
#include <stdio.h>

#include <algorithm>

#include "common.cuh"

namespace qsm {

template <typename T> struct CxT;
template <> struct CxT<double> { using type = cufftDoubleComplex; };
template <> struct CxT<float> { using type = cufftComplex; };

constexpr int TV_BLOCK = 256;
// Grid-stride kernels run a fixed, fully resident grid (the block partials of the
// reductions then have a fixed count and order): 5 blocks of 256 threads per SM
// in FP32 (<= 51 registers), 3 in FP64 (<= 85 registers).
template <typename T> struct TvOcc { static constexpr int minb = sizeof(T) == 4 ? 5 : 3; };
template <typename T> constexpr int tv_grid() { return 152 * TvOcc<T>::minb; }
// grad_shrink_k needs more registers in FP32 (it spills at 48): 4 blocks per SM
template <typename T> struct TvOccGS { static constexpr int minb = sizeof(T) == 4 ? 4 : 3; };
constexpr int TV_GRID_MAX = 152 * 5;
constexpr int TV_NSUM = 5;         // nr, na, nb, ||s||^2, ||rho grad' l||^2
// ADMM control state on the device (doubles): rho and its inverse, the last
// iteration's residuals and tolerances, the rho-schedule flag, done, iteration
enum { C_RHO, C_IRHO, C_NR, C_NS, C_NA, C_NB, C_EP, C_ED, C_FLAG, C_DONE, C_IT, C_N };

struct TvK {
    int nx, ny, nz, nxh;   // real dims, half-spectrum x extent
    double hx, hy, hz;     // voxel size
    double bx, by, bz;     // unit B0 direction
    double mu;
    bool oblique;          // B0 has two or more non-zero components
};

struct Vox {
    size_t l, NX, NY, NZ;
    int i, j, k;
};

// The voxels of a grid-stride loop in order, with their (i, j, k) advanced by
// carries instead of a 64-bit division per voxel: the stride is split into
// (si, sj, sk) once per thread.
struct VoxWalk {
    Vox v;
    size_t S;
    int si, sj, sk, nx, ny;
    __device__ __forceinline__ VoxWalk(size_t l0, size_t stride, const Dims &d)
    {
        nx = (int)d.nx;
        ny = (int)d.ny;
        v.l = l0;
        v.i = (int)(l0 % d.nx);
        v.j = (int)((l0 / d.nx) % d.ny);
        v.k = (int)(l0 / d.nxny());
        v.NX = d.nx - 1;
        v.NY = d.nx * (d.ny - 1);
        v.NZ = d.nxny() * (d.nz - 1);
        S = stride;
        si = (int)(stride % d.nx);
        sj = (int)((stride / d.nx) % d.ny);
        sk = (int)(stride / d.nxny());
    }
    __device__ __forceinline__ void next()
    {
        v.l += S;
        v.i += si;
        int c = v.i >= nx;
        v.i -= c ? nx : 0;
        v.j += sj + c;
        c = v.j >= ny;
        v.j -= c ? ny : 0;
        v.k += sk + c;
    }
};

#define VOX_LOOP(W, D)                                                                                  \
    for (VoxWalk W((size_t)blockIdx.x * blockDim.x + threadIdx.x, (size_t)gridDim.x * blockDim.x, D); \
         W.v.l < (D).n(); W.next())

__device__ __forceinline__ double fftfreq(int i, int n, double h) { return (double)(i <= (n - 1) / 2 ? i : i - n) / (n * h); }

// per-axis tables: frequencies fx[nxh] fy[ny] fz[nz], then the Laplacian terms
// Lx[nxh] Ly[ny] Lz[nz] (FP64)
__global__ void ktab_k(double *tab, TvK K)
{
    const int na[3] = {K.nxh, K.ny, K.nz}, nn[3] = {K.nx, K.ny, K.nz};
    const double hh[3] = {K.hx, K.hy, K.hz};
    const int tot = K.nxh + K.ny + K.nz;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += gridDim.x * blockDim.x) {
        int a = 0, i = t;
        while (i >= na[a]) i -= na[a++];
        tab[t] = fftfreq(i, nn[a], hh[a]);
        tab[tot + t] = (2.0 / (hh[a] * hh[a])) * (1.0 - cospi(2.0 * i / nn[a]));
    }
}

__device__ __forceinline__ double dipole_at(const TvK &K, double fx, double fy, double fz)
{
    const double kb = K.bx * fx + K.by * fy + K.bz * fz;
    const double k2 = fx * fx + fy * fy + fz * fz;
    return 1.0 / 3.0 - (kb * kb) / k2;
}

// D on the half spectrum, rounded to the working precision
template <typename T>
__global__ void dq_k(T *Dq, const double *__restrict__ tab, TvK K)
{
    const size_t nh = (size_t)K.nxh * K.ny * K.nz;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nh; q += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(q % K.nxh), j = (int)((q / K.nxh) % K.ny), k = (int)(q / ((size_t)K.nxh * K.ny));
        Dq[q] = q == 0 ? (T)0 : (T)dipole_at(K, tab[i], tab[K.nxh + j], tab[K.nxh + K.ny + k]);
    }
}

template <typename T>
__device__ __forceinline__ T inv_a(T K, T L, T rho)
{
    const T a = (T)1 / (K + rho * L);
    return isfinite(a) ? a : (T)0;
}

// X = iA .* (mu D .* fhat + R) / N in place of R (tv.m:172-175), in the working
// precision T
template <typename T>
__global__ void __launch_bounds__(TV_BLOCK, TvOcc<T>::minb) kmul_k(typename CxT<T>::type *R, const typename CxT<T>::type *__restrict__ fhat,
                       const T *__restrict__ Dq, const double *__restrict__ tab, TvK K, const double *ctl, double invn_)
{
    const int tot = K.nxh + K.ny + K.nz;
    const T mu = (T)K.mu, rho = (T)ctl[C_RHO], invn = (T)invn_;
    const Dims hd{(size_t)K.nxh, (size_t)K.ny, (size_t)K.nz};
    VOX_LOOP(wk, hd) {
        const size_t q = wk.v.l;
        const int i = wk.v.i, j = wk.v.j, k = wk.v.k;
        const T D = Dq[q];
        const T L = (T)((tab[tot + i] + tab[tot + K.nxh + j]) + tab[tot + K.nxh + K.ny + k]);
        T a = inv_a<T>(mu * D * D, L, rho), ad = a * (mu * D);
        if (K.oblique && ((2 * i == K.nx) || (2 * j == K.ny) || (2 * k == K.nz))) {
            // the negated index keeps Nyquist frequencies and flips the others
            const double fx = tab[i], fy = tab[K.nxh + j], fz = tab[K.nxh + K.ny + k];
            const double gx = 2 * i == K.nx ? fx : -fx, gy = 2 * j == K.ny ? fy : -fy, gz = 2 * k == K.nz ? fz : -fz;
            const T D2 = (T)dipole_at(K, gx, gy, gz);
            const T a2 = inv_a<T>(mu * D2 * D2, L, rho);
            ad = (T)0.5 * (ad + a2 * (mu * D2));
            a = (T)0.5 * (a + a2);
        }
        const typename CxT<T>::type fh = fhat[q], r = R[q];
        typename CxT<T>::type o;
        o.x = (ad * fh.x + a * r.x) * invn;
        o.y = (ad * fh.y + a * r.y) * invn;
        R[q] = o;
    }
}


// gradfp_adj_mex.c:156-257 of the field g_c(l) (h holds -1/h), with the
// reference's association order of the three axis terms.
template <typename T, typename G>
__device__ __forceinline__ T adj_at(const Vox &v, const Dims &d, const T *ih, G g)
{
    const size_t l = v.l;
    const T a = ih[0] * (g(0, l) - g(0, v.i > 0 ? l - 1 : l + v.NX));
    const T b = ih[1] * (g(1, l) - g(1, v.j > 0 ? l - d.nx : l + v.NY));
    const T c = ih[2] * (g(2, l) - g(2, v.k > 0 ? l - d.nxny() : l + v.NZ));
    return v.k == 0 ? (a + b) + c : v.j == 0 ? (c + a) + b : (c + b) + a;
}

// r = gradfp_adj(rho v - l) (tv.m:166-170).  Iteration ii also keeps u when
// the control state says iteration ii - 1 converged: the iterations the host
// launched past convergence overwrite u.
template <typename T>
__global__ void __launch_bounds__(TV_BLOCK, TvOcc<T>::minb) adj_rhs_k(T *r, const T *__restrict__ v, const T *__restrict__ lm, Dims d, T nx_, T ny_, T nz_,
                                       const double *ctl, int ii, T *usave, const T *__restrict__ u)
{
    const size_t N = d.n();
    const T ih[3] = {nx_, ny_, nz_};
    const T rho = (T)ctl[C_RHO];
    const bool save = ctl[C_DONE] != 0.0 && ctl[C_IT] == (double)(ii - 1);
    VOX_LOOP(wk, d) {
        if (save) usave[wk.v.l] = u[wk.v.l];
        r[wk.v.l] = adj_at<T>(wk.v, d, ih, [&](int c, size_t m) { return rho * v[c * N + m] - lm[c * N + m]; });
    }
}

template <int NS>
__device__ __forceinline__ void block_sums(double *part, double (&acc)[NS])
{
    __shared__ double red[NS][TV_BLOCK];
    const int t = threadIdx.x;
#pragma unroll
    for (int q = 0; q < NS; ++q) red[q][t] = acc[q];
    __syncthreads();
    for (int s = TV_BLOCK / 2; s > 0; s >>= 1) {
        if (t < s)
#pragma unroll
            for (int q = 0; q < NS; ++q) red[q][t] += red[q][t + s];
        __syncthreads();
    }
    if (t == 0)
#pragma unroll
        for (int q = 0; q < NS; ++q) part[q * gridDim.x + blockIdx.x] = red[q][0];
}

// grad, over-relaxation, shrinkage, multiplier update and the primal
// residual sums of one ADMM iteration (tv.m:185-221, :227-234)
template <typename T, bool ISO>
__global__ void __launch_bounds__(TV_BLOCK, TvOccGS<T>::minb)
grad_shrink_k(T *vn, const T *__restrict__ vo, T *lm, const T *__restrict__ u, Dims d, T hx, T hy, T hz, T alpha,
              const double *ctl, double *part)
{
    const T rho = (T)ctl[C_RHO], irho = (T)ctl[C_IRHO];
    const size_t N = d.n();
    PartialSum<T> ps[3];  // nr, na, nb
    VOX_LOOP(wk, d) {
        const Vox &v = wk.v;
        const size_t l = v.l;
        const T u0 = u[l];
        T dd[3];
        dd[0] = hx * ((v.i + 1 < (int)d.nx ? u[l + 1] : u[l - v.NX]) - u0);
        dd[1] = hy * ((v.j + 1 < (int)d.ny ? u[l + d.nx] : u[l - v.NY]) - u0);
        dd[2] = hz * ((v.k + 1 < (int)d.nz ? u[l + d.nxny()] : u[l - v.NZ]) - u0);
        T d1[3], r[3], w[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            d1[c] = alpha * dd[c] + ((T)1 - alpha) * vo[c * N + l];
            r[c] = d1[c] + irho * lm[c * N + l];
        }
        if (ISO) {
            T s = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            s = (s - irho) * (T)(s > irho) / s;
            if (!isfinite(s)) s = (T)0;
#pragma unroll
            for (int c = 0; c < 3; ++c) w[c] = r[c] * s;
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const T m = fabs(r[c]) - irho;
                const T sg = r[c] > (T)0 ? (T)1 : r[c] < (T)0 ? (T)-1 : (T)0;
                w[c] = (m > (T)0 ? m : (T)0) * sg;
            }
        }
        // per-voxel norms in the working precision (as MATLAB computes them in
        // the class of f), summed in FP64
        T e2 = 0, a2 = 0, b2 = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            vn[c * N + l] = w[c];
            lm[c * N + l] = lm[c * N + l] + rho * (d1[c] - w[c]);
            const T e = dd[c] - w[c];
            e2 += e * e;
            a2 += dd[c] * dd[c];
            b2 += w[c] * w[c];
        }
        ps[0].add(sqrt(e2));
        ps[1].add(sqrt(a2));
        ps[2].add(sqrt(b2));
    }
    double acc[3] = {ps[0].get(), ps[1].get(), ps[2].get()};
    block_sums<3>(part, acc);
}

// Anisotropic TV in FP32: grad_shrink_k and adj_norms_k in one pass.  Each
// thread also evaluates, for c = x, y, z, component c of the shrinkage at its
// backward neighbour along c -- the values the adjoint reads there -- with the
// neighbour owner's own arithmetic (bit-identical), so the new v and l are not
// read back; l is double-buffered (lmo in, lmn out) because neighbours read
// the old value.
template <typename T>
__global__ void __launch_bounds__(TV_BLOCK, TvOccGS<T>::minb)
grad_shrink_norms_k(T *vn, const T *__restrict__ vo, T *__restrict__ lmn, const T *__restrict__ lmo,
                    const T *__restrict__ u, Dims d, T hx, T hy, T hz, T alpha, const double *ctl, T nx_, T ny_, T nz_,
                    double *part)
{
    const T rho = (T)ctl[C_RHO], irho = (T)ctl[C_IRHO];
    const size_t N = d.n();
    const T hh[3] = {hx, hy, hz}, ih[3] = {nx_, ny_, nz_};
    PartialSum<T> ps[5];  // nr, na, nb, ||s||^2, ||rho grad' l||^2
    VOX_LOOP(wk, d) {
        const Vox &v = wk.v;
        const size_t l = v.l;
        const T u0 = u[l];
        const size_t fw[3] = {v.i + 1 < (int)d.nx ? l + 1 : l - v.NX, v.j + 1 < (int)d.ny ? l + d.nx : l - v.NY,
                              v.k + 1 < (int)d.nz ? l + d.nxny() : l - v.NZ};
        const size_t bw[3] = {v.i > 0 ? l - 1 : l + v.NX, v.j > 0 ? l - d.nx : l + v.NY,
                              v.k > 0 ? l - d.nxny() : l + v.NZ};
        T e2 = 0, a2 = 0, b2 = 0, gs[3], gt[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            // own voxel (grad_shrink_k, ISO = false)
            const T dd = hh[c] * (u[fw[c]] - u0);
            const T vo0 = vo[c * N + l], lo0 = lmo[c * N + l];
            const T d1 = alpha * dd + ((T)1 - alpha) * vo0;
            const T r = d1 + irho * lo0;
            const T mg = fabs(r) - irho;
            const T w = (mg > (T)0 ? mg : (T)0) * (r > (T)0 ? (T)1 : r < (T)0 ? (T)-1 : (T)0);
            const T ln = lo0 + rho * (d1 - w);
            vn[c * N + l] = w;
            lmn[c * N + l] = ln;
            const T e = dd - w;
            e2 += e * e;
            a2 += dd * dd;
            b2 += w * w;
            // component c at the backward neighbour m, whose forward neighbour along c is l
            const size_t m = bw[c];
            const T ddm = hh[c] * (u0 - u[m]);
            const T vom = vo[c * N + m], lom = lmo[c * N + m];
            const T d1m = alpha * ddm + ((T)1 - alpha) * vom;
            const T rm = d1m + irho * lom;
            const T mgm = fabs(rm) - irho;
            const T wm = (mgm > (T)0 ? mgm : (T)0) * (rm > (T)0 ? (T)1 : rm < (T)0 ? (T)-1 : (T)0);
            const T lnm = lom + rho * (d1m - wm);
            gs[c] = ih[c] * ((w - vo0) - (wm - vom));
            gt[c] = ih[c] * (ln - lnm);
        }
        ps[0].add(sqrt(e2));
        ps[1].add(sqrt(a2));
        ps[2].add(sqrt(b2));
        // adj_at's association order (gradfp_adj_mex.c regions)
        const T sa = v.k == 0 ? (gs[0] + gs[1]) + gs[2] : v.j == 0 ? (gs[2] + gs[0]) + gs[1] : (gs[2] + gs[1]) + gs[0];
        const T ta = v.k == 0 ? (gt[0] + gt[1]) + gt[2] : v.j == 0 ? (gt[2] + gt[0]) + gt[1] : (gt[2] + gt[1]) + gt[0];
        const T sv = rho * sa, tv = rho * ta;
        ps[3].add(sv * sv);
        ps[4].add(tv * tv);
    }
    double acc[5] = {ps[0].get(), ps[1].get(), ps[2].get(), ps[3].get(), ps[4].get()};
    block_sums<5>(part, acc);
}

// ||rho gradfp_adj(v - v_)||^2 and ||rho gradfp_adj(l)||^2 (tv.m:230, :239)
template <typename T>
__global__ void __launch_bounds__(TV_BLOCK, TvOcc<T>::minb)
adj_norms_k(const T *__restrict__ vn, const T *__restrict__ vo, const T *__restrict__ lm, Dims d, T nx_, T ny_, T nz_,
            const double *ctl, double *part)
{
    const T rho = (T)ctl[C_RHO];
    const size_t N = d.n();
    const T ih[3] = {nx_, ny_, nz_};
    PartialSum<T> ps[2];
    VOX_LOOP(wk, d) {
        const T s = rho * adj_at<T>(wk.v, d, ih, [&](int c, size_t m) { return vn[c * N + m] - vo[c * N + m]; });
        const T t = rho * adj_at<T>(wk.v, d, ih, [&](int c, size_t m) { return lm[c * N + m]; });
        ps[0].add(s * s);
        ps[1].add(t * t);
    }
    double acc[2] = {ps[0].get(), ps[1].get()};
    block_sums<2>(part, acc);
}

// initial v = grad(u), nr = sum |v| (tv.m:150-152)
template <typename T>
__global__ void __launch_bounds__(TV_BLOCK, TvOcc<T>::minb)
grad_init_k(T *v, const T *__restrict__ u, Dims d, T hx, T hy, T hz, double *part)
{
    const size_t N = d.n();
    PartialSum<T> ps;
    VOX_LOOP(wk, d) {
        const Vox &x = wk.v;
        const size_t l = x.l;
        const T u0 = u[l];
        const T a = hx * ((x.i + 1 < (int)d.nx ? u[l + 1] : u[l - x.NX]) - u0);
        const T b = hy * ((x.j + 1 < (int)d.ny ? u[l + d.nx] : u[l - x.NY]) - u0);
        const T c = hz * ((x.k + 1 < (int)d.nz ? u[l + d.nxny()] : u[l - x.NZ]) - u0);
        v[l] = a;
        v[N + l] = b;
        v[2 * N + l] = c;
        ps.add(sqrt(a * a + b * b + c * c));
    }
    double acc[1] = {ps.get()};
    block_sums<1>(part, acc);
}

// fold block partials in a fixed order: sums 0..ns1-1 have nblk1 partials
// each (at part), sums ns1..ns1+ns2-1 have nblk2 each (after them); thread t
// adds partials t, t + 256, ... of every sum in turn, then one shared-memory
// tree over all sums together (one block of 256 threads)
__global__ void __launch_bounds__(TV_BLOCK) fold_k(double *out, const double *__restrict__ part, int ns1, int nblk1,
                                                   int ns2, int nblk2)
{
    __shared__ double red[TV_NSUM][TV_BLOCK];
    const int t = threadIdx.x, ns = ns1 + ns2;
    for (int q = 0; q < TV_NSUM; ++q) {
        double s = 0.0;
        if (q < ns) {
            const double *p = q < ns1 ? part + q * nblk1 : part + ns1 * nblk1 + (q - ns1) * nblk2;
            const int nb = q < ns1 ? nblk1 : nblk2;
            for (int b = t; b < nb; b += TV_BLOCK) s += p[b];
        }
        red[q][t] = s;
    }
    __syncthreads();
    for (int h = TV_BLOCK / 2; h > 0; h >>= 1) {
        if (t < h)
#pragma unroll
            for (int q = 0; q < TV_NSUM; ++q) red[q][t] += red[q][t + h];
        __syncthreads();
    }
    if (t < ns) out[t] = red[t][0];
}

template <typename T, typename S>
__global__ void cvt_in_k(T *o, const S *__restrict__ a, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        o[l] = (T)a[l];
}

// x = mask .* u (tv.m:275)
template <typename T, typename S>
__global__ void mask_out_k(S *x, const T *__restrict__ u, const uint8_t *__restrict__ m, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        x[l] = (S)((m[l] ? (T)1 : (T)0) * u[l]);
}

static const char *cufft_str(cufftResult r)
{
    switch (r) {
    case CUFFT_SUCCESS: return "CUFFT_SUCCESS";
    case CUFFT_ALLOC_FAILED: return "CUFFT_ALLOC_FAILED";
    case CUFFT_INVALID_VALUE: return "CUFFT_INVALID_VALUE";
    case CUFFT_INVALID_SIZE: return "CUFFT_INVALID_SIZE";
    case CUFFT_EXEC_FAILED: return "CUFFT_EXEC_FAILED";
    default: return "cuFFT error";
    }
}

// tv.m's stopping test and rho schedule (tv.m:226-268) for iteration ii, in
// FP64 with the host's operations and order (no fused multiply-add on either
// side), from the five sums of the iteration.  Nothing changes once done.
struct TvCtlOpts {
    double rtol, atolp, atold, rtau, stau, gamma;
};

__global__ void tv_ctl_k(double *ctl, const double *__restrict__ sums, TvCtlOpts o, int ii)
{
    if (ctl[C_DONE] != 0.0) return;
    const double nrp = ctl[C_NR];
    const double nr = sums[0], na = sums[1], nb = sums[2], ns = sqrt(sums[3]);
    const double ep = o.atolp + o.rtol * (na < nb ? nb : na);
    const double ed = o.atold + o.rtol * sqrt(sums[4]);
    ctl[C_NR] = nr;
    ctl[C_NS] = ns;
    ctl[C_NA] = na;
    ctl[C_NB] = nb;
    ctl[C_EP] = ep;
    ctl[C_ED] = ed;
    ctl[C_IT] = (double)ii;
    if (nr < ep && ns < ed) {
        ctl[C_DONE] = 1.0;
        return;
    }
    double rho = ctl[C_RHO], flag = ctl[C_FLAG];
    if (nr > o.stau * ns || (nr > o.rtau * nrp && flag < 3.0)) {
        rho = o.gamma * rho;
        ctl[C_IRHO] = 1.0 / rho;
        if (flag > 5.0) flag = 0.0;
    } else if (nr < ns / o.stau) {
        rho = rho / (o.gamma * o.gamma);
        ctl[C_IRHO] = 1.0 / rho;
        flag = flag + 1.0;
    }
    ctl[C_RHO] = rho;
    ctl[C_FLAG] = flag;
}

#define QSM_FFT(call)                                                                           \
    do {                                                                                        \
        cufftResult r_ = (call);                                                                \
        if (r_ != CUFFT_SUCCESS) {                                                              \
            ::qsm::set_error(ctx, "%s:%d %s: %s", __FILE__, __LINE__, #call, cufft_str(r_));    \
            st = r_ == CUFFT_ALLOC_FAILED ? QSM_ERR_NOMEM : QSM_ERR_CUDA;                      \
            goto done;                                                                          \
        }                                                                                       \
    } while (0)

#define QSM_STEP(expr)           \
    do {                         \
        st = (expr);             \
        if (st != QSM_OK) goto done; \
    } while (0)

static qsm_status cuda_st(qsm_ctx *ctx, cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return QSM_OK;
    set_error(ctx, "%s: %s", what, cudaGetErrorString(e));
    return QSM_ERR_CUDA;
}

struct TvOpts {
    double mu, rtol, atol, rho, alpha, rtau, stau, gamma;
    int tv, maxit, verbose;
};

template <typename T, typename S>
static qsm_status tv_run(qsm_ctx *ctx, const Dims &d, const S *f, const uint8_t *mask, const double *h,
                         const double *bdir, TvOpts o, S *xout, qsm_tv_info *info)
{
    using C = typename CxT<T>::type;
    const size_t N = d.n();
    const int nxh = (int)(d.nx / 2 + 1);
    const size_t nh = (size_t)nxh * d.ny * d.nz;
    // u, r, v[2] (3 components each, N apart), l (3); fhat, R; partials + sums
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t rb = al(N * sizeof(T)), vb = al(3 * N * sizeof(T)), cb = al(nh * sizeof(C));
    const size_t tb = al(2 * (size_t)(nxh + d.ny + d.nz) * sizeof(double)), db = al(nh * sizeof(T));
    const size_t bytes = 3 * rb + 4 * vb + 2 * cb + tb + db + (TV_NSUM * TV_GRID_MAX + 64 + C_N) * sizeof(double);
    void *blk = nullptr;
    QSM_TRY(dalloc(ctx, &blk, bytes));
    char *c = (char *)blk;
    T *u = (T *)c; c += rb;
    T *r = (T *)c; c += rb;
    T *usave = (T *)c; c += rb;  // u of the converged iteration
    T *v[2];
    v[0] = (T *)c; c += vb;
    v[1] = (T *)c; c += vb;
    T *lmb[2];  // l, double-buffered where the fused FP32 pass reads the old value at neighbours
    lmb[0] = (T *)c; c += vb;
    lmb[1] = (T *)c; c += vb;
    int lc = 0;
    C *fhat = (C *)c; c += cb;
    C *R = (C *)c; c += cb;
    double *tab = (double *)c; c += tb;
    T *Dq = (T *)c; c += db;
    double *part = (double *)c;
    double *sums = part + TV_NSUM * TV_GRID_MAX;
    double *ctl = sums + 64;

    qsm_status st = QSM_OK;
    cufftHandle pf = 0, pi = 0;
    bool havef = false, havei = false;
    const cufftType tf = sizeof(T) == 8 ? CUFFT_D2Z : CUFFT_R2C, ti = sizeof(T) == 8 ? CUFFT_Z2D : CUFFT_C2R;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double hc[C_N] = {};
    int cur = 0;
    uint32_t it = 0;
    bool from_save = false;
    const double atolp = sqrt(3.0 * (double)N) * o.atol, atold = sqrt((double)N) * o.atol;
    TvK K;
    K.nx = (int)d.nx; K.ny = (int)d.ny; K.nz = (int)d.nz; K.nxh = nxh;
    K.hx = h[0]; K.hy = h[1]; K.hz = h[2];
    {
        const double bn = sqrt(bdir[0] * bdir[0] + bdir[1] * bdir[1] + bdir[2] * bdir[2]);
        K.bx = bdir[0] / bn; K.by = bdir[1] / bn; K.bz = bdir[2] / bn;
        K.oblique = ((bdir[0] != 0.0) + (bdir[1] != 0.0) + (bdir[2] != 0.0)) > 1;
    }
    K.mu = o.mu;
    const T ihx = (T)(1.0 / h[0]), ihy = (T)(1.0 / h[1]), ihz = (T)(1.0 / h[2]);
    const int TV_GRID = tv_grid<T>(), GS_GRID = 152 * TvOccGS<T>::minb;
    const dim3 g(TV_GRID), gs(GS_GRID), b(TV_BLOCK);
    const unsigned gk = (unsigned)std::min<size_t>((nh + TV_BLOCK - 1) / TV_BLOCK, (size_t)TV_GRID);

    QSM_STEP(cuda_st(ctx, cudaMemsetAsync(lmb[0], 0, 3 * N * sizeof(T), ctx->stream), "memset"));
    QSM_FFT(cufftPlan3d(&pf, (int)d.nz, (int)d.ny, (int)d.nx, tf));
    havef = true;
    QSM_FFT(cufftPlan3d(&pi, (int)d.nz, (int)d.ny, (int)d.nx, ti));
    havei = true;
    QSM_FFT(cufftSetStream(pf, ctx->stream));
    QSM_FFT(cufftSetStream(pi, ctx->stream));
    QSM_STEP(cuda_st(ctx, cudaEventCreate(&e0), "event"));
    QSM_STEP(cuda_st(ctx, cudaEventCreate(&e1), "event"));
    QSM_STEP(cuda_st(ctx, cudaEventRecord(e0, ctx->stream), "event"));

    // k-space tables and D (once per solve)
    ktab_k<<<1, 256, 0, ctx->stream>>>(tab, K);
    dq_k<T><<<gk, TV_BLOCK, 0, ctx->stream>>>(Dq, tab, K);
    // u = f; fhat = fft3(f) (F = mu conj(D) fhat is formed in kmul_k)
    cvt_in_k<T, S><<<g, b, 0, ctx->stream>>>(u, f, N);
    if (sizeof(T) == 8) QSM_FFT(cufftExecD2Z(pf, (cufftDoubleReal *)u, (cufftDoubleComplex *)fhat));
    else QSM_FFT(cufftExecR2C(pf, (cufftReal *)u, (cufftComplex *)fhat));
    grad_init_k<T><<<g, b, 0, ctx->stream>>>(v[0], u, d, ihx, ihy, ihz, part);
    fold_k<<<1, TV_BLOCK, 0, ctx->stream>>>(sums, part, 1, TV_GRID, 0, 0);
    // control state: rho, 1/rho (as the host forms it), nr of the initial v, flag 0
    hc[C_RHO] = o.rho;
    hc[C_IRHO] = 1.0 / o.rho;
    QSM_STEP(cuda_st(ctx, cudaMemcpyAsync(ctl, hc, C_N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "copy"));
    QSM_STEP(cuda_st(ctx, cudaMemcpyAsync(ctl + C_NR, sums, sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream), "copy"));
    if (o.verbose) printf("\niter\t\t||r||\t\teps_pri\t\t||s||\t\teps_dual\n");

    // Iterations are queued without waiting: tv_ctl_k applies the stopping
    // test and the rho schedule on the device, and the host reads the state
    // every `chunk` iterations (every iteration when printing).  Iterations
    // queued past convergence compute on with frozen rho; the converged u is
    // kept by the next adj_rhs_k, and the solve reports the converged state.
    {
        const TvCtlOpts co{o.rtol, atolp, atold, o.rtau, o.stau, o.gamma};
        const int chunk = o.verbose ? 1 : 8;
        int ii = 1, last = 0;
        bool done = false;
        while (ii <= o.maxit && !done) {
            const int end = std::min(o.maxit, ii + chunk - 1);
            for (; ii <= end; ++ii) {
                const int nxt = cur ^ 1;
                // u-subproblem
                adj_rhs_k<T><<<g, b, 0, ctx->stream>>>(r, v[cur], lmb[lc], d, -ihx, -ihy, -ihz, ctl, ii, usave, u);
                if (sizeof(T) == 8) QSM_FFT(cufftExecD2Z(pf, (cufftDoubleReal *)r, (cufftDoubleComplex *)R));
                else QSM_FFT(cufftExecR2C(pf, (cufftReal *)r, (cufftComplex *)R));
                kmul_k<T><<<gk, TV_BLOCK, 0, ctx->stream>>>(R, fhat, Dq, tab, K, ctl, 1.0 / (double)N);
                if (sizeof(T) == 8) QSM_FFT(cufftExecZ2D(pi, (cufftDoubleComplex *)R, (cufftDoubleReal *)u));
                else QSM_FFT(cufftExecC2R(pi, (cufftComplex *)R, (cufftReal *)u));
                // v-subproblem, multipliers, residuals
                if (sizeof(T) == 4 && o.tv == 1) {
                    grad_shrink_norms_k<T><<<gs, b, 0, ctx->stream>>>(v[nxt], v[cur], lmb[lc ^ 1], lmb[lc], u, d, ihx,
                                                                      ihy, ihz, (T)o.alpha, ctl, -ihx, -ihy, -ihz,
                                                                      part);
                    lc ^= 1;
                    fold_k<<<1, TV_BLOCK, 0, ctx->stream>>>(sums, part, TV_NSUM, GS_GRID, 0, 0);
                } else {
                    if (o.tv == 1)
                        grad_shrink_k<T, false><<<gs, b, 0, ctx->stream>>>(v[nxt], v[cur], lmb[lc], u, d, ihx, ihy,
                                                                           ihz, (T)o.alpha, ctl, part);
                    else
                        grad_shrink_k<T, true><<<gs, b, 0, ctx->stream>>>(v[nxt], v[cur], lmb[lc], u, d, ihx, ihy,
                                                                          ihz, (T)o.alpha, ctl, part);
                    adj_norms_k<T><<<g, b, 0, ctx->stream>>>(v[nxt], v[cur], lmb[lc], d, -ihx, -ihy, -ihz, ctl,
                                                             part + 3 * GS_GRID);
                    fold_k<<<1, TV_BLOCK, 0, ctx->stream>>>(sums, part, 3, GS_GRID, 2, TV_GRID);
                }
                tv_ctl_k<<<1, 1, 0, ctx->stream>>>(ctl, sums, co, ii);
                QSM_STEP(cuda_st(ctx, cudaGetLastError(), "launch"));
                cur = nxt;
            }
            last = ii - 1;
            QSM_STEP(cuda_st(ctx, cudaMemcpyAsync(hc, ctl, C_N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "copy"));
            QSM_STEP(cuda_st(ctx, cudaStreamSynchronize(ctx->stream), "sync"));
            done = hc[C_DONE] != 0.0;
            if (o.verbose)
                printf("%3d/%d\t\t%.4e\t%.4e\t%.4e\t%.4e\n", (int)hc[C_IT], o.maxit, hc[C_NR], hc[C_EP], hc[C_NS],
                       hc[C_ED]);
        }
        it = done ? (uint32_t)hc[C_IT] : (uint32_t)last;
        from_save = done && (int)hc[C_IT] < last;
    }
    if (o.verbose) printf("\n");
    QSM_STEP(cuda_st(ctx, cudaEventRecord(e1, ctx->stream), "event"));
    mask_out_k<T, S><<<g, b, 0, ctx->stream>>>(xout, from_save ? usave : u, mask, N);
    QSM_STEP(cuda_st(ctx, cudaGetLastError(), "launch"));
    QSM_STEP(cuda_st(ctx, cudaStreamSynchronize(ctx->stream), "sync"));
    if (info) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        info->iters = it;
        info->rho = hc[C_RHO];
        info->nr = hc[C_NR];
        info->eps_pri = hc[C_EP];
        info->ns = hc[C_NS];
        info->eps_dual = hc[C_ED];
        info->seconds = ms * 1e-3;
    }
done:
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (havef) cufftDestroy(pf);
    if (havei) cufftDestroy(pi);
    qsm_status st2 = dfree(ctx, blk);
    return st != QSM_OK ? st : st2;
}

}  // namespace qsm

using namespace qsm;

extern "C" qsm_status qsm_tv_admm(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], const void *f, const uint8_t *mask,
                                  const double vsz[3], const double bdir[3], double mu, int32_t tv, double rtol,
                                  double atol, int32_t maxit, double rho, double alpha, double rtau, double stau,
                                  double gamma, int32_t verbose, void *x, qsm_tv_info *info)
{
    Range nvtx_range("tv_admm");
    if (!ctx || !dims || !f || !mask || !vsz || !bdir || !x) return QSM_ERR_ARG;
    if (dt != QSM_F32 && dt != QSM_F64) return QSM_ERR_DTYPE;
    if (tv != 1 && tv != 2) return QSM_ERR_ARG;
    if (maxit < 0 || !(rho > 0.0)) return QSM_ERR_ARG;
    if (bdir[0] == 0.0 && bdir[1] == 0.0 && bdir[2] == 0.0) return QSM_ERR_ARG;
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    if (d.nx < 3 || d.ny < 3 || d.nz < 3) {
        set_error(ctx, "tv: every dimension must be >= 3 (padarray of the 3x3x3 Laplace kernel)");
        return QSM_ERR_DIMS;
    }
    if (d.nx > 0x7fffffff || d.ny > 0x7fffffff || d.nz > 0x7fffffff) return QSM_ERR_DIMS;
    const size_t es = dt == QSM_F32 ? 4 : 8;
    Staged sf, sm, sx;
    QSM_TRY(stage_in(ctx, sf, f, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sm, mask, d.n(), true));
    QSM_TRY(stage_in(ctx, sx, x, d.n() * es, false));
    TvOpts o{mu, rtol, atol, rho, alpha, rtau, stau, gamma, tv, maxit, verbose};
    qsm_status st;
    if (dt == QSM_F64)
        st = tv_run<double, double>(ctx, d, (const double *)sf.dev, (const uint8_t *)sm.dev, vsz, bdir, o,
                                    (double *)sx.dev, info);
    else
        st = tv_run<float, float>(ctx, d, (const float *)sf.dev, (const uint8_t *)sm.dev, vsz, bdir, o,
                                  (float *)sx.dev, info);
    stage_out(ctx, sf, false);
    stage_out(ctx, sm, false);
    if (st != QSM_OK) {
        stage_out(ctx, sx, false);
        return st;
    }
    return stage_out(ctx, sx, true);
}
