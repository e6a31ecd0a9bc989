// Multigrid-preconditioned CG Poisson solver and its pieces:
//   -Delta u = f in the mask G, u = 0 outside, on a grid padded by one voxel.
//
// Kernels evaluate the reference's per-voxel expressions in order without
// fused multiply-add (bit-identical to src/utils/poisson_solver/mex/*.c in
// FP32 and FP64).  Inner products and norms use the lane order of
// common.cu, as does the oracle's BLAS shim, so whole PCG solves are
// reproducible bit-for-bit.
//
//   red-black Gauss-Seidel  a pass only reads the other colour, so its voxels
//                           are independent and may run in any order.  Every
//                           level keeps its G voxels and its boundary band B
//                           as per-colour lists; a smoothing call runs its
//                           passes as one launch per pass (large lists), in
//                           one cooperative whole-GPU launch with a grid
//                           barrier per pass (mid-size), or in one cluster
//                           launch (small); full-grid passes remain for the
//                           public gauss_seidel_mex and grids without lists
//   coarsest level          the reference's <= 1024 x (128 reverse + 128
//                           forward sweeps + residual + norm) loop in one
//                           launch: z-slabs over a 16-CTA cluster in shared
//                           memory (small grids), over every SM with a grid
//                           barrier (large passes), or in one CTA; the norm
//                           keeps the lane order; no host round trips
//   PCG                     the BLAS-1 steps fused into four kernels on the
//                           lane-dot grid; scalars stay on the device and the
//                           host reads ||r|| once per iteration; where the
//                           iterate and residual are +0 outside G, warps visit
//                           only their lane-grid segments that hold G.  The
//                           mixed solver (FP32 V-cycle) contracts the FP64
//                           recurrence's multiply-adds into FMAs
#include <math.h>
#include <stdlib.h>
#include <algorithm>
#include <memory>
#include <mutex>
#include <set>
#include <vector>

#include "common.cuh"
#include "mg_pack.cuh"

namespace qsm {

template <typename T> struct GsC { T hx, hy, hz, hh; };

template <typename T> static GsC<T> gs_consts(const double *h)
{
    // gauss_seidel_mex.c:96-99 / :214-217
    GsC<T> c;
    c.hx = (T)(1.0 / (h[0] * h[0]));
    c.hy = (T)(1.0 / (h[1] * h[1]));
    c.hz = (T)(1.0 / (h[2] * h[2]));
    c.hh = (T)(1.0 / (2.0 * (double)(c.hx + c.hy + c.hz)));
    return c;
}

template <typename T> struct LapC { T hx, hy, hz, hh; };

template <typename T> static LapC<T> lap_consts(const double *h)
{
    // residual_mex.c:98-101 / lapmg_mex.c:87-90
    LapC<T> c;
    c.hx = (T)(1.0 / (h[0] * h[0]));
    c.hy = (T)(1.0 / (h[1] * h[1]));
    c.hz = (T)(1.0 / (h[2] * h[2]));
    c.hh = (T)(-2.0 * (c.hx + c.hy + c.hz));
    return c;
}

// ---------------------------------------------------------------------------
// thread-block cluster primitives (inline PTX)
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t cl_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cl_size()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
// all threads of all CTAs in the cluster; release / acquire at cluster scope
__device__ __forceinline__ void cl_sync()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// shared::cluster address of this shared-memory location in CTA `rank`
__device__ __forceinline__ uint32_t cl_map(const void *p, uint32_t rank)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ void cl_st(uint32_t a, double v)
{
    asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}
__device__ __forceinline__ void cl_st(uint32_t a, float v)
{
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}
// bitwise OR into a word of a CTA of the cluster (visible after the next cl_sync)
__device__ __forceinline__ void cl_or(uint32_t a, uint32_t v)
{
    asm volatile("red.relaxed.cluster.shared::cluster.or.b32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}

// ---------------------------------------------------------------------------
// Gauss-Seidel colour pass (gauss_seidel_mex.c:138-190 / :256-308)
// Pass over voxels with (i + j + k) = par (mod 2) in the interior, except
// x index skip_i.
// ---------------------------------------------------------------------------

template <typename T>
__global__ void gs_color_k(T *v, const T *__restrict__ f, const uint8_t *__restrict__ G, GsC<T> c, Dims d, int par,
                           size_t skip_i)
{
    const size_t j = 1 + (size_t)blockIdx.y * blockDim.y + threadIdx.y;
    const size_t k = 1 + (size_t)blockIdx.z * blockDim.z + threadIdx.z;
    if (j + 1 >= d.ny || k + 1 >= d.nz) return;
    const size_t i = 1 + ((1 + j + k + par) & 1) + 2 * ((size_t)blockIdx.x * blockDim.x + threadIdx.x);
    if (i + 1 >= d.nx || i == skip_i) return;
    const size_t nx = d.nx, nxny = d.nxny(), l = i + nx * j + nxny * k;
    if (!G[l]) return;
    v[l] = c.hh * (f[l] + (c.hx * (v[l - 1] + v[l + 1]) + c.hy * (v[l - nx] + v[l + nx]) + c.hz * (v[l - nxny] + v[l + nxny])));
}

template <typename T>
static qsm_status gauss_seidel(qsm_ctx *ctx, T *v, const T *f, const uint8_t *G, const double *h, const Dims &d,
                               int32_t iter, bool rev)
{
    if (d.nx < 3 || d.ny < 3 || d.nz < 3 || iter <= 0) return QSM_OK;
    const GsC<T> c = gs_consts<T>(h);
    const dim3 b(32, 4, 2);
    const dim3 g((unsigned)(((d.nx - 2 + 1) / 2 + 31) / 32), (unsigned)((d.ny - 2 + 3) / 4), (unsigned)((d.nz - 2 + 1) / 2));
    const int par0 = rev ? (int)((d.nx + 1) & 1) : 0;
    const size_t skip = rev ? d.nx - 2 : 1;
    for (int32_t s = 0; s < iter; ++s) {
        gs_color_k<T><<<g, b, 0, ctx->stream>>>(v, f, G, c, d, par0, (size_t)-1);
        gs_color_k<T><<<g, b, 0, ctx->stream>>>(v, f, G, c, d, par0 ^ 1, skip);
    }
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// ---------------------------------------------------------------------------
// residual / Laplacian (residual_mex.c:82-165, lapmg_mex.c:73-154)
// ---------------------------------------------------------------------------

#define MG_INTERIOR                                                           \
    const size_t i = 1 + (size_t)blockIdx.x * blockDim.x + threadIdx.x;       \
    const size_t j = 1 + (size_t)blockIdx.y * blockDim.y + threadIdx.y;       \
    const size_t k = 1 + (size_t)blockIdx.z * blockDim.z + threadIdx.z;       \
    if (i + 1 >= d.nx || j + 1 >= d.ny || k + 1 >= d.nz) return;             \
    const size_t nx = d.nx, nxny = d.nxny(), l = i + nx * j + nxny * k;

template <typename T>
__global__ void residual_k(T *r, const T *__restrict__ f, const T *__restrict__ x, const uint8_t *__restrict__ G,
                           LapC<T> c, Dims d)
{
    MG_INTERIOR
    if (!G[l]) return;
    r[l] = f[l] + (c.hh * x[l] + c.hx * (x[l - 1] + x[l + 1]) + c.hy * (x[l - nx] + x[l + nx]) + c.hz * (x[l - nxny] + x[l + nxny]));
}

template <typename T>
__global__ void lapmg_k(T *du, const T *__restrict__ u, const uint8_t *__restrict__ G, LapC<T> c, Dims d)
{
    MG_INTERIOR
    if (!G[l]) return;
    du[l] = c.hh * u[l] + c.hx * (u[l - 1] + u[l + 1]) + c.hy * (u[l - nx] + u[l + nx]) + c.hz * (u[l - nxny] + u[l + nxny]);
}

static inline dim3 interior_grid3(const Dims &d)
{
    Dims e{d.nx > 2 ? d.nx - 2 : 0, d.ny > 2 ? d.ny - 2 : 0, d.nz > 2 ? d.nz - 2 : 0};
    return vox_grid(e);
}

template <typename T>
static qsm_status residual(qsm_ctx *ctx, T *r, const T *f, const T *x, const uint8_t *G, const double *h, const Dims &d)
{
    const dim3 g = interior_grid3(d);
    if (g.x == 0 || g.y == 0 || g.z == 0) return QSM_OK;
    residual_k<T><<<g, vox_block(), 0, ctx->stream>>>(r, f, x, G, lap_consts<T>(h), d);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

template <typename T>
static qsm_status lapmg(qsm_ctx *ctx, T *du, const T *u, const uint8_t *G, const double *h, const Dims &d)
{
    const dim3 g = interior_grid3(d);
    if (g.x == 0 || g.y == 0 || g.z == 0) return QSM_OK;
    lapmg_k<T><<<g, vox_block(), 0, ctx->stream>>>(du, u, G, lap_consts<T>(h), d);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// ---------------------------------------------------------------------------
// grid transfer (restrict_mex.c:72-332, prolong/correct_mex.c:73-304)
// ---------------------------------------------------------------------------

template <typename T>
__global__ void restrict_k(T *x2, const T *__restrict__ x, const uint8_t *__restrict__ G2, Dims d2, Dims d)
{
    const size_t i2 = 1 + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t j2 = 1 + (size_t)blockIdx.y * blockDim.y + threadIdx.y;
    const size_t k2 = 1 + (size_t)blockIdx.z * blockDim.z + threadIdx.z;
    if (i2 + 1 >= d2.nx || j2 + 1 >= d2.ny || k2 + 1 >= d2.nz) return;
    const size_t l2 = i2 + d2.nx * j2 + d2.nxny() * k2;
    if (!G2[l2]) {
        x2[l2] = (T)0;
        return;
    }
    const size_t nx = d.nx, nxny = d.nxny();
    const size_t l = (2 * i2 - 1) + nx * (2 * j2 - 1) + nxny * (2 * k2 - 1);
#define X(a, b, c) x[(ptrdiff_t)l + (a) + (b) * (ptrdiff_t)nx + (c) * (ptrdiff_t)nxny]
    const T A = X(-1, -1, -1) + X(1, -1, -1) + X(-1, 1, -1) + X(1, 1, -1) + X(-1, -1, 1) + X(1, -1, 1) + X(-1, 1, 1) + X(1, 1, 1);
    const T B = X(0, -1, -1) + X(-1, 0, -1) + X(1, 0, -1) + X(0, 1, -1) + X(1, -1, 0) + X(-1, -1, 0) + X(-1, 1, 0) +
                X(1, 1, 0) + X(0, -1, 1) + X(-1, 0, 1) + X(1, 0, 1) + X(0, 1, 1);
    const T C = X(0, 0, -1) + X(0, -1, 0) + X(-1, 0, 0) + X(1, 0, 0) + X(0, 1, 0) + X(0, 0, 1);
#undef X
    x2[l2] = (T)0.015625 * A + (T)0.03125 * B + (T)0.0625 * C + (T)0.125 * x[l];
}

// Fine voxels (i, j, k) in [1, 2(n2-2)]^3: coarse parent i2 = (i+1)/2 and
// offset a = (i+1) mod 2 select the interpolation case.  One thread takes
// the two fine voxels i = 2 i2 - 1 (a = 0) and 2 i2 (a = 1) of one coarse
// column, so the case (b, c) is uniform across a warp (one x row) and the
// FP64 pipe never runs two cases' instructions for one warp.
// CLEAN (with ADD): x is +0 outside G, where the correction adds +0 and leaves
// it +0; those voxels are not touched.
template <typename T, bool ADD, bool CLEAN>
__global__ void prolong_k(T *x, const T *__restrict__ x2, const uint8_t *__restrict__ G, Dims d, Dims d2)
{
    const size_t i2 = 1 + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t j = 1 + (size_t)blockIdx.y * blockDim.y + threadIdx.y;
    const size_t k = 1 + (size_t)blockIdx.z * blockDim.z + threadIdx.z;
    if (i2 + 1 >= d2.nx || j > 2 * (d2.ny - 2) || k > 2 * (d2.nz - 2)) return;
    const size_t j2 = (j + 1) >> 1, k2 = (k + 1) >> 1;
    const int b = (int)((j + 1) & 1), c = (int)((k + 1) & 1);
    const size_t l2 = i2 + d2.nx * j2 + d2.nxny() * k2, ox = 1, oy = d2.nx, oz = d2.nxny();
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        const size_t lf = (2 * i2 - 1 + a) + d.nx * j + d.nxny() * k;
        if (ADD && CLEAN && !G[lf]) continue;
        T val = (T)0;
        if (G[lf]) {
            const T c0 = x2[l2];
            switch (a + 2 * b + 4 * c) {
            case 0: val = c0; break;
            case 1: val = (T)0.5 * (c0 + x2[l2 + ox]); break;
            case 2: val = (T)0.5 * (c0 + x2[l2 + oy]); break;
            case 4: val = (T)0.5 * (c0 + x2[l2 + oz]); break;
            case 3: val = (T)0.25 * (c0 + x2[l2 + ox] + x2[l2 + oy] + x2[l2 + ox + oy]); break;
            case 5: val = (T)0.25 * (c0 + x2[l2 + ox] + x2[l2 + oz] + x2[l2 + ox + oz]); break;
            case 6: val = (T)0.25 * (c0 + x2[l2 + oy] + x2[l2 + oz] + x2[l2 + oy + oz]); break;
            default:
                val = (T)0.125 * (c0 + x2[l2 + ox] + x2[l2 + oy] + x2[l2 + oz] + x2[l2 + ox + oy] + x2[l2 + ox + oz] +
                                  x2[l2 + oy + oz] + x2[l2 + ox + oy + oz]);
            }
        }
        x[lf] = ADD ? x[lf] + val : val;
    }
}

template <typename T>
static qsm_status restrict_(qsm_ctx *ctx, T *x2, const T *x, const uint8_t *G2, const Dims &d2, const Dims &d)
{
    const dim3 g = interior_grid3(d2);
    if (g.x == 0 || g.y == 0 || g.z == 0) return QSM_OK;
    restrict_k<T><<<g, vox_block(), 0, ctx->stream>>>(x2, x, G2, d2, d);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

template <typename T>
static qsm_status prolong(qsm_ctx *ctx, T *x, const T *x2, const uint8_t *G, const Dims &d, const Dims &d2, bool add,
                          bool clean = false)
{
    if (d2.nx < 3 || d2.ny < 3 || d2.nz < 3) return QSM_OK;
    const Dims e{d2.nx - 2, 2 * (d2.ny - 2), 2 * (d2.nz - 2)};
    const dim3 g = vox_grid(e);
    if (add && clean) prolong_k<T, true, true><<<g, vox_block(), 0, ctx->stream>>>(x, x2, G, d, d2);
    else if (add) prolong_k<T, true, false><<<g, vox_block(), 0, ctx->stream>>>(x, x2, G, d, d2);
    else prolong_k<T, false, false><<<g, vox_block(), 0, ctx->stream>>>(x, x2, G, d, d2);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// ---------------------------------------------------------------------------
// masks (coarsen_grid_mex.c:52-125, boundary_mask_mex.c:46-132,
// boundary_mask_l1_mex.c:49-117) -- integer, bit-exact
// ---------------------------------------------------------------------------

__global__ void coarsen_k(uint8_t *G2, const uint8_t *__restrict__ G, Dims d2, Dims d)
{
    const size_t i2 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t j2 = (size_t)blockIdx.y * blockDim.y + threadIdx.y;
    const size_t k2 = (size_t)blockIdx.z * blockDim.z + threadIdx.z;
    if (i2 >= d2.nx || j2 >= d2.ny || k2 >= d2.nz) return;
    const size_t l2 = i2 + d2.nx * j2 + d2.nxny() * k2;
    if (i2 == 0 || j2 == 0 || k2 == 0 || i2 + 1 >= d2.nx || j2 + 1 >= d2.ny || k2 + 1 >= d2.nz) {
        G2[l2] = 0;
        return;
    }
    const size_t i = 2 * i2 - 1, j = 2 * j2 - 1, k = 2 * k2 - 1;
    const size_t nx = d.nx, nxny = d.nxny(), l = i + nx * j + nxny * k;
    const bool bi = !(i < d.nx - 2), bj = !(j < d.ny - 2), bk = !(k < d.nz - 2);
    G2[l2] = (uint8_t)(G[l] && (bi || G[l + 1]) && (bj || G[l + nx]) && (bk || G[l + nxny]) &&
                       (bi || bj || G[l + 1 + nx]) && (bi || bk || G[l + 1 + nxny]) && (bj || bk || G[l + nx + nxny]) &&
                       (bi || bj || bk || G[l + 1 + nx + nxny]));
}

// b = G on the outermost interior shell and on 2x2x2 blocks (anchored at odd
// interior indices) that are not wholly inside G; b = 0 elsewhere.
__global__ void bmask_b_k(uint8_t *b, const uint8_t *__restrict__ G, Dims d)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t j = (size_t)blockIdx.y * blockDim.y + threadIdx.y;
    const size_t k = (size_t)blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= d.nx || j >= d.ny || k >= d.nz) return;
    const size_t nx = d.nx, nxny = d.nxny(), l = i + nx * j + nxny * k;
    uint8_t val = 0;
    const bool interior = i >= 1 && j >= 1 && k >= 1 && i + 2 <= d.nx && j + 2 <= d.ny && k + 2 <= d.nz;
    if (interior && (i == 1 || j == 1 || k == 1 || i == d.nx - 2 || j == d.ny - 2 || k == d.nz - 2)) val = G[l];
    // the block containing (i,j,k): anchor at the odd index <= each coordinate
    const size_t ai = (i & 1) ? i : i - 1, aj = (j & 1) ? j : j - 1, ak = (k & 1) ? k : k - 1;
    if (i >= 1 && j >= 1 && k >= 1 && ai + 2 <= d.nx && aj + 2 <= d.ny && ak + 2 <= d.nz) {
        const size_t la = ai + nx * aj + nxny * ak;
        const bool full = G[la] && G[la + 1] && G[la + nx] && G[la + nxny] && G[la + 1 + nx] && G[la + 1 + nxny] &&
                          G[la + nx + nxny] && G[la + 1 + nx + nxny];
        if (!full) val = G[l];
    }
    b[l] = val;
}

__global__ void bmask_grow_k(uint8_t *B, const uint8_t *__restrict__ b, const uint8_t *__restrict__ G, Dims d)
{
    MG_INTERIOR
    if (G[l]) B[l] = (uint8_t)(b[l - nxny] || b[l - nx] || b[l - 1] || b[l] || b[l + 1] || b[l + nx] || b[l + nxny]);
}

static qsm_status boundary_mask(qsm_ctx *ctx, uint8_t *B, const uint8_t *G, const Dims &d, uint8_t *scratch)
{
    if (d.nx < 3 || d.ny < 3 || d.nz < 3) return QSM_OK;
    bmask_b_k<<<vox_grid(d), vox_block(), 0, ctx->stream>>>(scratch, G, d);
    bmask_grow_k<<<interior_grid3(d), vox_block(), 0, ctx->stream>>>(B, scratch, G, d);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// ---------------------------------------------------------------------------
// boundary-band sweeps over voxel lists.  The band B is a thin shell of G; a
// full-grid colour pass over it would launch every voxel to update a few
// percent of them.  Each level keeps the linear indices of its B voxels,
// split by colour (i + j + k) mod 2, with flags for i == 1 and i == nx - 2
// (the voxels the reference's second colour pass skips).  A pass reads only
// the other colour, so the list order does not change the result.
// ---------------------------------------------------------------------------

constexpr uint32_t BL_I1 = 1u << 31, BL_INX2 = 1u << 30, BL_IDX = 0x3FFFFFFFu;

// The lists are in increasing index order: a pass over one then walks its
// level row by row, and the rows a warp's neighbours lie in are those the
// warps before it have just read (on the 256^3 FP32-V-cycle solve this took
// the solve from 19.7 to 17.9 ms against lists in atomic-append order).  Per
// x-row segment of 32 voxels (one warp of the interior grid, blockDim.x ==
// 32) the voxels of each colour are counted (COUNT: segc[p nseg + seg]), the
// counts are scanned, and each segment writes its voxels at its offset
// (segc then holds the offsets): the same lists every time, no atomics.
struct SegLists {
    uint32_t *l[4];  // B colour 0, B colour 1, G colour 0, G colour 1
};

template <bool FILL>
__global__ void blist_seg_k(SegLists out, unsigned *seg, const uint8_t *__restrict__ B, const uint8_t *__restrict__ G,
                            Dims d, size_t nseg)
{
    const size_t i = 1 + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t j = 1 + (size_t)blockIdx.y * blockDim.y + threadIdx.y;
    const size_t k = 1 + (size_t)blockIdx.z * blockDim.z + threadIdx.z;
    if (j + 1 >= d.ny || k + 1 >= d.nz) return;  // the whole warp (one row)
    bool onb = false, ong = false;
    int par = 0;
    uint32_t e = 0;
    if (i + 1 < d.nx) {
        const size_t l = i + d.nx * j + d.nxny() * k;
        onb = B[l] != 0;
        ong = G[l] != 0;
        par = (int)((i + j + k) & 1);
        e = (uint32_t)l | (i == 1 ? BL_I1 : 0u) | (i == d.nx - 2 ? BL_INX2 : 0u);
    }
    const int lane = threadIdx.x;
    const size_t sg = blockIdx.x + (size_t)gridDim.x * ((j - 1) + (d.ny - 2) * (k - 1));
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const bool on = (q < 2 ? onb : ong) && par == (q & 1);
        const unsigned m = __ballot_sync(0xffffffffu, on);
        if (!FILL) {
            if (lane == 0) seg[q * nseg + sg] = (unsigned)__popc(m);
        } else if (on) {
            // seg holds one exclusive scan over the four count arrays: rebase to array q
            out.l[q][seg[q * nseg + sg] - seg[q * nseg] + __popc(m & ((1u << lane) - 1u))] = e;
        }
    }
}

// exclusive scans of unsigned counts: blocks of SCAN_BLK elements scanned on
// their own (their totals to bs), the totals scanned the same way, then added
constexpr int SCAN_T = 256, SCAN_PER = 4, SCAN_BLK = SCAN_T * SCAN_PER;

__global__ void __launch_bounds__(SCAN_T) scan_blocks_k(const unsigned *__restrict__ a, unsigned *o, size_t n,
                                                        unsigned *bs)
{
    __shared__ unsigned sh[SCAN_T];
    const int tid = threadIdx.x;
    const size_t base = (size_t)blockIdx.x * SCAN_BLK + (size_t)tid * SCAN_PER;
    unsigned v[SCAN_PER], s = 0;
#pragma unroll
    for (int u = 0; u < SCAN_PER; ++u) {
        v[u] = base + u < n ? a[base + u] : 0u;
        s += v[u];
    }
    sh[tid] = s;
    __syncthreads();
    for (int off = 1; off < SCAN_T; off <<= 1) {
        const unsigned t = tid >= off ? sh[tid - off] : 0u;
        __syncthreads();
        sh[tid] += t;
        __syncthreads();
    }
    unsigned run = sh[tid] - s;
#pragma unroll
    for (int u = 0; u < SCAN_PER; ++u) {
        if (base + u < n) o[base + u] = run;
        run += v[u];
    }
    if (bs && tid == SCAN_T - 1) bs[blockIdx.x] = sh[tid];
}

__global__ void scan_add_k(unsigned *o, size_t n, const unsigned *__restrict__ bo)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) o[e] += bo[e / SCAN_BLK];
}

// the scratch (unsigned) exclusive_scan needs for n elements
static size_t scan_scratch(size_t n)
{
    size_t t = 0;
    for (size_t m = n; m > SCAN_BLK;) {
        const size_t nb = (m + SCAN_BLK - 1) / SCAN_BLK;
        t += 2 * nb;
        m = nb;
    }
    return t + 16;
}

static qsm_status exclusive_scan(qsm_ctx *ctx, const unsigned *a, unsigned *o, size_t n, unsigned *tmp)
{
    if (n == 0) return QSM_OK;
    const size_t nb = (n + SCAN_BLK - 1) / SCAN_BLK;
    scan_blocks_k<<<(unsigned)nb, SCAN_T, 0, ctx->stream>>>(a, o, n, nb > 1 ? tmp : nullptr);
    QSM_CUDA(cudaGetLastError());
    if (nb > 1) {
        unsigned *bo = tmp + nb;  // the block totals' exclusive scan
        QSM_TRY(exclusive_scan(ctx, tmp, bo, nb, bo + nb));
        scan_add_k<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(o, n, bo);
        QSM_CUDA(cudaGetLastError());
    }
    return QSM_OK;
}

// cnt[q] = the entries of list q (B colour 0, 1, G colour 0, 1) from the counts and their scan
__global__ void blist_total_k(const unsigned *__restrict__ segc, const unsigned *__restrict__ off, size_t nseg,
                              unsigned *cnt)
{
    const int q = threadIdx.x;
    if (q < 4 && nseg) {
        const size_t last = (size_t)(q + 1) * nseg - 1;
        cnt[q] = off[last] + segc[last] - off[(size_t)q * nseg];
    }
}

template <typename T>
__global__ void gs_list_k(T *v, const T *__restrict__ f, const uint32_t *__restrict__ list, unsigned cnt,
                          uint32_t skip, GsC<T> c, size_t nx, size_t nxny)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    const uint32_t e = list[t];
    if (e & skip) return;
    const size_t l = e & BL_IDX;
    v[l] = c.hh * (f[l] + (c.hx * (v[l - 1] + v[l + 1]) + c.hy * (v[l - nx] + v[l + nx]) + c.hz * (v[l - nxny] + v[l + nxny])));
}

// gs_list_k for FP32 passes, which are bound by load latency rather than by
// arithmetic: a thread takes GS_PER entries at a stride of the grid and issues
// all their loads before its first store.  A pass reads only the other
// colour, so the order of its updates does not change a bit.
constexpr int GS_PER = 4;
template <typename T>
__device__ __forceinline__ void gs_list_ilp_body(T *v, const T *__restrict__ f, const uint32_t *__restrict__ list, unsigned cnt,
                              uint32_t skip, GsC<T> c, size_t nx, size_t nxny, unsigned blk, unsigned nblk)
{
    const unsigned t0 = blk * blockDim.x + threadIdx.x, st = nblk * blockDim.x;
    size_t l[GS_PER];
    bool on[GS_PER];
#pragma unroll
    for (int u = 0; u < GS_PER; ++u) {
        const unsigned m = t0 + u * st;
        const uint32_t e = m < cnt ? list[m] : 0u;
        on[u] = m < cnt && !(e & skip);
        l[u] = e & BL_IDX;
    }
    T fv[GS_PER], a[GS_PER][6];
#pragma unroll
    for (int u = 0; u < GS_PER; ++u) {
        if (!on[u]) continue;
        const size_t q = l[u];
        fv[u] = f[q];
        a[u][0] = v[q - 1];
        a[u][1] = v[q + 1];
        a[u][2] = v[q - nx];
        a[u][3] = v[q + nx];
        a[u][4] = v[q - nxny];
        a[u][5] = v[q + nxny];
    }
#pragma unroll
    for (int u = 0; u < GS_PER; ++u)
        if (on[u])
            v[l[u]] = c.hh * (fv[u] + (c.hx * (a[u][0] + a[u][1]) + c.hy * (a[u][2] + a[u][3]) + c.hz * (a[u][4] + a[u][5])));
}

template <typename T>
__global__ void gs_list_ilp_k(T *v, const T *__restrict__ f, const uint32_t *__restrict__ list, unsigned cnt,
                              uint32_t skip, GsC<T> c, size_t nx, size_t nxny)
{
    gs_list_ilp_body<T>(v, f, list, cnt, skip, c, nx, nxny, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// All colour passes of one smoothing call on one thread-block cluster.  On a
// coarse level a pass updates a few thousand voxels and a launch per pass
// costs several times the pass itself; here the cluster's CTAs share each
// pass and meet at the cluster barrier between passes.  v stays in global
// memory (L2-resident at these sizes); its reads bypass L1 (ld.global.cg), so
// after the barrier's release / acquire a CTA reads what the others wrote.
// The list order within a pass is immaterial (a pass reads the other colour
// only), so results equal the per-pass launches bit for bit.
// ---------------------------------------------------------------------------

constexpr int SW_THREADS = 256;
enum { SW_LAUNCH = 0, SW_CLUSTER = 1, SW_GRID = 2 };
// per-colour list sizes: up to SW_CLUSTER_MAX on one cluster, up to SW_GRID_MAX
// over the whole GPU with a grid barrier, else a launch per pass.  Measured per
// pass (FP64, 256^3 hierarchy): cluster 2.1 us at 1.8k voxels, 3.5 us at 5-7k;
// grid 3.1 us at 7.4k, 3.6 us at 31k, 8.6 us at 126k (a thread then walks
// several entries one after another); launches 4.7 us at 31k, 7.8 us at 126k,
// 11 us at 334k.  So the grid takes lists of up to about one entry per thread.
constexpr unsigned SW_CLUSTER_MAX = 2500, SW_GRID_MAX = 45000;

// A thread's share of one list: at most SW_PER entries (longer lists keep one
// launch per pass), loaded once with their f values, since neither changes
// during the sweeps.
constexpr int SW_PER = 4;

template <typename T>
struct SwShare {
    uint32_t l[SW_PER];
    T f[SW_PER];
    uint32_t flags[SW_PER];
    int n;
    __device__ __forceinline__ void load(const uint32_t *list, unsigned cnt, const T *__restrict__ fg, unsigned t0,
                                         unsigned stride)
    {
        n = 0;
#pragma unroll
        for (int u = 0; u < SW_PER; ++u) {
            const unsigned m = t0 + u * stride;
            if (m < cnt) {
                const uint32_t e = list[m];
                l[u] = e & BL_IDX;
                flags[u] = e & ~BL_IDX;
                f[u] = fg[l[u]];
                n = u + 1;
            }
        }
    }
    __device__ __forceinline__ void pass(T *v, uint32_t skip, GsC<T> c, size_t nx, size_t nxny) const
    {
#pragma unroll
        for (int u = 0; u < SW_PER; ++u) {
            if (u >= n || (flags[u] & skip)) continue;
            const size_t q = l[u];
            v[q] = c.hh * (f[u] + (c.hx * (__ldcg(v + q - 1) + __ldcg(v + q + 1)) +
                                   c.hy * (__ldcg(v + q - nx) + __ldcg(v + q + nx)) +
                                   c.hz * (__ldcg(v + q - nxny) + __ldcg(v + q + nxny))));
        }
    }
};

// iter sweeps of (colour-a pass over la, colour-b pass over lb skipping the
// entries flagged skipb); the grid is exactly one cluster and each list holds
// at most SW_PER x (the grid's threads) entries.
template <typename T>
__global__ void __launch_bounds__(SW_THREADS) sweeps_cluster_k(T *v, const T *__restrict__ f,
                                                               const uint32_t *__restrict__ la, unsigned ca,
                                                               const uint32_t *__restrict__ lb, unsigned cb,
                                                               uint32_t skipb, int32_t iter, GsC<T> c, size_t nx,
                                                               size_t nxny)
{
    const unsigned stride = gridDim.x * SW_THREADS, t0 = blockIdx.x * SW_THREADS + threadIdx.x;
    SwShare<T> a, b;
    a.load(la, ca, f, t0, stride);
    b.load(lb, cb, f, t0, stride);
    for (int32_t s = 0; s < iter; ++s) {
        a.pass(v, 0u, c, nx, nxny);
        cl_sync();
        b.pass(v, skipb, c, nx, nxny);
        cl_sync();
    }
}

// Cluster size for sweeps_cluster_k (16, else 8, else 0 = not available),
// settled once per device.
template <typename T>
static int sweeps_cluster_size(qsm_ctx *ctx)
{
    static std::mutex mu;
    static int size[64];
    static bool done[64];
    std::lock_guard<std::mutex> lock(mu);
    const int dv = ctx->device & 63;
    if (done[dv]) return size[dv];
    done[dv] = true;
    size[dv] = 0;
    if (cudaFuncSetAttribute(sweeps_cluster_k<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    for (int cn = 16; cn >= 8; cn -= 8) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)cn;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3((unsigned)cn);
        cfg.blockDim = dim3(SW_THREADS);
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int ncl = 0;
        if (cudaOccupancyMaxActiveClusters(&ncl, sweeps_cluster_k<T>, &cfg) == cudaSuccess && ncl >= 1) {
            size[dv] = cn;
            break;
        }
        cudaGetLastError();
    }
    return size[dv];
}

template <typename T>
static qsm_status sweeps_cluster(qsm_ctx *ctx, int cn, T *v, const T *f, uint32_t *const lists[2],
                                 const unsigned cnt[2], const double *h, const Dims &d, int32_t iter, bool rev)
{
    const int par0 = rev ? (int)((d.nx + 1) & 1) : 0;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)cn;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)cn);
    cfg.blockDim = dim3(SW_THREADS);
    cfg.stream = ctx->stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    QSM_CUDA(cudaLaunchKernelEx(&cfg, sweeps_cluster_k<T>, v, f, (const uint32_t *)lists[par0], cnt[par0],
                                (const uint32_t *)lists[par0 ^ 1], cnt[par0 ^ 1], rev ? BL_INX2 : BL_I1, iter,
                                gs_consts<T>(h), d.nx, d.nxny()));
    return QSM_OK;
}

// ---------------------------------------------------------------------------
// Coarsest level over the whole GPU (mgpcg_mex.c:265-275).  When a colour
// pass of the coarsest grid is large (a shallow hierarchy, e.g. lbv's on a
// cropped volume: ~16k FP64 updates per colour), one cluster's 16 SMs are
// bound by their FP64 pipes (~5 us per pass).  Here one CTA per SM, launched
// cooperatively so that all are resident, takes every pass over the level's
// G colour lists and the CTAs meet at a grid barrier between passes.  The
// residual norm keeps the lane order: CTA b halves the 256-element blocks
// b, b + grid, ..., CTA 0 halves the 1024 block sums.  Every wait is bounded:
// a barrier that does not complete within CG_SPIN_LIMIT polls sets the error
// flag, and every CTA leaves at its next barrier.
// ---------------------------------------------------------------------------

constexpr int CG_THREADS = 256;
constexpr long long CG_SPIN_LIMIT = 1ll << 22;  // polls of the generation word (seconds)
constexpr unsigned CG_MIN_PASS = 6000;          // per-colour G count from which the grid beats a cluster

struct GridBar {
    unsigned *count;  // arrivals since the launch (zeroed by the host before it)
    int *err;
    unsigned extra;   // arrivals required beyond the grid's (0; 1 under QSM_DEBUG_GRID_BARRIER_TIMEOUT)
    long long limit;  // polls before a wait gives up
};

// Barrier number k (1, 2, ...) of the grid: each CTA adds one arrival with
// release semantics and polls the count with acquire loads until all
// gridDim.x x k arrivals are in.  False once any CTA's wait has run out
// (then every CTA leaves at its next barrier).
__device__ __forceinline__ bool grid_bar(const GridBar &g, unsigned &k)
{
    __shared__ int bad;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned target = ++k * gridDim.x + g.extra;
        __threadfence();
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(g.count) : "memory");
        long long spins = 0;
        for (;;) {
            unsigned cur;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(g.count) : "memory");
            if ((int)(cur - target) >= 0) break;
            if ((++spins & 1023) == 0 && *(volatile int *)g.err != 0) break;
            if (spins > g.limit) {
                atomicExch(g.err, 1);
                break;
            }
        }
        bad = *(volatile int *)g.err;
    }
    __syncthreads();
    return bad == 0;
}

// lane-order sum of src[e]^2, e < n (src written before the last barrier);
// part holds RED_NBLK + 1 values, entries nb .. RED_NBLK - 1 zero
template <typename T>
__device__ bool grid_lane_sum(const T *src, unsigned n, T *part, T *red, const GridBar &gb, unsigned &k, T *out)
{
    const int tid = threadIdx.x;
    const unsigned nb = (n + RED_BLOCK - 1) / RED_BLOCK;
    for (unsigned b = blockIdx.x; b < nb; b += gridDim.x) {
        const unsigned e = b * RED_BLOCK + tid;
        const T x = e < n ? __ldcg(src + e) : (T)0;
        red[tid] = x * x;
        __syncthreads();
        for (int st = RED_BLOCK / 2; st > 0; st >>= 1) {
            if (tid < st) red[tid] = red[tid] + red[tid + st];
            __syncthreads();
        }
        if (tid == 0) part[b] = red[0];
        __syncthreads();
    }
    if (!grid_bar(gb, k)) return false;
    if (blockIdx.x == 0) {
        const T tot = halve_partials(red, tid, part);
        if (tid == 0) part[RED_NBLK] = tot;
    }
    if (!grid_bar(gb, k)) return false;
    *out = __ldcg(part + RED_NBLK);
    return true;
}

template <typename T>
__device__ __forceinline__ void grid_pass(T *v, const T *__restrict__ f, const uint32_t *__restrict__ ls,
                                          unsigned cnt, uint32_t skip, GsC<T> c, size_t nx, size_t nxny)
{
    for (unsigned m = blockIdx.x * CG_THREADS + threadIdx.x; m < cnt; m += gridDim.x * CG_THREADS) {
        const uint32_t e = ls[m];
        if (e & skip) continue;
        const size_t l = e & BL_IDX;
        v[l] = c.hh * (f[l] + (c.hx * (__ldcg(v + l - 1) + __ldcg(v + l + 1)) +
                               c.hy * (__ldcg(v + l - nx) + __ldcg(v + l + nx)) +
                               c.hz * (__ldcg(v + l - nxny) + __ldcg(v + l + nxny))));
    }
}

template <typename T>
__global__ void __launch_bounds__(CG_THREADS) coarse_grid_k(T *v, const T *__restrict__ f, T *r,
                                                            const uint32_t *__restrict__ l0, unsigned c0,
                                                            const uint32_t *__restrict__ l1, unsigned c1, Dims d,
                                                            GsC<T> gc, LapC<T> lc, double tol, GridBar gb, T *part,
                                                            int *outer_out)
{
    __shared__ T red[RED_BLOCK];
    const size_t nx = d.nx, nxny = d.nxny();
    const unsigned n = (unsigned)d.n(), nb = (n + RED_BLOCK - 1) / RED_BLOCK;
    if (blockIdx.x == 0)
        for (unsigned b = nb + threadIdx.x; b < RED_NBLK; b += CG_THREADS) part[b] = (T)0;
    unsigned bk = 0;  // barriers passed
    T ff;
    if (!grid_lane_sum(f, n, part, red, gb, bk, &ff)) return;
    const double fn = sizeof(T) == 4 ? (double)sqrtf((float)ff) : sqrt((double)ff);
    const double reltol = tol * fn;
    const int rpar0 = (int)((d.nx + 1) & 1);
    const uint32_t *lr0 = rpar0 ? l1 : l0, *lr1 = rpar0 ? l0 : l1;
    const unsigned cr0 = rpar0 ? c1 : c0, cr1 = rpar0 ? c0 : c1;
    int outer = 0;
    for (int it = 0; it < 1024; ++it) {
        outer = it + 1;
        for (int s = 0; s < 128; ++s) {  // reverse sweeps
            grid_pass(v, f, lr0, cr0, 0u, gc, nx, nxny);
            if (!grid_bar(gb, bk)) return;
            grid_pass(v, f, lr1, cr1, BL_INX2, gc, nx, nxny);
            if (!grid_bar(gb, bk)) return;
        }
        for (int s = 0; s < 128; ++s) {  // forward sweeps
            grid_pass(v, f, l0, c0, 0u, gc, nx, nxny);
            if (!grid_bar(gb, bk)) return;
            grid_pass(v, f, l1, c1, BL_I1, gc, nx, nxny);
            if (!grid_bar(gb, bk)) return;
        }
        // residual of the interior G voxels (both colour lists), then its norm over all of r
        for (unsigned m = blockIdx.x * CG_THREADS + threadIdx.x; m < c0 + c1; m += gridDim.x * CG_THREADS) {
            const size_t l = (m < c0 ? l0[m] : l1[m - c0]) & BL_IDX;
            r[l] = f[l] + (lc.hh * __ldcg(v + l) + lc.hx * (__ldcg(v + l - 1) + __ldcg(v + l + 1)) +
                           lc.hy * (__ldcg(v + l - nx) + __ldcg(v + l + nx)) +
                           lc.hz * (__ldcg(v + l - nxny) + __ldcg(v + l + nxny)));
        }
        if (!grid_bar(gb, bk)) return;
        T rr;
        if (!grid_lane_sum(r, n, part, red, gb, bk, &rr)) return;
        const double rn = sizeof(T) == 4 ? (double)sqrtf((float)rr) : sqrt((double)rr);
        if (rn < reltol) break;
        if (c0 + c1 == 0) {  // no G voxel: every later outer iteration repeats this one exactly
            outer = 1024;
            break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && outer_out) *outer_out += outer;
}

// iter sweeps (colour-a pass over la, colour-b pass over lb skipping the
// entries flagged skipb) over the whole GPU with a grid barrier between
// passes: for lists too large for one cluster's 16 SMs but small enough that
// a launch per pass costs more than the barrier (~2.5 us).
template <typename T>
__global__ void __launch_bounds__(CG_THREADS) sweeps_grid_k(T *v, const T *__restrict__ f,
                                                            const uint32_t *__restrict__ la, unsigned ca,
                                                            const uint32_t *__restrict__ lb, unsigned cb,
                                                            uint32_t skipb, int32_t iter, GsC<T> c, size_t nx,
                                                            size_t nxny, GridBar gb)
{
    unsigned bk = 0;
    for (int32_t s = 0; s < iter; ++s) {
        grid_pass(v, f, la, ca, 0u, c, nx, nxny);
        if (!grid_bar(gb, bk)) return;
        grid_pass(v, f, lb, cb, skipb, c, nx, nxny);
        if (!grid_bar(gb, bk)) return;
    }
}

__global__ void bmask_l1_init_k(uint8_t *B, uint8_t *GL, const uint8_t *__restrict__ G, Dims d)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t j = (size_t)blockIdx.y * blockDim.y + threadIdx.y;
    const size_t k = (size_t)blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= d.nx || j >= d.ny || k >= d.nz) return;
    const size_t nx = d.nx, nxny = d.nxny(), l = i + nx * j + nxny * k;
    uint8_t v;
    if (i == 0 || j == 0 || k == 0 || i + 1 == d.nx || j + 1 == d.ny || k + 1 == d.nz)
        v = G[l];
    else
        v = (uint8_t)(G[l] && !(G[l - 1] && G[l + 1] && G[l - nx] && G[l + nx] && G[l - nxny] && G[l + nxny]));
    B[l] = v;
    GL[l] = v;
}

// One band step: a voxel that joins (GL: 0 -> L1+1) cannot change another
// voxel's test in the same step (that test looks for GL == L1), so the
// step is order-independent.
__global__ void bmask_l1_step_k(uint8_t *B, uint8_t *GL, const uint8_t *__restrict__ G, Dims d, size_t L1)
{
    const size_t i = L1 + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t j = L1 + (size_t)blockIdx.y * blockDim.y + threadIdx.y;
    const size_t k = L1 + (size_t)blockIdx.z * blockDim.z + threadIdx.z;
    if (i + L1 >= d.nx || j + L1 >= d.ny || k + L1 >= d.nz) return;
    const size_t nx = d.nx, nxny = d.nxny(), l = i + nx * j + nxny * k;
    if (G[l] && !GL[l] &&
        (GL[l - 1] == L1 || GL[l + 1] == L1 || GL[l - nx] == L1 || GL[l + nx] == L1 || GL[l - nxny] == L1 ||
         GL[l + nxny] == L1)) {
        B[l] = 1;
        GL[l] = (uint8_t)(L1 + 1);
    }
}

// ---------------------------------------------------------------------------
// pad / unpad / element-wise BLAS-1
// ---------------------------------------------------------------------------

template <typename T>
__global__ void pad_k(T *xp, const T *__restrict__ x, Dims d)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t j = (size_t)blockIdx.y * blockDim.y + threadIdx.y;
    const size_t k = (size_t)blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= d.nx || j >= d.ny || k >= d.nz) return;
    xp[(i + 1) + (d.nx + 2) * ((j + 1) + (d.ny + 2) * (k + 1))] = x[i + d.nx * (j + d.ny * k)];
}

template <typename T>
__global__ void unpad_k(T *x, const T *__restrict__ xp, Dims d)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t j = (size_t)blockIdx.y * blockDim.y + threadIdx.y;
    const size_t k = (size_t)blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= d.nx || j >= d.ny || k >= d.nz) return;
    x[i + d.nx * (j + d.ny * k)] = xp[(i + 1) + (d.nx + 2) * ((j + 1) + (d.ny + 2) * (k + 1))];
}

__global__ void mask01_pad_k(uint8_t *xp, const uint8_t *__restrict__ x, Dims d)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t j = (size_t)blockIdx.y * blockDim.y + threadIdx.y;
    const size_t k = (size_t)blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= d.nx || j >= d.ny || k >= d.nz) return;
    xp[(i + 1) + (d.nx + 2) * ((j + 1) + (d.ny + 2) * (k + 1))] = x[i + d.nx * (j + d.ny * k)] != 0;
}

// Scalar operands of the BLAS-1 kernels live in device memory:
// sc[idx] (negated when neg) or the immediate `imm` when idx < 0.
__device__ __forceinline__ double scal_of(const double *sc, int idx, bool neg, double imm)
{
    const double a = idx < 0 ? imm : sc[idx];
    return neg ? -a : a;
}

// x = a * x (sscal/dscal semantics; FP32 casts a to float)
template <typename T>
__global__ void scal_k(T *x, size_t n, const double *sc, int idx, bool neg, double imm)
{
    const T a = (T)scal_of(sc, idx, neg, imm);
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) x[l] = a * x[l];
}

// y = y + a * x (saxpy/daxpy semantics)
template <typename T>
__global__ void axpy_k(T *y, const T *__restrict__ x, size_t n, const double *sc, int idx, bool neg, double imm)
{
    const T a = (T)scal_of(sc, idx, neg, imm);
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) y[l] = y[l] + a * x[l];
}

template <typename T, typename S>
__global__ void cvt_k(T *o, const S *__restrict__ a, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) o[l] = (T)a[l];
}

// PCG scalar slots
enum { S_RHO = 0, S_PREV = 1, S_BETA = 2, S_A = 3, S_PQ = 4, S_RES = 5, S_TMP = 6, S_N = 8 };

__global__ void sqrt_k(double *dst, const double *src, bool f32)
{
    *dst = f32 ? (double)sqrtf((float)*src) : sqrt(*src);
}

template <typename T>
static qsm_status scal(qsm_ctx *ctx, T *x, size_t n, const double *sc, int idx, bool neg, double imm = 0.0)
{
    scal_k<T><<<1216, 256, 0, ctx->stream>>>(x, n, sc, idx, neg, imm);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

template <typename T>
static qsm_status axpy(qsm_ctx *ctx, T *y, const T *x, size_t n, const double *sc, int idx, bool neg, double imm = 0.0)
{
    axpy_k<T><<<1216, 256, 0, ctx->stream>>>(y, x, n, sc, idx, neg, imm);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// ||x||_2 in lane order into dst (device); FP32 sums in FP32 then sqrtf.
template <typename T>
static qsm_status nrm2(qsm_ctx *ctx, const T *x, size_t n, double *dst)
{
    QSM_TRY(lane_dot<T>(ctx, x, x, n, dst));
    sqrt_k<<<1, 1, 0, ctx->stream>>>(dst, dst, sizeof(T) == 4);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// ---------------------------------------------------------------------------
// coarsest level in one CTA (mgpcg_mex.c:265-275)
// ---------------------------------------------------------------------------

constexpr int CS_THREADS = 1024;

// Lane-order sum of sq[0..n) (n <= 2^18, so lane t holds sq[t] alone):
// 256-wide halving per block of lanes, then 1024-wide halving of the block
// sums (blocks past n contribute +0).  sq is clobbered.
template <typename T>
__device__ T cta_lane_sum(T *sq, T *blk, int n)
{
    const int tid = threadIdx.x;
    const int nb = (n + RED_BLOCK - 1) / RED_BLOCK;
    for (int s = RED_BLOCK / 2; s > 0; s >>= 1) {
        for (int t = tid; t < nb * RED_BLOCK; t += CS_THREADS) {
            const int o = t % RED_BLOCK;
            if (o < s) {
                const int a = t, b = t + s;
                const T va = a < n ? sq[a] : (T)0, vb = b < n ? sq[b] : (T)0;
                if (a < n || b < n) sq[a] = va + vb;  // a < n whenever the sum can be non-zero
            }
        }
        __syncthreads();
    }
    for (int b = tid; b < RED_NBLK; b += CS_THREADS) blk[b] = b < nb ? (b * RED_BLOCK < n ? sq[b * RED_BLOCK] : (T)0) : (T)0;
    __syncthreads();
    for (int s = RED_NBLK / 2; s > 0; s >>= 1) {
        for (int t = tid; t < s; t += CS_THREADS) blk[t] = blk[t] + blk[t + s];
        __syncthreads();
    }
    return blk[0];
}

template <typename T>
__device__ void cta_gs(T *v, const T *f, const uint8_t *G, GsC<T> c, Dims d, int par, int skip_i)
{
    const int nx = (int)d.nx, ny = (int)d.ny, nz = (int)d.nz, nxny = nx * ny;
    const int hx_ = (nx - 2 + 1) / 2, per_k = hx_ * (ny - 2), tot = per_k * (nz - 2);
    for (int t = threadIdx.x; t < tot; t += CS_THREADS) {
        const int k = 1 + t / per_k, rem = t % per_k, j = 1 + rem / hx_, ii = rem % hx_;
        const int i = 1 + ((1 + j + k + par) & 1) + 2 * ii;
        if (i + 1 >= nx || i == skip_i) continue;
        const int l = i + nx * j + nxny * k;
        if (!G[l]) continue;
        v[l] = c.hh * (f[l] + (c.hx * (v[l - 1] + v[l + 1]) + c.hy * (v[l - nx] + v[l + nx]) + c.hz * (v[l - nxny] + v[l + nxny])));
    }
    __syncthreads();
}

// One CTA's coarsest solve: list entries (v index, flags)
constexpr uint32_t CS_IDX = 0x0FFFFFFFu;
constexpr uint32_t CS_I1 = 1u << 28;    // i == 1
constexpr uint32_t CS_INX2 = 1u << 29;  // i == nx - 2
constexpr uint32_t CS_ABSENT = 1u << 30; // no entry (register-held shares)

// Shared memory of coarse_solve_k for an n-voxel grid: v, f, sq (n each),
// the lane-order block sums, G (n bytes), two colour lists of (n + 1) / 2
// entries.
__host__ __device__ inline size_t cs_smem(size_t n, size_t es)
{
    const size_t g = 3 * n * es + (size_t)RED_NBLK * es;
    return ((g + n + 15) & ~(size_t)15) + 2 * ((n + 1) / 2) * sizeof(uint32_t);
}

// one colour pass of the one-CTA solver over a colour list (entries with a
// `skip` flag are left alone): the expression of cta_gs, in any order
template <typename T>
__device__ __forceinline__ void cs_pass(T *v, const T *f, const uint32_t *list, int cnt, uint32_t skip, GsC<T> c,
                                        int nx, int nxny)
{
    for (int m = threadIdx.x; m < cnt; m += CS_THREADS) {
        const uint32_t e = list[m];
        if (e & skip) continue;
        const int l = (int)(e & CS_IDX);
        v[l] = c.hh * (f[l] + (c.hx * (v[l - 1] + v[l + 1]) + c.hy * (v[l - nx] + v[l + nx]) +
                               c.hz * (v[l - nxny] + v[l + nxny])));
    }
    __syncthreads();
}

// A thread's entries of one colour list, held in registers through the
// 512 passes of an outer iteration (the lists and f do not change during a
// call): at most CS_PER entries each, taken at a stride of the CTA, so lists
// of up to 2048 entries per colour are held.
constexpr int CS_PER = 2048 / CS_THREADS;
template <typename T>
struct CsShare {
    int l[CS_PER];
    T f[CS_PER];
    uint32_t fl[CS_PER];
    __device__ __forceinline__ void load(const uint32_t *list, int cnt, const T *fs)
    {
#pragma unroll
        for (int u = 0; u < CS_PER; ++u) {
            const int m = threadIdx.x + u * CS_THREADS;
            const uint32_t e = m < cnt ? list[m] : CS_ABSENT;
            l[u] = (int)(e & CS_IDX);
            fl[u] = e & ~CS_IDX;
            f[u] = m < cnt ? fs[l[u]] : (T)0;
        }
    }
    // one colour pass (entries flagged `skip` or absent are left alone), then the barrier
    __device__ __forceinline__ void pass(T *v, uint32_t skip, GsC<T> c, int nx, int nxny) const
    {
#pragma unroll
        for (int u = 0; u < CS_PER; ++u) {
            if (fl[u] & (skip | CS_ABSENT)) continue;
            const int q = l[u];
            v[q] = c.hh * (f[u] + (c.hx * (v[q - 1] + v[q + 1]) + c.hy * (v[q - nx] + v[q + nx]) +
                                   c.hz * (v[q - nxny] + v[q + nxny])));
        }
        __syncthreads();
    }
};

// 128 sweeps of (pass over a, pass over b skipping the entries flagged skipb)
template <typename T>
__device__ __forceinline__ void cs_sweeps(T *v, const CsShare<T> &a, const CsShare<T> &b, uint32_t skipb, GsC<T> c,
                                          int nx, int nxny)
{
    for (int s = 0; s < 128; ++s) {
        a.pass(v, 0u, c, nx, nxny);
        b.pass(v, skipb, c, nx, nxny);
    }
}

// The coarsest solve (mgpcg_mex.c:265-275) of a grid one CTA holds in shared
// memory.  The colour passes run from two lists of the interior G voxels
// built once per call (a pass reads only the other colour, so the order of
// its updates does not matter: the reference's result bit for bit), which
// leaves no index arithmetic in the 512 passes of an outer iteration.
template <typename T>
__device__ __forceinline__ void coarse_solve_body(T *gv, const T *__restrict__ gf, const uint8_t *__restrict__ gG,
                                                             T *gr, Dims d, GsC<T> gc, LapC<T> lc, double tol,
                                                             int *outer_out)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    const int n = (int)d.n();
    T *v = (T *)smraw;
    T *f = v + n;
    T *sq = f + n;
    T *blk = sq + n;
    uint8_t *G = (uint8_t *)(blk + RED_NBLK);
    const int cap = (n + 1) / 2;
    uint32_t *list = (uint32_t *)(smraw + (((size_t)3 * n * sizeof(T) + (size_t)RED_NBLK * sizeof(T) + n + 15) & ~(size_t)15));
    __shared__ int cnt[2];
    const int tid = threadIdx.x;
    const int nx = (int)d.nx, ny = (int)d.ny, nz = (int)d.nz, nxny = nx * ny;
    if (tid < 2) cnt[tid] = 0;
    for (int l = tid; l < n; l += CS_THREADS) {
        v[l] = gv[l];
        f[l] = gf[l];
        G[l] = gG[l];
        sq[l] = f[l] * f[l];
    }
    __syncthreads();
    for (int l = tid; l < n; l += CS_THREADS) {
        const int k = l / nxny, j = (l / nx) % ny, i = l % nx;
        if (i < 1 || i > nx - 2 || j < 1 || j > ny - 2 || k < 1 || k > nz - 2 || !G[l]) continue;
        const int par = (i + j + k) & 1;
        uint32_t e = (uint32_t)l;
        if (i == 1) e |= CS_I1;
        if (i == nx - 2) e |= CS_INX2;
        list[par * cap + atomicAdd(&cnt[par], 1)] = e;
    }
    // reltol = tol * nrm2(f)
    const T ff = cta_lane_sum<T>(sq, blk, n);
    const double fn = sizeof(T) == 4 ? (double)sqrtf((float)ff) : sqrt((double)ff);
    const double reltol = tol * fn;
    // An idle solve: no G voxel to update, or f and v all +0.  Its sweeps then
    // leave every value as it is (hh * (+0 + ...) is +0), so after the first
    // outer iteration (which writes the residual) every later one repeats it
    // exactly; the reference runs them all when its tolerance cannot be met
    // (tol * ||f|| = 0), and their result is that of the first.
    int nz_bits = 0;
    for (int l = tid; l < n; l += CS_THREADS) {
        if (sizeof(T) == 8)
            nz_bits |= (__double_as_longlong((double)v[l]) | __double_as_longlong((double)f[l])) != 0;
        else
            nz_bits |= (__float_as_int((float)v[l]) | __float_as_int((float)f[l])) != 0;
    }
    const bool idle = !__syncthreads_or(nz_bits) || (cnt[0] + cnt[1] == 0);
    __syncthreads();
    const int n0 = cnt[0], n1 = cnt[1];
    const uint32_t *list0 = list, *list1 = list + cap;
    const int rpar0 = (nx + 1) & 1;
    const uint32_t *lr0 = rpar0 ? list1 : list0, *lr1 = rpar0 ? list0 : list1;
    const int cr0 = rpar0 ? n1 : n0, cr1 = rpar0 ? n0 : n1;
    // lists that fit are held in registers (both colours, CS_PER entries per thread)
    const bool regs = n0 <= CS_PER * CS_THREADS && n1 <= CS_PER * CS_THREADS;
    CsShare<T> s0, s1;
    if (regs) {
        s0.load(list0, n0, f);
        s1.load(list1, n1, f);
    }
    int outer = 0;
    for (int it = 0; it < 1024; ++it) {
        outer = it + 1;
        if (regs) {
            if (rpar0) {  // reverse sweeps, then forward sweeps
                cs_sweeps<T>(v, s1, s0, CS_INX2, gc, nx, nxny);
            } else {
                cs_sweeps<T>(v, s0, s1, CS_INX2, gc, nx, nxny);
            }
            cs_sweeps<T>(v, s0, s1, CS_I1, gc, nx, nxny);
        } else {
            for (int s = 0; s < 128; ++s) {  // reverse sweeps
                cs_pass<T>(v, f, lr0, cr0, 0u, gc, nx, nxny);
                cs_pass<T>(v, f, lr1, cr1, CS_INX2, gc, nx, nxny);
            }
            for (int s = 0; s < 128; ++s) {  // forward sweeps
                cs_pass<T>(v, f, list0, n0, 0u, gc, nx, nxny);
                cs_pass<T>(v, f, list1, n1, CS_I1, gc, nx, nxny);
            }
        }
        // residual into r (global copy kept like the reference) and its norm
        for (int l = tid; l < n; l += CS_THREADS) {
            const int k = l / nxny, j = (l / nx) % ny, i = l % nx;
            T r = gr[l];
            if (i >= 1 && j >= 1 && k >= 1 && i + 1 < nx && j + 1 < ny && k + 1 < nz && G[l]) {
                r = f[l] + (lc.hh * v[l] + lc.hx * (v[l - 1] + v[l + 1]) + lc.hy * (v[l - nx] + v[l + nx]) +
                            lc.hz * (v[l - nxny] + v[l + nxny]));
                gr[l] = r;
            }
            sq[l] = r * r;
        }
        __syncthreads();
        const T rr = cta_lane_sum<T>(sq, blk, n);
        const double rn = sizeof(T) == 4 ? (double)sqrtf((float)rr) : sqrt((double)rr);
        __syncthreads();
        if (rn < reltol) break;
        if (idle) {
            outer = 1024;
            break;
        }
    }
    for (int l = tid; l < n; l += CS_THREADS) gv[l] = v[l];
    if (tid == 0 && outer_out) *outer_out += outer;
}

template <typename T>
__global__ void __launch_bounds__(CS_THREADS) coarse_solve_k(T *gv, const T *__restrict__ gf, const uint8_t *__restrict__ gG,
                                                             T *gr, Dims d, GsC<T> gc, LapC<T> lc, double tol,
                                                             int *outer_out)
{
    coarse_solve_body<T>(gv, gf, gG, gr, d, gc, lc, tol, outer_out);
}

// ---------------------------------------------------------------------------
// coarsest level on a thread-block cluster (mgpcg_mex.c:265-275)
//
// The one-CTA solver runs the reference's 256 sweeps per outer iteration on a
// single SM; in FP64 (two operations per clock per SM on this GPU) that is
// ~2.4 ms for an 18^3 grid.  Here the cn CTAs of a cluster split the interior
// z planes into slabs: CTA c owns planes [k0, k1) and keeps in shared memory
// v of planes k0-1 .. k1 (its slab plus one halo plane each side) and f, G of
// its slab.  Each colour pass updates the slab's voxels of that colour from a
// list built once (so no index arithmetic per pass), pushes the new values of
// its first and last plane into the neighbours' halo planes
// (st.shared::cluster), and ends at the cluster barrier, whose release /
// acquire makes the pushes visible.  A pass reads only the other colour, so
// the order of updates within a pass does not matter: results are those of
// the one-CTA solver, bit for bit.  The residual goes to global r, and its
// lane-order norm is formed as in cta_lane_sum: CTA c halves the 256-element
// blocks b = c, c + cn, ... and pushes the block sums into CTA 0, which
// halves the 1024 block sums and broadcasts the total.
// ---------------------------------------------------------------------------

constexpr int CC_THREADS = RED_BLOCK;
constexpr int CC_MAX_CTAS = 16;
constexpr uint32_t CC_IDX = 0x0FFFFFFFu;  // list entry: v index in the CTA's planes
constexpr uint32_t CC_I1 = 1u << 28;      // i == 1
constexpr uint32_t CC_INX2 = 1u << 29;    // i == nx - 2
constexpr uint32_t CC_DOWN = 1u << 30;    // first slab plane: push to CTA c - 1
constexpr uint32_t CC_UP = 1u << 31;      // last slab plane: push to CTA c + 1

// Shared-memory layout of one CTA (host and device agree on it).
struct CcLayout {
    size_t v, f, blk, red, bc, G, list, bytes;
    __host__ __device__ CcLayout(size_t nxny, int npmax, size_t es)
    {
        const size_t pl = (size_t)npmax * nxny;
        v = 0;
        f = v + (pl + 2 * nxny) * es;
        blk = f + pl * es;
        red = blk + (size_t)RED_NBLK * es;
        bc = red + (size_t)RED_BLOCK * es;
        G = (bc + 2 * sizeof(double) + 15) & ~(size_t)15;
        list = (G + pl + 15) & ~(size_t)15;
        bytes = list + 2 * pl * sizeof(uint32_t);
    }
};

// Lane-order sum of src[e]^2 over e < n (src in global memory, written
// before the last cluster barrier): the same pairing as cta_lane_sum.
template <typename T>
__device__ T cl_lane_sum(const T *src, int n, T *red, T *blk, T *bc, uint32_t c, uint32_t cn)
{
    const int tid = threadIdx.x;
    const int nb = (n + RED_BLOCK - 1) / RED_BLOCK;
    const uint32_t blk0 = cl_map(blk, 0);
    for (int b = (int)c; b < nb; b += (int)cn) {
        const int e = b * RED_BLOCK + tid;
        const T x = e < n ? __ldcg(src + e) : (T)0;
        red[tid] = x * x;
        __syncthreads();
        for (int s = RED_BLOCK / 2; s > 0; s >>= 1) {
            if (tid < s) red[tid] = red[tid] + red[tid + s];
            __syncthreads();
        }
        if (tid == 0) cl_st(blk0 + (uint32_t)(b * sizeof(T)), red[0]);
        __syncthreads();
    }
    cl_sync();
    if (c == 0) {
        // block sums b >= nb stay +0: never pushed, and t >= nb only ever adds +0 + +0
        for (int s = RED_NBLK / 2; s > 0; s >>= 1) {
            for (int t = tid; t < s; t += CC_THREADS) blk[t] = blk[t] + blk[t + s];
            __syncthreads();
        }
        if (tid < (int)cn) cl_st(cl_map(bc, (uint32_t)tid), blk[0]);
    }
    cl_sync();
    return bc[0];
}

template <typename T>
__device__ __forceinline__ void cc_pass(T *v, const T *f, const uint32_t *list, int cnt, uint32_t skip, GsC<T> c,
                                        int nx, int nxny, uint32_t vdn, uint32_t offdn, uint32_t vup, uint32_t offup)
{
    for (int m = threadIdx.x; m < cnt; m += CC_THREADS) {
        const uint32_t e = list[m];
        if (e & skip) continue;
        const int l = (int)(e & CC_IDX);
        const T val = c.hh * (f[l - nxny] + (c.hx * (v[l - 1] + v[l + 1]) + c.hy * (v[l - nx] + v[l + nx]) +
                                             c.hz * (v[l - nxny] + v[l + nxny])));
        v[l] = val;
        if (e & CC_DOWN) cl_st(vdn + (uint32_t)((l + offdn) * sizeof(T)), val);
        if (e & CC_UP) cl_st(vup + (uint32_t)((l - offup) * sizeof(T)), val);
    }
    cl_sync();
}

template <typename T>
__global__ void __launch_bounds__(CC_THREADS) coarse_cluster_k(T *gv, const T *__restrict__ gf,
                                                               const uint8_t *__restrict__ gG, T *gr, Dims d,
                                                               GsC<T> gc, LapC<T> lc, double tol, int npmax,
                                                               int *outer_out, int sweeps, int rev)
{
    // sweeps > 0: no coarsest solve, only that many sweeps (reverse when rev)
    // over the voxels of gG (a boundary band), then v is written back
    extern __shared__ __align__(16) unsigned char smraw[];
    const int nx = (int)d.nx, ny = (int)d.ny, nz = (int)d.nz, nxny = nx * ny, n = nxny * nz;
    const uint32_t c = cl_rank(), cn = cl_size();
    const int P = nz - 2;
    const int k0 = 1 + (int)((long long)P * c / cn), k1 = 1 + (int)((long long)P * (c + 1) / cn), np = k1 - k0;
    const int kp = 1 + (int)((long long)P * (c > 0 ? c - 1 : 0) / cn);  // first plane of CTA c - 1
    const CcLayout lay((size_t)nxny, npmax, sizeof(T));
    T *v = (T *)(smraw + lay.v), *f = (T *)(smraw + lay.f), *blk = (T *)(smraw + lay.blk);
    T *red = (T *)(smraw + lay.red), *bc = (T *)(smraw + lay.bc);
    uint8_t *G = smraw + lay.G;
    uint32_t *list = (uint32_t *)(smraw + lay.list);
    const int cap = npmax * nxny;
    __shared__ int cnt[2];
    __shared__ unsigned cflag;  // OR over the cluster: 1 = some G voxel to update, 2 = some v or f bit set
    const int tid = threadIdx.x;
    if (tid < 2) cnt[tid] = 0;
    if (tid == 0) cflag = 0u;
    for (int t = tid; t < RED_NBLK; t += CC_THREADS) blk[t] = (T)0;
    const size_t base = (size_t)(k0 - 1) * nxny;
    for (int t = tid; t < (np + 2) * nxny; t += CC_THREADS) v[t] = gv[base + t];
    for (int t = tid; t < np * nxny; t += CC_THREADS) {
        f[t] = gf[base + nxny + t];
        G[t] = gG[base + nxny + t];
    }
    __syncthreads();
    // colour lists of the slab's interior G voxels
    for (int t = tid; t < np * nxny; t += CC_THREADS) {
        const int kl = t / nxny, rem = t - kl * nxny, j = rem / nx, i = rem - j * nx, k = k0 + kl;
        if (i < 1 || i > nx - 2 || j < 1 || j > ny - 2 || !G[t]) continue;
        const int par = (i + j + k) & 1;
        uint32_t e = (uint32_t)(t + nxny);
        if (i == 1) e |= CC_I1;
        if (i == nx - 2) e |= CC_INX2;
        if (kl == 0 && c > 0) e |= CC_DOWN;
        if (kl == np - 1 && c + 1 < cn) e |= CC_UP;
        list[par * cap + atomicAdd(&cnt[par], 1)] = e;
    }
    // halo planes are loaded everywhere before any neighbour pushes into them
    cl_sync();
    const uint32_t vdn = c > 0 ? cl_map(v, c - 1) : 0u, vup = c + 1 < cn ? cl_map(v, c + 1) : 0u;
    const uint32_t offdn = (uint32_t)(nxny * (k0 - kp)), offup = (uint32_t)(nxny * np);
    const int n0 = cnt[0], n1 = cnt[1];
    const uint32_t *list0 = list, *list1 = list + cap;
    const int rpar0 = (nx + 1) & 1;
    const uint32_t *lr0 = rpar0 ? list1 : list0, *lr1 = rpar0 ? list0 : list1;
    const int cr0 = rpar0 ? n1 : n0, cr1 = rpar0 ? n0 : n1;
    if (sweeps > 0) {
        for (int s = 0; s < sweeps; ++s) {
            if (rev) {
                cc_pass<T>(v, f, lr0, cr0, 0u, gc, nx, nxny, vdn, offdn, vup, offup);
                cc_pass<T>(v, f, lr1, cr1, CC_INX2, gc, nx, nxny, vdn, offdn, vup, offup);
            } else {
                cc_pass<T>(v, f, list0, n0, 0u, gc, nx, nxny, vdn, offdn, vup, offup);
                cc_pass<T>(v, f, list1, n1, CC_I1, gc, nx, nxny, vdn, offdn, vup, offup);
            }
        }
        for (int t = tid; t < np * nxny; t += CC_THREADS) gv[base + nxny + t] = v[nxny + t];
        cl_sync();
        return;
    }

    // An idle solve (no G voxel to update anywhere, or every v and f bit clear):
    // its sweeps change nothing, so after the first outer iteration every
    // later one repeats it exactly (see coarse_solve_k).  The slab flags are
    // ORed into every CTA; the lane sum's cluster barriers make them visible.
    {
        int nzb = 0;
        for (int t = tid; t < (np + 2) * nxny; t += CC_THREADS)
            nzb |= sizeof(T) == 8 ? __double_as_longlong((double)v[t]) != 0 : __float_as_int((float)v[t]) != 0;
        for (int t = tid; t < np * nxny; t += CC_THREADS)
            nzb |= sizeof(T) == 8 ? __double_as_longlong((double)f[t]) != 0 : __float_as_int((float)f[t]) != 0;
        const unsigned bits = (cnt[0] + cnt[1] > 0 ? 1u : 0u) | (__syncthreads_or(nzb) ? 2u : 0u);
        if (tid < (int)cn && bits) cl_or(cl_map(&cflag, (uint32_t)tid), bits);
    }
    const T ff = cl_lane_sum<T>(gf, n, red, blk, bc, c, cn);
    const double fn = sizeof(T) == 4 ? (double)sqrtf((float)ff) : sqrt((double)ff);
    const double reltol = tol * fn;
    const bool idle = (cflag & 1u) == 0 || (cflag & 2u) == 0;
    int outer = 0;
    for (int it = 0; it < 1024; ++it) {
        outer = it + 1;
        for (int s = 0; s < 128; ++s) {  // reverse sweeps
            cc_pass<T>(v, f, lr0, cr0, 0u, gc, nx, nxny, vdn, offdn, vup, offup);
            cc_pass<T>(v, f, lr1, cr1, CC_INX2, gc, nx, nxny, vdn, offdn, vup, offup);
        }
        for (int s = 0; s < 128; ++s) {  // forward sweeps
            cc_pass<T>(v, f, list0, n0, 0u, gc, nx, nxny, vdn, offdn, vup, offup);
            cc_pass<T>(v, f, list1, n1, CC_I1, gc, nx, nxny, vdn, offdn, vup, offup);
        }
        // residual of the slab's interior G voxels into global r
        for (int q = 0; q < 2; ++q) {
            const uint32_t *ls = q ? list1 : list0;
            const int cq = q ? n1 : n0;
            for (int m = tid; m < cq; m += CC_THREADS) {
                const int l = (int)(ls[m] & CC_IDX);
                gr[base + l] = f[l - nxny] + (lc.hh * v[l] + lc.hx * (v[l - 1] + v[l + 1]) +
                                              lc.hy * (v[l - nx] + v[l + nx]) + lc.hz * (v[l - nxny] + v[l + nxny]));
            }
        }
        cl_sync();
        const T rr = cl_lane_sum<T>(gr, n, red, blk, bc, c, cn);
        const double rn = sizeof(T) == 4 ? (double)sqrtf((float)rr) : sqrt((double)rr);
        if (rn < reltol) break;
        if (idle) {
            outer = 1024;
            break;
        }
    }
    for (int t = tid; t < np * nxny; t += CC_THREADS) gv[base + nxny + t] = v[nxny + t];
    if (c == 0 && tid == 0 && outer_out) *outer_out += outer;
    cl_sync();  // no CTA leaves while a peer may still address its shared memory
}

// ---------------------------------------------------------------------------
// hierarchy and drivers (mgpcg_mex.c:126-332, mg_mex.c:94-207, fmg_mex.c:93-212)
// ---------------------------------------------------------------------------

template <typename T>
struct Level {
    Dims d;
    size_t n;
    T *v, *f, *r;
    // Invariant: on levels whose G is held as colour lists, f is +0 outside G from set-up
    // on (hier_init zeroes it, restrictions write only G): restrict_list_k writes f on G
    // only and relies on it, which is restrict_mex's result there.  Nothing may use a
    // coarse f as scratch outside G.
    uint8_t *G, *B;
    double h[3];
    uint32_t *bl[2];     // B voxels of each colour (null: full-grid passes over B)
    unsigned bn[2];
    uint32_t *gl[2];     // G voxels of each colour (null: full-grid passes)
    unsigned gn[2];
    uint8_t bmode, gmode;  // how a smoothing call runs the B / G passes (SW_LAUNCH, SW_CLUSTER, SW_GRID)
    int dsm_cn, dsm_npmax;  // > 0: long band sweeps run on z-slabs in a cluster's shared memory
    size_t dsm_smem;
};

template <typename T>
struct Hier {
    int nl;
    Level<T> L[16];
    void *blk;
    uint8_t *scratch;    // n(level 0) bytes for boundary-mask construction
    int *counters;       // device: coarse outer iterations
    bool coarse_in_smem;
    size_t coarse_smem;
    void *lists;         // the levels' colour lists (one allocation)
    int sw_ctas;         // cluster size of the list passes (0: not available)
    int sg_ctas;         // CTAs of the whole-GPU list passes (0: not available)
    bool v0_zero_outside; // level 0's v is +0 outside G whenever a cycle corrects it
    int host_outer;      // outer iterations of the host-driven coarsest solve
    int cg_ctas;         // > 0: the coarsest level runs on this many CTAs, cooperatively (wins over the cluster)
    GridBar gb;          // their barrier words (arrival count, error flag)
    void *gpart;         // RED_NBLK + 1 lane-order block sums
    int cc_ctas;         // > 0: the coarsest level runs on a cluster of this many CTAs
    int cc_npmax;        // planes per CTA (largest slab)
    size_t cc_smem;
};

static inline size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

// The coarse solver's dynamic shared-memory limit is a process-wide function
// attribute: raise it once per device to the opt-in maximum, so concurrent
// solves on several host threads never lower it under each other's launch.
// The limit is the opt-in maximum less the kernel's static shared memory; it
// is returned in *lim (0: the attribute could not be read).
template <typename T>
static qsm_status coarse_smem_limit(qsm_ctx *ctx, int maxsm, size_t *lim)
{
    static std::mutex mu;
    static std::set<int> done;
    *lim = 0;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, coarse_solve_k<T>) != cudaSuccess || (size_t)maxsm <= fa.sharedSizeBytes) {
        cudaGetLastError();
        return QSM_OK;
    }
    const size_t l = (size_t)maxsm - fa.sharedSizeBytes;
    std::lock_guard<std::mutex> lock(mu);
    if (!done.count(ctx->device)) {
        QSM_CUDA(cudaFuncSetAttribute(coarse_solve_k<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l));
        done.insert(ctx->device);
    }
    *lim = l;
    return QSM_OK;
}

// The cluster solver's dynamic shared-memory limit: the opt-in maximum less
// its static shared memory, raised once per device together with the
// permission for clusters of more than 8 CTAs.  0 if either is refused.
template <typename T>
static size_t cluster_smem_limit(qsm_ctx *ctx, int maxsm)
{
    static std::mutex mu;
    static std::set<int> done;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, coarse_cluster_k<T>) != cudaSuccess || (size_t)maxsm <= fa.sharedSizeBytes) {
        cudaGetLastError();
        return 0;
    }
    const size_t lim = (size_t)maxsm - fa.sharedSizeBytes;
    std::lock_guard<std::mutex> lock(mu);
    if (!done.count(ctx->device)) {
        if (cudaFuncSetAttribute(coarse_cluster_k<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim) !=
                cudaSuccess ||
            cudaFuncSetAttribute(coarse_cluster_k<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        done.insert(ctx->device);
    }
    return lim;
}

// Whether a cluster of cn CTAs with `smem` dynamic bytes each can be resident.
template <typename T>
static bool cluster_fits(int cn, size_t smem)
{
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)cn;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)cn);
    cfg.blockDim = dim3(CC_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, coarse_cluster_k<T>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return nclusters >= 1;
}

// Cluster shape for a grid held in z-slabs over up to 16 CTAs (at least one
// interior plane each) within the shared-memory limit; cn = 0 if none fits.
template <typename T>
static void plan_slabs(qsm_ctx *ctx, const Dims &dc, int maxsm, int *cn_out, int *npmax_out, size_t *smem_out)
{
    *cn_out = 0;
    const int P = (int)dc.nz - 2;
    if (dc.nx < 3 || dc.ny < 3 || P < 2 || dc.n() >= (1u << 27)) return;
    const size_t lim = cluster_smem_limit<T>(ctx, maxsm);
    for (int cn = P < CC_MAX_CTAS ? P : CC_MAX_CTAS; cn >= 2 && lim > 0; cn = cn > 8 ? 8 : cn - 1) {
        const int npmax = (P + cn - 1) / cn;
        const CcLayout lay(dc.nxny(), npmax, sizeof(T));
        if (lay.bytes > lim || !cluster_fits<T>(cn, lay.bytes)) continue;
        *cn_out = cn;
        *npmax_out = npmax;
        *smem_out = lay.bytes;
        return;
    }
}

// Cluster shape of the coarsest level.
template <typename T>
static void plan_cluster(qsm_ctx *ctx, Hier<T> &H, int maxsm)
{
    plan_slabs<T>(ctx, H.L[H.nl - 1].d, maxsm, &H.cc_ctas, &H.cc_npmax, &H.cc_smem);
}

template <typename T>
static qsm_status hier_init(qsm_ctx *ctx, Hier<T> &H, int nl, const Dims &dp, const double *h)
{
    memset(&H, 0, sizeof H);
    H.nl = nl;
    size_t bytes = 0;
    Dims d = dp;
    for (int i = 0; i < nl; ++i) {
        if (i > 0) d = Dims{((d.nx - 2 + 1) >> 1) + 2, ((d.ny - 2 + 1) >> 1) + 2, ((d.nz - 2 + 1) >> 1) + 2};
        H.L[i].d = d;
        H.L[i].n = d.n();
        for (int q = 0; q < 3; ++q) H.L[i].h[q] = i == 0 ? h[q] : H.L[i - 1].h[q] * 2.0;
        bytes += 3 * al256(d.n() * sizeof(T)) + 2 * al256(d.n());
    }
    bytes += al256(dp.n()) + 512 + al256((RED_NBLK + 1) * sizeof(double)) + 256;
    QSM_TRY(dalloc(ctx, &H.blk, bytes));
    QSM_CUDA(cudaMemsetAsync(H.blk, 0, bytes, ctx->stream));
    char *c = (char *)H.blk;
    for (int i = 0; i < nl; ++i) {
        const size_t n = H.L[i].n;
        H.L[i].v = (T *)c; c += al256(n * sizeof(T));
        H.L[i].f = (T *)c; c += al256(n * sizeof(T));
        H.L[i].r = (T *)c; c += al256(n * sizeof(T));
        H.L[i].G = (uint8_t *)c; c += al256(n);
        H.L[i].B = (uint8_t *)c; c += al256(n);
    }
    H.scratch = (uint8_t *)c; c += al256(dp.n());
    H.counters = (int *)c;
    c += 512;
    H.gpart = c;
    c += al256((RED_NBLK + 1) * sizeof(double));
    H.gb.count = (unsigned *)c;
    H.gb.err = (int *)c + 1;
    // test hook: barriers that can never complete, with a short wait, so the bounded wait runs out
    const bool short_bar = (ctx->debug & QSM_DEBUG_GRID_BARRIER_TIMEOUT) != 0;
    H.gb.extra = short_bar ? 1u : 0u;
    H.gb.limit = short_bar ? (1ll << 12) : CG_SPIN_LIMIT;
    const size_t nc = H.L[nl - 1].n;
    H.coarse_smem = cs_smem(nc, sizeof(T)) + 64;
    int maxsm = 0;
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    size_t cs_lim = 0;
    QSM_TRY(coarse_smem_limit<T>(ctx, maxsm, &cs_lim));
    H.coarse_in_smem = H.coarse_smem <= cs_lim && nc < (1u << 18);
    plan_cluster<T>(ctx, H, maxsm);
    // In FP32 one SM's FP32 rate keeps a colour pass of a small coarsest grid
    // under the cluster barrier's cost (157 against 214 us per 512-pass call
    // at 18^3): one CTA from colour lists, where it holds the grid.  FP64
    // passes need the cluster's 16 FP64 pipes.
    if (sizeof(T) == 4 && H.coarse_in_smem) H.cc_ctas = 0;
    // levels whose long band sweeps can run on z-slabs in a cluster
    for (int i = 0; i + 1 < nl; ++i)
        plan_slabs<T>(ctx, H.L[i].d, maxsm, &H.L[i].dsm_cn, &H.L[i].dsm_npmax, &H.L[i].dsm_smem);
    return QSM_OK;
}

// CTAs of the whole-GPU list passes: one per SM when cooperative launch is
// available, else 0.
template <typename T>
static int grid_sweep_ctas(qsm_ctx *ctx)
{
    int coop = 0, sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device) != cudaSuccess || !coop ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweeps_grid_k<T>, CG_THREADS, 0) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return 0;
    }
    return sms;
}

// The whole-GPU coarsest solver: for large colour passes, or where neither a
// cluster nor one CTA holds the grid; needs the coarsest level's G lists and
// cooperative launch.  cg_ctas = one CTA per SM, else 0.
template <typename T>
static void plan_coarse_grid(qsm_ctx *ctx, Hier<T> &H)
{
    H.cg_ctas = 0;
    const Level<T> &C = H.L[H.nl - 1];
    if (!C.gl[0] || C.d.nx < 3 || C.d.ny < 3 || C.d.nz < 3 || C.n >= (1u << 30)) return;
    const bool large = C.gn[0] > CG_MIN_PASS || C.gn[1] > CG_MIN_PASS;
    if (!large && (H.cc_ctas > 0 || H.coarse_in_smem)) return;
    int coop = 0, sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device) != cudaSuccess || !coop ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, coarse_grid_k<T>, CG_THREADS, 0) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return;
    }
    H.cg_ctas = sms;
}

// Colour lists of every level's G and boundary band B (counted, then filled
// into one allocation), and how each list's passes run (by its size).
// Grids of 2^30 voxels or more keep the full-grid passes.
template <typename T>
static qsm_status boundary_lists(qsm_ctx *ctx, Hier<T> &H)
{
    if (H.L[0].n >= ((size_t)1 << 30)) return QSM_OK;
    const int cn = sweeps_cluster_size<T>(ctx);
    unsigned *cnt = (unsigned *)H.counters + 8;  // B: 4i, 4i+1; G: 4i+2, 4i+3 (nl <= 16)
    QSM_CUDA(cudaMemsetAsync(cnt, 0, 4 * H.nl * sizeof(unsigned), ctx->stream));
    // per level: segment counts of its four lists (B and G, two colours each) and their scan
    size_t nseg[16] = {0}, tot_seg = 0, max_seg = 0;
    for (int i = 0; i < H.nl; ++i) {
        const dim3 g = interior_grid3(H.L[i].d);
        nseg[i] = (g.x && g.y && g.z) ? (size_t)g.x * (H.L[i].d.ny - 2) * (H.L[i].d.nz - 2) : 0;
        tot_seg += 2 * 2 * nseg[i];
        max_seg = std::max(max_seg, nseg[i]);
    }
    void *segblk = nullptr;
    const size_t segbytes = (2 * tot_seg + scan_scratch(4 * max_seg)) * sizeof(unsigned);
    QSM_TRY(dalloc(ctx, &segblk, segbytes));
    unsigned *segc = (unsigned *)segblk, *segoff = segc + tot_seg, *scan_tmp = segoff + tot_seg;
    for (size_t i = 0, o = 0; i < (size_t)H.nl; o += 4 * nseg[i], ++i) {
        const Level<T> &L = H.L[i];
        if (!nseg[i]) continue;
        const dim3 g = interior_grid3(L.d);
        blist_seg_k<false><<<g, vox_block(), 0, ctx->stream>>>(SegLists{}, segc + o, L.B, L.G, L.d, nseg[i]);
        QSM_CUDA(cudaGetLastError());
        QSM_TRY(exclusive_scan(ctx, segc + o, segoff + o, 4 * nseg[i], scan_tmp));
        blist_total_k<<<1, 32, 0, ctx->stream>>>(segc + o, segoff + o, nseg[i], cnt + 4 * i);
    }
    QSM_CUDA(cudaGetLastError());
    unsigned hc[64];
    QSM_CUDA(cudaMemcpyAsync(hc, cnt, 4 * H.nl * sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    size_t tot = 0;
    H.sg_ctas = grid_sweep_ctas<T>(ctx);
    auto mode = [&](unsigned c0, unsigned c1) -> uint8_t {
        const unsigned c = c0 > c1 ? c0 : c1;
        const unsigned cap = (unsigned)cn * SW_THREADS * SW_PER;
        // FP32 passes are not bound by 16 SMs' arithmetic: a cluster takes lists up to its capacity
        if (cn > 0 && c <= cap && (sizeof(T) == 4 || c <= SW_CLUSTER_MAX)) return SW_CLUSTER;
        if (H.sg_ctas > 0 && c <= SW_GRID_MAX) return SW_GRID;
        return SW_LAUNCH;
    };
    for (int i = 0; i < H.nl; ++i) {
        Level<T> &L = H.L[i];
        L.bmode = mode(hc[4 * i], hc[4 * i + 1]);
        L.gmode = mode(hc[4 * i + 2], hc[4 * i + 3]);
        for (int p = 0; p < 2; ++p)
            tot += al256((size_t)hc[4 * i + p] * sizeof(uint32_t)) + al256((size_t)hc[4 * i + 2 + p] * sizeof(uint32_t));
    }
    QSM_TRY(dalloc(ctx, &H.lists, tot + 256));
    H.sw_ctas = cn;
    char *c = (char *)H.lists;
    for (int i = 0; i < H.nl; ++i) {
        Level<T> &L = H.L[i];
        for (int p = 0; p < 2; ++p) {
            L.bl[p] = (uint32_t *)c;
            L.bn[p] = hc[4 * i + p];
            c += al256((size_t)hc[4 * i + p] * sizeof(uint32_t));
        }
        for (int p = 0; p < 2; ++p) {
            L.gl[p] = (uint32_t *)c;
            L.gn[p] = hc[4 * i + 2 + p];
            c += al256((size_t)hc[4 * i + 2 + p] * sizeof(uint32_t));
        }
    }
    for (size_t i = 0, o = 0; i < (size_t)H.nl; o += 4 * nseg[i], ++i) {
        const Level<T> &L = H.L[i];
        if (!nseg[i]) continue;
        const dim3 g = interior_grid3(L.d);
        blist_seg_k<true><<<g, vox_block(), 0, ctx->stream>>>(SegLists{{L.bl[0], L.bl[1], L.gl[0], L.gl[1]}},
                                                               segoff + o, L.B, L.G, L.d, nseg[i]);
    }
    QSM_CUDA(cudaGetLastError());
    QSM_TRY(dfree(ctx, segblk));
    plan_coarse_grid<T>(ctx, H);
    return QSM_OK;
}

// `iter` colour-pass pairs (gauss_seidel's order and skips) over colour lists,
// one launch per pass.
template <typename T>
static qsm_status list_sweeps(qsm_ctx *ctx, T *v, const T *f, uint32_t *const lists[2], const unsigned cnt[2],
                              const double *h, const Dims &d, int32_t iter, bool rev)
{
    const GsC<T> c = gs_consts<T>(h);
    const int par0 = rev ? (int)((d.nx + 1) & 1) : 0;
    const uint32_t skip = rev ? BL_INX2 : BL_I1;
    for (int32_t s = 0; s < iter; ++s)
        for (int q = 0; q < 2; ++q) {
            const int par = par0 ^ q;
            if (!cnt[par]) continue;
            if (sizeof(T) == 4)
                gs_list_ilp_k<T><<<(cnt[par] + 256 * GS_PER - 1) / (256 * GS_PER), 256, 0, ctx->stream>>>(
                    v, f, lists[par], cnt[par], q ? skip : 0u, c, d.nx, d.nxny());
            else
                gs_list_k<T><<<(cnt[par] + 255) / 256, 256, 0, ctx->stream>>>(v, f, lists[par], cnt[par],
                                                                             q ? skip : 0u, c, d.nx, d.nxny());
        }
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

template <typename T>
static qsm_status sweeps_grid(qsm_ctx *ctx, const Hier<T> &H, T *v, const T *f, uint32_t *const lists[2],
                              const unsigned cnt[2], const double *h, const Dims &d, int32_t iter, bool rev)
{
    const int par0 = rev ? (int)((d.nx + 1) & 1) : 0;
    T *vv = v;
    const T *ff = f;
    const uint32_t *la = lists[par0], *lb = lists[par0 ^ 1];
    unsigned ca = cnt[par0], cb = cnt[par0 ^ 1];
    uint32_t skipb = rev ? BL_INX2 : BL_I1;
    int32_t it = iter;
    GsC<T> gc = gs_consts<T>(h);
    size_t nx = d.nx, nxny = d.nxny();
    GridBar gb = H.gb;
    void *args[] = {&vv, &ff, &la, &ca, &lb, &cb, &skipb, &it, &gc, &nx, &nxny, &gb};
    QSM_CUDA(cudaMemsetAsync(H.gb.count, 0, sizeof(unsigned), ctx->stream));
    QSM_CUDA(cudaLaunchCooperativeKernel((const void *)sweeps_grid_k<T>, dim3((unsigned)H.sg_ctas), dim3(CG_THREADS),
                                         args, 0, ctx->stream));
    return QSM_OK;
}

// `iter` colour-pass pairs over a level's G (gauss_seidel over G): one
// cluster launch on small levels, else one launch per pass over the colour
// lists (full-grid passes only where there are no lists).
template <typename T>
static qsm_status smooth(qsm_ctx *ctx, const Hier<T> &H, Level<T> &L, int32_t iter, bool rev)
{
    if (!L.gl[0]) return gauss_seidel<T>(ctx, L.v, L.f, L.G, L.h, L.d, iter, rev);
    if (L.d.nx < 3 || L.d.ny < 3 || L.d.nz < 3 || iter <= 0) return QSM_OK;
    if (L.gmode == SW_CLUSTER) return sweeps_cluster<T>(ctx, H.sw_ctas, L.v, L.f, L.gl, L.gn, L.h, L.d, iter, rev);
    if (L.gmode == SW_GRID) return sweeps_grid<T>(ctx, H, L.v, L.f, L.gl, L.gn, L.h, L.d, iter, rev);
    return list_sweeps<T>(ctx, L.v, L.f, L.gl, L.gn, L.h, L.d, iter, rev);
}

// residual on G from its colour lists (residual_k restricted to G, in any order)
template <typename T>
__global__ void residual_list_k(T *r, const T *__restrict__ f, const T *__restrict__ x,
                                const uint32_t *__restrict__ l0, unsigned c0, const uint32_t *__restrict__ l1,
                                unsigned c1, LapC<T> c, size_t nx, size_t nxny)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c0 + c1) return;
    const size_t l = (t < c0 ? l0[t] : l1[t - c0]) & BL_IDX;
    r[l] = f[l] + (c.hh * x[l] + c.hx * (x[l - 1] + x[l + 1]) + c.hy * (x[l - nx] + x[l + nx]) + c.hz * (x[l - nxny] + x[l + nxny]));
}

// residual_list_k for FP32 levels (bound by load latency): GS_PER entries
// per thread at a stride of the grid, every load issued before a store.
template <typename T>
__device__ __forceinline__ void residual_list_ilp_body(T *r, const T *__restrict__ f, const T *__restrict__ x,
                                    const uint32_t *__restrict__ l0, unsigned c0, const uint32_t *__restrict__ l1,
                                    unsigned c1, LapC<T> c, size_t nx, size_t nxny, unsigned blk, unsigned nblk)
{
    const unsigned t0 = blk * blockDim.x + threadIdx.x, st = nblk * blockDim.x;
    size_t l[GS_PER];
    bool on[GS_PER];
#pragma unroll
    for (int u = 0; u < GS_PER; ++u) {
        const unsigned m = t0 + u * st;
        on[u] = m < c0 + c1;
        l[u] = on[u] ? ((m < c0 ? l0[m] : l1[m - c0]) & BL_IDX) : 0;
    }
    T fv[GS_PER], a[GS_PER][7];
#pragma unroll
    for (int u = 0; u < GS_PER; ++u) {
        if (!on[u]) continue;
        const size_t q = l[u];
        fv[u] = f[q];
        a[u][0] = x[q];
        a[u][1] = x[q - 1];
        a[u][2] = x[q + 1];
        a[u][3] = x[q - nx];
        a[u][4] = x[q + nx];
        a[u][5] = x[q - nxny];
        a[u][6] = x[q + nxny];
    }
#pragma unroll
    for (int u = 0; u < GS_PER; ++u)
        if (on[u])
            r[l[u]] = fv[u] + (c.hh * a[u][0] + c.hx * (a[u][1] + a[u][2]) + c.hy * (a[u][3] + a[u][4]) +
                               c.hz * (a[u][5] + a[u][6]));
}

template <typename T>
__global__ void residual_list_ilp_k(T *r, const T *__restrict__ f, const T *__restrict__ x,
                                    const uint32_t *__restrict__ l0, unsigned c0, const uint32_t *__restrict__ l1,
                                    unsigned c1, LapC<T> c, size_t nx, size_t nxny)
{
    residual_list_ilp_body<T>(r, f, x, l0, c0, l1, c1, c, nx, nxny, blockIdx.x, gridDim.x);
}

// The V-cycle's correction of an FP32 level whose v is +0 outside G
// (prolong_k<T, true, true>) from its G lists: x += the interpolated coarse
// value on each G voxel, GS_PER entries per thread.  The fine voxel
// (i, j, k) takes coarse parent i2 = (i + 1) / 2 and case bit (i + 1) mod 2
// per axis, as in prolong_k; the voxels of one colour in one x row share
// their case, so a warp's lanes mostly run one case.
template <typename T>
__device__ __forceinline__ void correct_list_body(T *x, const T *__restrict__ x2, const uint32_t *__restrict__ l0, unsigned c0,
                               const uint32_t *__restrict__ l1, unsigned c1, uint32_t nx, uint32_t nxny,
                               uint32_t nx2, uint32_t nxny2, unsigned blk, unsigned nblk)
{
    const unsigned t0 = blk * blockDim.x + threadIdx.x, st = nblk * blockDim.x;
    uint32_t l[GS_PER], l2[GS_PER];
    int cs[GS_PER];
    bool on[GS_PER];
#pragma unroll
    for (int u = 0; u < GS_PER; ++u) {
        const unsigned m = t0 + u * st;
        on[u] = m < c0 + c1;
        const uint32_t q = on[u] ? ((m < c0 ? l0[m] : l1[m - c0]) & BL_IDX) : 0u;
        const uint32_t k = q / nxny, rem = q - k * nxny, j = rem / nx, i = rem - j * nx;
        l[u] = q;
        l2[u] = (i + 1) / 2 + nx2 * ((j + 1) / 2) + nxny2 * ((k + 1) / 2);
        cs[u] = (int)(((i + 1) & 1) + 2 * ((j + 1) & 1) + 4 * ((k + 1) & 1));
    }
    T val[GS_PER], xv[GS_PER];
    const uint32_t ox = 1, oy = nx2, oz = nxny2;
#pragma unroll
    for (int u = 0; u < GS_PER; ++u) {
        if (!on[u]) continue;
        const uint32_t q2 = l2[u];
        const T c0v = x2[q2];
        xv[u] = x[l[u]];
        switch (cs[u]) {
        case 0: val[u] = c0v; break;
        case 1: val[u] = (T)0.5 * (c0v + x2[q2 + ox]); break;
        case 2: val[u] = (T)0.5 * (c0v + x2[q2 + oy]); break;
        case 4: val[u] = (T)0.5 * (c0v + x2[q2 + oz]); break;
        case 3: val[u] = (T)0.25 * (c0v + x2[q2 + ox] + x2[q2 + oy] + x2[q2 + ox + oy]); break;
        case 5: val[u] = (T)0.25 * (c0v + x2[q2 + ox] + x2[q2 + oz] + x2[q2 + ox + oz]); break;
        case 6: val[u] = (T)0.25 * (c0v + x2[q2 + oy] + x2[q2 + oz] + x2[q2 + oy + oz]); break;
        default:
            val[u] = (T)0.125 * (c0v + x2[q2 + ox] + x2[q2 + oy] + x2[q2 + oz] + x2[q2 + ox + oy] + x2[q2 + ox + oz] +
                                 x2[q2 + oy + oz] + x2[q2 + ox + oy + oz]);
        }
    }
#pragma unroll
    for (int u = 0; u < GS_PER; ++u)
        if (on[u]) x[l[u]] = xv[u] + val[u];
}

template <typename T>
__global__ void correct_list_k(T *x, const T *__restrict__ x2, const uint32_t *__restrict__ l0, unsigned c0,
                               const uint32_t *__restrict__ l1, unsigned c1, uint32_t nx, uint32_t nxny,
                               uint32_t nx2, uint32_t nxny2)
{
    correct_list_body<T>(x, x2, l0, c0, l1, c1, nx, nxny, nx2, nxny2, blockIdx.x, gridDim.x);
}

// restriction onto the coarse level's G voxels from its colour lists
// (restrict_k without its zero writes: the coarse f outside G is zeroed at
// set-up and nothing writes anything else there)
template <typename T>
__device__ __forceinline__ void restrict_list_body(T *x2, const T *__restrict__ x, const uint32_t *__restrict__ l0, unsigned c0,
                                const uint32_t *__restrict__ l1, unsigned c1, uint32_t nx2, uint32_t nxny2, Dims d, unsigned blk)
{
    const unsigned t = blk * blockDim.x + threadIdx.x;
    if (t >= c0 + c1) return;
    const uint32_t l2 = (t < c0 ? l0[t] : l1[t - c0]) & BL_IDX;
    const uint32_t k2 = l2 / nxny2, rem = l2 - k2 * nxny2, j2 = rem / nx2, i2 = rem - j2 * nx2;
    const size_t nx = d.nx, nxny = d.nxny();
    const size_t l = (2 * (size_t)i2 - 1) + nx * (2 * (size_t)j2 - 1) + nxny * (2 * (size_t)k2 - 1);
#define X(a, b, c) x[(ptrdiff_t)l + (a) + (b) * (ptrdiff_t)nx + (c) * (ptrdiff_t)nxny]
    const T A = X(-1, -1, -1) + X(1, -1, -1) + X(-1, 1, -1) + X(1, 1, -1) + X(-1, -1, 1) + X(1, -1, 1) + X(-1, 1, 1) + X(1, 1, 1);
    const T B = X(0, -1, -1) + X(-1, 0, -1) + X(1, 0, -1) + X(0, 1, -1) + X(1, -1, 0) + X(-1, -1, 0) + X(-1, 1, 0) +
                X(1, 1, 0) + X(0, -1, 1) + X(-1, 0, 1) + X(1, 0, 1) + X(0, 1, 1);
    const T C = X(0, 0, -1) + X(0, -1, 0) + X(-1, 0, 0) + X(1, 0, 0) + X(0, 1, 0) + X(0, 0, 1);
#undef X
    x2[l2] = (T)0.015625 * A + (T)0.03125 * B + (T)0.0625 * C + (T)0.125 * x[l];
}

template <typename T>
__global__ void restrict_list_k(T *x2, const T *__restrict__ x, const uint32_t *__restrict__ l0, unsigned c0,
                                const uint32_t *__restrict__ l1, unsigned c1, uint32_t nx2, uint32_t nxny2, Dims d)
{
    restrict_list_body<T>(x2, x, l0, c0, l1, c1, nx2, nxny2, d, blockIdx.x);
}

// the V-cycle's restriction of level l's residual onto level l + 1
template <typename T>
static qsm_status level_restrict(qsm_ctx *ctx, Level<T> &C, const Level<T> &L)
{
    if (!C.gl[0]) return restrict_<T>(ctx, C.f, L.r, C.G, C.d, L.d);
    const unsigned n = C.gn[0] + C.gn[1];
    if (n == 0 || C.d.nx < 3 || C.d.ny < 3 || C.d.nz < 3) return QSM_OK;
    restrict_list_k<T><<<(n + 255) / 256, 256, 0, ctx->stream>>>(C.f, L.r, C.gl[0], C.gn[0], C.gl[1], C.gn[1],
                                                                 (uint32_t)C.d.nx, (uint32_t)C.d.nxny(), L.d);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// the V-cycle's correction of level l from level l + 1 (clean: v is +0 outside G)
template <typename T>
static qsm_status level_correct(qsm_ctx *ctx, Level<T> &L, const Level<T> &C, bool clean)
{
    // from lists where they are long (~36 against ~43 us for a 258^3 level's 5.5M G voxels);
    // the grid kernel stays faster on small levels
    const unsigned n = L.gl[0] ? L.gn[0] + L.gn[1] : 0;
    if (sizeof(T) != 4 || !clean || n < (1u << 20) || L.n >= ((size_t)1 << 28) || C.d.nx < 3 || C.d.ny < 3 ||
        C.d.nz < 3)
        return prolong<T>(ctx, L.v, C.v, L.G, L.d, C.d, true, clean);
    correct_list_k<T><<<(n + 256 * GS_PER - 1) / (256 * GS_PER), 256, 0, ctx->stream>>>(
        L.v, C.v, L.gl[0], L.gn[0], L.gl[1], L.gn[1], (uint32_t)L.d.nx, (uint32_t)L.d.nxny(), (uint32_t)C.d.nx,
        (uint32_t)C.d.nxny());
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

template <typename T>
static qsm_status level_residual(qsm_ctx *ctx, Level<T> &L)
{
    if (!L.gl[0]) return residual<T>(ctx, L.r, L.f, L.v, L.G, L.h, L.d);
    const unsigned n = L.gn[0] + L.gn[1];
    if (n == 0 || L.d.nx < 3 || L.d.ny < 3 || L.d.nz < 3) return QSM_OK;
    if (sizeof(T) == 4)
        residual_list_ilp_k<T><<<(n + 256 * GS_PER - 1) / (256 * GS_PER), 256, 0, ctx->stream>>>(
            L.r, L.f, L.v, L.gl[0], L.gn[0], L.gl[1], L.gn[1], lap_consts<T>(L.h), L.d.nx, L.d.nxny());
    else
        residual_list_k<T><<<(n + 255) / 256, 256, 0, ctx->stream>>>(L.r, L.f, L.v, L.gl[0], L.gn[0], L.gl[1],
                                                                     L.gn[1], lap_consts<T>(L.h), L.d.nx, L.d.nxny());
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// `iter` colour-pass pairs over a level's boundary band (gauss_seidel over B):
// long sweeps (8 or more) on levels that fit run on z-slabs in a cluster's
// shared memory (coarse_cluster_k's sweep mode, ~0.7 us per pass instead of
// ~2 us with the level in L2); otherwise by list size.
template <typename T>
static qsm_status boundary_sweeps(qsm_ctx *ctx, const Hier<T> &H, Level<T> &L, int32_t iter, bool rev)
{
    if (!L.bl[0]) return gauss_seidel<T>(ctx, L.v, L.f, L.B, L.h, L.d, iter, rev);
    if (L.d.nx < 3 || L.d.ny < 3 || L.d.nz < 3 || iter <= 0) return QSM_OK;
    if (L.dsm_cn > 0 && iter >= 8) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)L.dsm_cn;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3((unsigned)L.dsm_cn);
        cfg.blockDim = dim3(CC_THREADS);
        cfg.dynamicSmemBytes = L.dsm_smem;
        cfg.stream = ctx->stream;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        QSM_CUDA(cudaLaunchKernelEx(&cfg, coarse_cluster_k<T>, L.v, (const T *)L.f, (const uint8_t *)L.B, L.r, L.d,
                                    gs_consts<T>(L.h), lap_consts<T>(L.h), 0.0, L.dsm_npmax, (int *)nullptr,
                                    (int)iter, rev ? 1 : 0));
        return QSM_OK;
    }
    if (L.bmode == SW_CLUSTER) return sweeps_cluster<T>(ctx, H.sw_ctas, L.v, L.f, L.bl, L.bn, L.h, L.d, iter, rev);
    if (L.bmode == SW_GRID) return sweeps_grid<T>(ctx, H, L.v, L.f, L.bl, L.bn, L.h, L.d, iter, rev);
    return list_sweeps<T>(ctx, L.v, L.f, L.bl, L.bn, L.h, L.d, iter, rev);
}

template <typename T>
static qsm_status hier_free(qsm_ctx *ctx, Hier<T> &H)
{
    if (H.lists) QSM_TRY(dfree(ctx, H.lists));
    H.lists = nullptr;
    return dfree(ctx, H.blk);
}

template <typename T>
static qsm_status hier_masks(qsm_ctx *ctx, Hier<T> &H, bool restrict_f)
{
    for (int i = 0; i < H.nl; ++i) {
        if (i > 0) {
            coarsen_k<<<vox_grid(H.L[i].d), vox_block(), 0, ctx->stream>>>(H.L[i].G, H.L[i - 1].G, H.L[i].d, H.L[i - 1].d);
            QSM_CUDA(cudaGetLastError());
            if (restrict_f) QSM_TRY(restrict_<T>(ctx, H.L[i].f, H.L[i - 1].f, H.L[i].G, H.L[i].d, H.L[i - 1].d));
        }
        QSM_TRY(boundary_mask(ctx, H.L[i].B, H.L[i].G, H.L[i].d, H.scratch));
    }
    return boundary_lists(ctx, H);
}

template <typename T>
static qsm_status coarse_solve(qsm_ctx *ctx, Hier<T> &H, int l, double *scal_dev)
{
    Level<T> &L = H.L[l];
    const double tol = sizeof(T) == 4 ? 1e-4 : 1e-8;
    if (H.cg_ctas > 0) {
        T *vv = L.v, *rr = L.r, *part = (T *)H.gpart;
        const T *ff = L.f;
        const uint32_t *la = L.gl[0], *lb = L.gl[1];
        unsigned ca = L.gn[0], cb = L.gn[1];
        Dims dd = L.d;
        GsC<T> gc = gs_consts<T>(L.h);
        LapC<T> lc = lap_consts<T>(L.h);
        double tl = tol;
        GridBar gb = H.gb;
        int *outer = H.counters;
        void *args[] = {&vv, &ff, &rr, &la, &ca, &lb, &cb, &dd, &gc, &lc, &tl, &gb, &part, &outer};
        QSM_CUDA(cudaMemsetAsync(H.gb.count, 0, sizeof(unsigned), ctx->stream));
        QSM_CUDA(cudaLaunchCooperativeKernel((const void *)coarse_grid_k<T>, dim3((unsigned)H.cg_ctas),
                                             dim3(CG_THREADS), args, 0, ctx->stream));
        return QSM_OK;
    }
    if (H.cc_ctas > 0) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)H.cc_ctas;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3((unsigned)H.cc_ctas);
        cfg.blockDim = dim3(CC_THREADS);
        cfg.dynamicSmemBytes = H.cc_smem;
        cfg.stream = ctx->stream;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        QSM_CUDA(cudaLaunchKernelEx(&cfg, coarse_cluster_k<T>, L.v, (const T *)L.f, (const uint8_t *)L.G, L.r, L.d,
                                    gs_consts<T>(L.h), lap_consts<T>(L.h), tol, H.cc_npmax, H.counters, 0, 0));
        return QSM_OK;
    }
    if (H.coarse_in_smem) {
        coarse_solve_k<T><<<1, CS_THREADS, H.coarse_smem, ctx->stream>>>(L.v, L.f, L.G, L.r, L.d, gs_consts<T>(L.h),
                                                                        lap_consts<T>(L.h), tol, H.counters);
        QSM_CUDA(cudaGetLastError());
        return QSM_OK;
    }
    // large coarsest grid (e.g. nlevels = 1): the same loop driven from the host
    double fn, rn;
    QSM_TRY(nrm2<T>(ctx, L.f, L.n, scal_dev + S_TMP));
    QSM_TRY(read_double(ctx, scal_dev + S_TMP, &fn));
    const double reltol = tol * fn;
    for (int i = 0; i < 1024; ++i) {
        QSM_TRY(gauss_seidel<T>(ctx, L.v, L.f, L.G, L.h, L.d, 128, true));
        QSM_TRY(gauss_seidel<T>(ctx, L.v, L.f, L.G, L.h, L.d, 128, false));
        QSM_TRY(residual<T>(ctx, L.r, L.f, L.v, L.G, L.h, L.d));
        QSM_TRY(nrm2<T>(ctx, L.r, L.n, scal_dev + S_TMP));
        QSM_TRY(read_double(ctx, scal_dev + S_TMP, &rn));
        ++H.host_outer;
        if (rn < reltol) break;
    }
    return QSM_OK;
}

template <typename T>
static qsm_status cycle(qsm_ctx *ctx, Hier<T> &H, int l, int mu, int pre, int post, int nb, double *sc)
{
    if (l < H.nl - 1) {
        Level<T> &L = H.L[l], &C = H.L[l + 1];
        const int32_t bs = (1 << l) * nb;
        QSM_TRY(smooth<T>(ctx, H, L, pre, true));
        QSM_TRY(boundary_sweeps<T>(ctx, H, L, bs, true));
        QSM_TRY(level_residual<T>(ctx, L));
        QSM_TRY(level_restrict<T>(ctx, C, L));
        QSM_CUDA(cudaMemsetAsync(C.v, 0, C.n * sizeof(T), ctx->stream));
        for (int i = 0; i < mu; ++i) {
            QSM_TRY(cycle<T>(ctx, H, l + 1, mu, pre, post, nb, sc));
            if (l + 1 == H.nl - 1) break;
        }
        // every level below the top is zeroed before its cycle; the PCG's top level too
        QSM_TRY(level_correct<T>(ctx, L, C, l > 0 || H.v0_zero_outside));
        QSM_TRY(boundary_sweeps<T>(ctx, H, L, bs, false));
        QSM_TRY(smooth<T>(ctx, H, L, post, false));
        return QSM_OK;
    }
    return coarse_solve<T>(ctx, H, l, sc);
}

// mx_mg: tol > 0 checks ||r|| < tol ||f|| before each cycle.
template <typename T>
static qsm_status mg_run(qsm_ctx *ctx, Hier<T> &H, double tol, int maxit, int mu, int pre, int post, int nb, double *sc,
                         int *cycles)
{
    int cyc = 0;
    if (tol > 0.0) {
        double fn, rn;
        QSM_TRY(nrm2<T>(ctx, H.L[0].f, H.L[0].n, sc + S_TMP));
        QSM_TRY(read_double(ctx, sc + S_TMP, &fn));
        const double reltol = tol * fn;
        for (int i = 0; i < maxit; ++i) {
            QSM_TRY(residual<T>(ctx, H.L[0].r, H.L[0].f, H.L[0].v, H.L[0].G, H.L[0].h, H.L[0].d));
            QSM_TRY(nrm2<T>(ctx, H.L[0].r, H.L[0].n, sc + S_TMP));
            QSM_TRY(read_double(ctx, sc + S_TMP, &rn));
            if (rn < reltol) break;
            QSM_TRY(cycle<T>(ctx, H, 0, mu, pre, post, nb, sc));
            ++cyc;
        }
    } else {
        for (int i = 0; i < maxit; ++i, ++cyc) QSM_TRY(cycle<T>(ctx, H, 0, mu, pre, post, nb, sc));
    }
    if (cycles) *cycles = cyc;
    return QSM_OK;
}

template <typename T>
static qsm_status pad(qsm_ctx *ctx, T *xp, const T *x, const Dims &d)
{
    pad_k<T><<<vox_grid(d), vox_block(), 0, ctx->stream>>>(xp, x, d);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

template <typename T>
static qsm_status unpad(qsm_ctx *ctx, T *x, const T *xp, const Dims &d)
{
    unpad_k<T><<<vox_grid(d), vox_block(), 0, ctx->stream>>>(x, xp, d);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

static qsm_status pad_mask(qsm_ctx *ctx, uint8_t *Gp, const uint8_t *G, const Dims &d)
{
    mask01_pad_k<<<vox_grid(d), vox_block(), 0, ctx->stream>>>(Gp, G, d);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// ---------------------------------------------------------------------------
// fused PCG vector steps (mgpcg_mex.c:160-205).  Each kernel runs on the
// lane_dot grid (RED_NBLK blocks of RED_BLOCK threads; thread t is lane t and
// visits elements t, t + 2^18, ... in increasing order), so the inner product
// it forms while it updates the vectors has lane_dot's order; the last block
// to finish folds the block partials and updates the PCG scalars, as the
// single-thread scalar kernels did.  Element updates keep the BLAS-1
// expressions: scal is a * x, axpy is y + a * x; multiplying by 1.0 is exact
// and multiplying by -1.0 is a sign flip, so those two are done without the
// FP64 pipe.
// ---------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ T neg_bits(T x)
{
    if (sizeof(T) == 8) return (T)__longlong_as_double(__double_as_longlong((double)x) ^ (long long)0x8000000000000000ull);
    return (T)__int_as_float(__float_as_int((float)x) ^ (int)0x80000000u);
}

// true in the last block to finish (all its threads), with the lane-order total
template <typename T>
__device__ __forceinline__ bool lane_fold(T *sm, T acc, T *part, unsigned *count, T *tot, unsigned blk)
{
    __shared__ bool last;
    const int tid = threadIdx.x;
    const T b = halve_block(sm, tid, acc);
    if (tid == 0) {
        part[blk] = b;
        __threadfence();
        last = atomicAdd(count, 1u) == RED_NBLK - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    *tot = halve_partials(sm, tid, part);
    return true;
}

// The mixed solver's PCG (an FP64 recurrence around an FP32 V-cycle, FM)
// contracts its multiply-adds into FP64 FMAs and converts between the two
// precisions in integer arithmetic: on this GPU the FP64 pipe bounds these
// steps, and that takes a third of their FP64 instructions off it.  The FP64
// and FP32 solvers keep the reference's separate products and sums.
template <bool FM, typename T>
__device__ __forceinline__ T pmad(T x, T y, T z)
{
    if constexpr (FM)
        return fma(x, y, z);
    else
        return x * y + z;
}
template <typename TP, typename TM>
__device__ __forceinline__ TP widen(TM v)
{
    if constexpr (sizeof(TP) == 8 && sizeof(TM) == 4)
        return f32_to_f64(v);
    else
        return (TP)v;
}
template <typename TM, typename TP>
__device__ __forceinline__ TM narrow(TP v)
{
    if constexpr (sizeof(TP) == 8 && sizeof(TM) == 4)
        return f64_to_f32(v);
    else
        return (TM)v;
}

// Voxels outside G in the PCG steps (sk: the level-0 mask, when the solve
// runs its masked form).  That form runs when the initial residual and
// iterate are exactly +0 outside G (pcg_zero_outside_k checks it per solve,
// after r = f - A x0); then r, p and x stay +0 there and q holds +-0, every
// update there leaves the value it had, and every product added to an
// inner product there is +-0.  A
// running sum that starts at +0 is never -0 in round-to-nearest, so adding
// +-0 to it changes nothing: skipping those voxels gives the same bits.
__device__ __forceinline__ bool pcg_on(const uint8_t *__restrict__ sk, size_t l) { return !sk || sk[l]; }

// Segments of the lane grid for the masked PCG steps.  Warp w of the lane
// grid (lanes 32 w .. 32 w + 31) visits the elements l = 32 w + lane +
// k RED_LANES, k = 0, 1, ...; segment (w, k) is those 32 elements.
// k[j * SEG_NW + w], j < cnt[w], lists in increasing k the segments that
// hold a voxel of G, and the masked steps visit only those: a warp whose 32
// elements all lie outside G then issues no FP64 instruction at all, where
// a per-element test leaves FP64 instructions with every lane predicated
// off, and those still take their slot in the FP64 pipe.  Each lane still
// visits its own elements of G in increasing k, so inner products keep
// the lane order and their bits.
constexpr uint32_t SEG_NW = (uint32_t)(RED_LANES / 32);

struct Segs {
    const uint32_t *k;    // nullptr: every element is visited
    const uint32_t *cnt;
};

static size_t seg_entries(size_t n) { return (n + RED_LANES - 1) / RED_LANES * SEG_NW; }

__global__ void __launch_bounds__(RED_BLOCK) pcg_segs_k(const uint8_t *__restrict__ sk, size_t n, uint32_t *segk,
                                                        uint32_t *segcnt)
{
    const size_t t = (size_t)blockIdx.x * RED_BLOCK + threadIdx.x;
    const uint32_t w = (uint32_t)(t >> 5);
    const bool lead = (threadIdx.x & 31) == 0;
    uint32_t c = 0;
    // k * RED_LANES < n is the same for the whole warp: every lane votes
    for (size_t k = 0, l = t; k * RED_LANES < n; ++k, l += RED_LANES) {
        const bool on = l < n && sk[l];
        if (__ballot_sync(0xffffffffu, on)) {
            if (lead) segk[(size_t)c * SEG_NW + w] = (uint32_t)k;
            ++c;
        }
    }
    if (lead) segcnt[w] = c;
}

// element indices of this warp's listed segments j .. j + 3 (n past the list
// end; the last segment may reach past n as well)
__device__ __forceinline__ void seg_group(const Segs &sg, size_t t, uint32_t w, uint32_t j, uint32_t c, size_t n,
                                          size_t *l)
{
#pragma unroll
    for (int u = 0; u < 4; ++u)
        l[u] = j + u < c ? t + (size_t)sg.k[(size_t)(j + u) * SEG_NW + w] * RED_LANES : n;
}

// flag = 1 if some voxel outside G holds a value other than +0 in a or b
template <typename T>
__global__ void pcg_zero_outside_k(const T *__restrict__ a, const T *__restrict__ b, const uint8_t *__restrict__ G,
                                   size_t n, int *flag)
{
    int bad = 0;
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
        if (G[l]) continue;
        if (sizeof(T) == 8) {
            bad |= __double_as_longlong((double)a[l]) != 0 || (b && __double_as_longlong((double)b[l]) != 0);
        } else {
            bad |= __float_as_int((float)a[l]) != 0 || (b && __float_as_int((float)b[l]) != 0);
        }
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(flag, 1);
}

// rho = r . q (q widened from the V-cycle's vm first when it runs in another
// precision); prevrho = old rho; beta = rho / prevrho
template <typename TP, typename TM>
__device__ __forceinline__ void pcg_rho_body(const TP *__restrict__ r, TP *__restrict__ q,
                                                       const TM *__restrict__ vm, const uint8_t *__restrict__ sk,
                                                       Segs sg, size_t n, TP *part, unsigned *count, double *sc, unsigned blk)
{
    constexpr bool FM = sizeof(TP) != sizeof(TM);
    __shared__ TP sm[RED_BLOCK];
    const size_t L = RED_LANES;
    size_t l = (size_t)blk * RED_BLOCK + threadIdx.x;
    TP acc = (TP)0;
    if (sg.k) {
        const uint32_t w = (uint32_t)(l >> 5), c = sg.cnt[w];
        for (uint32_t j = 0; j < c; j += 4) {
            size_t e[4];
            seg_group(sg, l, w, j, c, n, e);
            TP a[4] = {}, b[4] = {};
            bool on[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                on[u] = e[u] < n && sk[e[u]];
                if (e[u] < n) {
                    a[u] = r[e[u]];
                    b[u] = vm ? widen<TP, TM>(vm[e[u]]) : q[e[u]];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (!on[u]) continue;
                if (vm) q[e[u]] = b[u];
                acc = pmad<FM>(a[u], b[u], acc);
            }
        }
        l = n;
    }
    for (; l + 3 * L < n; l += 4 * L) {
        TP a[4], b[4];
        bool on[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            on[u] = pcg_on(sk, l + u * L);
            if (on[u]) {
                a[u] = r[l + u * L];
                b[u] = vm ? widen<TP, TM>(vm[l + u * L]) : q[l + u * L];
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (!on[u]) continue;
            if (vm) q[l + u * L] = b[u];
            acc = pmad<FM>(a[u], b[u], acc);
        }
    }
    for (; l < n; l += L) {
        if (!pcg_on(sk, l)) continue;
        const TP b = vm ? widen<TP, TM>(vm[l]) : q[l];
        if (vm) q[l] = b;
        acc = pmad<FM>(r[l], b, acc);
    }
    TP tot;
    if (lane_fold(sm, acc, part, count, &tot, blk) && threadIdx.x == 0) {
        sc[S_PREV] = sc[S_RHO];
        sc[S_RHO] = (double)tot;
        sc[S_BETA] = sc[S_RHO] / sc[S_PREV];
        *count = 0;
    }
}

template <typename TP, typename TM>
__global__ void __launch_bounds__(RED_BLOCK) pcg_rho_k(const TP *__restrict__ r, TP *__restrict__ q,
                                                       const TM *__restrict__ vm, const uint8_t *__restrict__ sk,
                                                       Segs sg, size_t n, TP *part, unsigned *count, double *sc)
{
    pcg_rho_body<TP, TM>(r, q, vm, sk, sg, n, part, count, sc, blockIdx.x);
}

// p = beta * p, then p = p + 1 * q (with segments: on the lane grid)
template <typename T, bool FM>
__device__ __forceinline__ void pcg_p_body(T *__restrict__ p, const T *__restrict__ q, const uint8_t *__restrict__ sk, Segs sg,
                        size_t n, const double *sc, unsigned blk, unsigned nblk)
{
    const T beta = (T)sc[S_BETA];
    if (sg.k) {
        const size_t t = (size_t)blk * blockDim.x + threadIdx.x;
        const uint32_t w = (uint32_t)(t >> 5), c = sg.cnt[w];
        for (uint32_t j = 0; j < c; j += 4) {
            size_t e[4];
            seg_group(sg, t, w, j, c, n, e);
            T pv[4] = {}, qv[4] = {};
            bool on[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                on[u] = e[u] < n && sk[e[u]];
                if (e[u] < n) {
                    pv[u] = p[e[u]];
                    qv[u] = q[e[u]];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (on[u]) p[e[u]] = pmad<FM>(beta, pv[u], qv[u]);
        }
        return;
    }
    for (size_t l = (size_t)blk * blockDim.x + threadIdx.x; l < n; l += (size_t)nblk * blockDim.x)
        if (pcg_on(sk, l)) p[l] = pmad<FM>(beta, p[l], q[l]);
}

template <typename T, bool FM>
__global__ void pcg_p_k(T *__restrict__ p, const T *__restrict__ q, const uint8_t *__restrict__ sk, Segs sg,
                        size_t n, const double *sc)
{
    pcg_p_body<T, FM>(p, q, sk, sg, n, sc, blockIdx.x, gridDim.x);
}

// q = lapmg(p) on G (interior), then q = -1 * q everywhere; pq = p . q;
// alpha = rho / pq
template <typename T, bool FM>
__device__ __forceinline__ T pcg_lap(const T *__restrict__ p, size_t l, size_t nx, size_t nxny, const LapC<T> &c, T pl)
{
    const T sx = p[l - 1] + p[l + 1], sy = p[l - nx] + p[l + nx], sz = p[l - nxny] + p[l + nxny];
    if constexpr (FM)
        return pmad<true>(c.hz, sz, pmad<true>(c.hy, sy, pmad<true>(c.hx, sx, c.hh * pl)));
    else
        return c.hh * pl + c.hx * sx + c.hy * sy + c.hz * sz;
}

template <typename T, bool FM>
__device__ __forceinline__ void pcg_q_body(T *__restrict__ q, const T *__restrict__ p,
                                                     const uint8_t *__restrict__ G, const uint8_t *__restrict__ sk,
                                                     Segs sg, LapC<T> c, Dims d, T *part, unsigned *count, double *sc, unsigned blk)
{
    __shared__ T sm[RED_BLOCK];
    const size_t nx = d.nx, ny = d.ny, nxny = d.nxny(), n = d.n();
    const size_t t = (size_t)blk * RED_BLOCK + threadIdx.x;
    T acc = (T)0;
    if (sg.k) {
        // sk is G here, whose one-voxel frame is 0: a voxel of G is interior and takes the stencil
        const uint32_t w = (uint32_t)(t >> 5), cn = sg.cnt[w];
        for (uint32_t jj = 0; jj < cn; jj += 4) {
            size_t e[4];
            seg_group(sg, t, w, jj, cn, n, e);
            bool on[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) on[u] = e[u] < n && sk[e[u]];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (!on[u]) continue;
                const size_t l = e[u];
                const T pl = p[l];
                const T qv = neg_bits(pcg_lap<T, FM>(p, l, nx, nxny, c, pl));
                q[l] = qv;
                acc = pmad<FM>(pl, qv, acc);
            }
        }
        T tot;
        if (lane_fold(sm, acc, part, count, &tot, blk) && threadIdx.x == 0) {
            sc[S_PQ] = (double)tot;
            sc[S_A] = sc[S_RHO] / sc[S_PQ];
            *count = 0;
        }
        return;
    }
    // (i, j, k) of l, then advanced by the lane stride in mixed radix (no division per element)
    size_t k = t / nxny, j = (t - k * nxny) / nx, i = t - k * nxny - j * nx;
    const size_t Lk = RED_LANES / nxny, Lj = (RED_LANES - Lk * nxny) / nx, Li = RED_LANES - Lk * nxny - Lj * nx;
    for (size_t l = t; l < n; l += RED_LANES) {
        if (pcg_on(sk, l)) {
            const T pl = p[l];
            T qv;
            if (i >= 1 && j >= 1 && k >= 1 && i + 1 < nx && j + 1 < d.ny && k + 1 < d.nz && G[l])
                qv = pcg_lap<T, FM>(p, l, nx, nxny, c, pl);
            else
                qv = q[l];
            qv = neg_bits(qv);
            q[l] = qv;
            acc = pmad<FM>(pl, qv, acc);
        }
        i += Li;
        const size_t cj = i >= nx;
        i -= cj * nx;
        j += Lj + cj;
        const size_t ck = j >= ny;
        j -= ck * ny;
        k += Lk + ck;
    }
    T tot;
    if (lane_fold(sm, acc, part, count, &tot, blk) && threadIdx.x == 0) {
        sc[S_PQ] = (double)tot;
        sc[S_A] = sc[S_RHO] / sc[S_PQ];
        *count = 0;
    }
}

template <typename T, bool FM>
__global__ void __launch_bounds__(RED_BLOCK) pcg_q_k(T *__restrict__ q, const T *__restrict__ p,
                                                     const uint8_t *__restrict__ G, const uint8_t *__restrict__ sk,
                                                     Segs sg, LapC<T> c, Dims d, T *part, unsigned *count, double *sc)
{
    pcg_q_body<T, FM>(q, p, G, sk, sg, c, d, part, count, sc, blockIdx.x);
}

// x = x + alpha * p; r = r + (-alpha) * q; ||r|| (and r in the V-cycle's
// precision for the next cycle when that differs)
template <typename TP, typename TM>
__device__ __forceinline__ void pcg_xr_body(TP *__restrict__ x, const TP *__restrict__ p,
                                                      TP *__restrict__ r, const TP *__restrict__ q,
                                                      TM *__restrict__ rm, const uint8_t *__restrict__ sk, Segs sg,
                                                      size_t n, TP *part, unsigned *count, double *sc, unsigned blk)
{
    constexpr bool FM = sizeof(TP) != sizeof(TM);
    __shared__ TP sm[RED_BLOCK];
    const TP a = (TP)sc[S_A], na = (TP)(-sc[S_A]);
    const size_t L = RED_LANES;
    size_t l = (size_t)blk * RED_BLOCK + threadIdx.x;
    TP acc = (TP)0;
    if (sg.k) {
        const uint32_t w = (uint32_t)(l >> 5), c = sg.cnt[w];
        for (uint32_t j = 0; j < c; j += 4) {
            size_t e[4];
            seg_group(sg, l, w, j, c, n, e);
            TP xv[4] = {}, pv[4] = {}, rv[4] = {}, qv[4] = {};
            bool on[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                on[u] = e[u] < n && sk[e[u]];
                if (e[u] < n) {
                    xv[u] = x[e[u]];
                    pv[u] = p[e[u]];
                    rv[u] = r[e[u]];
                    qv[u] = q[e[u]];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (!on[u]) continue;
                x[e[u]] = pmad<FM>(a, pv[u], xv[u]);
                const TP rn = pmad<FM>(na, qv[u], rv[u]);
                r[e[u]] = rn;
                if (rm) rm[e[u]] = narrow<TM, TP>(rn);
                acc = pmad<FM>(rn, rn, acc);
            }
        }
        l = n;
    }
    for (; l + 3 * L < n; l += 4 * L) {
        TP xv[4], pv[4], rv[4], qv[4];
        bool on[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            on[u] = pcg_on(sk, l + u * L);
            if (on[u]) {
                xv[u] = x[l + u * L];
                pv[u] = p[l + u * L];
                rv[u] = r[l + u * L];
                qv[u] = q[l + u * L];
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (!on[u]) continue;
            x[l + u * L] = pmad<FM>(a, pv[u], xv[u]);
            const TP rn = pmad<FM>(na, qv[u], rv[u]);
            r[l + u * L] = rn;
            if (rm) rm[l + u * L] = narrow<TM, TP>(rn);
            acc = pmad<FM>(rn, rn, acc);
        }
    }
    for (; l < n; l += L) {
        if (!pcg_on(sk, l)) continue;
        x[l] = pmad<FM>(a, p[l], x[l]);
        const TP rn = pmad<FM>(na, q[l], r[l]);
        r[l] = rn;
        if (rm) rm[l] = narrow<TM, TP>(rn);
        acc = pmad<FM>(rn, rn, acc);
    }
    TP tot;
    if (lane_fold(sm, acc, part, count, &tot, blk) && threadIdx.x == 0) {
        sc[S_RES] = sizeof(TP) == 4 ? (double)sqrtf((float)tot) : sqrt((double)tot);
        *count = 0;
    }
}

template <typename TP, typename TM>
__global__ void __launch_bounds__(RED_BLOCK) pcg_xr_k(TP *__restrict__ x, const TP *__restrict__ p,
                                                      TP *__restrict__ r, const TP *__restrict__ q,
                                                      TM *__restrict__ rm, const uint8_t *__restrict__ sk, Segs sg,
                                                      size_t n, TP *part, unsigned *count, double *sc)
{
    pcg_xr_body<TP, TM>(x, p, r, q, rm, sk, sg, n, part, count, sc, blockIdx.x);
}

// Which coarsest-level solver ran and its outer iterations (after the stream
// has been synchronised).
// (Also fails the solve if a whole-GPU coarsest solve's barrier ran out.)
template <typename T>
static qsm_status coarse_report(qsm_ctx *ctx, const Hier<T> &H, qsm_mg_info *info)
{
    if (H.cg_ctas > 0 || H.sg_ctas > 0) {
        int err = 0;
        QSM_CUDA(cudaMemcpy(&err, H.gb.err, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) {
            set_error(ctx, "multigrid: a grid barrier timed out");
            return QSM_ERR_TIMEOUT;
        }
    }
    if (!info) return QSM_OK;
    int dev_outer = 0;
    QSM_CUDA(cudaMemcpy(&dev_outer, H.counters, sizeof(int), cudaMemcpyDeviceToHost));
    info->coarse_ctas = H.cg_ctas > 0 ? -H.cg_ctas : H.cc_ctas > 0 ? H.cc_ctas : (H.coarse_in_smem ? 1 : 0);
    info->coarse_outer = dev_outer + H.host_outer;
    return QSM_OK;
}

// PCG (mx_pcg, mgpcg_mex.c:126-216).  TP = PCG precision, TM = V-cycle
// precision.  With TP == TM the V-cycle's level-0 v/f are the PCG q/r (as in
// the reference); with TM = float they are FP32 copies converted per call.
// A solve's state between iterations: pcg_setup runs everything before the
// loop, pcg_launch_iter enqueues one iteration (no host read), pcg_read_res
// reads its residual norm, pcg_finish writes the solution and frees the
// state.  pcg runs them in order; packed solves (pcg_pack_iter) advance
// several states per launch.
template <typename TP, typename TM>
struct PcgState {
    Dims d{}, dp{};
    size_t n = 0;
    Hier<TM> H;
    void *pv = nullptr;
    TP *x = nullptr, *p = nullptr, *r = nullptr, *q = nullptr;
    double *sc = nullptr;
    TP *part = nullptr;         // RED_NBLK lane-order block sums of the fused steps
    unsigned *count = nullptr;  // their last-block counter
    const uint8_t *sk = nullptr;
    Segs sg{nullptr, nullptr};
    LapC<TP> lc{};
    double res = 0.0, reltol = 0.0;
    int32_t it = 0, maxitcg = 0;
    double tolmg = 0.0;
    int32_t maxitmg = 0, mu = 1, npre = 1, npost = 1, nb = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool done() const { return it >= maxitcg || res <= reltol; }
};

template <typename TP, typename TM>
static qsm_status pcg_setup(qsm_ctx *ctx, PcgState<TP, TM> &S, const Dims &d, const TP *v0, const TP *f,
                            const uint8_t *mask, const double *h, double tolcg, int32_t maxitcg, double tolmg,
                            int32_t maxitmg, int32_t mu, int32_t npre, int32_t npost, int32_t nb, int32_t nl)
{
    constexpr bool same = sizeof(TP) == sizeof(TM);
    S.d = d;
    S.dp = Dims{d.nx + 2, d.ny + 2, d.nz + 2};
    const size_t n = S.n = S.dp.n();
    S.maxitcg = maxitcg;
    S.tolmg = tolmg;
    S.maxitmg = maxitmg;
    S.mu = mu;
    S.npre = npre;
    S.npost = npost;
    S.nb = nb;
    Hier<TM> &H = S.H;
    QSM_TRY(hier_init<TM>(ctx, H, nl, S.dp, h));
    H.v0_zero_outside = true;  // the preconditioner starts from v = 0 every time
    // PCG vectors: x, p (and r, q when the V-cycle runs in another precision), scalars,
    // the fused steps' block sums and counter, and the lane-grid segment lists of the
    // masked steps (built below when that form runs)
    const size_t vb = al256(n * sizeof(TP)), scb = al256(S_N * sizeof(double) + 256);
    const size_t pb = al256(RED_NBLK * sizeof(TP)) + 256;
    const size_t zb = (same ? 2 : 4) * vb + scb + pb;
    QSM_TRY(dalloc(ctx, &S.pv, zb + al256(seg_entries(n) * sizeof(uint32_t)) + SEG_NW * sizeof(uint32_t)));
    QSM_CUDA(cudaMemsetAsync(S.pv, 0, zb, ctx->stream));
    char *pv = (char *)S.pv;
    TP *x = S.x = (TP *)pv;
    S.p = (TP *)(pv + vb);
    TP *r = S.r = same ? (TP *)H.L[0].f : (TP *)(pv + 2 * vb);
    TP *q = S.q = same ? (TP *)H.L[0].v : (TP *)(pv + 3 * vb);
    double *sc = S.sc = (double *)(pv + (same ? 2 : 4) * vb);
    S.part = (TP *)(pv + (same ? 2 : 4) * vb + scb);
    S.count = (unsigned *)(pv + (same ? 2 : 4) * vb + scb + al256(RED_NBLK * sizeof(TP)));

    QSM_TRY(pad_mask(ctx, H.L[0].G, mask, d));
    QSM_TRY(hier_masks<TM>(ctx, H, false));
    if (v0) QSM_TRY(pad<TP>(ctx, x, v0, d));
    QSM_TRY(pad<TP>(ctx, r, f, d));

    QSM_CUDA(cudaEventCreate(&S.e0));
    QSM_CUDA(cudaEventCreate(&S.e1));
    QSM_CUDA(cudaEventRecord(S.e0, ctx->stream));
    QSM_CUDA(cudaMemsetAsync(sc, 0, S_N * sizeof(double), ctx->stream));
    // rho = 1 initially (mgpcg_mex.c:135-138)
    const double one = 1.0;
    QSM_CUDA(cudaMemcpyAsync(sc + S_RHO, &one, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    QSM_TRY(nrm2<TP>(ctx, r, n, sc + S_RES));
    QSM_TRY(read_double(ctx, sc + S_RES, &S.res));
    S.reltol = tolcg * S.res;
    QSM_CUDA(cudaMemsetAsync(q, 0, n * sizeof(TP), ctx->stream));
    QSM_TRY(lapmg<TP>(ctx, q, x, H.L[0].G, h, S.dp));
    QSM_TRY(scal<TP>(ctx, q, n, sc, -1, false, -1.0));
    QSM_TRY(axpy<TP>(ctx, r, q, n, sc, -1, false, -1.0));
    // The PCG steps skip the voxels outside G when the residual and the iterate are +0
    // there (f +-0 outside G becomes +0 in r = f - A x0, as -0 + +0 is +0).
    int *zflag = (int *)(pv + (same ? 2 : 4) * vb + S_N * sizeof(double));
    pcg_zero_outside_k<TP><<<1216, 256, 0, ctx->stream>>>(r, x, H.L[0].G, n, zflag);
    QSM_CUDA(cudaGetLastError());
    QSM_TRY(nrm2<TP>(ctx, r, n, sc + S_RES));
    QSM_TRY(read_double(ctx, sc + S_RES, &S.res));
    int hz = 1;
    QSM_CUDA(cudaMemcpyAsync(&hz, zflag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    S.sk = hz ? nullptr : H.L[0].G;
    if (S.sk) {
        uint32_t *segk = (uint32_t *)(pv + zb);
        uint32_t *segcnt = (uint32_t *)((char *)segk + al256(seg_entries(n) * sizeof(uint32_t)));
        pcg_segs_k<<<RED_NBLK, RED_BLOCK, 0, ctx->stream>>>(S.sk, n, segk, segcnt);
        QSM_CUDA(cudaGetLastError());
        S.sg = Segs{segk, segcnt};
    }
    S.lc = lap_consts<TP>(h);
    // the V-cycle's right-hand side in its own precision; pcg_xr_k refreshes it
    if (!same) cvt_k<TM, TP><<<1216, 256, 0, ctx->stream>>>(H.L[0].f, r, n);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

template <typename TP, typename TM>
static qsm_status pcg_launch_iter(qsm_ctx *ctx, PcgState<TP, TM> &S)
{
    constexpr bool same = sizeof(TP) == sizeof(TM);
    Hier<TM> &H = S.H;
    const size_t n = S.n;
    if (same)
        QSM_CUDA(cudaMemsetAsync(S.q, 0, n * sizeof(TP), ctx->stream));
    else
        QSM_CUDA(cudaMemsetAsync(H.L[0].v, 0, n * sizeof(TM), ctx->stream));
    {
        Range cyc("mgpcg/preconditioner");
        QSM_TRY(mg_run<TM>(ctx, H, S.tolmg, S.maxitmg, S.mu, S.npre, S.npost, S.nb, S.sc, nullptr));
    }
    pcg_rho_k<TP, TM><<<RED_NBLK, RED_BLOCK, 0, ctx->stream>>>(S.r, S.q, same ? nullptr : H.L[0].v, S.sk, S.sg, n,
                                                               S.part, S.count, S.sc);
    // with segments pcg_p_k runs on the lane grid
    pcg_p_k<TP, !same><<<S.sg.k ? RED_NBLK : 1216, RED_BLOCK, 0, ctx->stream>>>(S.p, S.q, S.sk, S.sg, n, S.sc);
    pcg_q_k<TP, !same><<<RED_NBLK, RED_BLOCK, 0, ctx->stream>>>(S.q, S.p, H.L[0].G, S.sk, S.sg, S.lc, S.dp, S.part,
                                                                S.count, S.sc);
    pcg_xr_k<TP, TM><<<RED_NBLK, RED_BLOCK, 0, ctx->stream>>>(S.x, S.p, S.r, S.q, same ? nullptr : H.L[0].f, S.sk,
                                                              S.sg, n, S.part, S.count, S.sc);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

template <typename TP, typename TM>
static qsm_status pcg_read_res(qsm_ctx *ctx, PcgState<TP, TM> &S)
{
    QSM_TRY(read_double(ctx, S.sc + S_RES, &S.res));
    S.it += 1;
    return QSM_OK;
}

// Writes the solution (vout: unpadded, device) and the statistics and frees the state.
template <typename TP, typename TM>
static qsm_status pcg_finish(qsm_ctx *ctx, PcgState<TP, TM> &S, TP *vout, qsm_mg_info *info)
{
    if (S.e1) QSM_CUDA(cudaEventRecord(S.e1, ctx->stream));
    if (vout) QSM_TRY(unpad<TP>(ctx, vout, S.x, S.d));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    if (S.e0 && S.e1) cudaEventElapsedTime(&ms, S.e0, S.e1);
    if (S.e0) cudaEventDestroy(S.e0);
    if (S.e1) cudaEventDestroy(S.e1);
    S.e0 = S.e1 = nullptr;
    if (info) {
        info->iters = S.it;
        info->resnorm = S.res;
        info->seconds = ms * 1e-3;
    }
    const qsm_status rep = coarse_report(ctx, S.H, info);  // a timed-out solve still frees its state
    if (S.pv) QSM_TRY(dfree(ctx, S.pv));
    S.pv = nullptr;
    QSM_TRY(hier_free(ctx, S.H));
    return rep;
}

template <typename TP, typename TM>
static qsm_status pcg(qsm_ctx *ctx, const Dims &d, const TP *v0, const TP *f, const uint8_t *mask, const double *h,
                      double tolcg, int32_t maxitcg, double tolmg, int32_t maxitmg, int32_t mu, int32_t npre,
                      int32_t npost, int32_t nb, int32_t nl, int32_t verbose, TP *vout, qsm_mg_info *info)
{
    Range nvtx_range("mgpcg");
    PcgState<TP, TM> S;
    QSM_TRY(pcg_setup(ctx, S, d, v0, f, mask, h, tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nb, nl));
    if (verbose) printf("\niter%6s\tresidual\n", "");
    while (!S.done()) {
        QSM_TRY(pcg_launch_iter(ctx, S));
        QSM_TRY(pcg_read_res(ctx, S));
        if (info && info->resnorm_hist) info->resnorm_hist[S.it - 1] = S.res;
        if (verbose) printf("%5d/%d\t%1.3e\n", S.it - 1, maxitcg, S.res);
    }
    if (verbose) printf("\n");
    return pcg_finish(ctx, S, vout, info);
}

// ---------------------------------------------------------------------------
// Packed PCG solves (qsm_mgpcg_batch and session steps): up to MV_MAX solves
// with the same multigrid options advance together, one PCG iteration at a
// time, each kernel of the iteration launched once for all of them.  A
// packed launch's descriptor set (one kernel parameter) gives each solve its
// arrays, lists and block range; the bodies are those of the one-solve
// kernels, so every solve's result is its solve alone bit for bit:
// colour passes, residuals, restrictions and corrections from the levels'
// voxel lists (any order within a pass or a level gives the same bits),
// the coarsest level on one CTA per solve (the one-CTA solver, whose
// results the cluster and whole-GPU solvers reproduce), and the four PCG
// steps on one lane grid per solve with its own block sums.
// ---------------------------------------------------------------------------
constexpr int MV_MAX = 16;

template <typename T>
struct MvGs {  // one solve's share of a packed colour pass
    T *v;
    const T *f;
    const uint32_t *list;
    unsigned cnt, blk0, nblk;
    uint32_t skip;
    GsC<T> c;
    size_t nx, nxny;
};
template <typename T>
struct MvGsSet {
    MvGs<T> m[MV_MAX];
    int n;
};

template <typename T>
struct MvLev {  // one solve's level l (residual, restriction onto l + 1, correction from l + 1)
    T *v, *f, *r, *v2, *f2;
    const uint32_t *l0, *l1, *c0l, *c1l;  // level l's and level l+1's G lists
    unsigned n0, n1, m0, m1, blk0, nblk;
    LapC<T> c;
    uint32_t nx, nxny, nx2, nxny2;
    Dims d;
};
template <typename T>
struct MvLevSet {
    MvLev<T> m[MV_MAX];
    int n;
};

template <typename T>
struct MvCs {  // one solve's coarsest level (CTA blockIdx.x)
    T *v, *r;
    const T *f;
    const uint8_t *G;
    Dims d;
    GsC<T> gc;
    LapC<T> lc;
    double tol;
    int *outer;
};
template <typename T>
struct MvCsSet {
    MvCs<T> m[MV_MAX];
    int n;
};

template <typename TP, typename TM>
struct MvPcg {  // one solve's PCG vectors and scratch (blocks k RED_NBLK .. (k + 1) RED_NBLK - 1)
    TP *x, *p, *r, *q, *part;
    TM *vm, *rm;  // the V-cycle's level-0 v and f in its precision (null when they are q and r)
    const uint8_t *sk, *G;
    Segs sg;
    unsigned *count;
    double *sc;
    size_t n;
    LapC<TP> lc;
    Dims dp;
};
template <typename TP, typename TM>
struct MvPcgSet {
    MvPcg<TP, TM> m[MV_MAX];
    int n;
};

template <typename T>
struct MvSw {  // one solve's smoothing call on a thread-block cluster of its own
    T *v;
    const T *f;
    const uint32_t *la, *lb;
    unsigned ca, cb;
    uint32_t skipb;
    GsC<T> c;
    size_t nx, nxny;
};
template <typename T>
struct MvSwSet {
    MvSw<T> m[MV_MAX];
    int n;
};

__device__ __forceinline__ uint32_t cl_id()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}

// iter sweeps (pass over la, pass over lb skipping skipb) of solve `cluster id`
// on its cluster: sweeps_cluster_k's body, each cluster on its own solve
// (clusters never wait for one another)
template <typename T>
__global__ void __launch_bounds__(SW_THREADS) sweeps_pack_k(const __grid_constant__ MvSwSet<T> P, int32_t iter)
{
    const MvSw<T> &m = P.m[cl_id()];
    const unsigned stride = cl_size() * SW_THREADS, t0 = cl_rank() * SW_THREADS + threadIdx.x;
    SwShare<T> a, b;
    a.load(m.la, m.ca, m.f, t0, stride);
    b.load(m.lb, m.cb, m.f, t0, stride);
    for (int32_t s = 0; s < iter; ++s) {
        a.pass(m.v, 0u, m.c, m.nx, m.nxny);
        cl_sync();
        b.pass(m.v, m.skipb, m.c, m.nx, m.nxny);
        cl_sync();
    }
}

// the solve that owns this block of a list launch: blk0 <= blockIdx.x < blk0 + nblk
template <typename D>
__device__ __forceinline__ const D &mv_of(const D *m, int n)
{
    int k = 0;
    for (int q = 1; q < n; ++q)
        if (m[q].blk0 <= blockIdx.x) k = q;
    return m[k];
}

template <typename T>
__global__ void __launch_bounds__(256) gs_pack_k(const __grid_constant__ MvGsSet<T> P)
{
    const MvGs<T> &m = mv_of(P.m, P.n);
    gs_list_ilp_body<T>(m.v, m.f, m.list, m.cnt, m.skip, m.c, m.nx, m.nxny, blockIdx.x - m.blk0, m.nblk);
}

template <typename T>
__global__ void __launch_bounds__(256) residual_pack_k(const __grid_constant__ MvLevSet<T> P)
{
    const MvLev<T> &m = mv_of(P.m, P.n);
    residual_list_ilp_body<T>(m.r, m.f, m.v, m.l0, m.n0, m.l1, m.n1, m.c, m.nx, m.nxny, blockIdx.x - m.blk0,
                              m.nblk);
}

template <typename T>
__global__ void __launch_bounds__(256) restrict_pack_k(const __grid_constant__ MvLevSet<T> P)
{
    const MvLev<T> &m = mv_of(P.m, P.n);
    restrict_list_body<T>(m.f2, m.r, m.c0l, m.m0, m.c1l, m.m1, m.nx2, m.nxny2, m.d, blockIdx.x - m.blk0);
}

template <typename T>
__global__ void __launch_bounds__(256) correct_pack_k(const __grid_constant__ MvLevSet<T> P)
{
    const MvLev<T> &m = mv_of(P.m, P.n);
    correct_list_body<T>(m.v, m.v2, m.l0, m.n0, m.l1, m.n1, m.nx, m.nxny, m.nx2, m.nxny2, blockIdx.x - m.blk0,
                         m.nblk);
}

template <typename T>
__global__ void __launch_bounds__(CS_THREADS) coarse_pack_k(const __grid_constant__ MvCsSet<T> P)
{
    const MvCs<T> &m = P.m[blockIdx.x];
    coarse_solve_body<T>(m.v, m.f, m.G, m.r, m.d, m.gc, m.lc, m.tol, m.outer);
}

template <typename TP, typename TM>
__global__ void __launch_bounds__(RED_BLOCK) pcg_rho_pack_k(const __grid_constant__ MvPcgSet<TP, TM> P)
{
    const MvPcg<TP, TM> &m = P.m[blockIdx.x / RED_NBLK];
    pcg_rho_body<TP, TM>(m.r, m.q, m.vm, m.sk, m.sg, m.n, m.part, m.count, m.sc, blockIdx.x % RED_NBLK);
}

template <typename TP, typename TM>
__global__ void __launch_bounds__(RED_BLOCK) pcg_p_pack_k(const __grid_constant__ MvPcgSet<TP, TM> P)
{
    const MvPcg<TP, TM> &m = P.m[blockIdx.x / RED_NBLK];
    pcg_p_body<TP, sizeof(TP) != sizeof(TM)>(m.p, m.q, m.sk, m.sg, m.n, m.sc, blockIdx.x % RED_NBLK, RED_NBLK);
}

template <typename TP, typename TM>
__global__ void __launch_bounds__(RED_BLOCK) pcg_q_pack_k(const __grid_constant__ MvPcgSet<TP, TM> P)
{
    const MvPcg<TP, TM> &m = P.m[blockIdx.x / RED_NBLK];
    pcg_q_body<TP, sizeof(TP) != sizeof(TM)>(m.q, m.p, m.G, m.sk, m.sg, m.lc, m.dp, m.part, m.count, m.sc,
                                             blockIdx.x % RED_NBLK);
}

template <typename TP, typename TM>
__global__ void __launch_bounds__(RED_BLOCK) pcg_xr_pack_k(const __grid_constant__ MvPcgSet<TP, TM> P)
{
    const MvPcg<TP, TM> &m = P.m[blockIdx.x / RED_NBLK];
    pcg_xr_body<TP, TM>(m.x, m.p, m.r, m.q, m.rm, m.sk, m.sg, m.n, m.part, m.count, m.sc, blockIdx.x % RED_NBLK);
}

static unsigned blocks_for(unsigned entries, unsigned per_block) { return (entries + per_block - 1) / per_block; }

// `iter` sweeps of one kind of list (G or the band B) on level l of every solve
// Clusters of the packed smoothing calls: 8 CTAs (portable), so that 16 solves' clusters
// are resident at once.
constexpr int MV_CLUSTER = 8;

// The whole smoothing call on one cluster per solve, where every solve's lists of
// that kind fit its cluster (as sweeps_cluster's capacity rule); false if not.
template <typename T>
static bool pack_sweeps_cluster(qsm_ctx *ctx, Hier<T> *const *H, int ns, int l, bool band, int32_t iter, bool rev,
                                qsm_status *st)
{
    *st = QSM_OK;
    const unsigned cap = MV_CLUSTER * SW_THREADS * SW_PER;
    MvSwSet<T> P;
    P.n = 0;
    for (int k = 0; k < ns; ++k) {
        const Level<T> &L = H[k]->L[l];
        if (L.d.nx < 3 || L.d.ny < 3 || L.d.nz < 3) continue;
        const int par0 = rev ? (int)((L.d.nx + 1) & 1) : 0;
        const unsigned *cnt = band ? L.bn : L.gn;
        uint32_t *const *lists = band ? L.bl : L.gl;
        const unsigned c = std::max(cnt[0], cnt[1]);
        if (c > cap || (sizeof(T) == 8 && c > SW_CLUSTER_MAX)) return false;
        if (!cnt[0] && !cnt[1]) continue;
        MvSw<T> &m = P.m[P.n++];
        m.v = L.v;
        m.f = L.f;
        m.la = lists[par0];
        m.ca = cnt[par0];
        m.lb = lists[par0 ^ 1];
        m.cb = cnt[par0 ^ 1];
        m.skipb = rev ? BL_INX2 : BL_I1;
        m.c = gs_consts<T>(L.h);
        m.nx = L.d.nx;
        m.nxny = L.d.nxny();
    }
    if (!P.n) return true;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = MV_CLUSTER;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(P.n * MV_CLUSTER));
    cfg.blockDim = dim3(SW_THREADS);
    cfg.stream = ctx->stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, sweeps_pack_k<T>, P, iter);
    if (e != cudaSuccess) {
        set_error(ctx, "%s", cudaGetErrorString(e));
        *st = QSM_ERR_CUDA;
    }
    return true;
}

template <typename T>
static qsm_status pack_sweeps(qsm_ctx *ctx, Hier<T> *const *H, int ns, int l, bool band, int32_t iter, bool rev)
{
    if (iter <= 0) return QSM_OK;
    qsm_status cst;
    if (pack_sweeps_cluster<T>(ctx, H, ns, l, band, iter, rev, &cst)) return cst;
    for (int32_t s = 0; s < iter; ++s)
        for (int pass = 0; pass < 2; ++pass) {
            MvGsSet<T> P;
            P.n = 0;
            unsigned blk = 0;
            for (int k = 0; k < ns; ++k) {
                const Level<T> &L = H[k]->L[l];
                if (L.d.nx < 3 || L.d.ny < 3 || L.d.nz < 3) continue;
                const int par = (rev ? (int)((L.d.nx + 1) & 1) : 0) ^ pass;
                const unsigned cnt = band ? L.bn[par] : L.gn[par];
                if (!cnt) continue;
                MvGs<T> &m = P.m[P.n++];
                m.v = L.v;
                m.f = L.f;
                m.list = band ? L.bl[par] : L.gl[par];
                m.cnt = cnt;
                m.skip = pass ? (rev ? BL_INX2 : BL_I1) : 0u;
                m.c = gs_consts<T>(L.h);
                m.nx = L.d.nx;
                m.nxny = L.d.nxny();
                m.blk0 = blk;
                m.nblk = blocks_for(cnt, 256 * GS_PER);
                blk += m.nblk;
            }
            if (!P.n) continue;
            gs_pack_k<T><<<blk, 256, 0, ctx->stream>>>(P);
        }
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

enum { MV_RESIDUAL, MV_RESTRICT, MV_CORRECT };

// the residual of level l, its restriction onto level l + 1, or level l's correction from l + 1
template <typename T>
static qsm_status pack_level(qsm_ctx *ctx, Hier<T> *const *H, int ns, int l, int what)
{
    MvLevSet<T> P;
    P.n = 0;
    unsigned blk = 0;
    for (int k = 0; k < ns; ++k) {
        Level<T> &L = H[k]->L[l];
        Level<T> &C = H[k]->L[l + 1];
        if (L.d.nx < 3 || L.d.ny < 3 || L.d.nz < 3) continue;
        if (what != MV_RESIDUAL && (C.d.nx < 3 || C.d.ny < 3 || C.d.nz < 3)) continue;
        const unsigned nf = L.gn[0] + L.gn[1], nc = C.gn[0] + C.gn[1];
        const unsigned work = what == MV_RESTRICT ? nc : nf;
        if (!work) continue;
        MvLev<T> &m = P.m[P.n++];
        m.v = L.v;
        m.f = L.f;
        m.r = L.r;
        m.v2 = C.v;
        m.f2 = C.f;
        m.l0 = L.gl[0];
        m.l1 = L.gl[1];
        m.n0 = L.gn[0];
        m.n1 = L.gn[1];
        m.c0l = C.gl[0];
        m.c1l = C.gl[1];
        m.m0 = C.gn[0];
        m.m1 = C.gn[1];
        m.c = lap_consts<T>(L.h);
        m.nx = (uint32_t)L.d.nx;
        m.nxny = (uint32_t)L.d.nxny();
        m.nx2 = (uint32_t)C.d.nx;
        m.nxny2 = (uint32_t)C.d.nxny();
        m.d = L.d;
        m.blk0 = blk;
        m.nblk = blocks_for(work, what == MV_RESTRICT ? 256 : 256 * GS_PER);
        blk += m.nblk;
    }
    if (!P.n) return QSM_OK;
    if (what == MV_RESIDUAL)
        residual_pack_k<T><<<blk, 256, 0, ctx->stream>>>(P);
    else if (what == MV_RESTRICT)
        restrict_pack_k<T><<<blk, 256, 0, ctx->stream>>>(P);
    else
        correct_pack_k<T><<<blk, 256, 0, ctx->stream>>>(P);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// The packed coarsest solve's dynamic shared-memory limit (as coarse_smem_limit).
template <typename T>
static qsm_status coarse_pack_smem_limit(qsm_ctx *ctx, size_t *lim)
{
    static std::mutex mu;
    static std::set<int> done;
    *lim = 0;
    int maxsm = 0;
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, coarse_pack_k<T>) != cudaSuccess || (size_t)maxsm <= fa.sharedSizeBytes) {
        cudaGetLastError();
        return QSM_OK;
    }
    const size_t l = (size_t)maxsm - fa.sharedSizeBytes;
    std::lock_guard<std::mutex> lock(mu);
    if (!done.count(ctx->device)) {
        QSM_CUDA(cudaFuncSetAttribute(coarse_pack_k<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l));
        done.insert(ctx->device);
    }
    *lim = l;
    return QSM_OK;
}

template <typename T>
static qsm_status pack_coarse(qsm_ctx *ctx, Hier<T> *const *H, int ns, int l)
{
    MvCsSet<T> P;
    P.n = 0;
    size_t smem = 0;
    for (int k = 0; k < ns; ++k) {
        Level<T> &L = H[k]->L[l];
        MvCs<T> &m = P.m[P.n++];
        m.v = L.v;
        m.r = L.r;
        m.f = L.f;
        m.G = L.G;
        m.d = L.d;
        m.gc = gs_consts<T>(L.h);
        m.lc = lap_consts<T>(L.h);
        m.tol = sizeof(T) == 4 ? 1e-4 : 1e-8;
        m.outer = H[k]->counters;
        smem = std::max(smem, H[k]->coarse_smem);
    }
    if (!P.n) return QSM_OK;
    coarse_pack_k<T><<<(unsigned)P.n, CS_THREADS, smem, ctx->stream>>>(P);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// The V-cycle (cycle) on level l of every solve
template <typename T>
static qsm_status cycle_pack(qsm_ctx *ctx, Hier<T> *const *H, int ns, int l, int mu, int pre, int post, int nb)
{
    const int nl = H[0]->nl;
    if (l < nl - 1) {
        const int32_t bs = (1 << l) * nb;
        QSM_TRY(pack_sweeps<T>(ctx, H, ns, l, false, pre, true));
        QSM_TRY(pack_sweeps<T>(ctx, H, ns, l, true, bs, true));
        QSM_TRY(pack_level<T>(ctx, H, ns, l, MV_RESIDUAL));
        QSM_TRY(pack_level<T>(ctx, H, ns, l, MV_RESTRICT));
        for (int k = 0; k < ns; ++k)
            QSM_CUDA(cudaMemsetAsync(H[k]->L[l + 1].v, 0, H[k]->L[l + 1].n * sizeof(T), ctx->stream));
        for (int i = 0; i < mu; ++i) {
            QSM_TRY(cycle_pack<T>(ctx, H, ns, l + 1, mu, pre, post, nb));
            if (l + 1 == nl - 1) break;
        }
        QSM_TRY(pack_level<T>(ctx, H, ns, l, MV_CORRECT));
        QSM_TRY(pack_sweeps<T>(ctx, H, ns, l, true, bs, false));
        QSM_TRY(pack_sweeps<T>(ctx, H, ns, l, false, post, false));
        return QSM_OK;
    }
    return pack_coarse<T>(ctx, H, ns, l);
}

// Whether a set-up solve can run packed: fixed V-cycle count (tolmg <= 0), voxel lists on
// every level, and a coarsest grid one CTA holds.
template <typename TP, typename TM>
static bool pcg_packable(qsm_ctx *ctx, const PcgState<TP, TM> &S)
{
    if (S.tolmg > 0.0) return false;
    for (int i = 0; i < S.H.nl; ++i)
        if (!S.H.L[i].gl[0] || !S.H.L[i].bl[0]) return false;
    size_t lim = 0;
    if (coarse_pack_smem_limit<TM>(ctx, &lim) != QSM_OK || lim == 0) return false;
    const Level<TM> &C = S.H.L[S.H.nl - 1];
    return S.H.coarse_smem <= lim && C.n < (1u << 18);
}

// Packed solves must agree on the options that shape an iteration's launches.
template <typename TP, typename TM>
static bool pcg_same_shape(const PcgState<TP, TM> &a, const PcgState<TP, TM> &b)
{
    return a.H.nl == b.H.nl && a.mu == b.mu && a.npre == b.npre && a.npost == b.npost && a.nb == b.nb &&
           a.maxitmg == b.maxitmg;
}

// One PCG iteration of ns (<= MV_MAX) packable solves of one shape that are not done;
// their residual norms are read back (h_res: ns pinned doubles).
template <typename TP, typename TM>
static qsm_status pcg_pack_iter(qsm_ctx *ctx, PcgState<TP, TM> *const *S, int ns, double *h_res)
{
    constexpr bool same = sizeof(TP) == sizeof(TM);
    if (ns <= 0) return QSM_OK;
    if (ns > MV_MAX) return QSM_ERR_ARG;
    Range nvtx_range("mgpcg/packed iteration");
    Hier<TM> *H[MV_MAX];
    for (int k = 0; k < ns; ++k) {
        H[k] = &S[k]->H;
        if (same)
            QSM_CUDA(cudaMemsetAsync(S[k]->q, 0, S[k]->n * sizeof(TP), ctx->stream));
        else
            QSM_CUDA(cudaMemsetAsync(H[k]->L[0].v, 0, S[k]->n * sizeof(TM), ctx->stream));
    }
    for (int c = 0; c < S[0]->maxitmg; ++c)
        QSM_TRY(cycle_pack<TM>(ctx, H, ns, 0, S[0]->mu, S[0]->npre, S[0]->npost, S[0]->nb));
    MvPcgSet<TP, TM> P;
    P.n = ns;
    for (int k = 0; k < ns; ++k) {
        PcgState<TP, TM> &s = *S[k];
        MvPcg<TP, TM> &m = P.m[k];
        m.x = s.x;
        m.p = s.p;
        m.r = s.r;
        m.q = s.q;
        m.part = s.part;
        m.vm = same ? nullptr : H[k]->L[0].v;
        m.rm = same ? nullptr : H[k]->L[0].f;
        m.sk = s.sk;
        m.G = H[k]->L[0].G;
        m.sg = s.sg;
        m.count = s.count;
        m.sc = s.sc;
        m.n = s.n;
        m.lc = s.lc;
        m.dp = s.dp;
    }
    const unsigned grid = (unsigned)ns * RED_NBLK;
    pcg_rho_pack_k<TP, TM><<<grid, RED_BLOCK, 0, ctx->stream>>>(P);
    pcg_p_pack_k<TP, TM><<<grid, RED_BLOCK, 0, ctx->stream>>>(P);
    pcg_q_pack_k<TP, TM><<<grid, RED_BLOCK, 0, ctx->stream>>>(P);
    pcg_xr_pack_k<TP, TM><<<grid, RED_BLOCK, 0, ctx->stream>>>(P);
    QSM_CUDA(cudaGetLastError());
    for (int k = 0; k < ns; ++k)
        QSM_CUDA(cudaMemcpyAsync(h_res + k, S[k]->sc + S_RES, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < ns; ++k) {
        S[k]->res = h_res[k];
        S[k]->it += 1;
    }
    return QSM_OK;
}

// count solves with shared options: set up in groups of MV_MAX, the packable ones of a group
// advanced together (pcg_pack_iter), any other one by itself; then each finished.
template <typename TM>
static qsm_status mgpcg_batch_t(qsm_ctx *ctx, uint32_t count, const Dims *d, const double *const *v0,
                                const double *const *f, const uint8_t *const *mask, const double *h, double tolcg,
                                int32_t maxitcg, double tolmg, int32_t maxitmg, int32_t mu, int32_t npre,
                                int32_t npost, int32_t nb, int32_t nl, double *const *out, qsm_mg_info *info,
                                double *h_res)
{
    using St = PcgState<double, TM>;
    for (uint32_t g0 = 0; g0 < count; g0 += MV_MAX) {
        const uint32_t g1 = std::min<uint32_t>(count, g0 + MV_MAX);
        std::vector<std::unique_ptr<St>> st;
        qsm_status err = QSM_OK;
        auto release = [&]() {
            for (auto &sp : st)
                if (sp && sp->pv) pcg_finish(ctx, *sp, (double *)nullptr, (qsm_mg_info *)nullptr);
        };
        std::vector<St *> pack;
        for (uint32_t b = g0; b < g1 && err == QSM_OK; ++b) {
            st.emplace_back(new St());
            St &S = *st.back();
            err = pcg_setup(ctx, S, d[b], v0 ? v0[b] : nullptr, f[b], mask[b], h, tolcg, maxitcg, tolmg, maxitmg,
                            mu, npre, npost, nb, nl);
            if (err != QSM_OK) break;
            if (pcg_packable(ctx, S) && (pack.empty() || pcg_same_shape(*pack[0], S))) {
                // the one-CTA form reports its coarsest solver as such
                S.H.cc_ctas = 0;
                S.H.cg_ctas = 0;
                pack.push_back(&S);
                continue;
            }
            while (err == QSM_OK && !S.done()) {
                err = pcg_launch_iter(ctx, S);
                if (err == QSM_OK) err = pcg_read_res(ctx, S);
                if (err == QSM_OK && info && info[b].resnorm_hist) info[b].resnorm_hist[S.it - 1] = S.res;
            }
        }
        while (err == QSM_OK) {
            St *act[MV_MAX];
            int na = 0;
            for (St *sp : pack)
                if (!sp->done()) act[na++] = sp;
            if (!na) break;
            err = pcg_pack_iter(ctx, act, na, h_res);
            if (err == QSM_OK && info)
                for (int k = 0; k < na; ++k) {
                    const uint32_t b = g0 + (uint32_t)(std::find_if(st.begin(), st.end(),
                                                                    [&](const std::unique_ptr<St> &u) {
                                                                        return u.get() == act[k];
                                                                    }) - st.begin());
                    if (info[b].resnorm_hist) info[b].resnorm_hist[act[k]->it - 1] = act[k]->res;
                }
        }
        if (err != QSM_OK) {
            release();
            return err;
        }
        for (uint32_t b = g0; b < g1; ++b) {
            const qsm_status fs = pcg_finish(ctx, *st[b - g0], out[b], info ? info + b : nullptr);
            if (fs != QSM_OK && err == QSM_OK) err = fs;
        }
        if (err != QSM_OK) {
            release();
            return err;
        }
    }
    return QSM_OK;
}

// Session interface (mg_pack.cuh): a solve is one PcgState in the precision
// its V-cycle asks for.
struct MgPackSolve {
    bool mixed = true, packable = false;
    PcgState<double, float> sm;
    PcgState<double, double> sd;
};

qsm_status mgpack_setup(qsm_ctx *ctx, bool mixed, const Dims &d, const double *v0, const double *f,
                        const uint8_t *mask, const double vsz[3], double tolcg, int32_t maxitcg, double tolmg,
                        int32_t maxitmg, int32_t mu, int32_t npre, int32_t npost, int32_t nb, int32_t nl,
                        MgPackSolve **out)
{
    *out = nullptr;
    std::unique_ptr<MgPackSolve> p(new MgPackSolve());
    p->mixed = mixed;
    qsm_status st;
    if (mixed) {
        st = pcg_setup(ctx, p->sm, d, v0, f, mask, vsz, tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nb, nl);
        if (st == QSM_OK) p->packable = pcg_packable(ctx, p->sm);
        if (p->packable) p->sm.H.cc_ctas = p->sm.H.cg_ctas = 0;
    } else {
        st = pcg_setup(ctx, p->sd, d, v0, f, mask, vsz, tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nb, nl);
        if (st == QSM_OK) p->packable = pcg_packable(ctx, p->sd);
        if (p->packable) p->sd.H.cc_ctas = p->sd.H.cg_ctas = 0;
    }
    if (st != QSM_OK) {
        if (p->sm.pv) pcg_finish(ctx, p->sm, (double *)nullptr, (qsm_mg_info *)nullptr);
        if (p->sd.pv) pcg_finish(ctx, p->sd, (double *)nullptr, (qsm_mg_info *)nullptr);
        return st;
    }
    *out = p.release();
    return QSM_OK;
}

bool mgpack_done(const MgPackSolve *s) { return s->mixed ? s->sm.done() : s->sd.done(); }

template <typename TM>
static qsm_status mgpack_step_t(qsm_ctx *ctx, std::vector<PcgState<double, TM> *> &todo, double *h_res)
{
    while (!todo.empty()) {
        PcgState<double, TM> *grp[MV_MAX];
        int ng = 0;
        std::vector<PcgState<double, TM> *> rest;
        for (auto *sp : todo)
            if (ng < MV_MAX && (ng == 0 || pcg_same_shape(*grp[0], *sp)))
                grp[ng++] = sp;
            else
                rest.push_back(sp);
        QSM_TRY(pcg_pack_iter(ctx, grp, ng, h_res));
        todo.swap(rest);
    }
    return QSM_OK;
}

qsm_status mgpack_step(qsm_ctx *ctx, MgPackSolve *const *s, int n, double *h_res)
{
    std::vector<PcgState<double, float> *> pm;
    std::vector<PcgState<double, double> *> pd;
    for (int k = 0; k < n; ++k) {
        MgPackSolve *p = s[k];
        if (mgpack_done(p)) continue;
        if (p->packable) {
            if (p->mixed)
                pm.push_back(&p->sm);
            else
                pd.push_back(&p->sd);
        } else if (p->mixed) {
            QSM_TRY(pcg_launch_iter(ctx, p->sm));
            QSM_TRY(pcg_read_res(ctx, p->sm));
        } else {
            QSM_TRY(pcg_launch_iter(ctx, p->sd));
            QSM_TRY(pcg_read_res(ctx, p->sd));
        }
    }
    QSM_TRY(mgpack_step_t<float>(ctx, pm, h_res));
    return mgpack_step_t<double>(ctx, pd, h_res);
}

qsm_status mgpack_finish(qsm_ctx *ctx, MgPackSolve *s, double *vout, qsm_mg_info *info)
{
    std::unique_ptr<MgPackSolve> p(s);
    return p->mixed ? pcg_finish(ctx, p->sm, vout, info) : pcg_finish(ctx, p->sd, vout, info);
}

template <typename T>
static qsm_status mg_solve(qsm_ctx *ctx, const Dims &d, const T *v0, const T *f, const uint8_t *mask, const double *h,
                           double tol, int32_t maxit, int32_t mu, int32_t npre, int32_t npost, int32_t nb, int32_t nl,
                           T *vout, qsm_mg_info *info, bool full)
{
    Range nvtx_range("mg");
    const Dims dp{d.nx + 2, d.ny + 2, d.nz + 2};
    Hier<T> H;
    QSM_TRY(hier_init<T>(ctx, H, nl, dp, h));
    void *sv = nullptr;
    QSM_TRY(dalloc(ctx, &sv, S_N * sizeof(double)));
    double *sc = (double *)sv;
    QSM_TRY(pad_mask(ctx, H.L[0].G, mask, d));
    QSM_TRY(pad<T>(ctx, H.L[0].f, f, d));
    if (v0) QSM_TRY(pad<T>(ctx, H.L[0].v, v0, d));
    QSM_TRY(hier_masks<T>(ctx, H, full));
    cudaEvent_t e0, e1;
    QSM_CUDA(cudaEventCreate(&e0));
    QSM_CUDA(cudaEventCreate(&e1));
    QSM_CUDA(cudaEventRecord(e0, ctx->stream));
    int cycles = 0;
    if (!full) {
        QSM_TRY(mg_run<T>(ctx, H, tol, maxit, mu, npre, npost, nb, sc, &cycles));
    } else {
        // mx_fmg (fmg_mex.c:93-119), unrolled from the coarsest level up
        for (int l = H.nl - 1; l >= 0; --l) {
            if (l < H.nl - 1) QSM_TRY(prolong<T>(ctx, H.L[l].v, H.L[l + 1].v, H.L[l].G, H.L[l].d, H.L[l + 1].d, false));
            if (l == 0 && tol > 0.0) {
                double fn, rn;
                QSM_TRY(nrm2<T>(ctx, H.L[0].f, H.L[0].n, sc + S_TMP));
                QSM_TRY(read_double(ctx, sc + S_TMP, &fn));
                const double reltol = tol * fn;
                for (int i = 0; i < 1000 * maxit; ++i) {
                    QSM_TRY(residual<T>(ctx, H.L[0].r, H.L[0].f, H.L[0].v, H.L[0].G, H.L[0].h, H.L[0].d));
                    QSM_TRY(nrm2<T>(ctx, H.L[0].r, H.L[0].n, sc + S_TMP));
                    QSM_TRY(read_double(ctx, sc + S_TMP, &rn));
                    if (rn < reltol) break;
                    QSM_TRY(cycle<T>(ctx, H, 0, mu, npre, npost, nb, sc));
                    ++cycles;
                }
            } else {
                for (int i = 0; i < maxit; ++i) QSM_TRY(cycle<T>(ctx, H, l, mu, npre, npost, nb, sc));
                if (l == 0) cycles += maxit;
            }
        }
    }
    QSM_CUDA(cudaEventRecord(e1, ctx->stream));
    QSM_TRY(unpad<T>(ctx, vout, H.L[0].v, d));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (info) {
        info->iters = cycles;
        info->resnorm = 0.0;
        info->seconds = ms * 1e-3;
    }
    const qsm_status rep = coarse_report(ctx, H, info);  // a timed-out solve still frees its state
    QSM_TRY(dfree(ctx, sv));
    QSM_TRY(hier_free(ctx, H));
    return rep;
}

// ---------------------------------------------------------------------------
// pairwise masked norm (norm2_mex.c:83-131): leaves of <= 128 elements are
// summed sequentially in parallel, then combined along the same binary tree
// by one thread.
// ---------------------------------------------------------------------------

static void leaves(size_t off, size_t n, std::vector<unsigned long long> &out)
{
    if (n <= 128) {
        out.push_back(((unsigned long long)off << 8) | (unsigned long long)n);
        return;
    }
    const size_t m = n >> 1;
    leaves(off, m, out);
    leaves(off + m, n - m, out);
}

template <typename T>
__global__ void leaf_sum_k(T *out, const unsigned long long *lv, size_t nleaf, const T *__restrict__ x,
                           const uint8_t *__restrict__ G)
{
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nleaf) return;
    const size_t off = lv[t] >> 8, n = lv[t] & 0xFF;
    T s = G[off] ? x[off] * x[off] : (T)0;
    for (size_t i = 1; i < n; ++i)
        if (G[off + i]) s += x[off + i] * x[off + i];
    out[t] = s;
}

template <typename T>
__device__ T tree_combine(const T *leaf, size_t n, size_t &li)
{
    // explicit stack: (n, partial, state)
    struct Fr { size_t n; T a; int st; };
    Fr stk[64];
    int sp = 0;
    stk[0] = {n, (T)0, 0};
    T ret = (T)0;
    while (sp >= 0) {
        Fr &fr = stk[sp];
        if (fr.n <= 128) {
            ret = leaf[li++];
            --sp;
            continue;
        }
        if (fr.st == 0) {
            fr.st = 1;
            stk[sp + 1] = {fr.n >> 1, (T)0, 0};
            ++sp;
        } else if (fr.st == 1) {
            fr.a = ret;
            fr.st = 2;
            stk[sp + 1] = {fr.n - (fr.n >> 1), (T)0, 0};
            ++sp;
        } else {
            ret = fr.a + ret;
            --sp;
        }
    }
    return ret;
}

template <typename T>
__global__ void tree_k(double *out, const T *leaf, size_t n)
{
    size_t li = 0;
    const T s = tree_combine<T>(leaf, n, li);
    *out = sizeof(T) == 4 ? (double)sqrtf((float)s) : sqrt((double)s);
}

}  // namespace qsm

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

using namespace qsm;

static bool bad_dt(qsm_dtype dt) { return dt != QSM_F32 && dt != QSM_F64; }

extern "C" {

qsm_status qsm_gauss_seidel(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], void *v, const void *f,
                            const uint8_t *G, const double vsz[3], int32_t iter, int32_t reverse)
{
    if (!ctx || !dims || !v || !f || !G || !vsz) return QSM_ERR_ARG;
    if (bad_dt(dt)) return QSM_ERR_DTYPE;
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    const size_t es = dt == QSM_F32 ? 4 : 8;
    Staged sv, sf, sg;
    QSM_TRY(stage_in(ctx, sv, v, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sf, f, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sg, G, d.n(), true));
    qsm_status s = dt == QSM_F32 ? gauss_seidel<float>(ctx, (float *)sv.dev, (const float *)sf.dev, (const uint8_t *)sg.dev, vsz, d, iter, reverse != 0)
                                 : gauss_seidel<double>(ctx, (double *)sv.dev, (const double *)sf.dev, (const uint8_t *)sg.dev, vsz, d, iter, reverse != 0);
    QSM_TRY(stage_out(ctx, sv, true));
    QSM_TRY(stage_out(ctx, sf, false));
    QSM_TRY(stage_out(ctx, sg, false));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return s;
}

qsm_status qsm_residual(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], void *r, const void *f, const void *x,
                        const uint8_t *G, const double vsz[3])
{
    if (!ctx || !dims || !r || !f || !x || !G || !vsz) return QSM_ERR_ARG;
    if (bad_dt(dt)) return QSM_ERR_DTYPE;
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    const size_t es = dt == QSM_F32 ? 4 : 8;
    Staged sr, sf, sx, sg;
    QSM_TRY(stage_in(ctx, sr, r, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sf, f, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sx, x, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sg, G, d.n(), true));
    qsm_status s = dt == QSM_F32 ? residual<float>(ctx, (float *)sr.dev, (const float *)sf.dev, (const float *)sx.dev, (const uint8_t *)sg.dev, vsz, d)
                                 : residual<double>(ctx, (double *)sr.dev, (const double *)sf.dev, (const double *)sx.dev, (const uint8_t *)sg.dev, vsz, d);
    QSM_TRY(stage_out(ctx, sr, true));
    QSM_TRY(stage_out(ctx, sf, false));
    QSM_TRY(stage_out(ctx, sx, false));
    QSM_TRY(stage_out(ctx, sg, false));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return s;
}

qsm_status qsm_lapmg(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], void *d2u, const void *u, const uint8_t *G,
                     const double vsz[3])
{
    if (!ctx || !dims || !d2u || !u || !G || !vsz) return QSM_ERR_ARG;
    if (bad_dt(dt)) return QSM_ERR_DTYPE;
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    const size_t es = dt == QSM_F32 ? 4 : 8;
    Staged so, su, sg;
    QSM_TRY(stage_in(ctx, so, d2u, d.n() * es, true));
    QSM_TRY(stage_in(ctx, su, u, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sg, G, d.n(), true));
    qsm_status s = dt == QSM_F32 ? lapmg<float>(ctx, (float *)so.dev, (const float *)su.dev, (const uint8_t *)sg.dev, vsz, d)
                                 : lapmg<double>(ctx, (double *)so.dev, (const double *)su.dev, (const uint8_t *)sg.dev, vsz, d);
    QSM_TRY(stage_out(ctx, so, true));
    QSM_TRY(stage_out(ctx, su, false));
    QSM_TRY(stage_out(ctx, sg, false));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return s;
}

static bool transfer_dims_ok(const size_t *d2, const size_t *d)
{
    for (int q = 0; q < 3; ++q) {
        if (d2[q] < 2 || d[q] < 1) return false;
        if (d2[q] >= 3 && 2 * (d2[q] - 2) > d[q] - 1) return false;
    }
    return true;
}

qsm_status qsm_restrict(qsm_ctx *ctx, qsm_dtype dt, const size_t dims2[3], void *x2, const size_t dims[3],
                        const void *x, const uint8_t *G2)
{
    if (!ctx || !dims2 || !dims || !x2 || !x || !G2) return QSM_ERR_ARG;
    if (bad_dt(dt)) return QSM_ERR_DTYPE;
    if (!transfer_dims_ok(dims2, dims)) {
        set_error(ctx, "coarse grid does not fit the fine grid");
        return QSM_ERR_DIMS;
    }
    cudaSetDevice(ctx->device);
    const Dims d2 = make_dims(dims2), d = make_dims(dims);
    const size_t es = dt == QSM_F32 ? 4 : 8;
    Staged s2, s1, sg;
    QSM_TRY(stage_in(ctx, s2, x2, d2.n() * es, true));
    QSM_TRY(stage_in(ctx, s1, x, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sg, G2, d2.n(), true));
    qsm_status s = dt == QSM_F32 ? restrict_<float>(ctx, (float *)s2.dev, (const float *)s1.dev, (const uint8_t *)sg.dev, d2, d)
                                 : restrict_<double>(ctx, (double *)s2.dev, (const double *)s1.dev, (const uint8_t *)sg.dev, d2, d);
    QSM_TRY(stage_out(ctx, s2, true));
    QSM_TRY(stage_out(ctx, s1, false));
    QSM_TRY(stage_out(ctx, sg, false));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return s;
}

static qsm_status prolong_api(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], void *x, const size_t dims2[3],
                              const void *x2, const uint8_t *G, bool add)
{
    if (!ctx || !dims2 || !dims || !x2 || !x || !G) return QSM_ERR_ARG;
    if (bad_dt(dt)) return QSM_ERR_DTYPE;
    if (!transfer_dims_ok(dims2, dims)) {
        set_error(ctx, "coarse grid does not fit the fine grid");
        return QSM_ERR_DIMS;
    }
    cudaSetDevice(ctx->device);
    const Dims d2 = make_dims(dims2), d = make_dims(dims);
    const size_t es = dt == QSM_F32 ? 4 : 8;
    Staged s1, s2, sg;
    QSM_TRY(stage_in(ctx, s1, x, d.n() * es, true));
    QSM_TRY(stage_in(ctx, s2, x2, d2.n() * es, true));
    QSM_TRY(stage_in(ctx, sg, G, d.n(), true));
    qsm_status s = dt == QSM_F32 ? prolong<float>(ctx, (float *)s1.dev, (const float *)s2.dev, (const uint8_t *)sg.dev, d, d2, add)
                                 : prolong<double>(ctx, (double *)s1.dev, (const double *)s2.dev, (const uint8_t *)sg.dev, d, d2, add);
    QSM_TRY(stage_out(ctx, s1, true));
    QSM_TRY(stage_out(ctx, s2, false));
    QSM_TRY(stage_out(ctx, sg, false));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return s;
}

qsm_status qsm_prolong(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], void *x, const size_t dims2[3], const void *x2,
                       const uint8_t *G)
{
    return prolong_api(ctx, dt, dims, x, dims2, x2, G, false);
}

qsm_status qsm_correct(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], void *x, const size_t dims2[3], const void *x2,
                       const uint8_t *G)
{
    return prolong_api(ctx, dt, dims, x, dims2, x2, G, true);
}

qsm_status qsm_coarsen_grid(qsm_ctx *ctx, const size_t dims2[3], uint8_t *G2, const size_t dims[3], const uint8_t *G)
{
    if (!ctx || !dims2 || !dims || !G2 || !G) return QSM_ERR_ARG;
    if (!transfer_dims_ok(dims2, dims)) {
        set_error(ctx, "coarse grid does not fit the fine grid");
        return QSM_ERR_DIMS;
    }
    cudaSetDevice(ctx->device);
    const Dims d2 = make_dims(dims2), d = make_dims(dims);
    Staged s2, s1;
    QSM_TRY(stage_in(ctx, s2, G2, d2.n(), false));
    QSM_TRY(stage_in(ctx, s1, G, d.n(), true));
    coarsen_k<<<vox_grid(d2), vox_block(), 0, ctx->stream>>>((uint8_t *)s2.dev, (const uint8_t *)s1.dev, d2, d);
    QSM_CUDA(cudaGetLastError());
    QSM_TRY(stage_out(ctx, s2, true));
    QSM_TRY(stage_out(ctx, s1, false));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return QSM_OK;
}

qsm_status qsm_boundary_mask(qsm_ctx *ctx, const size_t dims[3], uint8_t *B, const uint8_t *G)
{
    if (!ctx || !dims || !B || !G) return QSM_ERR_ARG;
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    Staged sb, sg;
    QSM_TRY(stage_in(ctx, sb, B, d.n(), true));
    QSM_TRY(stage_in(ctx, sg, G, d.n(), true));
    void *scr = nullptr;
    QSM_TRY(dalloc(ctx, &scr, d.n()));
    qsm_status s = boundary_mask(ctx, (uint8_t *)sb.dev, (const uint8_t *)sg.dev, d, (uint8_t *)scr);
    QSM_TRY(dfree(ctx, scr));
    QSM_TRY(stage_out(ctx, sb, true));
    QSM_TRY(stage_out(ctx, sg, false));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return s;
}

qsm_status qsm_boundary_mask_l1(qsm_ctx *ctx, const size_t dims[3], uint8_t *B, const uint8_t *G, uint8_t l1)
{
    if (!ctx || !dims || !B || !G) return QSM_ERR_ARG;
    if (dims[0] == 0 || dims[1] == 0 || dims[2] == 0) return QSM_ERR_DIMS;
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    Staged sb, sg;
    QSM_TRY(stage_in(ctx, sb, B, d.n(), true));
    QSM_TRY(stage_in(ctx, sg, G, d.n(), true));
    void *gl = nullptr;
    QSM_TRY(dalloc(ctx, &gl, d.n()));
    bmask_l1_init_k<<<vox_grid(d), vox_block(), 0, ctx->stream>>>((uint8_t *)sb.dev, (uint8_t *)gl, (const uint8_t *)sg.dev, d);
    for (size_t L1 = 1; L1 < l1; ++L1) {
        if (2 * L1 >= d.nx || 2 * L1 >= d.ny || 2 * L1 >= d.nz) break;
        const Dims e{d.nx - 2 * L1, d.ny - 2 * L1, d.nz - 2 * L1};
        bmask_l1_step_k<<<vox_grid(e), vox_block(), 0, ctx->stream>>>((uint8_t *)sb.dev, (uint8_t *)gl, (const uint8_t *)sg.dev, d, L1);
    }
    QSM_CUDA(cudaGetLastError());
    QSM_TRY(dfree(ctx, gl));
    QSM_TRY(stage_out(ctx, sb, true));
    QSM_TRY(stage_out(ctx, sg, false));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return QSM_OK;
}

qsm_status qsm_norm2(qsm_ctx *ctx, qsm_dtype dt, size_t n, const void *x, const uint8_t *G, double *out)
{
    if (!ctx || !x || !G || !out) return QSM_ERR_ARG;
    if (bad_dt(dt)) return QSM_ERR_DTYPE;
    if (n == 0) return QSM_ERR_DIMS;
    cudaSetDevice(ctx->device);
    const size_t es = dt == QSM_F32 ? 4 : 8;
    std::vector<unsigned long long> lv;
    leaves(0, n, lv);
    Staged sx, sg;
    QSM_TRY(stage_in(ctx, sx, x, n * es, true));
    QSM_TRY(stage_in(ctx, sg, G, n, true));
    void *buf = nullptr;
    QSM_TRY(dalloc(ctx, &buf, lv.size() * (8 + es) + 64));
    unsigned long long *dl = (unsigned long long *)buf;
    void *leafv = (char *)buf + lv.size() * 8;
    QSM_CUDA(cudaMemcpyAsync(dl, lv.data(), lv.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    const unsigned g = (unsigned)((lv.size() + 255) / 256);
    if (dt == QSM_F32) {
        leaf_sum_k<float><<<g, 256, 0, ctx->stream>>>((float *)leafv, dl, lv.size(), (const float *)sx.dev, (const uint8_t *)sg.dev);
        tree_k<float><<<1, 1, 0, ctx->stream>>>(ctx->red_out, (const float *)leafv, n);
    } else {
        leaf_sum_k<double><<<g, 256, 0, ctx->stream>>>((double *)leafv, dl, lv.size(), (const double *)sx.dev, (const uint8_t *)sg.dev);
        tree_k<double><<<1, 1, 0, ctx->stream>>>(ctx->red_out, (const double *)leafv, n);
    }
    QSM_CUDA(cudaGetLastError());
    double r;
    QSM_TRY(read_double(ctx, ctx->red_out, &r));
    QSM_TRY(dfree(ctx, buf));
    QSM_TRY(stage_out(ctx, sx, false));
    QSM_TRY(stage_out(ctx, sg, false));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = r;
    return QSM_OK;
}

static qsm_status solver_checks(qsm_ctx *ctx, const size_t *dims, int32_t nl)
{
    if (nl > 16) {
        set_error(ctx, "nlevels too large. Increase MAX_DEPTH.");
        return QSM_ERR_DEPTH;
    }
    if (nl < 1) {
        set_error(ctx, "nlevels must be >= 1");
        return QSM_ERR_ARG;
    }
    if (dims[0] == 0 || dims[1] == 0 || dims[2] == 0) return QSM_ERR_DIMS;
    return QSM_OK;
}

qsm_status qsm_mgpcg(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], const void *v0, const void *f,
                     const uint8_t *mask, const double vsz[3], double tolcg, int32_t maxitcg, double tolmg,
                     int32_t maxitmg, int32_t mu, int32_t npre, int32_t npost, int32_t nboundary, int32_t nlevels,
                     int32_t verbose, void *v_out, qsm_mg_info *info)
{
    if (!ctx || !dims || !f || !mask || !vsz || !v_out) return QSM_ERR_ARG;
    if (bad_dt(dt)) return QSM_ERR_DTYPE;
    QSM_TRY(solver_checks(ctx, dims, nlevels));
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    const size_t es = dt == QSM_F32 ? 4 : 8;
    Staged s0, sf, sm, so;
    if (v0) QSM_TRY(stage_in(ctx, s0, v0, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sf, f, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sm, mask, d.n(), true));
    QSM_TRY(stage_in(ctx, so, v_out, d.n() * es, false));
    qsm_status s;
    if (dt == QSM_F32)
        s = pcg<float, float>(ctx, d, v0 ? (const float *)s0.dev : nullptr, (const float *)sf.dev, (const uint8_t *)sm.dev, vsz,
                              tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nboundary, nlevels, verbose, (float *)so.dev, info);
    else
        s = pcg<double, double>(ctx, d, v0 ? (const double *)s0.dev : nullptr, (const double *)sf.dev, (const uint8_t *)sm.dev,
                                vsz, tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nboundary, nlevels, verbose,
                                (double *)so.dev, info);
    if (v0) QSM_TRY(stage_out(ctx, s0, false));
    QSM_TRY(stage_out(ctx, sf, false));
    QSM_TRY(stage_out(ctx, sm, false));
    QSM_TRY(stage_out(ctx, so, s == QSM_OK));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return s;
}

qsm_status qsm_mgpcg_mixed(qsm_ctx *ctx, const size_t dims[3], const double *v0, const double *f, const uint8_t *mask,
                           const double vsz[3], double tolcg, int32_t maxitcg, double tolmg, int32_t maxitmg, int32_t mu,
                           int32_t npre, int32_t npost, int32_t nboundary, int32_t nlevels, int32_t verbose,
                           double *v_out, qsm_mg_info *info)
{
    if (!ctx || !dims || !f || !mask || !vsz || !v_out) return QSM_ERR_ARG;
    QSM_TRY(solver_checks(ctx, dims, nlevels));
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    Staged s0, sf, sm, so;
    if (v0) QSM_TRY(stage_in(ctx, s0, v0, d.n() * 8, true));
    QSM_TRY(stage_in(ctx, sf, f, d.n() * 8, true));
    QSM_TRY(stage_in(ctx, sm, mask, d.n(), true));
    QSM_TRY(stage_in(ctx, so, v_out, d.n() * 8, false));
    qsm_status s = pcg<double, float>(ctx, d, v0 ? (const double *)s0.dev : nullptr, (const double *)sf.dev,
                                      (const uint8_t *)sm.dev, vsz, tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost,
                                      nboundary, nlevels, verbose, (double *)so.dev, info);
    if (v0) QSM_TRY(stage_out(ctx, s0, false));
    QSM_TRY(stage_out(ctx, sf, false));
    QSM_TRY(stage_out(ctx, sm, false));
    QSM_TRY(stage_out(ctx, so, s == QSM_OK));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return s;
}

qsm_status qsm_mgpcg_batch(qsm_ctx *ctx, int32_t mixed, uint32_t count, const size_t *dims, const double *const *v0,
                           const double *const *f, const uint8_t *const *mask, const double vsz[3], double tolcg,
                           int32_t maxitcg, double tolmg, int32_t maxitmg, int32_t mu, int32_t npre, int32_t npost,
                           int32_t nboundary, int32_t nlevels, double *const *v_out, qsm_mg_info *info)
{
    if (!ctx || !dims || !f || !mask || !vsz || !v_out) return QSM_ERR_ARG;
    if (count == 0) return QSM_OK;
    for (uint32_t b = 0; b < count; ++b) {
        if (!f[b] || !mask[b] || !v_out[b]) return QSM_ERR_ARG;
        QSM_TRY(solver_checks(ctx, dims + 3 * b, nlevels));
    }
    cudaSetDevice(ctx->device);
    std::vector<Dims> d(count);
    std::vector<Staged> s0(count), sf(count), sm(count), so(count);
    std::vector<const double *> pv0(count, nullptr), pf(count);
    std::vector<const uint8_t *> pm(count);
    std::vector<double *> po(count);
    for (uint32_t b = 0; b < count; ++b) {
        d[b] = make_dims(dims + 3 * b);
        const size_t n = d[b].n();
        if (v0 && v0[b]) {
            QSM_TRY(stage_in(ctx, s0[b], v0[b], n * 8, true));
            pv0[b] = (const double *)s0[b].dev;
        }
        QSM_TRY(stage_in(ctx, sf[b], f[b], n * 8, true));
        QSM_TRY(stage_in(ctx, sm[b], mask[b], n, true));
        QSM_TRY(stage_in(ctx, so[b], v_out[b], n * 8, false));
        pf[b] = (const double *)sf[b].dev;
        pm[b] = (const uint8_t *)sm[b].dev;
        po[b] = (double *)so[b].dev;
    }
    double *h_res = nullptr;
    QSM_CUDA(cudaMallocHost((void **)&h_res, MV_MAX * sizeof(double)));
    const qsm_status s =
        mixed ? mgpcg_batch_t<float>(ctx, count, d.data(), pv0.data(), pf.data(), pm.data(), vsz, tolcg, maxitcg, tolmg,
                                     maxitmg, mu, npre, npost, nboundary, nlevels, po.data(), info, h_res)
              : mgpcg_batch_t<double>(ctx, count, d.data(), pv0.data(), pf.data(), pm.data(), vsz, tolcg, maxitcg,
                                      tolmg, maxitmg, mu, npre, npost, nboundary, nlevels, po.data(), info, h_res);
    cudaFreeHost(h_res);
    for (uint32_t b = 0; b < count; ++b) {
        if (v0 && v0[b]) QSM_TRY(stage_out(ctx, s0[b], false));
        QSM_TRY(stage_out(ctx, sf[b], false));
        QSM_TRY(stage_out(ctx, sm[b], false));
        QSM_TRY(stage_out(ctx, so[b], s == QSM_OK));
    }
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return s;
}

static qsm_status mg_api(qsm_ctx *ctx, qsm_dtype dt, const size_t *dims, const void *v0, const void *f, const uint8_t *mask,
                         const double *vsz, double tol, int32_t maxit, int32_t mu, int32_t npre, int32_t npost,
                         int32_t nb, int32_t nl, void *v_out, qsm_mg_info *info, bool full)
{
    if (!ctx || !dims || !f || !mask || !vsz || !v_out) return QSM_ERR_ARG;
    if (bad_dt(dt)) return QSM_ERR_DTYPE;
    QSM_TRY(solver_checks(ctx, dims, nl));
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    const size_t es = dt == QSM_F32 ? 4 : 8;
    Staged s0, sf, sm, so;
    if (v0) QSM_TRY(stage_in(ctx, s0, v0, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sf, f, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sm, mask, d.n(), true));
    QSM_TRY(stage_in(ctx, so, v_out, d.n() * es, false));
    qsm_status s;
    if (dt == QSM_F32)
        s = mg_solve<float>(ctx, d, v0 ? (const float *)s0.dev : nullptr, (const float *)sf.dev, (const uint8_t *)sm.dev, vsz,
                            tol, maxit, mu, npre, npost, nb, nl, (float *)so.dev, info, full);
    else
        s = mg_solve<double>(ctx, d, v0 ? (const double *)s0.dev : nullptr, (const double *)sf.dev, (const uint8_t *)sm.dev,
                             vsz, tol, maxit, mu, npre, npost, nb, nl, (double *)so.dev, info, full);
    if (v0) QSM_TRY(stage_out(ctx, s0, false));
    QSM_TRY(stage_out(ctx, sf, false));
    QSM_TRY(stage_out(ctx, sm, false));
    QSM_TRY(stage_out(ctx, so, s == QSM_OK));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    return s;
}

qsm_status qsm_mg(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], const void *v0, const void *f, const uint8_t *mask,
                  const double vsz[3], double tol, int32_t maxit, int32_t mu, int32_t npre, int32_t npost,
                  int32_t nboundary, int32_t nlevels, void *v_out, qsm_mg_info *info)
{
    return mg_api(ctx, dt, dims, v0, f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels, v_out, info, false);
}

qsm_status qsm_fmg(qsm_ctx *ctx, qsm_dtype dt, const size_t dims[3], const void *f, const uint8_t *mask,
                   const double vsz[3], double tol, int32_t maxit, int32_t mu, int32_t npre, int32_t npost,
                   int32_t nboundary, int32_t nlevels, void *v_out, qsm_mg_info *info)
{
    return mg_api(ctx, dt, dims, nullptr, f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels, v_out, info, true);
}

}  // extern "C"
