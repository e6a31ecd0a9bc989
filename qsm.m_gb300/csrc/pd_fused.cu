// Primal-dual TGV / TV inversion, mixed-precision fused path.
//
// One kernel per iteration does the dual update, the primal update and the
// extragradient for a 3-D tile of the interior:
//
//   1. the dual (nu, p, q) is evaluated on the tile plus the one-voxel layer
//      on its low side (which the primal's backward differences read) and
//      nu alone on the high-side faces (the primal's Laplacian reads them),
//      into shared memory; halo points are recomputed by every tile that
//      needs them, with identical arithmetic, instead of synchronising the
//      grid;
//   2. the primal (chi, eta, w) of the tile reads the dual from shared
//      memory and writes the next iterate.
//
// Storage (all FP32, component-major): the primal family {chi, eta, w1..3}
// is triple-buffered and the extragradient point chi_ = chi^n + (chi^n -
// chi^(n-1)) is formed where it is read, so it is never stored; the dual
// family {nu, p1..3, q1..6} is double-buffered.  Per iteration each voxel
// reads chi^n, chi^(n-1) (5+5 arrays), the dual (10), f (1) and one mask
// byte, and writes chi^(n+1) (5) and the dual (10): 36 arrays + 1 B =
// 145 B, against 51 arrays + 2 B (206 B) for the reference's two sweeps.
//
// Per voxel the FP32 expressions and their association order are those of
// update_dualf / update_primalf (pd_tgv_mex.c:332-485, :659-812; TV:
// pd_tv_mex.c:314-412, :524-622); the file is built without fused
// multiply-add, so chi is bit-identical to the reference's mx_pdf.
//
// Convergence monitors (every 10th iteration) accumulate in FP64 inside the
// kernel from the old and new chi/eta held in registers: block partials,
// then the last block reduces them in a fixed order (deterministic).
#include <math.h>

#include "common.cuh"
#include "pd.cuh"

namespace qsm {

constexpr int FT_X = 32, FT_Y = 8, FT_Z = 4;           // tile of interior voxels
constexpr int FB_X = FT_X + 2, FB_Y = FT_Y + 2, FB_Z = FT_Z + 2;  // dual box (+-1)
constexpr int FB_N = FB_X * FB_Y * FB_Z;
constexpr int F_THREADS = FT_X * FT_Y;                  // 256
constexpr size_t TGV_SMEM = 10 * FB_N * sizeof(float);  // dynamic shared memory of tgv_fused_k

// mask byte: bit 0 = m (primal update), bit 1 = mi (dual update)
__global__ void pack_masks_k(uint8_t *mm, const uint8_t *__restrict__ m, const uint8_t *__restrict__ mi, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        mm[l] = (uint8_t)((m[l] ? 1 : 0) | (mi[l] ? 2 : 0));
}

struct FusedTgv {
    const float *Pc[5];   // chi^n, eta^n, w1^n, w2^n, w3^n
    const float *Pp[5];   // iterate n-1
    float *Pn[5];         // iterate n+1 (written)
    const float *Dc[10];  // nu, p1..3, q1..6 at n
    float *Dn[10];        // at n+1 (written)
    const float *f;
    const uint8_t *mm;
    double *part;         // 4 * gridsize partial monitor sums
    unsigned int *count;
    PdCtl *ctl;
};

// extragradient point (pd_tgv_mex.c:804-810): x_ = x^n + 1*(x^n - x^(n-1))
__device__ __forceinline__ float xbar(const float *__restrict__ c, const float *__restrict__ p, size_t l)
{
    const float cn = __ldg(c + l);
    return cn + 1.0f * (cn - __ldg(p + l));
}

template <bool CHECK>
__global__ void __launch_bounds__(F_THREADS, 2)
tgv_fused_k(FusedTgv s, DualC<float> dc, PrimalC<float> pc, Dims d, double tol, uint32_t it)
{
    extern __shared__ float shd[];  // 10 x FB_N floats
    if (s.ctl->done) return;
    const size_t nx = d.nx, nxny = d.nxny(), N = d.n();
    const size_t x0 = 1 + (size_t)blockIdx.x * FT_X, y0 = 1 + (size_t)blockIdx.y * FT_Y, z0 = 1 + (size_t)blockIdx.z * FT_Z;
    const int tid = threadIdx.x;

    // ---- 1. dual on the box [x0-1, x0+FT_X] x ... (low layer + tile + high faces)
    for (int p = tid; p < FB_N; p += F_THREADS) {
        const int bx = p % FB_X, by = (p / FB_X) % FB_Y, bz = p / (FB_X * FB_Y);
        const size_t x = x0 - 1 + bx, y = y0 - 1 + by, z = z0 - 1 + bz;
        const bool hx = bx == FB_X - 1, hy = by == FB_Y - 1, hz = bz == FB_Z - 1;
        const int nhigh = (int)hx + (int)hy + (int)hz;
        float v[10];
#pragma unroll
        for (int q = 0; q < 10; ++q) v[q] = 0.0f;
        if (nhigh <= 1 && x < d.nx && y < d.ny && z < d.nz) {
            const size_t l = x + nx * y + nxny * z;
            const bool inside = (__ldg(s.mm + l) & 2) != 0;  // mi: all 6 neighbours in the mask (never on a face)
            if (nhigh == 1) {
                // high face: the primal only reads nu here
                float nu = __ldg(s.Dc[0] + l);
                if (inside) {
                    const float c0 = xbar(s.Pc[0], s.Pp[0], l);
                    const float lap = dc.lhh * xbar(s.Pc[1], s.Pp[1], l) +
                                      dc.lhx * (xbar(s.Pc[1], s.Pp[1], l - 1) + xbar(s.Pc[1], s.Pp[1], l + 1)) +
                                      dc.lhy * (xbar(s.Pc[1], s.Pp[1], l - nx) + xbar(s.Pc[1], s.Pp[1], l + nx)) +
                                      dc.lhz * (xbar(s.Pc[1], s.Pp[1], l - nxny) + xbar(s.Pc[1], s.Pp[1], l + nxny));
                    const float wav = dc.whh * c0 +
                                      dc.whx * (xbar(s.Pc[0], s.Pp[0], l - 1) + xbar(s.Pc[0], s.Pp[0], l + 1)) +
                                      dc.why * (xbar(s.Pc[0], s.Pp[0], l - nx) + xbar(s.Pc[0], s.Pp[0], l + nx)) +
                                      dc.whz * (xbar(s.Pc[0], s.Pp[0], l - nxny) + xbar(s.Pc[0], s.Pp[0], l + nxny));
                    nu = nu + ((lap - wav) + __ldg(s.f + l));
                }
                v[0] = nu;
            } else {
#pragma unroll
                for (int q = 0; q < 10; ++q) v[q] = __ldg(s.Dc[q] + l);
                if (inside) {
                    // chi_ and eta_ at the 7-point stencil, w_ at the +1 points
                    const float c0 = xbar(s.Pc[0], s.Pp[0], l);
                    const float cxm = xbar(s.Pc[0], s.Pp[0], l - 1), cxp = xbar(s.Pc[0], s.Pp[0], l + 1);
                    const float cym = xbar(s.Pc[0], s.Pp[0], l - nx), cyp = xbar(s.Pc[0], s.Pp[0], l + nx);
                    const float czm = xbar(s.Pc[0], s.Pp[0], l - nxny), czp = xbar(s.Pc[0], s.Pp[0], l + nxny);
                    const float lap = dc.lhh * xbar(s.Pc[1], s.Pp[1], l) +
                                      dc.lhx * (xbar(s.Pc[1], s.Pp[1], l - 1) + xbar(s.Pc[1], s.Pp[1], l + 1)) +
                                      dc.lhy * (xbar(s.Pc[1], s.Pp[1], l - nx) + xbar(s.Pc[1], s.Pp[1], l + nx)) +
                                      dc.lhz * (xbar(s.Pc[1], s.Pp[1], l - nxny) + xbar(s.Pc[1], s.Pp[1], l + nxny));
                    const float wav = dc.whh * c0 + dc.whx * (cxm + cxp) + dc.why * (cym + cyp) + dc.whz * (czm + czp);
                    v[0] = v[0] + ((lap - wav) + __ldg(s.f + l));

                    const float w1 = xbar(s.Pc[2], s.Pp[2], l), w2 = xbar(s.Pc[3], s.Pp[3], l), w3 = xbar(s.Pc[4], s.Pp[4], l);
                    float a1 = v[1] + dc.hx * (cxp - c0) - dc.sg * w1;
                    float a2 = v[2] + dc.hy * (cyp - c0) - dc.sg * w2;
                    float a3 = v[3] + dc.hz * (czp - c0) - dc.sg * w3;
                    float t = a1 * a1 + a2 * a2 + a3 * a3;
                    if (t > dc.alp12) {
                        t = dc.alp1 / sqrtf(t);
                        a1 = a1 * t; a2 = a2 * t; a3 = a3 * t;
                    }
                    v[1] = a1; v[2] = a2; v[3] = a3;

                    const float w1x = xbar(s.Pc[2], s.Pp[2], l + 1), w1y = xbar(s.Pc[2], s.Pp[2], l + nx), w1z = xbar(s.Pc[2], s.Pp[2], l + nxny);
                    const float w2x = xbar(s.Pc[3], s.Pp[3], l + 1), w2y = xbar(s.Pc[3], s.Pp[3], l + nx), w2z = xbar(s.Pc[3], s.Pp[3], l + nxny);
                    const float w3x = xbar(s.Pc[4], s.Pp[4], l + 1), w3y = xbar(s.Pc[4], s.Pp[4], l + nx), w3z = xbar(s.Pc[4], s.Pp[4], l + nxny);
                    float b1 = v[4] + dc.hx * (w1x - w1);
                    float b2 = v[5] + dc.hx2 * (w2x - w2) + dc.hy2 * (w1y - w1);
                    float b3 = v[6] + dc.hx2 * (w3x - w3) + dc.hz2 * (w1z - w1);
                    float b4 = v[7] + dc.hy * (w2y - w2);
                    float b5 = v[8] + dc.hy2 * (w3y - w3) + dc.hz2 * (w2z - w2);
                    float b6 = v[9] + dc.hz * (w3z - w3);
                    t = b1 * b1 + b4 * b4 + b6 * b6 + 2.0f * (b2 * b2 + b3 * b3 + b5 * b5);
                    if (t > dc.alp02) {
                        t = dc.alp0 / sqrtf(t);
                        b1 = b1 * t; b2 = b2 * t; b3 = b3 * t; b4 = b4 * t; b5 = b5 * t; b6 = b6 * t;
                    }
                    v[4] = b1; v[5] = b2; v[6] = b3; v[7] = b4; v[8] = b5; v[9] = b6;
                    // the owning tile stores the new dual
                    if (bx >= 1 && by >= 1 && bz >= 1) {
#pragma unroll
                        for (int q = 0; q < 10; ++q) s.Dn[q][l] = v[q];
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 10; ++q) shd[(q) * FB_N + p] = v[q];
    }
    __syncthreads();

    // ---- 2. primal + extragradient on the tile
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int tx = tid % FT_X, ty = tid / FT_X;
    const size_t x = x0 + tx, y = y0 + ty;
    if (x + 1 < d.nx && y + 1 < d.ny) {
        for (int tz = 0; tz < FT_Z; ++tz) {
            const size_t z = z0 + tz;
            if (z + 1 >= d.nz) break;
            const size_t l = x + nx * y + nxny * z;
            if (!(__ldg(s.mm + l) & 1)) continue;
            const int b = (tx + 1) + FB_X * ((ty + 1) + FB_Y * (tz + 1));
            const int sx = 1, sy = FB_X, sz = FB_X * FB_Y;
            const float nu0 = shd[(0) * FB_N + b];
            const float xs = shd[(0) * FB_N + b - sx] + shd[(0) * FB_N + b + sx];
            const float ys = shd[(0) * FB_N + b - sy] + shd[(0) * FB_N + b + sy];
            const float zs = shd[(0) * FB_N + b - sz] + shd[(0) * FB_N + b + sz];
            const float en = __ldg(s.Pc[1] + l), cn = __ldg(s.Pc[0] + l);
            const float w1n = __ldg(s.Pc[2] + l), w2n = __ldg(s.Pc[3] + l), w3n = __ldg(s.Pc[4] + l);
            const float e1 = pc.tau1 * (en - pc.lhh * nu0 - pc.lhx * xs - pc.lhy * ys - pc.lhz * zs);
            const float c1 = cn + (pc.hx * (shd[(1) * FB_N + b] - shd[(1) * FB_N + b - sx]) + pc.hy * (shd[(2) * FB_N + b] - shd[(2) * FB_N + b - sy]) +
                                   pc.hz * (shd[(3) * FB_N + b] - shd[(3) * FB_N + b - sz]) +
                                   (pc.whh * nu0 + pc.whx * xs + pc.why * ys + pc.whz * zs));
            const float u1 = w1n + (pc.tt * shd[(1) * FB_N + b] + pc.hx * (shd[(4) * FB_N + b] - shd[(4) * FB_N + b - sx] + shd[(5) * FB_N + b] - shd[(5) * FB_N + b - sy] +
                                                                  shd[(6) * FB_N + b] - shd[(6) * FB_N + b - sz]));
            const float u2 = w2n + (pc.tt * shd[(2) * FB_N + b] + pc.hy * (shd[(5) * FB_N + b] - shd[(5) * FB_N + b - sx] + shd[(7) * FB_N + b] - shd[(7) * FB_N + b - sy] +
                                                                  shd[(8) * FB_N + b] - shd[(8) * FB_N + b - sz]));
            const float u3 = w3n + (pc.tt * shd[(3) * FB_N + b] + pc.hz * (shd[(6) * FB_N + b] - shd[(6) * FB_N + b - sx] + shd[(8) * FB_N + b] - shd[(8) * FB_N + b - sy] +
                                                                  shd[(9) * FB_N + b] - shd[(9) * FB_N + b - sz]));
            s.Pn[0][l] = c1;
            s.Pn[1][l] = e1;
            s.Pn[2][l] = u1;
            s.Pn[3][l] = u2;
            s.Pn[4][l] = u3;
            if (CHECK) {
                double a, bb, c, e;
                mon_terms(c1, cn, e1, en, a, bb, c, e);
                acc[0] += a; acc[1] += bb; acc[2] += c; acc[3] += e;
            }
        }
    }
    (void)N;
    if (!CHECK) return;

    // ---- 3. monitor sums: block tree, then the last block in fixed order
    __shared__ double red[4][F_THREADS];
    __shared__ bool last;
    const unsigned int nblk = gridDim.x * gridDim.y * gridDim.z;
    const unsigned int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
#pragma unroll
    for (int q = 0; q < 4; ++q) red[q][tid] = acc[q];
    __syncthreads();
    for (int st = F_THREADS / 2; st > 0; st >>= 1) {
        if (tid < st)
#pragma unroll
            for (int q = 0; q < 4; ++q) red[q][tid] += red[q][tid + st];
        __syncthreads();
    }
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) s.part[(size_t)q * nblk + bid] = red[q][0];
        __threadfence();
        last = atomicAdd(s.count, 1u) == nblk - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        double a = 0.0;
        for (unsigned int b2 = tid; b2 < nblk; b2 += F_THREADS) a += __ldcg(s.part + (size_t)q * nblk + b2);
        red[q][tid] = a;
    }
    __syncthreads();
    for (int st = F_THREADS / 2; st > 0; st >>= 1) {
        if (tid < st)
#pragma unroll
            for (int q = 0; q < 4; ++q) red[q][tid] += red[q][tid + st];
        __syncthreads();
    }
    if (tid == 0) {
        double r[4] = {red[0][0], red[1][0], red[2][0], red[3][0]};
        pd_finish(s.ctl, r, tol, it);
        *s.count = 0;
    }
}

// ---------------------------------------------------------------------------
// TV: primal {chi, eta}, dual {nu, p1..3}
// ---------------------------------------------------------------------------

struct FusedTv {
    const float *Pc[2];
    const float *Pp[2];
    float *Pn[2];
    const float *Dc[4];
    float *Dn[4];
    const float *f;
    const uint8_t *mm;
    double *part;
    unsigned int *count;
    PdCtl *ctl;
};

template <bool CHECK>
__global__ void __launch_bounds__(F_THREADS, 2)
tv_fused_k(FusedTv s, DualC<float> dc, PrimalC<float> pc, Dims d, double tol, uint32_t it)
{
    __shared__ float sh[4][FB_N];
    if (s.ctl->done) return;
    const size_t nx = d.nx, nxny = d.nxny();
    const size_t x0 = 1 + (size_t)blockIdx.x * FT_X, y0 = 1 + (size_t)blockIdx.y * FT_Y, z0 = 1 + (size_t)blockIdx.z * FT_Z;
    const int tid = threadIdx.x;
    for (int p = tid; p < FB_N; p += F_THREADS) {
        const int bx = p % FB_X, by = (p / FB_X) % FB_Y, bz = p / (FB_X * FB_Y);
        const size_t x = x0 - 1 + bx, y = y0 - 1 + by, z = z0 - 1 + bz;
        const bool hx = bx == FB_X - 1, hy = by == FB_Y - 1, hz = bz == FB_Z - 1;
        const int nhigh = (int)hx + (int)hy + (int)hz;
        float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (nhigh <= 1 && x < d.nx && y < d.ny && z < d.nz) {
            const size_t l = x + nx * y + nxny * z;
            const bool inside = (__ldg(s.mm + l) & 2) != 0;
            const int nq = nhigh == 1 ? 1 : 4;
            for (int q = 0; q < nq; ++q) v[q] = __ldg(s.Dc[q] + l);
            if (inside) {
                const float c0 = xbar(s.Pc[0], s.Pp[0], l);
                const float cxm = xbar(s.Pc[0], s.Pp[0], l - 1), cxp = xbar(s.Pc[0], s.Pp[0], l + 1);
                const float cym = xbar(s.Pc[0], s.Pp[0], l - nx), cyp = xbar(s.Pc[0], s.Pp[0], l + nx);
                const float czm = xbar(s.Pc[0], s.Pp[0], l - nxny), czp = xbar(s.Pc[0], s.Pp[0], l + nxny);
                const float lap = dc.lhh * xbar(s.Pc[1], s.Pp[1], l) +
                                  dc.lhx * (xbar(s.Pc[1], s.Pp[1], l - 1) + xbar(s.Pc[1], s.Pp[1], l + 1)) +
                                  dc.lhy * (xbar(s.Pc[1], s.Pp[1], l - nx) + xbar(s.Pc[1], s.Pp[1], l + nx)) +
                                  dc.lhz * (xbar(s.Pc[1], s.Pp[1], l - nxny) + xbar(s.Pc[1], s.Pp[1], l + nxny));
                const float wav = dc.whh * c0 + dc.whx * (cxm + cxp) + dc.why * (cym + cyp) + dc.whz * (czm + czp);
                v[0] = v[0] + ((lap - wav) + __ldg(s.f + l));
                if (nhigh == 0) {
                    float a1 = v[1] + dc.hx * (cxp - c0);
                    float a2 = v[2] + dc.hy * (cyp - c0);
                    float a3 = v[3] + dc.hz * (czp - c0);
                    float t = a1 * a1 + a2 * a2 + a3 * a3;
                    if (t > dc.alp12) {
                        t = dc.alp1 / sqrtf(t);
                        a1 = a1 * t; a2 = a2 * t; a3 = a3 * t;
                    }
                    v[1] = a1; v[2] = a2; v[3] = a3;
                    if (bx >= 1 && by >= 1 && bz >= 1) {
#pragma unroll
                        for (int q = 0; q < 4; ++q) s.Dn[q][l] = v[q];
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) sh[q][p] = v[q];
    }
    __syncthreads();

    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int tx = tid % FT_X, ty = tid / FT_X;
    const size_t x = x0 + tx, y = y0 + ty;
    if (x + 1 < d.nx && y + 1 < d.ny) {
        for (int tz = 0; tz < FT_Z; ++tz) {
            const size_t z = z0 + tz;
            if (z + 1 >= d.nz) break;
            const size_t l = x + nx * y + nxny * z;
            if (!(__ldg(s.mm + l) & 1)) continue;
            const int b = (tx + 1) + FB_X * ((ty + 1) + FB_Y * (tz + 1));
            const int sx = 1, sy = FB_X, sz = FB_X * FB_Y;
            const float nu0 = sh[0][b];
            const float xs = sh[0][b - sx] + sh[0][b + sx];
            const float ys = sh[0][b - sy] + sh[0][b + sy];
            const float zs = sh[0][b - sz] + sh[0][b + sz];
            const float en = __ldg(s.Pc[1] + l), cn = __ldg(s.Pc[0] + l);
            const float e1 = pc.tau1 * (en - pc.lhh * nu0 - pc.lhx * xs - pc.lhy * ys - pc.lhz * zs);
            const float c1 = cn + (pc.hx * (sh[1][b] - sh[1][b - sx]) + pc.hy * (sh[2][b] - sh[2][b - sy]) +
                                   pc.hz * (sh[3][b] - sh[3][b - sz]) +
                                   (pc.whh * nu0 + pc.whx * xs + pc.why * ys + pc.whz * zs));
            s.Pn[0][l] = c1;
            s.Pn[1][l] = e1;
            if (CHECK) {
                double a, bb, c, e;
                mon_terms(c1, cn, e1, en, a, bb, c, e);
                acc[0] += a; acc[1] += bb; acc[2] += c; acc[3] += e;
            }
        }
    }
    if (!CHECK) return;
    __shared__ double red[4][F_THREADS];
    __shared__ bool last;
    const unsigned int nblk = gridDim.x * gridDim.y * gridDim.z;
    const unsigned int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
#pragma unroll
    for (int q = 0; q < 4; ++q) red[q][tid] = acc[q];
    __syncthreads();
    for (int st = F_THREADS / 2; st > 0; st >>= 1) {
        if (tid < st)
#pragma unroll
            for (int q = 0; q < 4; ++q) red[q][tid] += red[q][tid + st];
        __syncthreads();
    }
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) s.part[(size_t)q * nblk + bid] = red[q][0];
        __threadfence();
        last = atomicAdd(s.count, 1u) == nblk - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        double a = 0.0;
        for (unsigned int b2 = tid; b2 < nblk; b2 += F_THREADS) a += __ldcg(s.part + (size_t)q * nblk + b2);
        red[q][tid] = a;
    }
    __syncthreads();
    for (int st = F_THREADS / 2; st > 0; st >>= 1) {
        if (tid < st)
#pragma unroll
            for (int q = 0; q < 4; ++q) red[q][tid] += red[q][tid + st];
        __syncthreads();
    }
    if (tid == 0) {
        double r[4] = {red[0][0], red[1][0], red[2][0], red[3][0]};
        pd_finish(s.ctl, r, tol, it);
        *s.count = 0;
    }
}

// ---------------------------------------------------------------------------
// driver
// ---------------------------------------------------------------------------

qsm_status pd_fused(qsm_ctx *ctx, bool tgv, const Dims &d, qsm_dtype dt, const void *d2f, const uint8_t *mask,
                    const double *h, double lam, double alpha, double tol, uint32_t maxiter, uint32_t verbose,
                    void *chi_out, qsm_pd_info *info)
{
    const size_t N = d.n();
    const int np = tgv ? 5 : 2, nd = tgv ? 10 : 4;
    const size_t stride = (N * sizeof(float) + 255) & ~(size_t)255;
    const dim3 grid((unsigned)((d.nx > 2 ? d.nx - 2 : 0) + FT_X - 1) / FT_X,
                    (unsigned)((d.ny > 2 ? d.ny - 2 : 0) + FT_Y - 1) / FT_Y,
                    (unsigned)((d.nz > 2 ? d.nz - 2 : 0) + FT_Z - 1) / FT_Z);
    const size_t nblk = (size_t)grid.x * grid.y * grid.z;
    const bool empty = nblk == 0;
    // 3 primal buffers + 2 dual buffers + f + scratch masks + partials + ctl
    const size_t bytes = stride * (3 * np + 2 * nd + 1) + 3 * ((N + 255) & ~(size_t)255) +
                         4 * (nblk + 1) * sizeof(double) + 512;
    void *blk = nullptr;
    QSM_TRY(dalloc(ctx, &blk, bytes));
    QSM_CUDA(cudaMemsetAsync(blk, 0, bytes, ctx->stream));
    char *c = (char *)blk;
    float *P[3][5], *D[2][10];
    for (int b = 0; b < 3; ++b)
        for (int q = 0; q < np; ++q, c += stride) P[b][q] = (float *)c;
    for (int b = 0; b < 2; ++b)
        for (int q = 0; q < nd; ++q, c += stride) D[b][q] = (float *)c;
    float *f = (float *)c;
    c += stride;
    const size_t mstride = (N + 255) & ~(size_t)255;
    uint8_t *m = (uint8_t *)c, *mi = m + mstride, *mm = mi + mstride;
    c += 3 * mstride;
    double *part = (double *)c;
    c += 4 * (nblk + 1) * sizeof(double);
    PdCtl *ctl = (PdCtl *)(((uintptr_t)c + 255) & ~(uintptr_t)255);

    double tau, sigma;
    pd_steps(h, &tau, &sigma);
    if (tgv) {
        QSM_CUDA(cudaFuncSetAttribute(tgv_fused_k<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TGV_SMEM));
        QSM_CUDA(cudaFuncSetAttribute(tgv_fused_k<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TGV_SMEM));
    }
    QSM_TRY(launch_masks(ctx, m, mi, mask, d));
    pack_masks_k<<<2048, 256, 0, ctx->stream>>>(mm, m, mi, N);
    QSM_CUDA(cudaGetLastError());
    if (dt == QSM_F32)
        QSM_TRY((launch_scale<float, float>(ctx, f, (const float *)d2f, sigma, N)));
    else
        QSM_TRY((launch_scale<float, double>(ctx, f, (const double *)d2f, sigma, N)));
    const DualC<float> dc = tgv ? make_dual_c<float>(sigma, h, alpha * lam, lam) : make_dual_c<float>(sigma, h, 0.0, lam);
    const PrimalC<float> pc = make_primal_c<float>(tau, h);

    cudaEvent_t e0, e1;
    QSM_CUDA(cudaEventCreate(&e0));
    QSM_CUDA(cudaEventCreate(&e1));
    QSM_CUDA(cudaEventRecord(e0, ctx->stream));
    if (verbose) printf("Iter\t\t||delta chi||\t||delta eta||\n");
    const uint32_t pmod = maxiter ? maxiter / (verbose > 4 ? (verbose < maxiter ? verbose : maxiter) : (4 < maxiter ? 4 : maxiter)) : 1;
    PdCtl hctl;
    memset(&hctl, 0, sizeof hctl);
    uint32_t enq = 0;
    for (uint32_t it = 0; it < maxiter; ++it) {
        const int cur = it % 3, prv = (it + 2) % 3, nxt = (it + 1) % 3;
        const int dcur = it % 2, dnxt = (it + 1) % 2;
        const bool chk = ((it + 1) % 10) == 0;
        if (!empty) {
            if (tgv) {
                FusedTgv s;
                for (int q = 0; q < 5; ++q) { s.Pc[q] = P[cur][q]; s.Pp[q] = P[prv][q]; s.Pn[q] = P[nxt][q]; }
                for (int q = 0; q < 10; ++q) { s.Dc[q] = D[dcur][q]; s.Dn[q] = D[dnxt][q]; }
                s.f = f; s.mm = mm; s.part = part; s.count = ctx->red_count + 1; s.ctl = ctl;
                if (chk) tgv_fused_k<true><<<grid, F_THREADS, TGV_SMEM, ctx->stream>>>(s, dc, pc, d, tol, it + 1);
                else tgv_fused_k<false><<<grid, F_THREADS, TGV_SMEM, ctx->stream>>>(s, dc, pc, d, tol, it + 1);
            } else {
                FusedTv s;
                for (int q = 0; q < 2; ++q) { s.Pc[q] = P[cur][q]; s.Pp[q] = P[prv][q]; s.Pn[q] = P[nxt][q]; }
                for (int q = 0; q < 4; ++q) { s.Dc[q] = D[dcur][q]; s.Dn[q] = D[dnxt][q]; }
                s.f = f; s.mm = mm; s.part = part; s.count = ctx->red_count + 1; s.ctl = ctl;
                if (chk) tv_fused_k<true><<<grid, F_THREADS, 0, ctx->stream>>>(s, dc, pc, d, tol, it + 1);
                else tv_fused_k<false><<<grid, F_THREADS, 0, ctx->stream>>>(s, dc, pc, d, tol, it + 1);
            }
            QSM_CUDA(cudaGetLastError());
        }
        enq = it + 1;
        const bool print = verbose && (it == 0 || it == maxiter - 1 || ((it + 1) % pmod) == 0);
        if (print || (chk && ((it + 1) % 100) == 0)) {
            QSM_CUDA(cudaMemcpyAsync(&hctl, ctl, sizeof(PdCtl), cudaMemcpyDeviceToHost, ctx->stream));
            QSM_CUDA(cudaStreamSynchronize(ctx->stream));
            if (verbose && (print || hctl.done))
                printf("%5d/%d\t%.3e\t%.3e\n", hctl.done ? hctl.iters : it + 1, maxiter, hctl.checks ? hctl.n1 : 1.0,
                       hctl.checks ? hctl.n2 : 1.0);
            if (hctl.done) break;
        }
    }
    QSM_CUDA(cudaEventRecord(e1, ctx->stream));
    QSM_CUDA(cudaMemcpyAsync(&hctl, ctl, sizeof(PdCtl), cudaMemcpyDeviceToHost, ctx->stream));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    const uint32_t iters = hctl.done ? hctl.iters : enq;
    const float *chi = P[iters % 3][0];
    if (dt == QSM_F32)
        QSM_CUDA(cudaMemcpyAsync(chi_out, chi, N * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    else
        QSM_TRY((launch_convert<double, float>(ctx, (double *)chi_out, chi, N)));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (info) {
        info->iters = iters;
        info->monitor_chi = hctl.checks ? hctl.n1 : 1.0;
        info->monitor_eta = hctl.checks ? hctl.n2 : 1.0;
        info->seconds = ms * 1e-3;
    }
    return dfree(ctx, blk);
}

}  // namespace qsm
