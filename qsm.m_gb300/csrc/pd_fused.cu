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
// Only tiles holding mask voxels are launched: outside m and mi the
// reference never changes anything, so the primal and the dual stay 0 there
// in every buffer.  Inside a tile, the dual is only read where mi holds (it
// is identically 0 elsewhere).
//
// Storage (all FP32, component-major): the primal family {chi, eta, w1..3}
// is triple-buffered and the extragradient point chi_ = chi^n + (chi^n -
// chi^(n-1)) is formed where it is read, so it is never stored; the dual
// family {nu, p1..3, q1..6} is double-buffered.  Per iteration an active
// voxel reads chi^n, chi^(n-1) (5+5 arrays), the dual (10), f (1) and one
// mask byte, and writes chi^(n+1) (5) and the dual (10): 36 arrays + 1 B =
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
//
// Tile shapes: a few compiled variants; the first solve on a grid size times
// each for a few iterations and keeps the fastest (an in-process table,
// optionally persisted in the file named by QSM_AUTOTUNE_CACHE);
// QSM_FUSED_VARIANT=<index> forces one.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "pd.cuh"
#include "pd_fused.cuh"

namespace qsm {

// mask byte: bit 0 = m (primal update), bit 1 = mi (dual update)
__global__ void pack_masks_k(uint8_t *mm, const uint8_t *__restrict__ m, const uint8_t *__restrict__ mi, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        mm[l] = (uint8_t)((m[l] ? 1 : 0) | (mi[l] ? 2 : 0));
}

// A tile is active iff one of its voxels is in m (primal update) or in mi
// (dual update).
__global__ void tile_flags_k(uint8_t *flag, const uint8_t *__restrict__ mm, Dims d, unsigned gx, unsigned gy, int tx,
                             int ty, int tz)
{
    const unsigned t = blockIdx.x;
    const size_t x0 = 1 + (size_t)(t % gx) * tx, y0 = 1 + (size_t)((t / gx) % gy) * ty, z0 = 1 + (size_t)(t / (gx * gy)) * tz;
    int any = 0;
    for (int p = threadIdx.x; p < tx * ty * tz; p += blockDim.x) {
        const size_t x = x0 + p % tx, y = y0 + (p / tx) % ty, z = z0 + p / (tx * ty);
        if (x + 1 < d.nx && y + 1 < d.ny && z + 1 < d.nz && mm[x + d.nx * (y + d.ny * z)]) any = 1;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) flag[t] = (uint8_t)any;
}

// ---------------------------------------------------------------------------
// TGV
// ---------------------------------------------------------------------------

template <int TX, int TY, int TZ, int MINB, bool CHECK>
__global__ void __launch_bounds__(TX * TY, MINB)
tgv_fused_k(FusedArgs s, DualC<float> dc, PrimalC<float> pc, Dims d, double tol, uint32_t it)
{
    constexpr int BX = TX + 2, BY = TY + 2, BZ = TZ + 2, BN = BX * BY * BZ, THREADS = TX * TY;
    extern __shared__ double shd_raw[];  // 10 x BN floats of the dual (reused for the monitor reduction)
    float *shd = (float *)shd_raw;
    if (s.ctl->done) return;
    const size_t nx = d.nx, nxny = d.nxny();
    const unsigned tile = s.tiles[blockIdx.x];
    const size_t x0 = 1 + (size_t)(tile % s.gx) * TX, y0 = 1 + (size_t)((tile / s.gx) % s.gy) * TY,
                 z0 = 1 + (size_t)(tile / (s.gx * s.gy)) * TZ;
    const int tid = threadIdx.x;

    // ---- 1. dual on the box [x0-1, x0+TX] x ... (low layer + tile + high faces)
    for (int p = tid; p < BN; p += THREADS) {
        const int bx = p % BX, by = (p / BX) % BY, bz = p / (BX * BY);
        const size_t x = x0 - 1 + bx, y = y0 - 1 + by, z = z0 - 1 + bz;
        const int nhigh = (int)(bx == BX - 1) + (int)(by == BY - 1) + (int)(bz == BZ - 1);
        float v[10];
#pragma unroll
        for (int q = 0; q < 10; ++q) v[q] = 0.0f;
        if (nhigh <= 1 && x < d.nx && y < d.ny && z < d.nz) {
            const size_t l = x + nx * y + nxny * z;
            // mi: all six neighbours in the mask (never true on a face); the dual is 0 outside it
            const bool inside = (__ldg(s.mm + l) & 2) != 0;
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
                v[0] = __ldg(s.Dc[0] + l) + ((lap - wav) + __ldg(s.f + l));
                if (nhigh == 0) {
#pragma unroll
                    for (int q = 1; q < 10; ++q) v[q] = __ldg(s.Dc[q] + l);
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
        for (int q = 0; q < 10; ++q) shd[q * BN + p] = v[q];
    }
    __syncthreads();

    // ---- 2. primal + extragradient on the tile
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int tx = tid % TX, ty = tid / TX;
    const size_t x = x0 + tx, y = y0 + ty;
    if (x + 1 < d.nx && y + 1 < d.ny) {
#pragma unroll 1
        for (int tz = 0; tz < TZ; ++tz) {
            const size_t z = z0 + tz;
            if (z + 1 >= d.nz) break;
            const size_t l = x + nx * y + nxny * z;
            if (!(__ldg(s.mm + l) & 1)) continue;
            const int b = (tx + 1) + BX * ((ty + 1) + BY * (tz + 1));
            constexpr int sx = 1, sy = BX, sz = BX * BY;
#define SH(q, o) shd[(q) * BN + b + (o)]
            const float nu0 = SH(0, 0);
            const float xs = SH(0, -sx) + SH(0, sx);
            const float ys = SH(0, -sy) + SH(0, sy);
            const float zs = SH(0, -sz) + SH(0, sz);
            const float en = __ldg(s.Pc[1] + l), cn = __ldg(s.Pc[0] + l);
            const float w1n = __ldg(s.Pc[2] + l), w2n = __ldg(s.Pc[3] + l), w3n = __ldg(s.Pc[4] + l);
            const float e1 = pc.tau1 * (en - pc.lhh * nu0 - pc.lhx * xs - pc.lhy * ys - pc.lhz * zs);
            const float c1 = cn + (pc.hx * (SH(1, 0) - SH(1, -sx)) + pc.hy * (SH(2, 0) - SH(2, -sy)) +
                                   pc.hz * (SH(3, 0) - SH(3, -sz)) + (pc.whh * nu0 + pc.whx * xs + pc.why * ys + pc.whz * zs));
            const float u1 = w1n + (pc.tt * SH(1, 0) + pc.hx * (SH(4, 0) - SH(4, -sx) + SH(5, 0) - SH(5, -sy) + SH(6, 0) - SH(6, -sz)));
            const float u2 = w2n + (pc.tt * SH(2, 0) + pc.hy * (SH(5, 0) - SH(5, -sx) + SH(7, 0) - SH(7, -sy) + SH(8, 0) - SH(8, -sz)));
            const float u3 = w3n + (pc.tt * SH(3, 0) + pc.hz * (SH(6, 0) - SH(6, -sx) + SH(8, 0) - SH(8, -sy) + SH(9, 0) - SH(9, -sz)));
#undef SH
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
    if (CHECK) monitor_reduce<THREADS>(s, shd_raw, acc, tol, it);
}

// ---------------------------------------------------------------------------
// TV: primal {chi, eta}, dual {nu, p1..3}
// ---------------------------------------------------------------------------

template <int TX, int TY, int TZ, int MINB, bool CHECK>
__global__ void __launch_bounds__(TX * TY, MINB)
tv_fused_k(FusedArgs s, DualC<float> dc, PrimalC<float> pc, Dims d, double tol, uint32_t it)
{
    constexpr int BX = TX + 2, BY = TY + 2, BZ = TZ + 2, BN = BX * BY * BZ, THREADS = TX * TY;
    extern __shared__ double shd_raw[];  // 4 x BN floats
    float *shd = (float *)shd_raw;
    if (s.ctl->done) return;
    const size_t nx = d.nx, nxny = d.nxny();
    const unsigned tile = s.tiles[blockIdx.x];
    const size_t x0 = 1 + (size_t)(tile % s.gx) * TX, y0 = 1 + (size_t)((tile / s.gx) % s.gy) * TY,
                 z0 = 1 + (size_t)(tile / (s.gx * s.gy)) * TZ;
    const int tid = threadIdx.x;
    for (int p = tid; p < BN; p += THREADS) {
        const int bx = p % BX, by = (p / BX) % BY, bz = p / (BX * BY);
        const size_t x = x0 - 1 + bx, y = y0 - 1 + by, z = z0 - 1 + bz;
        const int nhigh = (int)(bx == BX - 1) + (int)(by == BY - 1) + (int)(bz == BZ - 1);
        float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (nhigh <= 1 && x < d.nx && y < d.ny && z < d.nz) {
            const size_t l = x + nx * y + nxny * z;
            const bool inside = (__ldg(s.mm + l) & 2) != 0;  // the dual is 0 outside mi
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
                v[0] = __ldg(s.Dc[0] + l) + ((lap - wav) + __ldg(s.f + l));
                if (nhigh == 0) {
                    float a1 = __ldg(s.Dc[1] + l) + dc.hx * (cxp - c0);
                    float a2 = __ldg(s.Dc[2] + l) + dc.hy * (cyp - c0);
                    float a3 = __ldg(s.Dc[3] + l) + dc.hz * (czp - c0);
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
        for (int q = 0; q < 4; ++q) shd[q * BN + p] = v[q];
    }
    __syncthreads();

    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int tx = tid % TX, ty = tid / TX;
    const size_t x = x0 + tx, y = y0 + ty;
    if (x + 1 < d.nx && y + 1 < d.ny) {
#pragma unroll 1
        for (int tz = 0; tz < TZ; ++tz) {
            const size_t z = z0 + tz;
            if (z + 1 >= d.nz) break;
            const size_t l = x + nx * y + nxny * z;
            if (!(__ldg(s.mm + l) & 1)) continue;
            const int b = (tx + 1) + BX * ((ty + 1) + BY * (tz + 1));
            constexpr int sx = 1, sy = BX, sz = BX * BY;
            const float nu0 = shd[b];
            const float xs = shd[b - sx] + shd[b + sx];
            const float ys = shd[b - sy] + shd[b + sy];
            const float zs = shd[b - sz] + shd[b + sz];
            const float en = __ldg(s.Pc[1] + l), cn = __ldg(s.Pc[0] + l);
            const float e1 = pc.tau1 * (en - pc.lhh * nu0 - pc.lhx * xs - pc.lhy * ys - pc.lhz * zs);
            const float c1 = cn + (pc.hx * (shd[BN + b] - shd[BN + b - sx]) + pc.hy * (shd[2 * BN + b] - shd[2 * BN + b - sy]) +
                                   pc.hz * (shd[3 * BN + b] - shd[3 * BN + b - sz]) +
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
    if (CHECK) monitor_reduce<THREADS>(s, shd_raw, acc, tol, it);
}

// ---------------------------------------------------------------------------
// variants, launch, autotuning
// ---------------------------------------------------------------------------

struct Variant {
    int tx, ty, tz;   // tile of interior voxels (z: chunk of planes for the streaming kernel)
    bool stream;      // pd_stream.cu column-streaming kernel, else the 3-D tile kernel here
};
// 3-D tiles: threads = tx * ty; streaming: threads = (tx + 4) * (ty + 4)
static const Variant kVariants[] = {{32, 8, 4, false}, {32, 8, 2, false}, {32, 4, 4, false}, {32, 16, 2, false},
                                    {28, 12, 8, true},   {28, 12, 16, true},  {28, 12, 32, true},  {28, 12, 64, true}};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

static size_t smem_bytes(const Variant &v, bool tgv)
{
    if (v.stream) return stream_smem(v.tx, v.ty, tgv);
    const size_t bn = (size_t)(v.tx + 2) * (v.ty + 2) * (v.tz + 2);
    const size_t dual = (tgv ? 10 : 4) * bn * sizeof(float);
    const size_t red = 4 * (size_t)v.tx * v.ty * sizeof(double);
    return std::max(dual, red);
}

template <int TX, int TY, int TZ, int MINB>
static void launch_t(qsm_ctx *ctx, bool tgv, bool chk, unsigned nact, const FusedArgs &s, const DualC<float> &dc,
                     const PrimalC<float> &pc, const Dims &d, double tol, uint32_t it, size_t smem)
{
    if (tgv) {
        if (chk) tgv_fused_k<TX, TY, TZ, MINB, true><<<nact, TX * TY, smem, ctx->stream>>>(s, dc, pc, d, tol, it);
        else tgv_fused_k<TX, TY, TZ, MINB, false><<<nact, TX * TY, smem, ctx->stream>>>(s, dc, pc, d, tol, it);
    } else {
        if (chk) tv_fused_k<TX, TY, TZ, MINB, true><<<nact, TX * TY, smem, ctx->stream>>>(s, dc, pc, d, tol, it);
        else tv_fused_k<TX, TY, TZ, MINB, false><<<nact, TX * TY, smem, ctx->stream>>>(s, dc, pc, d, tol, it);
    }
}

template <int TX, int TY, int TZ, int MINB>
static qsm_status set_smem_t(qsm_ctx *ctx, size_t tgv_smem, size_t tv_smem)
{
    QSM_CUDA(cudaFuncSetAttribute(tgv_fused_k<TX, TY, TZ, MINB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tgv_smem));
    QSM_CUDA(cudaFuncSetAttribute(tgv_fused_k<TX, TY, TZ, MINB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tgv_smem));
    QSM_CUDA(cudaFuncSetAttribute(tv_fused_k<TX, TY, TZ, MINB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tv_smem));
    QSM_CUDA(cudaFuncSetAttribute(tv_fused_k<TX, TY, TZ, MINB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tv_smem));
    return QSM_OK;
}

static qsm_status launch_variant(qsm_ctx *ctx, int v, bool tgv, bool chk, unsigned nact, const FusedArgs &s,
                                 const DualC<float> &dc, const PrimalC<float> &pc, const Dims &d, double tol, uint32_t it)
{
    const size_t sm = smem_bytes(kVariants[v], tgv);
    if (kVariants[v].stream)
        return stream_launch(ctx, kVariants[v].tx, kVariants[v].ty, kVariants[v].tz, tgv, chk, nact, s, dc, pc, d, tol, it);
    switch (v) {
    case 0: launch_t<32, 8, 4, 2>(ctx, tgv, chk, nact, s, dc, pc, d, tol, it, sm); break;
    case 1: launch_t<32, 8, 2, 3>(ctx, tgv, chk, nact, s, dc, pc, d, tol, it, sm); break;
    case 2: launch_t<32, 4, 4, 4>(ctx, tgv, chk, nact, s, dc, pc, d, tol, it, sm); break;
    case 3: launch_t<32, 16, 2, 1>(ctx, tgv, chk, nact, s, dc, pc, d, tol, it, sm); break;
    default: return QSM_ERR_ARG;
    }
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

static qsm_status set_all_smem(qsm_ctx *ctx)
{
    QSM_TRY((set_smem_t<32, 8, 4, 2>(ctx, smem_bytes(kVariants[0], true), smem_bytes(kVariants[0], false))));
    QSM_TRY((set_smem_t<32, 8, 2, 3>(ctx, smem_bytes(kVariants[1], true), smem_bytes(kVariants[1], false))));
    QSM_TRY((set_smem_t<32, 4, 4, 4>(ctx, smem_bytes(kVariants[2], true), smem_bytes(kVariants[2], false))));
    QSM_TRY((set_smem_t<32, 16, 2, 1>(ctx, smem_bytes(kVariants[3], true), smem_bytes(kVariants[3], false))));
    return stream_set_smem(ctx);
}

// process-wide tuning table: (tgv, nx, ny, nz) -> variant
using TuneKey = std::tuple<int, size_t, size_t, size_t>;
static std::map<TuneKey, int> g_tuned;
static std::mutex g_tune_mu;
static bool g_tune_loaded = false;

static void tune_load_locked()
{
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char *path = getenv("QSM_AUTOTUNE_CACHE");
    if (!path || !*path) return;
    FILE *fp = fopen(path, "r");
    if (!fp) return;
    int tg, v;
    size_t a, b, c;
    while (fscanf(fp, "%d %zu %zu %zu %d", &tg, &a, &b, &c, &v) == 5)
        if (v >= 0 && v < kNumVariants) g_tuned[TuneKey(tg, a, b, c)] = v;
    fclose(fp);
}

static void tune_store_locked(const TuneKey &k, int v)
{
    g_tuned[k] = v;
    const char *path = getenv("QSM_AUTOTUNE_CACHE");
    if (!path || !*path) return;
    FILE *fp = fopen(path, "a");
    if (!fp) return;
    fprintf(fp, "%d %zu %zu %zu %d\n", std::get<0>(k), std::get<1>(k), std::get<2>(k), std::get<3>(k), v);
    fclose(fp);
}

// ---------------------------------------------------------------------------
// driver
// ---------------------------------------------------------------------------

struct TileList {
    unsigned gx = 0, gy = 0, gz = 0, nact = 0;
    unsigned *dev = nullptr;  // inside the state block
    uint64_t active_vox = 0;
};

qsm_status pd_fused(qsm_ctx *ctx, bool tgv, const Dims &d, qsm_dtype dt, const void *d2f, const uint8_t *mask,
                    const double *h, double lam, double alpha, double tol, uint32_t maxiter, uint32_t verbose,
                    void *chi_out, qsm_pd_info *info)
{
    const size_t N = d.n();
    const int np = tgv ? 5 : 2, nd = tgv ? 10 : 4;
    const size_t stride = (N * sizeof(float) + 255) & ~(size_t)255;
    const size_t mstride = (N + 255) & ~(size_t)255;
    const size_t ix = d.nx > 2 ? d.nx - 2 : 0, iy = d.ny > 2 ? d.ny - 2 : 0, iz = d.nz > 2 ? d.nz - 2 : 0;

    // tile grids of every variant
    TileList tl[kNumVariants];
    size_t ntiles_total = 0, nblk_max = 0;
    for (int v = 0; v < kNumVariants; ++v) {
        tl[v].gx = (unsigned)((ix + kVariants[v].tx - 1) / kVariants[v].tx);
        tl[v].gy = (unsigned)((iy + kVariants[v].ty - 1) / kVariants[v].ty);
        tl[v].gz = (unsigned)((iz + kVariants[v].tz - 1) / kVariants[v].tz);
        const size_t nb = (size_t)tl[v].gx * tl[v].gy * tl[v].gz;
        ntiles_total += nb;
        nblk_max = std::max(nblk_max, nb);
    }

    // 3 primal buffers + 2 dual buffers + f + masks + tile lists + partials + ctl
    const size_t bytes = stride * (3 * np + 2 * nd + 1) + 3 * mstride + (ntiles_total + 64) * sizeof(unsigned) +
                         (nblk_max + 64) + 4 * (nblk_max + 1) * sizeof(double) + 1024;
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
    uint8_t *m = (uint8_t *)c, *mi = m + mstride, *mm = mi + mstride;
    c += 3 * mstride;
    unsigned *tiles_base = (unsigned *)c;
    c += (ntiles_total + 64) * sizeof(unsigned);
    uint8_t *tflag = (uint8_t *)c;
    c += nblk_max + 64;
    c = (char *)(((uintptr_t)c + 255) & ~(uintptr_t)255);
    double *part = (double *)c;
    c += 4 * (nblk_max + 1) * sizeof(double);
    PdCtl *ctl = (PdCtl *)(((uintptr_t)c + 255) & ~(uintptr_t)255);
    const size_t state_bytes = stride * (3 * np + 2 * nd);  // primal + dual buffers (zeroed again after tuning)

    double tau, sigma;
    pd_steps(h, &tau, &sigma);
    QSM_TRY(set_all_smem(ctx));
    QSM_TRY(launch_masks(ctx, m, mi, mask, d));
    pack_masks_k<<<2048, 256, 0, ctx->stream>>>(mm, m, mi, N);
    QSM_CUDA(cudaGetLastError());
    if (dt == QSM_F32)
        QSM_TRY((launch_scale<float, float>(ctx, f, (const float *)d2f, sigma, N)));
    else
        QSM_TRY((launch_scale<float, double>(ctx, f, (const double *)d2f, sigma, N)));

    // active tiles of every variant, ascending (fixed order of the monitor partials)
    {
        unsigned *tp = tiles_base;
        for (int v = 0; v < kNumVariants; ++v) {
            const size_t nb = (size_t)tl[v].gx * tl[v].gy * tl[v].gz;
            tl[v].dev = tp;
            tp += nb;
            if (!nb) continue;
            tile_flags_k<<<(unsigned)nb, 256, 0, ctx->stream>>>(tflag, mm, d, tl[v].gx, tl[v].gy, kVariants[v].tx,
                                                                kVariants[v].ty, kVariants[v].tz);
            QSM_CUDA(cudaGetLastError());
            std::vector<uint8_t> hf(nb);
            QSM_CUDA(cudaMemcpyAsync(hf.data(), tflag, nb, cudaMemcpyDeviceToHost, ctx->stream));
            QSM_CUDA(cudaStreamSynchronize(ctx->stream));
            std::vector<unsigned> ht;
            ht.reserve(nb);
            for (size_t t = 0; t < nb; ++t) {
                if (!hf[t]) continue;
                ht.push_back((unsigned)t);
                const size_t ttx = t % tl[v].gx, tty = (t / tl[v].gx) % tl[v].gy, ttz = t / ((size_t)tl[v].gx * tl[v].gy);
                tl[v].active_vox += std::min((size_t)kVariants[v].tx, ix - ttx * kVariants[v].tx) *
                                    std::min((size_t)kVariants[v].ty, iy - tty * kVariants[v].ty) *
                                    std::min((size_t)kVariants[v].tz, iz - ttz * kVariants[v].tz);
            }
            tl[v].nact = (unsigned)ht.size();
            if (!ht.empty())
                QSM_CUDA(cudaMemcpyAsync(tl[v].dev, ht.data(), ht.size() * sizeof(unsigned), cudaMemcpyHostToDevice, ctx->stream));
            QSM_CUDA(cudaStreamSynchronize(ctx->stream));
        }
    }

    const DualC<float> dc = tgv ? make_dual_c<float>(sigma, h, alpha * lam, lam) : make_dual_c<float>(sigma, h, 0.0, lam);
    const PrimalC<float> pc = make_primal_c<float>(tau, h);

    auto args_for = [&](int v, uint32_t it) {
        FusedArgs s;
        memset(&s, 0, sizeof s);
        const int cur = it % 3, prv = (it + 2) % 3, nxt = (it + 1) % 3, dcur = it % 2, dnxt = (it + 1) % 2;
        for (int q = 0; q < np; ++q) { s.Pc[q] = P[cur][q]; s.Pp[q] = P[prv][q]; s.Pn[q] = P[nxt][q]; }
        for (int q = 0; q < nd; ++q) { s.Dc[q] = D[dcur][q]; s.Dn[q] = D[dnxt][q]; }
        s.f = f; s.mm = mm; s.part = part; s.count = ctx->red_count + 1; s.ctl = ctl;
        s.tiles = tl[v].dev; s.gx = tl[v].gx; s.gy = tl[v].gy;
        return s;
    };

    // choose the tile variant
    int var = 0;
    const char *force = getenv("QSM_FUSED_VARIANT");
    const TuneKey key((int)tgv, d.nx, d.ny, d.nz);
    bool tuned = false;
    if (force && *force) {
        var = std::min(std::max(atoi(force), 0), kNumVariants - 1);
        tuned = true;
    } else {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        tune_load_locked();
        auto itk = g_tuned.find(key);
        if (itk != g_tuned.end()) {
            var = itk->second;
            tuned = true;
        }
    }
    if (!tuned && tl[0].nact > 0 && maxiter >= 20) {
        // time each variant over a few iterations on this problem, then reset the state
        cudaEvent_t t0, t1;
        QSM_CUDA(cudaEventCreate(&t0));
        QSM_CUDA(cudaEventCreate(&t1));
        float best = 1e30f;
        for (int v = 0; v < kNumVariants; ++v) {
            for (uint32_t it = 0; it < 2; ++it)
                QSM_TRY(launch_variant(ctx, v, tgv, false, tl[v].nact, args_for(v, it), dc, pc, d, tol, it + 1));
            QSM_CUDA(cudaEventRecord(t0, ctx->stream));
            for (uint32_t it = 2; it < 8; ++it)
                QSM_TRY(launch_variant(ctx, v, tgv, false, tl[v].nact, args_for(v, it), dc, pc, d, tol, it + 1));
            QSM_CUDA(cudaEventRecord(t1, ctx->stream));
            QSM_CUDA(cudaEventSynchronize(t1));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, t0, t1);
            if (ms < best) {
                best = ms;
                var = v;
            }
        }
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        QSM_CUDA(cudaMemsetAsync(P[0][0], 0, state_bytes, ctx->stream));
        std::lock_guard<std::mutex> lock(g_tune_mu);
        tune_store_locked(key, var);
    }
    const unsigned nact = tl[var].nact;
    const bool empty = nact == 0;

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
        const bool chk = ((it + 1) % 10) == 0;
        if (!empty) QSM_TRY(launch_variant(ctx, var, tgv, chk, nact, args_for(var, it), dc, pc, d, tol, it + 1));
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
        info->active_voxels = tl[var].active_vox;
        info->tile[0] = (uint32_t)kVariants[var].tx;
        info->tile[1] = (uint32_t)kVariants[var].ty;
        info->tile[2] = (uint32_t)kVariants[var].tz;
    }
    return dfree(ctx, blk);
}

}  // namespace qsm
