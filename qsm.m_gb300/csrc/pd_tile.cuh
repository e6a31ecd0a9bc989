// Device bodies of the fused mixed-precision TGV/TV iteration, shared by the
// one-volume kernels (pd_fused.cu: 3-D tiles; pd_stream.cu: z-streaming
// columns) and the persistent many-volume kernels (pd_batch.cu).
//
// 3-D tile (tile_tgv / tile_tv, TX x TY threads):
//   1. the dual (nu, p, q) is evaluated on the tile plus the one-voxel layer
//      on its low side (which the primal's backward differences read) and
//      nu alone on the high-side faces (the primal's Laplacian reads them),
//      into shared memory; halo points are recomputed by every tile that
//      needs them, with identical arithmetic, instead of synchronising the
//      grid;
//   2. the primal (chi, eta, w) of the tile reads the dual from shared
//      memory and writes the next iterate.
//
// Column (column_pd, (TX+4) x (TY+4) threads): each thread walks its column
// upwards one plane per step:
//
//   step j:  (a) read the primal iterates n and n-1 at plane j+1 of its own
//                column and form the extragradient point (chi_, eta_, w_);
//                keep it in registers (z-neighbours) and publish it in
//                shared memory (x/y-neighbours of plane j+1)
//            (b) the dual at plane j (threads of the one-voxel ring and the
//                tile) from registers (z) and shared memory (x, y): written
//                to shared memory, and to HBM by the owning threads
//            (c) the primal + extragradient at plane j-1 (tile threads), from
//                the dual of planes j-2 (registers), j-1 (shared memory, x/y
//                neighbours) and j (own value)
//            (b) ends with an arrival on the step's mbarrier; step j+1 waits
//            for every thread's arrival before it reads plane j+1's shared
//            values (triple-buffered planes, see column_pd)
//
// so every input value of a plane is read from HBM once per CTA (the ring
// re-reads neighbouring tiles' edges, mostly from L2) and the dual is
// evaluated once per plane and column (plus the ring), not on a 3-D halo.
// Only the two planes below a chunk are recomputed.
//
// Both skip voxels outside the mask (their state is identically 0).  Per
// voxel the FP32 expressions are those of update_dualf / update_primalf
// (pd_tgv_mex.c:332-485, :659-812; TV: pd_tv_mex.c:314-412, :524-622) in the
// reference's association order; the files are built without fused
// multiply-add, so chi is bit-identical to the reference's mx_pdf.
//
// Monitor terms (every check iteration): x^2, e^2, (x - x0)^2, (e - e0)^2 per
// voxel in FP32, summed per thread with compensation (PartialSum<float>) and
// handed to the FP64 block fold as one value per thread: converting and adding
// every voxel's terms in FP64 made a check iteration cost 1.8 plain ones, FP64
// running at 1/64 of the FP32 rate.
#pragma once

#include <math.h>

#include "common.cuh"
#include "pd.cuh"
#include "pd_fused.cuh"
#include "tma.cuh"

namespace qsm {

// One 3-D tile of the fused TGV iteration; shd holds 10 x (TX+2)(TY+2)(TZ+2)
// floats; acc receives this thread's monitor sums when check is set.
template <int TX, int TY, int TZ>
__device__ __forceinline__ void tile_tgv(const FusedArgs &s, const DualC<float> &dc, const PrimalC<float> &pc,
                                         const Dims &d, unsigned tile, bool check, float *shd, double *acc)
{
    constexpr int BX = TX + 2, BY = TY + 2, BZ = TZ + 2, BN = BX * BY * BZ, THREADS = TX * TY;
    const size_t nx = d.nx, nxny = d.nxny();
    const size_t x0 = 1 + (size_t)(tile % s.gx) * TX, y0 = 1 + (size_t)((tile / s.gx) % s.gy) * TY,
                 z0 = 1 + (size_t)(tile / (s.gx * s.gy)) * TZ;
    const int tid = threadIdx.x;
    PartialSum<float> mon[4];

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
                // (chi_, eta_, w1_, w2_) at the voxel and its six neighbours
                float C[4], Xm[4], Xp[4], Ym[4], Yp[4], Zm[4], Zp[4];
                bar_head<true>(s, l, C);
                bar_head<true>(s, l - 1, Xm);
                bar_head<true>(s, l + 1, Xp);
                bar_head<true>(s, l - nx, Ym);
                bar_head<true>(s, l + nx, Yp);
                bar_head<true>(s, l - nxny, Zm);
                bar_head<true>(s, l + nxny, Zp);
                const float c0 = C[0];
                const float cxm = Xm[0], cxp = Xp[0], cym = Ym[0], cyp = Yp[0], czm = Zm[0], czp = Zp[0];
                const float lap = dc.lhh * C[1] + dc.lhx * (Xm[1] + Xp[1]) + dc.lhy * (Ym[1] + Yp[1]) +
                                  dc.lhz * (Zm[1] + Zp[1]);
                const float wav = dc.whh * c0 + dc.whx * (cxm + cxp) + dc.why * (cym + cyp) + dc.whz * (czm + czp);
                const float4 da = __ldg(s.Dca + l);
                v[0] = da.x + ((lap - wav) + __ldg(s.f + l));
                if (nhigh == 0) {
                    const float4 db = __ldg(s.Dcb + l);
                    const float2 dd = __ldg(s.Dcc + l);
                    v[1] = da.y; v[2] = da.z; v[3] = da.w;
                    v[4] = db.x; v[5] = db.y; v[6] = db.z; v[7] = db.w; v[8] = dd.x; v[9] = dd.y;
                    const float w1 = C[2], w2 = C[3], w3 = xbar(s.Pc1, s.Pp1, l);
                    float a1 = v[1] + dc.hx * (cxp - c0) - dc.sg * w1;
                    float a2 = v[2] + dc.hy * (cyp - c0) - dc.sg * w2;
                    float a3 = v[3] + dc.hz * (czp - c0) - dc.sg * w3;
                    float t = a1 * a1 + a2 * a2 + a3 * a3;
                    if (t > dc.alp12) {
                        t = dc.alp1 / sqrtf(t);
                        a1 = a1 * t; a2 = a2 * t; a3 = a3 * t;
                    }
                    v[1] = a1; v[2] = a2; v[3] = a3;
                    const float w1x = Xp[2], w1y = Yp[2], w1z = Zp[2];
                    const float w2x = Xp[3], w2y = Yp[3], w2z = Zp[3];
                    const float w3x = xbar(s.Pc1, s.Pp1, l + 1), w3y = xbar(s.Pc1, s.Pp1, l + nx),
                                w3z = xbar(s.Pc1, s.Pp1, l + nxny);
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
                    if (bx >= 1 && by >= 1 && bz >= 1) store_dual<true>(s, l, v);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 10; ++q) shd[q * BN + p] = v[q];
    }
    __syncthreads();

    // ---- 2. primal + extragradient on the tile
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
            float pn[5];
            load_primal<true>(s.Pc, s.Pc1, l, pn);
            const float cn = pn[0], en = pn[1], w1n = pn[2], w2n = pn[3], w3n = pn[4];
            const float e1 = pc.tau1 * (en - pc.lhh * nu0 - pc.lhx * xs - pc.lhy * ys - pc.lhz * zs);
            const float c1 = cn + (pc.hx * (SH(1, 0) - SH(1, -sx)) + pc.hy * (SH(2, 0) - SH(2, -sy)) +
                                   pc.hz * (SH(3, 0) - SH(3, -sz)) + (pc.whh * nu0 + pc.whx * xs + pc.why * ys + pc.whz * zs));
            const float u1 = w1n + (pc.tt * SH(1, 0) + pc.hx * (SH(4, 0) - SH(4, -sx) + SH(5, 0) - SH(5, -sy) + SH(6, 0) - SH(6, -sz)));
            const float u2 = w2n + (pc.tt * SH(2, 0) + pc.hy * (SH(5, 0) - SH(5, -sx) + SH(7, 0) - SH(7, -sy) + SH(8, 0) - SH(8, -sz)));
            const float u3 = w3n + (pc.tt * SH(3, 0) + pc.hz * (SH(6, 0) - SH(6, -sx) + SH(8, 0) - SH(8, -sy) + SH(9, 0) - SH(9, -sz)));
#undef SH
            const float pv[5] = {c1, e1, u1, u2, u3};
            store_primal<true>(s.Pn, s.Pn1, l, pv);
            if (check) {
                mon[0].add(c1 * c1);
                mon[1].add(e1 * e1);
                mon[2].add((c1 - cn) * (c1 - cn));
                mon[3].add((e1 - en) * (e1 - en));
            }
        }
    }
    if (check)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] += mon[q].get();
    (void)THREADS;
}

// One 3-D tile of the fused TV iteration; shd holds 4 x (TX+2)(TY+2)(TZ+2) floats.
template <int TX, int TY, int TZ>
__device__ __forceinline__ void tile_tv(const FusedArgs &s, const DualC<float> &dc, const PrimalC<float> &pc,
                                        const Dims &d, unsigned tile, bool check, float *shd, double *acc)
{
    constexpr int BX = TX + 2, BY = TY + 2, BZ = TZ + 2, BN = BX * BY * BZ, THREADS = TX * TY;
    const size_t nx = d.nx, nxny = d.nxny();
    const size_t x0 = 1 + (size_t)(tile % s.gx) * TX, y0 = 1 + (size_t)((tile / s.gx) % s.gy) * TY,
                 z0 = 1 + (size_t)(tile / (s.gx * s.gy)) * TZ;
    const int tid = threadIdx.x;
    PartialSum<float> mon[4];
    for (int p = tid; p < BN; p += THREADS) {
        const int bx = p % BX, by = (p / BX) % BY, bz = p / (BX * BY);
        const size_t x = x0 - 1 + bx, y = y0 - 1 + by, z = z0 - 1 + bz;
        const int nhigh = (int)(bx == BX - 1) + (int)(by == BY - 1) + (int)(bz == BZ - 1);
        float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (nhigh <= 1 && x < d.nx && y < d.ny && z < d.nz) {
            const size_t l = x + nx * y + nxny * z;
            const bool inside = (__ldg(s.mm + l) & 2) != 0;  // the dual is 0 outside mi
            if (inside) {
                float C[2], Xm[2], Xp[2], Ym[2], Yp[2], Zm[2], Zp[2];
                bar_head<false>(s, l, C);
                bar_head<false>(s, l - 1, Xm);
                bar_head<false>(s, l + 1, Xp);
                bar_head<false>(s, l - nx, Ym);
                bar_head<false>(s, l + nx, Yp);
                bar_head<false>(s, l - nxny, Zm);
                bar_head<false>(s, l + nxny, Zp);
                const float c0 = C[0];
                const float cxm = Xm[0], cxp = Xp[0], cym = Ym[0], cyp = Yp[0], czm = Zm[0], czp = Zp[0];
                const float lap = dc.lhh * C[1] + dc.lhx * (Xm[1] + Xp[1]) + dc.lhy * (Ym[1] + Yp[1]) +
                                  dc.lhz * (Zm[1] + Zp[1]);
                const float wav = dc.whh * c0 + dc.whx * (cxm + cxp) + dc.why * (cym + cyp) + dc.whz * (czm + czp);
                const float4 da = __ldg(s.Dca + l);
                v[0] = da.x + ((lap - wav) + __ldg(s.f + l));
                if (nhigh == 0) {
                    float a1 = da.y + dc.hx * (cxp - c0);
                    float a2 = da.z + dc.hy * (cyp - c0);
                    float a3 = da.w + dc.hz * (czp - c0);
                    float t = a1 * a1 + a2 * a2 + a3 * a3;
                    if (t > dc.alp12) {
                        t = dc.alp1 / sqrtf(t);
                        a1 = a1 * t; a2 = a2 * t; a3 = a3 * t;
                    }
                    v[1] = a1; v[2] = a2; v[3] = a3;
                    if (bx >= 1 && by >= 1 && bz >= 1) store_dual<false>(s, l, v);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) shd[q * BN + p] = v[q];
    }
    __syncthreads();

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
            float pn[2];
            load_primal<false>(s.Pc, s.Pc1, l, pn);
            const float cn = pn[0], en = pn[1];
            const float e1 = pc.tau1 * (en - pc.lhh * nu0 - pc.lhx * xs - pc.lhy * ys - pc.lhz * zs);
            const float c1 = cn + (pc.hx * (shd[BN + b] - shd[BN + b - sx]) + pc.hy * (shd[2 * BN + b] - shd[2 * BN + b - sy]) +
                                   pc.hz * (shd[3 * BN + b] - shd[3 * BN + b - sz]) +
                                   (pc.whh * nu0 + pc.whx * xs + pc.why * ys + pc.whz * zs));
            const float pv[2] = {c1, e1};
            store_primal<false>(s.Pn, s.Pn1, l, pv);
            if (check) {
                mon[0].add(c1 * c1);
                mon[1].add(e1 * e1);
                mon[2].add((c1 - cn) * (c1 - cn));
                mon[3].add((e1 - en) * (e1 - en));
            }
        }
    }
    if (check)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] += mon[q].get();
    (void)THREADS;
}

// One TX x TY column tile, planes [zs, zs + cz) of the interior, of the
// fused TGV (TGV) or TV iteration with (TX+4)(TY+4) threads; smem holds
// P x (NB + ND) planes of (TX+4)(TY+4) floats (and, for TGV, three
// mbarriers).  acc receives this thread's monitor sums when check is set.
//
// TGV steps are ordered by split arrive/wait barriers instead of one barrier
// per plane: step k publishes the extragradient point of plane j+1 and the
// dual of plane j, arrives on barrier k % 3 and then runs the primal of
// plane j-1, which reads only what step k-1 published; step k+1 starts by
// waiting for every thread's step-k arrival.  A warp may so run up to a step
// ahead of the others.  The exchange planes are triple-buffered (P = 3): a
// fast warp at step k+1 writes the buffers step k-1 read, and its wait for
// step k proves that every thread is done with step k-1.  TV, whose steps
// are a third as long, keeps one barrier at the end of each step and two
// buffers (P = 2): measured 5-10 % faster there (the split form gains 1 % on
// TGV).
constexpr uint32_t kColumnWaitLimit = 1u << 22;
template <int TX, int TY, bool TGV>
__device__ __forceinline__ void column_pd(const FusedArgs &s, const DualC<float> &dc, const PrimalC<float> &pc,
                                          const Dims &d, int cz, unsigned tile, bool check, float *smem, double *acc)
{
    constexpr int WX = TX + 4, WY = TY + 4, NT = WX * WY;
    constexpr int NB = TGV ? 5 : 2;   // extragradient arrays: chi_, eta_, w1_, w2_, w3_
    constexpr int ND = TGV ? 10 : 4;  // dual arrays: nu, p1..3, q1..6
    constexpr bool SPLIT = TGV;       // split step barriers (else one barrier per step)
    constexpr int P = SPLIT ? 3 : 2;  // exchange buffers
    float *B = smem;                  // [P][NB][NT]  extragradient point of one plane
    float *S = B + P * NB * NT;       // [P][ND][NT]  dual of one plane
    uint64_t *sbar = (uint64_t *)(S + P * ND * NT);  // [3] step barriers (SPLIT)
    const long x0 = 1 + (long)(tile % s.gx) * TX, y0 = 1 + (long)((tile / s.gx) % s.gy) * TY;
    const long zs = 1 + (long)(tile / (s.gx * s.gy)) * cz;
    const long ze = min(zs + (long)cz, (long)d.nz - 1);
    const int tid = threadIdx.x, tx = tid % WX, ty = tid / WX;
    const long x = x0 - 2 + tx, y = y0 - 2 + ty;
    PartialSum<float> mon[4];
    const bool valid = x >= 0 && y >= 0 && x < (long)d.nx && y < (long)d.ny;
    const bool ring1 = tx >= 1 && tx <= TX + 2 && ty >= 1 && ty <= TY + 2;  // dual is evaluated here
    const bool owned = tx >= 2 && tx <= TX + 1 && ty >= 2 && ty <= TY + 1 && x + 1 < (long)d.nx && y + 1 < (long)d.ny;
    const size_t nxny = d.nxny();
    const size_t col = valid ? (size_t)x + d.nx * (size_t)y : 0;
    const long nz = (long)d.nz;

    // Every global input is fetched one plane step before it is used, so the
    // memory latency of a plane overlaps the arithmetic of the previous one.
    // The mask bytes that decide which inputs to fetch come from a register
    // ring loaded further ahead, so no fetch waits for a mask load first.
    auto mask_at = [&](long z) -> unsigned {
        return (valid && z >= 0 && z < nz) ? (unsigned)__ldg(s.mm + col + nxny * (size_t)z) : 0u;
    };
    //   raw iterates n, n-1 (+ mask bit m) of the own column, plane j+2
    float rc[NB], rp[NB];
    bool rm = false;
    auto fetch_bars = [&](long z, unsigned mb) {
        rm = (mb & 1u) != 0;
        const size_t l = col + nxny * (size_t)(rm ? z : 0);  // an in-bounds address even when unused
        if (rm) {
            load_primal<TGV>(s.Pc, s.Pc1, l, rc);
            load_primal<TGV>(s.Pp, s.Pp1, l, rp);
        } else {
#pragma unroll
            for (int q = 0; q < NB; ++q) rc[q] = rp[q] = 0.0f;
        }
    };
    auto make_bars = [&](float *v) {
#pragma unroll
        for (int q = 0; q < NB; ++q) v[q] = rm ? rc[q] + 1.0f * (rc[q] - rp[q]) : 0.0f;
    };
    //   dual state n and f at plane j+1 (ring threads inside mi)
    float rd[ND], rf = 0.0f;
    bool rmi = false;
    auto fetch_dual = [&](long z, unsigned mb) {
        rmi = ring1 && z >= 1 && z + 1 < nz && (mb & 2u);
        const size_t l = col + nxny * (size_t)(rmi ? z : 0);
        if (rmi) {
            load_dual<TGV>(s, l, rd);
            rf = __ldg(s.f + l);
        } else {
#pragma unroll
            for (int q = 0; q < ND; ++q) rd[q] = 0.0f;
            rf = 0.0f;
        }
    };
    //   iterate n at plane j (primal of the next step), owned threads inside m
    float rpc[NB];
    bool rpm = false;
    auto fetch_primal = [&](long z, unsigned mb) {
        rpm = owned && z >= zs && z < ze && (mb & 1u);
        const size_t l = col + nxny * (size_t)(rpm ? z : 0);
        if (rpm) {
            load_primal<TGV>(s.Pc, s.Pc1, l, rpc);
        } else {
#pragma unroll
            for (int q = 0; q < NB; ++q) rpc[q] = 0.0f;
        }
    };

    // mask ring: byte k of mr = mask of plane j+k (k = 0..3) at step j;
    // mnext = plane j+4, loaded one step earlier
    unsigned mr = 0;
    for (int k = 0; k < 4; ++k) mr |= mask_at(zs - 1 + k) << (8 * k);
    unsigned mnext = mask_at(zs + 3);

    // registers: extragradient point of planes j-1, j, j+1 (own column)
    float bm[NB], b0[NB], bp[NB];
    fetch_bars(zs - 2, mask_at(zs - 2));
    make_bars(bm);
    fetch_bars(zs - 1, mr & 0xffu);
    make_bars(b0);
#pragma unroll
    for (int q = 0; q < NB; ++q) B[q * NT + tid] = b0[q];  // plane zs - 1: buffer of step 0
    if (SPLIT && tid == 0)
        for (int q = 0; q < 3; ++q) mbar_init(sbar + q, NT);
    fetch_bars(zs, (mr >> 8) & 0xffu);
    fetch_dual(zs - 1, mr & 0xffu);
    // own dual of planes j-1 (vp) and j-2 (the z-1 neighbours of the primal
    // at j-1), kept in registers: the primal reads only x/y neighbours from
    // shared memory
    float vp[ND];
#pragma unroll
    for (int q = 0; q < ND; ++q) vp[q] = 0.0f;
    float nu_m2 = 0.f, p3_m2 = 0.f, q3_m2 = 0.f, q5_m2 = 0.f, q6_m2 = 0.f;
    bool waited = true;
    __syncthreads();

    for (long j = zs - 1; j <= ze; ++j) {
        const int k = (int)(j - (zs - 1));                      // step
        float *Bj = B + (k % P) * NB * NT;                      // extragradient of plane j (step k-1)
        float *Bn = B + ((k + 1) % P) * NB * NT;                // plane j+1 (written now)
        float *Sj = S + (k % P) * ND * NT;                      // dual of plane j (written now)
        const float *Sm = S + ((k + P - 1) % P) * ND * NT;      // dual of plane j-1 (step k-1)

        // (a) extragradient point of plane j+1 (fetched last step); fetch plane j+2.  Its buffer
        // was last read by step k-2, which every thread finished before step k-1's arrival.
        make_bars(bp);
#pragma unroll
        for (int q = 0; q < NB; ++q) Bn[q * NT + tid] = bp[q];
        const unsigned mfar = mask_at(j + 5);
        fetch_bars(j + 2, (mr >> 16) & 0xffu);
        // the x/y neighbours of plane j come from step k-1
        if (SPLIT && k > 0 && !mbar_wait(sbar + (k - 1) % 3, (uint32_t)(((k - 1) / 3) & 1), kColumnWaitLimit))
            waited = false;

        // (b) dual at plane j from the state fetched last step; fetch plane j+1
        float v[ND];
        const bool do_dual = rmi;
        float dcur[ND], fcur = rf;
#pragma unroll
        for (int q = 0; q < ND; ++q) dcur[q] = rd[q];
        // the primal's iterate of plane j-1 (fetched last step)
        float pcur[NB];
        const bool do_primal = rpm;
#pragma unroll
        for (int q = 0; q < NB; ++q) pcur[q] = rpc[q];
        fetch_dual(j + 1, (mr >> 8) & 0xffu);
        fetch_primal(j, mr & 0xffu);
#pragma unroll
        for (int q = 0; q < ND; ++q) v[q] = 0.0f;
        if (do_dual) {
            const size_t l = col + nxny * (size_t)j;
            const float c0 = b0[0];
            const float cxm = Bj[tid - 1], cxp = Bj[tid + 1], cym = Bj[tid - WX], cyp = Bj[tid + WX];
            const float czm = bm[0], czp = bp[0];
            const float *E = Bj + NT;
            const float lap = dc.lhh * b0[1] + dc.lhx * (E[tid - 1] + E[tid + 1]) +
                              dc.lhy * (E[tid - WX] + E[tid + WX]) + dc.lhz * (bm[1] + bp[1]);
            const float wav = dc.whh * c0 + dc.whx * (cxm + cxp) + dc.why * (cym + cyp) + dc.whz * (czm + czp);
            v[0] = dcur[0] + ((lap - wav) + fcur);
            if (TGV) {
                const float w1 = b0[2], w2 = b0[3], w3 = b0[4];
                float a1 = dcur[1] + dc.hx * (cxp - c0) - dc.sg * w1;
                float a2 = dcur[2] + dc.hy * (cyp - c0) - dc.sg * w2;
                float a3 = dcur[3] + dc.hz * (czp - c0) - dc.sg * w3;
                float t = a1 * a1 + a2 * a2 + a3 * a3;
                if (t > dc.alp12) {
                    t = dc.alp1 / sqrtf(t);
                    a1 = a1 * t; a2 = a2 * t; a3 = a3 * t;
                }
                v[1] = a1; v[2] = a2; v[3] = a3;
                const float *W1 = Bj + 2 * NT, *W2 = Bj + 3 * NT, *W3 = Bj + 4 * NT;
                const float w1x = W1[tid + 1], w1y = W1[tid + WX], w1z = bp[2];
                const float w2x = W2[tid + 1], w2y = W2[tid + WX], w2z = bp[3];
                const float w3x = W3[tid + 1], w3y = W3[tid + WX], w3z = bp[4];
                float r1 = dcur[4] + dc.hx * (w1x - w1);
                float r2 = dcur[5] + dc.hx2 * (w2x - w2) + dc.hy2 * (w1y - w1);
                float r3 = dcur[6] + dc.hx2 * (w3x - w3) + dc.hz2 * (w1z - w1);
                float r4 = dcur[7] + dc.hy * (w2y - w2);
                float r5 = dcur[8] + dc.hy2 * (w3y - w3) + dc.hz2 * (w2z - w2);
                float r6 = dcur[9] + dc.hz * (w3z - w3);
                t = r1 * r1 + r4 * r4 + r6 * r6 + 2.0f * (r2 * r2 + r3 * r3 + r5 * r5);
                if (t > dc.alp02) {
                    t = dc.alp0 / sqrtf(t);
                    r1 = r1 * t; r2 = r2 * t; r3 = r3 * t; r4 = r4 * t; r5 = r5 * t; r6 = r6 * t;
                }
                v[4] = r1; v[5] = r2; v[6] = r3; v[7] = r4; v[8] = r5; v[9] = r6;
            } else {
                float a1 = dcur[1] + dc.hx * (cxp - c0);
                float a2 = dcur[2] + dc.hy * (cyp - c0);
                float a3 = dcur[3] + dc.hz * (czp - c0);
                float t = a1 * a1 + a2 * a2 + a3 * a3;
                if (t > dc.alp12) {
                    t = dc.alp1 / sqrtf(t);
                    a1 = a1 * t; a2 = a2 * t; a3 = a3 * t;
                }
                v[1] = a1; v[2] = a2; v[3] = a3;
            }
            if (owned && j >= zs && j < ze) store_dual<TGV>(s, l, v);
        }
#pragma unroll
        for (int q = 0; q < ND; ++q) Sj[q * NT + tid] = v[q];
        if (SPLIT) mbar_arrive(sbar + k % 3);

        // (c) primal + extragradient at plane j-1
        if (do_primal) {
            const size_t l = col + nxny * (size_t)(j - 1);
            const float nu0 = vp[0];
            const float xs = Sm[tid - 1] + Sm[tid + 1];
            const float ys = Sm[tid - WX] + Sm[tid + WX];
            const float zs_ = nu_m2 + v[0];
            const float cn = pcur[0], en = pcur[1];
            const float e1 = pc.tau1 * (en - pc.lhh * nu0 - pc.lhx * xs - pc.lhy * ys - pc.lhz * zs_);
            const float *P1 = Sm + NT, *P2 = Sm + 2 * NT;  // p3's z-neighbour comes from registers
            const float c1 = cn + (pc.hx * (vp[1] - P1[tid - 1]) + pc.hy * (vp[2] - P2[tid - WX]) +
                                   pc.hz * (vp[3] - p3_m2) +
                                   (pc.whh * nu0 + pc.whx * xs + pc.why * ys + pc.whz * zs_));
            float pv[NB];
            pv[0] = c1;
            pv[1] = e1;
            if (TGV) {
                const float *Q1 = Sm + 4 * NT, *Q2 = Sm + 5 * NT, *Q3 = Sm + 6 * NT, *Q4 = Sm + 7 * NT,
                            *Q5 = Sm + 8 * NT;  // q6 is only read along z (registers)
                const float u1 = pcur[2] + (pc.tt * vp[1] + pc.hx * (vp[4] - Q1[tid - 1] + vp[5] - Q2[tid - WX] +
                                                                      vp[6] - q3_m2));
                const float u2 = pcur[3] + (pc.tt * vp[2] + pc.hy * (vp[5] - Q2[tid - 1] + vp[7] - Q4[tid - WX] +
                                                                      vp[8] - q5_m2));
                const float u3 = pcur[4] + (pc.tt * vp[3] + pc.hz * (vp[6] - Q3[tid - 1] + vp[8] - Q5[tid - WX] +
                                                                      vp[9] - q6_m2));
                pv[2] = u1;
                pv[3] = u2;
                pv[4] = u3;
            }
            store_primal<TGV>(s.Pn, s.Pn1, l, pv);
            if (check) {
                mon[0].add(c1 * c1);
                mon[1].add(e1 * e1);
                mon[2].add((c1 - cn) * (c1 - cn));
                mon[3].add((e1 - en) * (e1 - en));
            }
        }
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            bm[q] = b0[q];
            b0[q] = bp[q];
        }
        nu_m2 = vp[0];
        p3_m2 = vp[3];
        if (TGV) {
            q3_m2 = vp[6];
            q5_m2 = vp[8];
            q6_m2 = vp[9];
        }
#pragma unroll
        for (int q = 0; q < ND; ++q) vp[q] = v[q];
        mr = (mr >> 8) | (mnext << 24);
        mnext = mfar;
        if (!SPLIT) __syncthreads();
    }
    if (SPLIT) {
        if (!waited) atomicOr(&s.ctl->stalled, 1u);
        // every thread's last arrival is in: the barriers are retired before the
        // shared memory is used again
        __syncthreads();
        if (tid == 0)
            for (int q = 0; q < 3; ++q) mbar_inval(sbar + q);
        __syncthreads();
    }
    if (check)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] += mon[q].get();
}

}  // namespace qsm
