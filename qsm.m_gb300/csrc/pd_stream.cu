// Primal-dual TGV / TV, mixed-precision fused path: z-streaming kernel.
//
// A CTA owns a TX x TY column tile of the interior and a chunk of planes
// [zs, ze).  Its (TX+4) x (TY+4) threads map one-to-one onto the tile plus a
// two-voxel ring; each thread walks its column upwards one plane per step:
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
//            one __syncthreads
//
// so every input value of a plane is read from HBM once per CTA (the ring
// re-reads neighbouring tiles' edges, mostly from L2) and the dual is
// evaluated once per plane and column (plus the ring), not on a 3-D halo.
// Only the two planes below a chunk are recomputed.  Voxels outside the
// mask are skipped (their state is identically 0).
//
// Per voxel the FP32 expressions are those of pd_tgv_mex.c:332-485 and
// :659-812 (TV: pd_tv_mex.c:314-412, :524-622) in the reference's order,
// built without fused multiply-add: chi is bit-identical to mx_pdf.
#include <math.h>

#include "common.cuh"
#include "pd.cuh"
#include "pd_fused.cuh"

namespace qsm {

template <int TX, int TY, bool TGV, bool CHECK>
__global__ void __launch_bounds__((TX + 4) * (TY + 4), 1)
stream_k(FusedArgs s, DualC<float> dc, PrimalC<float> pc, Dims d, int cz, double tol, uint32_t it)
{
    constexpr int WX = TX + 4, WY = TY + 4, NT = WX * WY;
    constexpr int NB = TGV ? 5 : 2;   // extragradient arrays: chi_, eta_, w1_, w2_, w3_
    constexpr int ND = TGV ? 10 : 4;  // dual arrays: nu, p1..3, q1..6
    extern __shared__ double smem_raw[];
    float *B = (float *)smem_raw;     // [2][NB][NT]  extragradient point of one plane
    float *S = B + 2 * NB * NT;       // [2][ND][NT]  dual of one plane
    if (s.ctl->done) return;

    const unsigned tile = s.tiles[blockIdx.x];
    const long x0 = 1 + (long)(tile % s.gx) * TX, y0 = 1 + (long)((tile / s.gx) % s.gy) * TY;
    const long zs = 1 + (long)(tile / (s.gx * s.gy)) * cz;
    const long ze = min(zs + (long)cz, (long)d.nz - 1);
    const int tid = threadIdx.x, tx = tid % WX, ty = tid / WX;
    const long x = x0 - 2 + tx, y = y0 - 2 + ty;
    const bool valid = x >= 0 && y >= 0 && x < (long)d.nx && y < (long)d.ny;
    const bool ring1 = tx >= 1 && tx <= TX + 2 && ty >= 1 && ty <= TY + 2;  // dual is evaluated here
    const bool owned = tx >= 2 && tx <= TX + 1 && ty >= 2 && ty <= TY + 1 && x + 1 < (long)d.nx && y + 1 < (long)d.ny;
    const size_t nxny = d.nxny();
    const size_t col = valid ? (size_t)x + d.nx * (size_t)y : 0;
    const long nz = (long)d.nz;

    // Every global input is fetched one plane step before it is used, so the
    // memory latency of a plane overlaps the arithmetic of the previous one.
    //   raw iterates n, n-1 (+ mask bit m) of the own column, plane j+2
    float rc[NB], rp[NB];
    bool rm = false;
    auto fetch_bars = [&](long z) {
        rm = valid && z >= 0 && z < nz && (__ldg(s.mm + col + nxny * (size_t)z) & 1);
        const size_t l = col + nxny * (size_t)(rm ? z : 0);  // an in-bounds address even when unused
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            rc[q] = rm ? __ldg(s.Pc[q] + l) : 0.0f;
            rp[q] = rm ? __ldg(s.Pp[q] + l) : 0.0f;
        }
    };
    auto make_bars = [&](float *v) {
#pragma unroll
        for (int q = 0; q < NB; ++q) v[q] = rm ? rc[q] + 1.0f * (rc[q] - rp[q]) : 0.0f;
    };
    //   dual state n and f at plane j+1 (ring threads inside mi)
    float rd[ND], rf = 0.0f;
    bool rmi = false;
    auto fetch_dual = [&](long z) {
        rmi = ring1 && valid && z >= 1 && z + 1 < nz && (__ldg(s.mm + col + nxny * (size_t)z) & 2);
        const size_t l = col + nxny * (size_t)(rmi ? z : 0);
#pragma unroll
        for (int q = 0; q < ND; ++q) rd[q] = rmi ? __ldg(s.Dc[q] + l) : 0.0f;
        rf = rmi ? __ldg(s.f + l) : 0.0f;
    };
    //   iterate n at plane j (primal of the next step), owned threads inside m
    float rpc[NB];
    bool rpm = false;
    auto fetch_primal = [&](long z) {
        rpm = owned && z >= zs && z < ze && (__ldg(s.mm + col + nxny * (size_t)z) & 1);
        const size_t l = col + nxny * (size_t)(rpm ? z : 0);
#pragma unroll
        for (int q = 0; q < NB; ++q) rpc[q] = rpm ? __ldg(s.Pc[q] + l) : 0.0f;
    };

    // registers: extragradient point of planes j-1, j, j+1 (own column)
    float bm[NB], b0[NB], bp[NB];
    fetch_bars(zs - 2);
    make_bars(bm);
    fetch_bars(zs - 1);
    make_bars(b0);
    {
        float *Bw = B + ((zs - 1) & 1) * NB * NT;
#pragma unroll
        for (int q = 0; q < NB; ++q) Bw[q * NT + tid] = b0[q];
    }
    fetch_bars(zs);
    fetch_dual(zs - 1);
    // own dual of plane j-2 (read by the primal at j-1 through its z-1 neighbour)
    float nu_m2 = 0.f, p3_m2 = 0.f, q3_m2 = 0.f, q5_m2 = 0.f, q6_m2 = 0.f;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    __syncthreads();

    for (long j = zs - 1; j <= ze; ++j) {
        float *Bj = B + (j & 1) * NB * NT;              // extragradient of plane j (written last step)
        float *Bn = B + ((j + 1) & 1) * NB * NT;        // plane j+1 (written now)
        float *Sj = S + (j & 1) * ND * NT;              // dual of plane j (written now; held plane j-2)
        const float *Sm = S + ((j + 1) & 1) * ND * NT;  // dual of plane j-1

        // own dual values of plane j-2 before plane j overwrites them
        if (owned && j - 1 >= zs) {
            nu_m2 = Sj[tid];
            p3_m2 = Sj[3 * NT + tid];
            if (TGV) {
                q3_m2 = Sj[6 * NT + tid];
                q5_m2 = Sj[8 * NT + tid];
                q6_m2 = Sj[9 * NT + tid];
            }
        }

        // (a) extragradient point of plane j+1 (fetched last step); fetch plane j+2
        make_bars(bp);
#pragma unroll
        for (int q = 0; q < NB; ++q) Bn[q * NT + tid] = bp[q];
        fetch_bars(j + 2);

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
        fetch_dual(j + 1);
        fetch_primal(j);
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
            if (owned && j >= zs && j < ze) {
#pragma unroll
                for (int q = 0; q < ND; ++q) s.Dn[q][l] = v[q];
            }
        }
#pragma unroll
        for (int q = 0; q < ND; ++q) Sj[q * NT + tid] = v[q];

        // (c) primal + extragradient at plane j-1
        if (do_primal) {
            const size_t l = col + nxny * (size_t)(j - 1);
            const float nu0 = Sm[tid];
            const float xs = Sm[tid - 1] + Sm[tid + 1];
            const float ys = Sm[tid - WX] + Sm[tid + WX];
            const float zs_ = nu_m2 + v[0];
            const float cn = pcur[0], en = pcur[1];
            const float e1 = pc.tau1 * (en - pc.lhh * nu0 - pc.lhx * xs - pc.lhy * ys - pc.lhz * zs_);
            const float *P1 = Sm + NT, *P2 = Sm + 2 * NT, *P3 = Sm + 3 * NT;
            const float c1 = cn + (pc.hx * (P1[tid] - P1[tid - 1]) + pc.hy * (P2[tid] - P2[tid - WX]) +
                                   pc.hz * (P3[tid] - p3_m2) +
                                   (pc.whh * nu0 + pc.whx * xs + pc.why * ys + pc.whz * zs_));
            s.Pn[0][l] = c1;
            s.Pn[1][l] = e1;
            if (TGV) {
                const float *Q1 = Sm + 4 * NT, *Q2 = Sm + 5 * NT, *Q3 = Sm + 6 * NT, *Q4 = Sm + 7 * NT,
                            *Q5 = Sm + 8 * NT, *Q6 = Sm + 9 * NT;
                const float u1 = pcur[2] + (pc.tt * P1[tid] + pc.hx * (Q1[tid] - Q1[tid - 1] + Q2[tid] - Q2[tid - WX] +
                                                                        Q3[tid] - q3_m2));
                const float u2 = pcur[3] + (pc.tt * P2[tid] + pc.hy * (Q2[tid] - Q2[tid - 1] + Q4[tid] - Q4[tid - WX] +
                                                                        Q5[tid] - q5_m2));
                const float u3 = pcur[4] + (pc.tt * P3[tid] + pc.hz * (Q3[tid] - Q3[tid - 1] + Q5[tid] - Q5[tid - WX] +
                                                                        Q6[tid] - q6_m2));
                s.Pn[2][l] = u1;
                s.Pn[3][l] = u2;
                s.Pn[4][l] = u3;
            }
            if (CHECK) {
                double a, b, c, e;
                mon_terms(c1, cn, e1, en, a, b, c, e);
                acc[0] += a; acc[1] += b; acc[2] += c; acc[3] += e;
            }
        }
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            bm[q] = b0[q];
            b0[q] = bp[q];
        }
        __syncthreads();
    }
    if (CHECK) monitor_reduce<NT>(s, smem_raw, acc, tol, it);
}

size_t stream_smem(int tx, int ty, bool tgv)
{
    const size_t nt = (size_t)(tx + 4) * (ty + 4);
    const size_t planes = 2 * ((tgv ? 5 : 2) + (tgv ? 10 : 4)) * nt * sizeof(float);
    return std::max(planes, 4 * nt * sizeof(double));
}

template <int TX, int TY>
static qsm_status set_t(qsm_ctx *ctx)
{
    const int t = (int)stream_smem(TX, TY, true), v = (int)stream_smem(TX, TY, false);
    QSM_CUDA(cudaFuncSetAttribute(stream_k<TX, TY, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, t));
    QSM_CUDA(cudaFuncSetAttribute(stream_k<TX, TY, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, t));
    QSM_CUDA(cudaFuncSetAttribute(stream_k<TX, TY, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, v));
    QSM_CUDA(cudaFuncSetAttribute(stream_k<TX, TY, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, v));
    return QSM_OK;
}

qsm_status stream_set_smem(qsm_ctx *ctx)
{
    QSM_TRY((set_t<28, 12>(ctx)));
    return QSM_OK;
}

template <int TX, int TY>
static void launch_t(qsm_ctx *ctx, bool tgv, bool chk, unsigned nact, const FusedArgs &s, const DualC<float> &dc,
                     const PrimalC<float> &pc, const Dims &d, int cz, double tol, uint32_t it)
{
    const size_t sm = stream_smem(TX, TY, tgv);
    const int nt = (TX + 4) * (TY + 4);
    if (tgv) {
        if (chk) stream_k<TX, TY, true, true><<<nact, nt, sm, ctx->stream>>>(s, dc, pc, d, cz, tol, it);
        else stream_k<TX, TY, true, false><<<nact, nt, sm, ctx->stream>>>(s, dc, pc, d, cz, tol, it);
    } else {
        if (chk) stream_k<TX, TY, false, true><<<nact, nt, sm, ctx->stream>>>(s, dc, pc, d, cz, tol, it);
        else stream_k<TX, TY, false, false><<<nact, nt, sm, ctx->stream>>>(s, dc, pc, d, cz, tol, it);
    }
}

qsm_status stream_launch(qsm_ctx *ctx, int tx, int ty, int cz, bool tgv, bool chk, unsigned nact, const FusedArgs &s,
                         const DualC<float> &dc, const PrimalC<float> &pc, const Dims &d, double tol, uint32_t it)
{
    if (tx == 28 && ty == 12) launch_t<28, 12>(ctx, tgv, chk, nact, s, dc, pc, d, cz, tol, it);
    else return QSM_ERR_ARG;
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

}  // namespace qsm
