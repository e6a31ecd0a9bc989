// Column tile of the fused TGV/TV iteration with asynchronous staging
// (cp.async) of the state two planes ahead.
//
// The arithmetic, the thread layout ((TX+4) x (TY+4) threads: a TX x TY
// column tile plus a two-voxel ring) and the plane walk are those of
// column_pd (pd_tile.cuh).  What changes is how the inputs arrive: each
// thread copies the values of its own column that it will need
//   - iterate n and n-1 of plane j+3 (extragradient at step j+2),
//   - dual state n and f of plane j+2 (dual at step j+2),
// straight from global into shared-memory rings with cp.async at step j,
// and waits for them two steps later.  The copies occupy no registers and
// cannot be moved next to their use by the compiler, so two planes of HBM
// latency are covered by the intervening arithmetic; a thread reads back
// only what it copied itself, so no barrier is needed for them.  Voxels
// outside the mask are zero-filled by the copy (src-size 0: nothing is
// read from HBM), which is the value the state has there.  Iterate n stays
// in its ring for five planes, so the primal of plane j-1 reads it from
// shared memory too.
//
// Shared memory (floats): B [2][NB][NT], S [2][ND][NT] as in column_pd,
// PC [5][NB][NT] (iterate n), PP [3][NB][NT] (iterate n-1),
// DQ [3][ND+1][NT] (dual state n, f).
#pragma once

#include <math.h>

#include "common.cuh"
#include "pd.cuh"
#include "pd_fused.cuh"

namespace qsm {

__device__ __forceinline__ void cp_async4(float *dst, const float *src, bool ok)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(ok ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <bool TGV>
constexpr size_t async_smem_floats(int tx, int ty)
{
    return (size_t)(tx + 4) * (ty + 4) * ((2 + 5) * (TGV ? 5 : 2) + 2 * (TGV ? 10 : 4) + 3 * (TGV ? 5 : 2) +
                                           3 * ((TGV ? 10 : 4) + 1));
}

template <int TX, int TY, bool TGV>
__device__ __forceinline__ void column_async(const FusedArgs &s, const DualC<float> &dc, const PrimalC<float> &pc,
                                             const Dims &d, int cz, unsigned tile, bool check, float *smem,
                                             double *acc)
{
    constexpr int WX = TX + 4, WY = TY + 4, NT = WX * WY;
    constexpr int NB = TGV ? 5 : 2;   // primal family: chi, eta, w1..3
    constexpr int ND = TGV ? 10 : 4;  // dual family: nu, p1..3, q1..6
    constexpr int DIST = 2;           // steps between a copy and its use
    float *B = smem;                  // [2][NB][NT]  extragradient point of one plane
    float *S = B + 2 * NB * NT;       // [2][ND][NT]  dual of one plane
    float *PC = S + 2 * ND * NT;      // [5][NB][NT]  iterate n of planes mod 5
    float *PP = PC + 5 * NB * NT;     // [3][NB][NT]  iterate n-1 of planes mod 3
    float *DQ = PP + 3 * NB * NT;     // [3][ND+1][NT] dual state n and f of planes mod 3

    const long x0 = 1 + (long)(tile % s.gx) * TX, y0 = 1 + (long)((tile / s.gx) % s.gy) * TY;
    const long zs = 1 + (long)(tile / (s.gx * s.gy)) * cz;
    const long ze = min(zs + (long)cz, (long)d.nz - 1);
    const int tid = threadIdx.x, tx = tid % WX, ty = tid / WX;
    const long x = x0 - 2 + tx, y = y0 - 2 + ty;
    const bool valid = x >= 0 && y >= 0 && x < (long)d.nx && y < (long)d.ny;
    const bool ring1 = tx >= 1 && tx <= TX + 2 && ty >= 1 && ty <= TY + 2;  // the dual is evaluated here
    const bool owned = tx >= 2 && tx <= TX + 1 && ty >= 2 && ty <= TY + 1 && x + 1 < (long)d.nx && y + 1 < (long)d.ny;
    const size_t nxny = d.nxny();
    const size_t col = valid ? (size_t)x + d.nx * (size_t)y : 0;
    const long nz = (long)d.nz;
    auto slot5 = [](long p) { return (int)((p + 5) % 5); };
    auto slot3 = [](long p) { return (int)((p + 3) % 3); };

    // mask bytes of the own column, planes p (0 outside the volume)
    auto mask_at = [&](long p) -> unsigned {
        return (valid && p >= 0 && p < nz) ? (unsigned)__ldg(s.mm + col + nxny * (size_t)p) : 0u;
    };
    // copies of iterate n, n-1 at plane p (zero-filled outside m)
    auto issue_primal = [&](long p, unsigned mb) {
        const bool ok = (mb & 1u) != 0;
        const size_t l = col + nxny * (size_t)(ok ? p : 0);
        float *pc5 = PC + slot5(p) * NB * NT + tid, *pp3 = PP + slot3(p) * NB * NT + tid;
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            cp_async4(pc5 + q * NT, s.Pc[q] + l, ok);
            cp_async4(pp3 + q * NT, s.Pp[q] + l, ok);
        }
    };
    // copies of the dual state n and f at plane p (ring threads inside mi)
    auto issue_dual = [&](long p, unsigned mb) {
        if (!(ring1 && p >= 1 && p + 1 < nz && (mb & 2u))) return;
        const size_t l = col + nxny * (size_t)p;
        float *dq = DQ + slot3(p) * (ND + 1) * NT + tid;
#pragma unroll
        for (int q = 0; q < ND; ++q) cp_async4(dq + q * NT, s.Dc[q] + l, true);
        cp_async4(dq + ND * NT, s.f + l, true);
    };

    // mask ring: byte k of mr = mask of plane j-1+k (k = 0..4) at step j
    unsigned long long mr = 0;
    for (int k = 0; k < 5; ++k) mr |= (unsigned long long)mask_at(zs - 2 + k) << (8 * k);
    unsigned mnext = mask_at(zs + 3);  // plane j+4 for the first step

    // extragradient of planes zs-2, zs-1 (own column), read directly
    float bm[NB], b0[NB];
    {
        const unsigned m2 = mask_at(zs - 2), m1 = mask_at(zs - 1);
        const size_t l2 = col + nxny * (size_t)((m2 & 1u) ? zs - 2 : 0), l1 = col + nxny * (size_t)((m1 & 1u) ? zs - 1 : 0);
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const float c2 = (m2 & 1u) ? __ldg(s.Pc[q] + l2) : 0.0f, p2 = (m2 & 1u) ? __ldg(s.Pp[q] + l2) : 0.0f;
            const float c1 = (m1 & 1u) ? __ldg(s.Pc[q] + l1) : 0.0f, p1 = (m1 & 1u) ? __ldg(s.Pp[q] + l1) : 0.0f;
            bm[q] = (m2 & 1u) ? c2 + 1.0f * (c2 - p2) : 0.0f;
            b0[q] = (m1 & 1u) ? c1 + 1.0f * (c1 - p1) : 0.0f;
        }
        float *Bw = B + ((zs - 1) & 1) * NB * NT;
#pragma unroll
        for (int q = 0; q < NB; ++q) Bw[q * NT + tid] = b0[q];
    }
    // the copies the first two steps consume: planes zs, zs+1 (primal), zs-1, zs (dual)
    issue_primal(zs, (unsigned)(mr >> 16) & 0xffu);
    issue_dual(zs - 1, (unsigned)(mr >> 8) & 0xffu);
    cp_async_commit();
    issue_primal(zs + 1, (unsigned)(mr >> 24) & 0xffu);
    issue_dual(zs, (unsigned)(mr >> 16) & 0xffu);
    cp_async_commit();
    // own dual values of plane j-2 (the primal at j-1 reads them as z-1 neighbours)
    float nu_m2 = 0.f, p3_m2 = 0.f, q3_m2 = 0.f, q5_m2 = 0.f, q6_m2 = 0.f;
    __syncthreads();

    for (long j = zs - 1; j <= ze; ++j) {
        float *Bj = B + (j & 1) * NB * NT;              // extragradient of plane j (written last step)
        float *Bn = B + ((j + 1) & 1) * NB * NT;        // plane j+1 (written now)
        float *Sj = S + (j & 1) * ND * NT;              // dual of plane j (written now; held plane j-2)
        const float *Sm = S + ((j + 1) & 1) * ND * NT;  // dual of plane j-1
        // masks of planes j-1 .. j+3
        const unsigned mj_1 = (unsigned)mr & 0xffu, mj = (unsigned)(mr >> 8) & 0xffu;

        // copies for plane j+3 (iterates) and j+2 (dual state); fetch the mask of plane j+5
        issue_primal(j + 1 + DIST, (unsigned)(mr >> 32) & 0xffu);
        issue_dual(j + DIST, (unsigned)(mr >> 24) & 0xffu);
        cp_async_commit();
        const unsigned mfar = mask_at(j + 5);
        cp_async_wait<DIST>();  // this thread's copies for planes j+1 (iterates) and j (dual state) landed

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

        // (a) extragradient point of plane j+1
        float bp[NB];
        {
            const float *c5 = PC + slot5(j + 1) * NB * NT + tid, *p3 = PP + slot3(j + 1) * NB * NT + tid;
#pragma unroll
            for (int q = 0; q < NB; ++q) {
                const float c = c5[q * NT];
                bp[q] = c + 1.0f * (c - p3[q * NT]);
                Bn[q * NT + tid] = bp[q];
            }
        }

        // (b) dual at plane j
        float v[ND];
#pragma unroll
        for (int q = 0; q < ND; ++q) v[q] = 0.0f;
        const bool do_dual = ring1 && valid && j >= 1 && j + 1 < nz && (mj & 2u);
        if (do_dual) {
            const float *dq = DQ + slot3(j) * (ND + 1) * NT + tid;
            const size_t l = col + nxny * (size_t)j;
            const float c0 = b0[0];
            const float cxm = Bj[tid - 1], cxp = Bj[tid + 1], cym = Bj[tid - WX], cyp = Bj[tid + WX];
            const float czm = bm[0], czp = bp[0];
            const float *E = Bj + NT;
            const float lap = dc.lhh * b0[1] + dc.lhx * (E[tid - 1] + E[tid + 1]) +
                              dc.lhy * (E[tid - WX] + E[tid + WX]) + dc.lhz * (bm[1] + bp[1]);
            const float wav = dc.whh * c0 + dc.whx * (cxm + cxp) + dc.why * (cym + cyp) + dc.whz * (czm + czp);
            v[0] = dq[0] + ((lap - wav) + dq[ND * NT]);
            if (TGV) {
                const float w1 = b0[2], w2 = b0[3], w3 = b0[4];
                float a1 = dq[1 * NT] + dc.hx * (cxp - c0) - dc.sg * w1;
                float a2 = dq[2 * NT] + dc.hy * (cyp - c0) - dc.sg * w2;
                float a3 = dq[3 * NT] + dc.hz * (czp - c0) - dc.sg * w3;
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
                float r1 = dq[4 * NT] + dc.hx * (w1x - w1);
                float r2 = dq[5 * NT] + dc.hx2 * (w2x - w2) + dc.hy2 * (w1y - w1);
                float r3 = dq[6 * NT] + dc.hx2 * (w3x - w3) + dc.hz2 * (w1z - w1);
                float r4 = dq[7 * NT] + dc.hy * (w2y - w2);
                float r5 = dq[8 * NT] + dc.hy2 * (w3y - w3) + dc.hz2 * (w2z - w2);
                float r6 = dq[9 * NT] + dc.hz * (w3z - w3);
                t = r1 * r1 + r4 * r4 + r6 * r6 + 2.0f * (r2 * r2 + r3 * r3 + r5 * r5);
                if (t > dc.alp02) {
                    t = dc.alp0 / sqrtf(t);
                    r1 = r1 * t; r2 = r2 * t; r3 = r3 * t; r4 = r4 * t; r5 = r5 * t; r6 = r6 * t;
                }
                v[4] = r1; v[5] = r2; v[6] = r3; v[7] = r4; v[8] = r5; v[9] = r6;
            } else {
                float a1 = dq[1 * NT] + dc.hx * (cxp - c0);
                float a2 = dq[2 * NT] + dc.hy * (cyp - c0);
                float a3 = dq[3 * NT] + dc.hz * (czp - c0);
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
        if (owned && j - 1 >= zs && j - 1 < ze && (mj_1 & 1u)) {
            const float *pn = PC + slot5(j - 1) * NB * NT + tid;
            const size_t l = col + nxny * (size_t)(j - 1);
            const float nu0 = Sm[tid];
            const float xs = Sm[tid - 1] + Sm[tid + 1];
            const float ys = Sm[tid - WX] + Sm[tid + WX];
            const float zs_ = nu_m2 + v[0];
            const float cn = pn[0], en = pn[NT];
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
                const float u1 = pn[2 * NT] + (pc.tt * P1[tid] + pc.hx * (Q1[tid] - Q1[tid - 1] + Q2[tid] - Q2[tid - WX] +
                                                                           Q3[tid] - q3_m2));
                const float u2 = pn[3 * NT] + (pc.tt * P2[tid] + pc.hy * (Q2[tid] - Q2[tid - 1] + Q4[tid] - Q4[tid - WX] +
                                                                           Q5[tid] - q5_m2));
                const float u3 = pn[4 * NT] + (pc.tt * P3[tid] + pc.hz * (Q3[tid] - Q3[tid - 1] + Q5[tid] - Q5[tid - WX] +
                                                                           Q6[tid] - q6_m2));
                s.Pn[2][l] = u1;
                s.Pn[3][l] = u2;
                s.Pn[4][l] = u3;
            }
            if (check) {
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
        mr = (mr >> 8) | ((unsigned long long)mnext << 32);
        mnext = mfar;
        __syncthreads();
    }
    cp_async_wait<0>();  // copies for planes past the chunk: land before shared memory is reused
    __syncthreads();
}

}  // namespace qsm
