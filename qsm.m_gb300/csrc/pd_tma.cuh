// Fused TGV column body with TMA-staged primal iterates.
//
// The same column walk as column_pd (pd_tile.cuh): each of (TX+4)(TY+4)
// threads owns one column of a TX x TY tile plus a two-voxel ring and steps
// up the planes of a z-chunk, forming the extragradient point of plane j+1,
// the dual of plane j and the primal of plane j-1 per step, with one
// barrier per plane.  The difference is where the primal iterates come from:
// instead of every thread loading its column's iterates n and n-1 into
// registers a step ahead (26 registers of prefetched values, plus their
// address and mask arithmetic), one thread issues per plane four
// cp.async.bulk.tensor loads -- the (TX+4) x (TY+4) box of family A
// (chi, eta, w1, w2) and of family B (w3) at iterates n and n-1 -- into a
// ring of shared-memory plane slots that complete on an mbarrier:
//
//   iterate n:   4 slots (plane j+2 in flight, j+1 read for the
//                extragradient, j-1 read by the primal, j waiting for it)
//   iterate n-1: 2 slots (plane j+2 in flight, j+1 read)
//
// The loads bring whole boxes: outside the mask the iterates are zero in
// every buffer (nothing ever writes there), so the extragradient point there
// is computed as 0 + 1*(0 - 0) = +0 without a mask test, as the register
// path's select gives, and halo voxels outside the volume read the TMA's
// zero fill.  The dual state (needed only where mi holds) keeps its
// mask-selective register prefetch.  The freed registers let a 28 x 20 tile
// (768 threads, 24 warps per SM) run without spills.
//
// Family B is a float array: a box must start at a multiple of 4 elements,
// so its box starts at x rounded down to a multiple of 4 and is 4 wider.
// The per-voxel arithmetic and its order are column_pd's, so chi is
// bit-identical to it and to the reference's mx_pdf (update_dualf /
// update_primalf, pd_tgv_mex.c:332-485, :659-812).
//
// Waits on the plane barriers are bounded; a wait that gives up marks the
// solve (PdCtl::stalled) and the step continues, so every thread still
// reaches every __syncthreads and the kernel ends.
#pragma once

#include "pd_tile.cuh"
#include "tma.cuh"

namespace qsm {

constexpr size_t tma_al128(size_t b) { return (b + 127) & ~(size_t)127; }
constexpr uint32_t kTmaWaitLimit = 1u << 20;

template <int TX, int TY>
struct TmaLayout {
    static constexpr int WX = TX + 4, WY = TY + 4, NT = WX * WY;
    static constexpr int WB = WX + 4;  // family-B box width
    static constexpr int NA = 4, NP = 2;
    static constexpr uint32_t A_BYTES = NT * 16, B_BYTES = WB * WY * 4;
    static constexpr uint32_t PLANE_TX = 2 * (A_BYTES + B_BYTES);  // bytes of one plane's four loads
    static constexpr size_t SA = tma_al128(A_BYTES), SB = tma_al128(B_BYTES);
    static constexpr size_t O_BAR = 0;  // NA mbarriers
    static constexpr size_t O_AN = 128;
    static constexpr size_t O_BN = O_AN + NA * SA;
    static constexpr size_t O_AP = O_BN + NA * SB;
    static constexpr size_t O_BP = O_AP + NP * SA;
    static constexpr size_t O_X = O_BP + NP * SB;  // exchange buffers: [2][5][NT] + [2][10][NT] floats
    static constexpr size_t BYTES = O_X + 2 * 15 * (size_t)NT * sizeof(float);
    // dynamic shared memory to request: the layout plus room to align its base
    static constexpr size_t REQUEST = BYTES + 128;
};

// Aligns the dynamic shared memory base to 128 bytes (TMA destinations).
__device__ __forceinline__ char *tma_smem_base(unsigned char *raw)
{
    return (char *)raw + ((128u - (smem_addr(raw) & 127u)) & 127u);
}

template <int TX, int TY>
__device__ __forceinline__ void column_tma(const TmaMaps &tm, const FusedArgs &s, const DualC<float> &dc,
                                           const PrimalC<float> &pc, const Dims &d, int cz, unsigned tile,
                                           bool check, char *smem, double *acc)
{
    using L = TmaLayout<TX, TY>;
    constexpr int WX = L::WX, NT = L::NT, WB = L::WB;
    constexpr int NB = 5, ND = 10;
    uint64_t *bar = (uint64_t *)(smem + L::O_BAR);
    float *B = (float *)(smem + L::O_X);  // [2][NB][NT]  extragradient point of one plane
    float *S = B + 2 * NB * NT;           // [2][ND][NT]  dual of one plane
    const long x0 = 1 + (long)(tile % s.gx) * TX, y0 = 1 + (long)((tile / s.gx) % s.gy) * TY;
    const long zs = 1 + (long)(tile / (s.gx * s.gy)) * cz;
    const long ze = min(zs + (long)cz, (long)d.nz - 1);
    const int tid = threadIdx.x, tx = tid % WX, ty = tid / WX;
    const long x = x0 - 2 + tx, y = y0 - 2 + ty;
    const int xa = (int)(x0 - 2), ya = (int)(y0 - 2);
    const int xb = xa & ~3;             // family-B box start (a multiple of 4; may be -4)
    const int bi = ty * WB + tx + (xa - xb);  // own column in a family-B box
    PartialSum<float> mon[4];
    const bool valid = x >= 0 && y >= 0 && x < (long)d.nx && y < (long)d.ny;
    const bool ring1 = tx >= 1 && tx <= TX + 2 && ty >= 1 && ty <= TY + 2;  // dual is evaluated here
    const bool owned = tx >= 2 && tx <= TX + 1 && ty >= 2 && ty <= TY + 1 && x + 1 < (long)d.nx && y + 1 < (long)d.ny;
    const size_t nxny = d.nxny();
    const size_t col = valid ? (size_t)x + d.nx * (size_t)y : 0;
    const long nz = (long)d.nz;
    const long q0 = zs - 2;  // plane of the first load; a plane's slot follows from p - q0
    bool ok = true;

    auto issue = [&](long p) {  // thread 0: the four loads of plane p
        const long q = p - q0;
        const int sa = (int)(q & 3), sp = (int)(q & 1);
        uint64_t *b = bar + sa;
        mbar_arrive_expect_tx(b, L::PLANE_TX);
        tma_load_3d(smem + L::O_AN + sa * L::SA, &tm.ac, 4 * xa, ya, (int)p, b);
        tma_load_3d(smem + L::O_BN + sa * L::SB, &tm.bc, xb, ya, (int)p, b);
        tma_load_3d(smem + L::O_AP + sp * L::SA, &tm.ap, 4 * xa, ya, (int)p, b);
        tma_load_3d(smem + L::O_BP + sp * L::SB, &tm.bp, xb, ya, (int)p, b);
    };
    auto wait_plane = [&](long p) {
        const long q = p - q0;
        if (!mbar_wait(bar + (q & 3), (uint32_t)((q >> 2) & 1), kTmaWaitLimit)) ok = false;
    };
    // extragradient point of the own column at (loaded) plane p
    auto bars_at = [&](long p, float *v) {
        const long q = p - q0;
        const float4 c = ((const float4 *)(smem + L::O_AN + (q & 3) * L::SA))[tid];
        const float4 o = ((const float4 *)(smem + L::O_AP + (q & 1) * L::SA))[tid];
        const float cb = ((const float *)(smem + L::O_BN + (q & 3) * L::SB))[bi];
        const float ob = ((const float *)(smem + L::O_BP + (q & 1) * L::SB))[bi];
        v[0] = bar1(c.x, o.x);
        v[1] = bar1(c.y, o.y);
        v[2] = bar1(c.z, o.z);
        v[3] = bar1(c.w, o.w);
        v[4] = bar1(cb, ob);
    };
    auto mask_at = [&](long z) -> unsigned {
        return (valid && z >= 0 && z < nz) ? (unsigned)__ldg(s.mm + col + nxny * (size_t)z) : 0u;
    };
    //   dual state n and f at plane j+1 (ring threads inside mi)
    float rd[ND], rf = 0.0f;
    bool rmi = false;
    auto fetch_dual = [&](long z, unsigned mb) {
        rmi = ring1 && z >= 1 && z + 1 < nz && (mb & 2u);
        if (rmi) {
            const size_t l = col + nxny * (size_t)z;
            load_dual<true>(s, l, rd);
            rf = __ldg(s.f + l);
        }
    };

    if (tid == 0) {
        for (int k = 0; k < L::NA; ++k) mbar_init(bar + k, 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (tid == 0) {
        issue(zs - 2);
        issue(zs - 1);
    }
    // mask ring: byte k of mr = mask of plane j+k (k = 0..3) at step j
    unsigned mr = 0;
    for (int k = 0; k < 4; ++k) mr |= mask_at(zs - 1 + k) << (8 * k);
    unsigned mnext = mask_at(zs + 3);

    // registers: extragradient point of planes j-1, j, j+1 (own column)
    float bm[NB], b0[NB], bp[NB];
    wait_plane(zs - 2);
    bars_at(zs - 2, bm);
    wait_plane(zs - 1);
    bars_at(zs - 1, b0);
    {
        float *Bw = B + ((zs - 1) & 1) * NB * NT;
#pragma unroll
        for (int q = 0; q < NB; ++q) Bw[q * NT + tid] = b0[q];
    }
    fetch_dual(zs - 1, mr & 0xffu);
    float vp[ND];
#pragma unroll
    for (int q = 0; q < ND; ++q) vp[q] = 0.0f;
    float nu_m2 = 0.f, p3_m2 = 0.f, q3_m2 = 0.f, q5_m2 = 0.f, q6_m2 = 0.f;
    bool pm = false;  // primal due at plane j-1 (owned, inside m)
    __syncthreads();  // the first two planes' iterate n-1 slots are read: plane zs may reuse one
    if (tid == 0) issue(zs);

    for (long j = zs - 1; j <= ze; ++j) {
        float *Bj = B + (j & 1) * NB * NT;              // extragradient of plane j (written last step)
        float *Bn = B + ((j + 1) & 1) * NB * NT;        // plane j+1 (written now)
        float *Sj = S + (j & 1) * ND * NT;              // dual of plane j (written now; held plane j-2)
        const float *Sm = S + ((j + 1) & 1) * ND * NT;  // dual of plane j-1

        // plane j+2's loads reuse the slots of planes j-2 (iterate n: last read by the primal of
        // step j-1) and j (iterate n-1: last read at step j-1); only planes up to ze+1 are read
        if (tid == 0 && j + 2 <= ze + 1) issue(j + 2);

        // (a) extragradient point of plane j+1
        wait_plane(j + 1);
        bars_at(j + 1, bp);
#pragma unroll
        for (int q = 0; q < NB; ++q) Bn[q * NT + tid] = bp[q];
        const unsigned mfar = mask_at(j + 5);

        // (b) dual at plane j from the state fetched last step; fetch plane j+1
        float v[ND];
        const bool do_dual = rmi;
        float dcur[ND], fcur = rf;
#pragma unroll
        for (int q = 0; q < ND; ++q) dcur[q] = rd[q];
        fetch_dual(j + 1, (mr >> 8) & 0xffu);
        const bool do_primal = pm;
        pm = owned && j >= zs && j < ze && (mr & 1u);
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
            if (owned && j >= zs && j < ze) store_dual<true>(s, l, v);
        }
#pragma unroll
        for (int q = 0; q < ND; ++q) Sj[q * NT + tid] = v[q];

        // (c) primal + extragradient at plane j-1, iterate n from its slot
        if (do_primal) {
            const long q = (j - 1) - q0;
            const float4 ca = ((const float4 *)(smem + L::O_AN + (q & 3) * L::SA))[tid];
            const float cb = ((const float *)(smem + L::O_BN + (q & 3) * L::SB))[bi];
            const size_t l = col + nxny * (size_t)(j - 1);
            const float nu0 = vp[0];
            const float xs = Sm[tid - 1] + Sm[tid + 1];
            const float ys = Sm[tid - WX] + Sm[tid + WX];
            const float zs_ = nu_m2 + v[0];
            const float cn = ca.x, en = ca.y;
            const float e1 = pc.tau1 * (en - pc.lhh * nu0 - pc.lhx * xs - pc.lhy * ys - pc.lhz * zs_);
            const float *P1 = Sm + NT, *P2 = Sm + 2 * NT;
            const float c1 = cn + (pc.hx * (vp[1] - P1[tid - 1]) + pc.hy * (vp[2] - P2[tid - WX]) +
                                   pc.hz * (vp[3] - p3_m2) +
                                   (pc.whh * nu0 + pc.whx * xs + pc.why * ys + pc.whz * zs_));
            const float *Q1 = Sm + 4 * NT, *Q2 = Sm + 5 * NT, *Q3 = Sm + 6 * NT, *Q4 = Sm + 7 * NT,
                        *Q5 = Sm + 8 * NT;
            const float u1 = ca.z + (pc.tt * vp[1] + pc.hx * (vp[4] - Q1[tid - 1] + vp[5] - Q2[tid - WX] +
                                                               vp[6] - q3_m2));
            const float u2 = ca.w + (pc.tt * vp[2] + pc.hy * (vp[5] - Q2[tid - 1] + vp[7] - Q4[tid - WX] +
                                                               vp[8] - q5_m2));
            const float u3 = cb + (pc.tt * vp[3] + pc.hz * (vp[6] - Q3[tid - 1] + vp[8] - Q5[tid - WX] +
                                                             vp[9] - q6_m2));
            const float pv[NB] = {c1, e1, u1, u2, u3};
            store_primal<true>(s.Pn, s.Pn1, l, pv);
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
        q3_m2 = vp[6];
        q5_m2 = vp[8];
        q6_m2 = vp[9];
#pragma unroll
        for (int q = 0; q < ND; ++q) vp[q] = v[q];
        mr = (mr >> 8) | (mnext << 24);
        mnext = mfar;
        __syncthreads();
    }
    if (!ok) atomicOr(&s.ctl->stalled, 1u);
    if (check)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] += mon[q].get();
}

}  // namespace qsm
