// Shared pieces of the fused mixed-precision TGV/TV kernels (pd_fused.cu:
// 3-D tiles; pd_stream.cu: z-streaming column tiles).
#pragma once

#include "common.cuh"
#include "pd.cuh"

namespace qsm {

struct FusedArgs {
    const float *Pc[5];     // chi^n, eta^n, w1^n, w2^n, w3^n (TV: chi, eta)
    const float *Pp[5];     // iterate n-1
    float *Pn[5];           // iterate n+1 (written)
    const float *Dc[10];    // nu, p1..3, q1..6 at n (TV: nu, p1..3)
    float *Dn[10];          // at n+1 (written)
    const float *f;
    const uint8_t *mm;
    double *part;           // 4 x gridDim.x partial monitor sums
    unsigned int *count;
    PdCtl *ctl;
    const unsigned *tiles;  // active tile indices (x fastest), one per block
    unsigned gx, gy;        // tiles per row / per plane
};

// extragradient point (pd_tgv_mex.c:804-810): x_ = x^n + 1*(x^n - x^(n-1))
__device__ __forceinline__ float xbar(const float *__restrict__ c, const float *__restrict__ p, size_t l)
{
    const float cn = __ldg(c + l);
    return cn + 1.0f * (cn - __ldg(p + l));
}

// Monitor sums of one block, then the last block folds the partials in
// block order and applies the stopping test.  red aliases dynamic shared
// memory (4 x THREADS doubles) that is free once the primal has finished.
template <int THREADS>
__device__ __forceinline__ void monitor_reduce(const FusedArgs &s, double *red, const double *acc, double tol,
                                               uint32_t it)
{
    __shared__ bool last;
    const int tid = threadIdx.x;
    const unsigned int nblk = gridDim.x, bid = blockIdx.x;
    __syncthreads();  // everyone is done reading the dual from shared memory
#pragma unroll
    for (int q = 0; q < 4; ++q) red[q * THREADS + tid] = acc[q];
    __syncthreads();
    for (int st = THREADS / 2; st > 0; st >>= 1) {
        if (tid < st)
#pragma unroll
            for (int q = 0; q < 4; ++q) red[q * THREADS + tid] += red[q * THREADS + tid + st];
        __syncthreads();
    }
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) s.part[(size_t)q * nblk + bid] = red[q * THREADS];
        __threadfence();
        last = atomicAdd(s.count, 1u) == nblk - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        double a = 0.0;
        for (unsigned int b2 = tid; b2 < nblk; b2 += THREADS) a += __ldcg(s.part + (size_t)q * nblk + b2);
        red[q * THREADS + tid] = a;
    }
    __syncthreads();
    for (int st = THREADS / 2; st > 0; st >>= 1) {
        if (tid < st)
#pragma unroll
            for (int q = 0; q < 4; ++q) red[q * THREADS + tid] += red[q * THREADS + tid + st];
        __syncthreads();
    }
    if (tid == 0) {
        double r[4] = {red[0], red[THREADS], red[2 * THREADS], red[3 * THREADS]};
        pd_finish(s.ctl, r, tol, it);
        *s.count = 0;
    }
}


size_t stream_smem(int tx, int ty, bool tgv);
qsm_status stream_set_smem(qsm_ctx *ctx);
qsm_status stream_launch(qsm_ctx *ctx, int tx, int ty, int cz, bool tgv, bool chk, unsigned nact, const FusedArgs &s,
                         const DualC<float> &dc, const PrimalC<float> &pc, const Dims &d, double tol, uint32_t it);

}  // namespace qsm
