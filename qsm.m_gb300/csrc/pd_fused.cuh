// Shared pieces of the fused mixed-precision TGV/TV kernels (pd_fused.cu:
// 3-D tiles; pd_stream.cu: z-streaming column tiles).
#pragma once

#include <vector>

#include "common.cuh"
#include "pd.cuh"

namespace qsm {

// Device state of the fused path, interleaved per voxel so that one address
// and one 8/16-byte access serve several fields (SoA across voxels, AoS
// within a family):
//   primal family A: TGV (chi, eta, w1, w2) as float4, TV (chi, eta) as float2
//   primal family B: TGV w3 as float
//   dual families:   (nu, p1, p2, p3) float4; TGV also (q1, q2, q3, q4) float4
//                    and (q5, q6) float2
// Families A/B are triple-buffered (iterates n-1, n, n+1), the dual
// families double-buffered.
struct FusedArgs {
    const void *Pc, *Pp;    // family A at iterate n, n-1
    void *Pn;               // family A at n+1 (written)
    const float *Pc1, *Pp1; // family B at n, n-1
    float *Pn1;             // family B at n+1
    const float4 *Dca, *Dcb;
    const float2 *Dcc;      // dual at n
    float4 *Dna, *Dnb;
    float2 *Dnc;            // dual at n+1 (written)
    const float *f;
    const uint8_t *mm;
    double *part;           // 4 x gridDim.x partial monitor sums
    unsigned int *count;
    PdCtl *ctl;
    const unsigned *tiles;  // active tile indices (x fastest), one per block
    unsigned gx, gy;        // tiles per row / per plane
    // replayed graphs: the iteration count comes from a device counter
    const uint32_t *gbase;  // null: the launch's `it` is the iteration count
    uint32_t start, maxiter;
};

// extragradient point (pd_tgv_mex.c:804-810): x_ = x^n + 1*(x^n - x^(n-1))
__device__ __forceinline__ float bar1(float c, float p) { return c + 1.0f * (c - p); }
__device__ __forceinline__ float xbar(const float *__restrict__ c, const float *__restrict__ p, size_t l)
{
    return bar1(__ldg(c + l), __ldg(p + l));
}

// the primal family of voxel l: TGV v = (chi, eta, w1, w2, w3), TV v = (chi, eta)
template <bool TGV>
__device__ __forceinline__ void load_primal(const void *A, const float *B, size_t l, float *v)
{
    if (TGV) {
        const float4 a = __ldg((const float4 *)A + l);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = __ldg(B + l);
    } else {
        const float2 a = __ldg((const float2 *)A + l);
        v[0] = a.x; v[1] = a.y;
    }
}
template <bool TGV>
__device__ __forceinline__ void store_primal(void *A, float *B, size_t l, const float *v)
{
    if (TGV) {
        ((float4 *)A)[l] = make_float4(v[0], v[1], v[2], v[3]);
        B[l] = v[4];
    } else {
        ((float2 *)A)[l] = make_float2(v[0], v[1]);
    }
}
// the dual of voxel l: TGV v = (nu, p1..3, q1..6), TV v = (nu, p1..3)
template <bool TGV>
__device__ __forceinline__ void load_dual(const FusedArgs &s, size_t l, float *v)
{
    const float4 a = __ldg(s.Dca + l);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    if (TGV) {
        const float4 b = __ldg(s.Dcb + l);
        const float2 c = __ldg(s.Dcc + l);
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w; v[8] = c.x; v[9] = c.y;
    }
}
template <bool TGV>
__device__ __forceinline__ void store_dual(const FusedArgs &s, size_t l, const float *v)
{
    s.Dna[l] = make_float4(v[0], v[1], v[2], v[3]);
    if (TGV) {
        s.Dnb[l] = make_float4(v[4], v[5], v[6], v[7]);
        s.Dnc[l] = make_float2(v[8], v[9]);
    }
}
// (chi_, eta_) of family A at l, and for TGV also (w1_, w2_)
template <bool TGV>
__device__ __forceinline__ void bar_head(const FusedArgs &s, size_t l, float *v)
{
    if (TGV) {
        const float4 c = __ldg((const float4 *)s.Pc + l), p = __ldg((const float4 *)s.Pp + l);
        v[0] = bar1(c.x, p.x); v[1] = bar1(c.y, p.y); v[2] = bar1(c.z, p.z); v[3] = bar1(c.w, p.w);
    } else {
        const float2 c = __ldg((const float2 *)s.Pc + l), p = __ldg((const float2 *)s.Pp + l);
        v[0] = bar1(c.x, p.x); v[1] = bar1(c.y, p.y);
    }
}

// Iteration count this launch completes, 0 if it must do nothing.  Direct
// launches pass it = the count; a graph replayed from a device iteration
// base passes it = the node's offset in the graph and sets gbase.
__device__ __forceinline__ uint32_t launch_iter(const FusedArgs &s, uint32_t it)
{
    if (!s.gbase) return it;
    const uint32_t l = *s.gbase + it - s.start;
    return l < s.maxiter ? l + 1 : 0;
}

// Monitor sums of one tile (block), then the last of the nblk tiles folds
// the partials in tile order and applies the stopping test.  red aliases
// dynamic shared memory (4 x THREADS doubles) that is free once the primal
// has finished.  After the call the shared memory is free again only after
// the next __syncthreads.
template <int THREADS>
__device__ __forceinline__ void monitor_fold(double *part, unsigned int *count, PdCtl *ctl, unsigned int nblk,
                                             unsigned int bid, double *red, const double *acc, double tol,
                                             uint32_t it)
{
    __shared__ bool last;
    const int tid = threadIdx.x;
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
        for (int q = 0; q < 4; ++q) part[(size_t)q * nblk + bid] = red[q * THREADS];
        __threadfence();
        last = atomicAdd(count, 1u) == nblk - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        double a = 0.0;
        for (unsigned int b2 = tid; b2 < nblk; b2 += THREADS) a += __ldcg(part + (size_t)q * nblk + b2);
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
        pd_finish(ctl, r, tol, it);
        *count = 0;
    }
}

// one block per active tile
template <int THREADS>
__device__ __forceinline__ void monitor_reduce(const FusedArgs &s, double *red, const double *acc, double tol,
                                               uint32_t it)
{
    monitor_fold<THREADS>(s.part, s.count, s.ctl, gridDim.x, blockIdx.x, red, acc, tol, it);
}

// Tensor maps of the TGV primal families at iterates n (c) and n-1 (p) for
// the TMA column kernel (pd_tma.cuh): family A as floats (4 nx, ny, nz)
// with a (4 (TX+4), TY+4, 1) box, family B as (nx, ny, nz) with a
// (TX+8, TY+4, 1) box.
struct TmaMaps {
    CUtensorMap ac, ap, bc, bp;
};

size_t stream_smem(int tx, int ty, bool tgv);
size_t stream_tma_smem(int tx, int ty);
qsm_status stream_set_smem(qsm_ctx *ctx);
// tm: the TMA column kernel (TGV) with these maps; null: the register-prefetch one
qsm_status stream_launch(qsm_ctx *ctx, cudaStream_t st, int tx, int ty, int cz, bool tgv, bool chk, unsigned nact,
                         const FusedArgs &s, const DualC<float> &dc, const PrimalC<float> &pc, const Dims &d,
                         double tol, uint32_t it, const TmaMaps *tm);

// ---------------------------------------------------------------------------
// Tile variants and the device state of one fused solve (pd_fused.cu), shared
// with the many-volume session (pd_batch.cu).
// ---------------------------------------------------------------------------

struct Variant {
    int tx, ty, tz;   // tile of interior voxels (z: chunk of planes for the column kernel)
    bool stream;      // column-streaming kernel, else the 3-D tile kernel
    bool tma;         // column kernel with TMA-staged primal iterates (TGV, nx a multiple of 4)
};
constexpr int kNumVariants = 13;
// register-prefetch column variant (28 x 16, 16 planes) that stands in for a
// TMA variant where that cannot run (TV, nx not a multiple of 4, packed
// many-volume launches)
constexpr int kTmaFallback = 8;
const Variant &variant(int v);
size_t variant_smem(int v, bool tgv);
int variant_threads(int v);

struct TileList {
    unsigned gx = 0, gy = 0, gz = 0, nact = 0;
    unsigned *dev = nullptr;  // active tile indices, ascending (inside the state block)
    uint64_t active_vox = 0;  // interior voxels covered by the active tiles
};

// Device state of one solve: triple-buffered primal, double-buffered dual,
// scaled data, masks, the active-tile lists of every variant and the monitor
// scratch, in one allocation.
struct PdVolume {
    bool tgv = false;
    Dims d{};
    int np = 0, nd = 0;
    void *blk = nullptr;
    void *PA[3] = {};           // primal family A of iterates (rotating)
    float *PB[3] = {};          // primal family B (TGV w3)
    float4 *DA[2] = {}, *DB[2] = {};
    float2 *DC[2] = {};         // dual families
    float *f = nullptr;
    uint8_t *mm = nullptr;       // bit 0 m, bit 1 mi
    TileList tl[kNumVariants];
    double *part = nullptr;      // 4 x (max tiles) monitor partials
    unsigned *count = nullptr;   // arrival counter of the monitor fold
    PdCtl *ctl = nullptr;
    size_t state_bytes = 0;      // primal + dual buffers (from PA[0])
    DualC<float> dc{};
    PrimalC<float> pc{};
    int var = 0;                 // chosen tile variant
    // TMA maps per (variant, iterate rotation it % 3), filled for the TMA
    // variants; empty when they cannot run on this volume
    std::vector<TmaMaps> maps;
};

// Whether variant var can run on this volume.
bool variant_ok(const PdVolume &v, int var);

// Device bytes one solve holds (the allocation pd_volume_init makes).
size_t pd_volume_bytes(bool tgv, const Dims &d);
// Allocates and initialises the state from device d2f (dtype dt) and mask.
qsm_status pd_volume_init(qsm_ctx *ctx, PdVolume *v, bool tgv, const Dims &d, qsm_dtype dt, const void *d2f,
                          const uint8_t *mask, const double *h, double lam, double alpha);
// Kernel arguments of variant var for the iteration that reads iterate `it`.
FusedArgs pd_volume_args(const PdVolume &v, int var, uint32_t it);
// Picks v->var: QSM_FUSED_VARIANT, the tuning table, or timing each variant
// on this volume for a few iterations (the state is zeroed again after).
qsm_status pd_volume_tune(qsm_ctx *ctx, PdVolume *v, uint32_t maxiter);
// One iteration of variant v->var on stream st (the one-volume kernels); s
// from pd_volume_args(v, v.var, rot), it the kernel's iteration argument.
qsm_status pd_volume_launch(qsm_ctx *ctx, cudaStream_t st, const PdVolume &v, bool chk, const FusedArgs &s,
                            double tol, uint32_t it, uint32_t rot);
// chi after `iters` iterations, converted to dt.
qsm_status pd_volume_result(qsm_ctx *ctx, const PdVolume &v, uint32_t iters, qsm_dtype dt, void *chi);
qsm_status pd_volume_free(qsm_ctx *ctx, PdVolume *v);

}  // namespace qsm
