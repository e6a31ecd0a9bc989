// Shared device/host infrastructure of the GB300 QSM library: status codes,
// the per-device context (stream + stream-ordered memory pool), staging of
// caller pointers that may live in host or device memory, launch geometry,
// and the deterministic "lane order" reductions.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <stdio.h>
#include <string.h>

#include "../../include/qsm_gpu.h"

#include <nvtx3/nvToolsExt.h>

namespace qsm {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------

void set_error(qsm_ctx *ctx, const char *fmt, ...);

#define QSM_CUDA(call)                                                              \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            ::qsm::set_error(ctx, "%s:%d %s: %s", __FILE__, __LINE__, #call,        \
                             cudaGetErrorString(e_));                               \
            return QSM_ERR_CUDA;                                                    \
        }                                                                           \
    } while (0)

#define QSM_TRY(expr)                                                               \
    do {                                                                            \
        qsm_status s_ = (expr);                                                     \
        if (s_ != QSM_OK) return s_;                                                \
    } while (0)

// ---------------------------------------------------------------------------
// geometry
// ---------------------------------------------------------------------------

// A named NVTX range over a scope, shown by profilers (Nsight Systems,
// Nsight Compute's range filters); with no profiler attached a push/pop is a
// call through an unset function pointer.
struct Range {
    explicit Range(const char *name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range &) = delete;
    Range &operator=(const Range &) = delete;
};

struct Dims {
    size_t nx, ny, nz;
    __host__ __device__ size_t nxny() const { return nx * ny; }
    __host__ __device__ size_t n() const { return nx * ny * nz; }
};

static inline Dims make_dims(const size_t *d) { return Dims{d[0], d[1], d[2]}; }

// A thread's partial sum for the FP64 block reductions.  FP64 arithmetic runs at
// 1/64 of the FP32 rate on this GPU, so an FP32 kernel that converted and added
// every voxel's term in FP64 would be bound by the FP64 pipe: FP32 terms are
// summed per thread with compensation (Kahan; exact under -fmad=false), and
// only the thread's total goes to FP64.  FP64 terms are summed in FP64.
template <typename T> struct PartialSum;
template <> struct PartialSum<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double get() const { return s; }
};
template <> struct PartialSum<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x)
    {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double get() const { return (double)s - (double)c; }
};

// One thread per voxel: block 32 x 4 x 2 over (x, y, z).
static inline dim3 vox_block() { return dim3(32, 4, 2); }
static inline dim3 vox_grid(const Dims &d)
{
    return dim3((unsigned)((d.nx + 31) / 32), (unsigned)((d.ny + 3) / 4), (unsigned)((d.nz + 1) / 2));
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------

}  // namespace qsm

struct qsm_ctx {
    int device;
    cudaStream_t stream;
    bool own_stream;
    cudaMemPool_t pool;
    int verbose;
    char err[512];
    // lane-order reduction scratch (partials + results), grown on demand
    double *red_partial;   // 4 * QSM_RED_NBLK doubles
    double *red_out;       // 8 doubles
    unsigned int *red_count;
    double *host_out;      // pinned, 8 doubles
    uint32_t debug;        // QSM_DEBUG_* test hooks (qsm_ctx_set_debug)
};

namespace qsm {

// device allocation from the context's pool, ordered on its stream
qsm_status dalloc(qsm_ctx *ctx, void **p, size_t bytes);
qsm_status dfree(qsm_ctx *ctx, void *p);

// Where a caller pointer lives.
bool is_device_ptr(const void *p);

// A caller array that may be host or device memory.  stage_in() gives a
// device pointer (copying host data in when `copy_in`); stage_out() copies a
// staged array back to the host buffer and releases the staging copy.
struct Staged {
    void *host;      // caller's host pointer (null if caller passed device memory)
    void *dev;       // device pointer used by kernels
    size_t bytes;
    bool owned;
};

qsm_status stage_in(qsm_ctx *ctx, Staged &s, const void *p, size_t bytes, bool copy_in);
qsm_status stage_out(qsm_ctx *ctx, Staged &s, bool copy_out);

// ---------------------------------------------------------------------------
// lane-order reductions
//
// Element i of an n-vector goes to lane i mod 2^18; each lane sums its
// elements in increasing i from +0.0 (no fused multiply-add); lanes form
// 1024 blocks of 256 reduced by halving (s = 128..1: a[t] += a[t+s]); the
// 1024 block sums are reduced by the same halving.  The CPU oracle and its
// BLAS shim use exactly this order, so results agree bit-for-bit.
// ---------------------------------------------------------------------------

constexpr int RED_BLOCK = 256;
constexpr int RED_NBLK = QSM_RED_NBLK;
constexpr size_t RED_LANES = (size_t)RED_BLOCK * RED_NBLK;

template <typename T>
__device__ __forceinline__ T halve_block(T *sm, int tid, T v)
{
    sm[tid] = v;
    __syncthreads();
    for (int s = RED_BLOCK / 2; s > 0; s >>= 1) {
        if (tid < s) sm[tid] = sm[tid] + sm[tid + s];
        __syncthreads();
    }
    return sm[0];
}

// Final halving over the RED_NBLK block partials by one block of RED_BLOCK
// threads: level s = 512 is done by each thread for t and t + 256, then the
// remaining levels in shared memory.
template <typename T>
__device__ __forceinline__ T halve_partials(T *sm, int tid, const T *part)
{
    static_assert(RED_NBLK == 4 * RED_BLOCK, "lane order layout");
    T a = __ldcg(part + tid), b = __ldcg(part + tid + 256), c = __ldcg(part + tid + 512), d = __ldcg(part + tid + 768);
    // s = 512: a[t] += a[t+512] for t < 512
    sm[tid] = a + c;
    T hi = b + d;  // element t + 256 after the s = 512 level
    __syncthreads();
    // s = 256: a[t] += a[t+256]
    T v = sm[tid] + hi;
    __syncthreads();
    return halve_block(sm, tid, v);
}

// FP32 -> FP64 (exact) and FP64 -> FP32 (round to nearest, ties to even)
// in integer arithmetic, from the IEEE 754 binary32 / binary64 encodings:
// the bits of the device's own conversions (a NaN keeps its payload and is
// made quiet), but issued on the integer pipes rather than the FP64 pipe,
// which this GPU runs at 1/64 of the FP32 rate.  qsm_fp_convert_check
// compares them with the device's conversions.
__device__ __forceinline__ double f32_to_f64(float f)
{
    const uint32_t u = __float_as_uint(f);
    const uint64_t s = (uint64_t)(u >> 31) << 63;
    const uint32_t e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    uint64_t r;
    if (e == 0xffu) {  // infinity, NaN (quiet bit set)
        r = s | (0x7ffull << 52) | ((uint64_t)m << 29) | (m ? (1ull << 51) : 0ull);
    } else if (e == 0u) {  // zero, or a subnormal made normal: its leading 1 moves to bit 23
        if (m == 0u) {
            r = s;
        } else {
            const int sh = __clz(m) - 8;
            r = s | ((uint64_t)(897 - sh) << 52) | ((uint64_t)((m << sh) & 0x7fffffu) << 29);
        }
    } else {  // exponent bias 127 -> 1023
        r = s | ((uint64_t)(e + 896u) << 52) | ((uint64_t)m << 29);
    }
    return __longlong_as_double((long long)r);
}

__device__ __forceinline__ float f64_to_f32(double d)
{
    const uint64_t u = (uint64_t)__double_as_longlong(d);
    const uint32_t s = (uint32_t)(u >> 63) << 31;
    const int e = (int)((u >> 52) & 0x7ffu);
    const uint64_t m = u & ((1ull << 52) - 1);
    uint32_t r;
    if (e == 0x7ff) {  // infinity, NaN (quiet bit set, top payload bits kept)
        r = m ? (0x7fc00000u | (uint32_t)(m >> 29)) : 0x7f800000u;
    } else if (e >= 1151) {  // 2^128 or more: infinity
        r = 0x7f800000u;
    } else if (e >= 897) {  // a normal float: keep 23 fraction bits, round on the other 29
        const uint32_t hi = (uint32_t)(m >> 29), rem = (uint32_t)(m & ((1u << 29) - 1));
        const uint32_t up = rem > (1u << 28) || (rem == (1u << 28) && (hi & 1u));
        r = (((uint32_t)(e - 896) << 23) | hi) + up;  // a carry moves into the exponent (up to infinity)
    } else {  // a subnormal float or zero: the significand in units of 2^-149, rounded
        const int sh = 926 - e;
        if (sh >= 54) {
            r = 0u;  // below half the smallest subnormal
        } else {
            const uint64_t M = e ? (m | (1ull << 52)) : m;
            const uint64_t q = M >> sh, rem = M & ((1ull << sh) - 1), half = 1ull << (sh - 1);
            r = (uint32_t)q + (uint32_t)(rem > half || (rem == half && (q & 1)));
        }
    }
    return __uint_as_float(s | r);
}

// out[0] = dot(x, y) (or sum x*x when y == x) in lane order, on ctx->stream,
// written to device memory `dout`.  T in {float, double}; FP32 inputs
// accumulate in FP32 like sdot and the result is widened.
template <typename T>
qsm_status lane_dot(qsm_ctx *ctx, const T *x, const T *y, size_t n, double *dout);

// Reads back one device double (synchronises the stream).
qsm_status read_double(qsm_ctx *ctx, const double *d, double *h);

// A tiled TMA tensor map of a 3-D array (tma.cuh): element type dt, extents
// dims[0..2] (dims[0] fastest), byte strides of dims 1 and 2 (multiples of
// 16), box extents box[0..2]; zeros are read outside the extents.  Fails
// with QSM_ERR_ARG where the driver refuses the description.
qsm_status tma_encode_3d(qsm_ctx *ctx, CUtensorMap *map, CUtensorMapDataType dt, const void *base,
                         const uint64_t dims[3], const uint64_t strides[2], const uint32_t box[3]);

}  // namespace qsm
