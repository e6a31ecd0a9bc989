// Context, staging and lane-order reductions.
#include <stdarg.h>
#include <stdlib.h>

#include "common.cuh"

namespace qsm {

void set_error(qsm_ctx *ctx, const char *fmt, ...)
{
    if (!ctx) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(ctx->err, sizeof ctx->err, fmt, ap);
    va_end(ap);
}

qsm_status dalloc(qsm_ctx *ctx, void **p, size_t bytes)
{
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMallocFromPoolAsync(p, bytes, ctx->pool, ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error(ctx, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        *p = nullptr;
        return QSM_ERR_NOMEM;
    }
    return QSM_OK;
}

qsm_status dfree(qsm_ctx *ctx, void *p)
{
    if (!p) return QSM_OK;
    QSM_CUDA(cudaFreeAsync(p, ctx->stream));
    return QSM_OK;
}

bool is_device_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

qsm_status stage_in(qsm_ctx *ctx, Staged &s, const void *p, size_t bytes, bool copy_in)
{
    s.host = nullptr;
    s.dev = nullptr;
    s.bytes = bytes;
    s.owned = false;
    if (is_device_ptr(p)) {
        s.dev = const_cast<void *>(p);
        return QSM_OK;
    }
    s.host = const_cast<void *>(p);
    QSM_TRY(dalloc(ctx, &s.dev, bytes));
    s.owned = true;
    if (copy_in && bytes) QSM_CUDA(cudaMemcpyAsync(s.dev, p, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return QSM_OK;
}

qsm_status stage_out(qsm_ctx *ctx, Staged &s, bool copy_out)
{
    if (!s.owned) return QSM_OK;
    if (copy_out && s.bytes) QSM_CUDA(cudaMemcpyAsync(s.host, s.dev, s.bytes, cudaMemcpyDeviceToHost, ctx->stream));
    qsm_status st = dfree(ctx, s.dev);
    s.dev = nullptr;
    s.owned = false;
    return st;
}

// ---------------------------------------------------------------------------
// lane-order dot product
// ---------------------------------------------------------------------------

// Throughput probe: eight independent chains x = x * m + c per thread (a
// multiply and an add each, -fmad=false), 16 operations per iteration.
template <typename T>
__global__ void __launch_bounds__(256) fp_rate_k(T *out, T m, T c, int iters)
{
    T a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) a[u] = (T)(threadIdx.x + u);
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int u = 0; u < 8; ++u) a[u] = a[u] * m + c;
    T s = (T)0;
#pragma unroll
    for (int u = 0; u < 8; ++u) s = s + a[u];
    if (s == (T)-1) out[0] = s;  // keeps the chains live; never true for these inputs
}

// f32_to_f64 / f64_to_f32 against the device's conversions: every float
// (base .. base + count), and `count` doubles from a 64-bit mix of the index,
// one in eight drawn at random and the rest aimed at the cases that need
// care (float rounding ties, the float exponent range and its edges,
// subnormal and overflowing results).
__device__ __forceinline__ uint64_t cvt_mix(uint64_t z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__global__ void cvt_check_k(unsigned long long nfloat, unsigned long long ndouble, unsigned long long *bad)
{
    unsigned long long nb = 0;
    const unsigned long long st = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < nfloat; i += st) {
        const float f = __uint_as_float((uint32_t)i);
        nb += __double_as_longlong((double)f) != __double_as_longlong(f32_to_f64(f));
    }
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < ndouble; i += st) {
        uint64_t u = cvt_mix(i);
        const uint64_t sign = u & 0x8000000000000000ull, ex = cvt_mix(i ^ 0x5bd1e995ull);
        switch (i & 7) {
        case 1:  // exponents around the float range
            u = (u & 0x800fffffffffffffull) | ((860 + ex % 300) << 52);
            break;
        case 2:  // exact ties between two floats
            u = (u & 0xfff0000000000000ull) | (((u >> 12) & 0x7fffffull) << 29) | (1ull << 28);
            break;
        case 3:  // ties or float-exact values near the subnormal and overflow edges
            u = sign | ((860 + ex % 300) << 52) | (((u >> 20) & 0x7fffffull) << 29) | ((ex >> 40) & 1 ? (1ull << 28) : 0);
            break;
        case 4:  // next to 2^128
            u = (u & 0x800fffffffffffffull) | ((1140 + ex % 20) << 52);
            break;
        case 5:  // double subnormals and tiny normals
            u = (u & 0x800fffffffffffffull) | ((ex % 40) << 52);
            break;
        default:
            break;
        }
        const double d = __longlong_as_double((long long)u);
        nb += __float_as_uint((float)d) != __float_as_uint(f64_to_f32(d));
    }
    if (nb) atomicAdd(bad, nb);
}

template <typename T>
__global__ void __launch_bounds__(RED_BLOCK) lane_dot_kernel(const T *__restrict__ x, const T *__restrict__ y,
                                                             size_t n, T *part, unsigned int *count, double *out)
{
    __shared__ T sm[RED_BLOCK];
    __shared__ bool last;
    const int tid = threadIdx.x;
    const size_t t = (size_t)blockIdx.x * RED_BLOCK + tid;
    T acc = (T)0;
    size_t i = t;
    // four elements' loads in flight per thread; the lane still adds them in
    // increasing i
    for (; i + 3 * RED_LANES < n; i += 4 * RED_LANES) {
        const T x0 = x[i], x1 = x[i + RED_LANES], x2 = x[i + 2 * RED_LANES], x3 = x[i + 3 * RED_LANES];
        const T y0 = y[i], y1 = y[i + RED_LANES], y2 = y[i + 2 * RED_LANES], y3 = y[i + 3 * RED_LANES];
        acc = acc + x0 * y0;
        acc = acc + x1 * y1;
        acc = acc + x2 * y2;
        acc = acc + x3 * y3;
    }
    for (; i < n; i += RED_LANES) acc = acc + x[i] * y[i];
    T b = halve_block(sm, tid, acc);
    if (tid == 0) {
        part[blockIdx.x] = b;
        __threadfence();
        last = atomicAdd(count, 1u) == RED_NBLK - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    T r = halve_partials(sm, tid, part);
    if (tid == 0) {
        out[0] = (double)r;
        *count = 0;
    }
}

template <typename T>
qsm_status lane_dot(qsm_ctx *ctx, const T *x, const T *y, size_t n, double *dout)
{
    lane_dot_kernel<T><<<RED_NBLK, RED_BLOCK, 0, ctx->stream>>>(x, y, n, (T *)ctx->red_partial, ctx->red_count, dout);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

template qsm_status lane_dot<float>(qsm_ctx *, const float *, const float *, size_t, double *);
template qsm_status lane_dot<double>(qsm_ctx *, const double *, const double *, size_t, double *);

qsm_status read_double(qsm_ctx *ctx, const double *d, double *h)
{
    QSM_CUDA(cudaMemcpyAsync(ctx->host_out, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    *h = ctx->host_out[0];
    return QSM_OK;
}

namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
}  // namespace

qsm_status tma_encode_3d(qsm_ctx *ctx, CUtensorMap *map, CUtensorMapDataType dt, const void *base,
                         const uint64_t dims[3], const uint64_t strides[2], const uint32_t box[3])
{
    static EncodeTiledFn encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        QSM_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !fn) {
            set_error(ctx, "cuTensorMapEncodeTiled is not available from the driver");
            return QSM_ERR_CUDA;
        }
        encode = (EncodeTiledFn)fn;
    }
    const cuuint64_t gd[3] = {dims[0], dims[1], dims[2]};
    const cuuint64_t gs[2] = {strides[0], strides[1]};
    const cuuint32_t bx[3] = {box[0], box[1], box[2]};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = encode(map, dt, 3, const_cast<void *>(base), gd, gs, bx, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error(ctx, "cuTensorMapEncodeTiled failed (%d): dims %llu %llu %llu box %u %u %u", (int)r,
                  (unsigned long long)dims[0], (unsigned long long)dims[1], (unsigned long long)dims[2], box[0],
                  box[1], box[2]);
        return QSM_ERR_ARG;
    }
    return QSM_OK;
}

}  // namespace qsm

// ---------------------------------------------------------------------------
// C ABI: context
// ---------------------------------------------------------------------------

using namespace qsm;

extern "C" {

int qsm_abi_version(void) { return QSM_GPU_ABI_VERSION; }

const char *qsm_status_string(qsm_status s)
{
    switch (s) {
    case QSM_OK: return "ok";
    case QSM_ERR_ARG: return "invalid argument";
    case QSM_ERR_DIMS: return "invalid dimensions";
    case QSM_ERR_DTYPE: return "invalid dtype";
    case QSM_ERR_NOMEM: return "out of device memory";
    case QSM_ERR_CUDA: return "CUDA error";
    case QSM_ERR_NONFINITE: return "non-finite convergence monitor";
    case QSM_ERR_DEPTH: return "nlevels too large. Increase MAX_DEPTH.";
    case QSM_ERR_BUSY: return "busy";
    case QSM_ERR_TIMEOUT: return "timeout";
    }
    return "unknown status";
}

const char *qsm_last_error(const qsm_ctx *ctx) { return ctx ? ctx->err : "no context"; }

qsm_status qsm_ctx_create(int device, qsm_ctx **out)
{
    if (!out) return QSM_ERR_ARG;
    *out = nullptr;
    qsm_ctx *ctx = (qsm_ctx *)calloc(1, sizeof(qsm_ctx));
    if (!ctx) return QSM_ERR_NOMEM;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        ctx->own_stream = true;
        cudaMemPoolProps props;
        memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        e = cudaMemPoolCreate(&ctx->pool, &props);
    }
    if (e == cudaSuccess) {
        uint64_t thr = UINT64_MAX;  // keep freed blocks cached in the pool
        e = cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->red_partial, 4 * RED_NBLK * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->red_out, 8 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->red_count, 8 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(ctx->red_count, 0, 8 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&ctx->host_out, 8 * sizeof(double));
    if (e != cudaSuccess) {
        snprintf(ctx->err, sizeof ctx->err, "context creation failed: %s", cudaGetErrorString(e));
        fprintf(stderr, "qsm_ctx_create: %s\n", ctx->err);
        qsm_ctx_destroy(ctx);
        return QSM_ERR_CUDA;
    }
    *out = ctx;
    return QSM_OK;
}

qsm_status qsm_ctx_set_debug(qsm_ctx *ctx, uint32_t flags)
{
    if (!ctx) return QSM_ERR_ARG;
    if (flags & ~(uint32_t)QSM_DEBUG_GRID_BARRIER_TIMEOUT) return QSM_ERR_ARG;
    ctx->debug = flags;
    return QSM_OK;
}

qsm_status qsm_ctx_destroy(qsm_ctx *ctx)
{
    if (!ctx) return QSM_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->red_partial) cudaFree(ctx->red_partial);
    if (ctx->red_out) cudaFree(ctx->red_out);
    if (ctx->red_count) cudaFree(ctx->red_count);
    if (ctx->host_out) cudaFreeHost(ctx->host_out);
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    free(ctx);
    return QSM_OK;
}

qsm_status qsm_ctx_set_stream(qsm_ctx *ctx, void *stream)
{
    if (!ctx) return QSM_ERR_ARG;
    cudaStreamSynchronize(ctx->stream);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    ctx->own_stream = false;
    ctx->stream = (cudaStream_t)stream;
    return QSM_OK;
}

void *qsm_ctx_get_stream(qsm_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

qsm_status qsm_ctx_set_verbose(qsm_ctx *ctx, int verbose)
{
    if (!ctx) return QSM_ERR_ARG;
    ctx->verbose = verbose;
    return QSM_OK;
}

qsm_status qsm_fp_pipe_rate(qsm_ctx *ctx, qsm_dtype dtype, double *ops_per_s)
{
    if (!ctx || !ops_per_s) return QSM_ERR_ARG;
    if (dtype != QSM_F32 && dtype != QSM_F64) return QSM_ERR_DTYPE;
    cudaSetDevice(ctx->device);
    int sms = 0;
    QSM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const dim3 grid((unsigned)sms * 8), block(256);
    const int iters = dtype == QSM_F64 ? 1000 : 40000;
    cudaEvent_t e0, e1;
    QSM_CUDA(cudaEventCreate(&e0));
    QSM_CUDA(cudaEventCreate(&e1));
    float best = 0.f;
    for (int rep = 0; rep < 4; ++rep) {
        QSM_CUDA(cudaEventRecord(e0, ctx->stream));
        if (dtype == QSM_F64)
            fp_rate_k<double><<<grid, block, 0, ctx->stream>>>(ctx->red_out, 0.999999, 1e-3, iters);
        else
            fp_rate_k<float><<<grid, block, 0, ctx->stream>>>((float *)ctx->red_out, 0.9999f, 1e-3f, iters);
        QSM_CUDA(cudaEventRecord(e1, ctx->stream));
        QSM_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        QSM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // launch 0 warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ops_per_s = (double)grid.x * block.x * 16.0 * iters / (best * 1e-3);
    return QSM_OK;
}

qsm_status qsm_fp_convert_check(qsm_ctx *ctx, unsigned long long *mismatches)
{
    if (!ctx || !mismatches) return QSM_ERR_ARG;
    cudaSetDevice(ctx->device);
    int sms = 0;
    QSM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    unsigned long long *bad = (unsigned long long *)ctx->red_out;
    QSM_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), ctx->stream));
    cvt_check_k<<<(unsigned)sms * 8, 256, 0, ctx->stream>>>(1ull << 32, 1ull << 30, bad);
    QSM_CUDA(cudaGetLastError());
    QSM_CUDA(cudaMemcpyAsync(ctx->host_out, bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    *mismatches = *(unsigned long long *)ctx->host_out;
    return QSM_OK;
}

qsm_status qsm_dot(qsm_ctx *ctx, qsm_dtype dtype, size_t n, const void *x, const void *y, double *out)
{
    if (!ctx || !x || !y || !out) return QSM_ERR_ARG;
    cudaSetDevice(ctx->device);
    const size_t es = dtype == QSM_F32 ? 4 : 8;
    if (dtype != QSM_F32 && dtype != QSM_F64) return QSM_ERR_DTYPE;
    Staged sx, sy;
    QSM_TRY(stage_in(ctx, sx, x, n * es, true));
    QSM_TRY(stage_in(ctx, sy, y, n * es, true));
    if (dtype == QSM_F32)
        QSM_TRY(lane_dot<float>(ctx, (const float *)sx.dev, (const float *)sy.dev, n, ctx->red_out));
    else
        QSM_TRY(lane_dot<double>(ctx, (const double *)sx.dev, (const double *)sy.dev, n, ctx->red_out));
    QSM_TRY(stage_out(ctx, sx, false));
    QSM_TRY(stage_out(ctx, sy, false));
    return read_double(ctx, ctx->red_out, out);
}

}  // extern "C"
