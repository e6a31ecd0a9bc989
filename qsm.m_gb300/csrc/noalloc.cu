// qsm_norm2_noalloc: the masked pairwise 2-norm of norm2_mex, for callers
// that cannot allocate device memory.
//
// Who needs it: applications that own every byte of device memory
// themselves -- a MATLAB session hands its MEX files gpuArray memory from
// MATLAB's own pool, and latency-critical pipelines allocate everything
// once at start-up -- and must not let a library call cudaMalloc/cudaFree
// mid-run (those calls synchronise the device and can stall other streams).
// This variant takes only device pointers and a stream, and keeps its
// scratch (one partial sum per leaf of the pairwise tree) in a fixed
// file-scope device array instead of allocating it.
//
// Limits and sharing:
//   - n must satisfy 1 <= n <= QSM_NORM2_NOALLOC_MAX_N (2^25 elements); the
//     scratch holds at most n/64 + 1 leaf sums (4 MiB of doubles), and every
//     GPU that loads the library keeps that array until the process exits;
//   - every call shares the one array, and it keeps the last call's
//     contents (each call rewrites every leaf sum it reads, so nothing has
//     to start at zero); calls that overlap on the GPU -- on two streams, or
//     from two host threads -- race on it;
//   - the first call on each device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current) and caches it with
//     the id of the CUDA context that was current; make that first call
//     before any stream capture.  A device reset (cudaDeviceReset, MATLAB's
//     reset(gpuDevice)) destroys the context and unloads the array, so the
//     next call sees a new context id and looks the address up again: the
//     first call after a reset is a set-up call too, and also belongs
//     outside stream capture.
#include <cuda.h>
#include <cuda_runtime.h>
#include <mutex>
#include <stdint.h>

#include "../../include/qsm_gpu.h"

namespace {

constexpr size_t kMaxN = QSM_NORM2_NOALLOC_MAX_N;
constexpr size_t kMaxLeaves = kMaxN / 64 + 1;  // leaves hold 64..128 elements when n > 128
constexpr int kLeaf = 128;                      // norm2_mex.c BLOCK_SIZE
constexpr int kMaxDevices = 64;

// Per-leaf partial sums (doubles; FP32 sums use the first half as floats).
static __device__ __align__(256) double g_norm2_leaf_sums[kMaxLeaves];

// Device address of g_norm2_leaf_sums per device, with the id of the
// context it was looked up in (0: not looked up yet).
struct ScratchSlot {
    unsigned long long ctx_id;
    double *ptr;
};
ScratchSlot g_scratch[kMaxDevices];
std::mutex g_scratch_mu;

// The driver's context queries, reached through the runtime (the library
// does not link libcuda itself).
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

// Id of the calling thread's current CUDA context; 0 when none is current
// yet.  False when the driver does not offer the queries.
bool current_ctx_id(unsigned long long &id)
{
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult ra, rb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 4000, cudaEnableDefault, &ra) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &rb) != cudaSuccess ||
            ra != cudaDriverEntryPointSuccess || rb != cudaDriverEntryPointSuccess || !a || !b) {
            cudaGetLastError();
            return false;
        }
        get_current = (CtxGetCurrentFn)a;
        get_id = (CtxGetIdFn)b;
    }
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS) return false;
    id = 0;
    return !c || get_id(c, &id) == CUDA_SUCCESS;
}

// (L(a), L(a+1)): leaf counts of the pairwise tree for sizes a and a+1.
// A node of size s > 128 splits into s/2 (rounded down) and the rest.
__host__ __device__ inline void leaf_pair(size_t a, size_t &la, size_t &la1)
{
    if (a + 1 <= (size_t)kLeaf) {
        la = 1;
        la1 = 1;
        return;
    }
    size_t lb, lb1;
    leaf_pair(a >> 1, lb, lb1);
    const size_t b = a >> 1;
    if ((a & 1) == 0) {  // a = 2b, a+1 = 2b+1
        la = a <= (size_t)kLeaf ? 1 : lb + lb;
        la1 = lb + lb1;
    } else {             // a = 2b+1, a+1 = 2b+2
        la = lb + lb1;
        la1 = lb1 + lb1;
    }
    (void)b;
}

__host__ __device__ inline size_t leaf_count(size_t s)
{
    if (s <= (size_t)kLeaf) return 1;
    size_t l0, l1;
    leaf_pair(s, l0, l1);
    return l0;
}

// Leaf t of the tree over [0, n): its offset and length.
__device__ inline void leaf_at(size_t n, size_t t, size_t &off, size_t &len)
{
    off = 0;
    size_t s = n;
    while (s > (size_t)kLeaf) {
        const size_t m = s >> 1;
        const size_t lm = leaf_count(m);
        if (t < lm) {
            s = m;
        } else {
            t -= lm;
            off += m;
            s -= m;
        }
    }
    len = s;
}

// One thread per leaf: the sequential masked sum of squares of
// norm2_mex.c:83-131 (FP32 input sums in FP32).
template <typename T>
__global__ void leaf_sums_k(T *sums, size_t nleaf, size_t n, const T *__restrict__ x, const uint8_t *__restrict__ G)
{
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nleaf) return;
    size_t off, len;
    leaf_at(n, t, off, len);
    T s = G[off] ? x[off] * x[off] : (T)0;
    for (size_t i = 1; i < len; ++i)
        if (G[off + i]) s += x[off + i] * x[off + i];
    sums[t] = s;
}

// One thread combines the leaf sums along the tree (left + right at every
// node, as the recursion does) and writes sqrt of the total to *out.
template <typename T>
__global__ void combine_k(double *out, const T *sums, size_t n)
{
    struct Frame { size_t n; T left; int state; };
    Frame stk[64];
    int sp = 0;
    size_t li = 0;
    T ret = (T)0;
    stk[0] = {n, (T)0, 0};
    while (sp >= 0) {
        Frame &f = stk[sp];
        if (f.n <= (size_t)kLeaf) {
            ret = sums[li++];
            --sp;
        } else if (f.state == 0) {
            f.state = 1;
            stk[sp + 1] = {f.n >> 1, (T)0, 0};
            ++sp;
        } else if (f.state == 1) {
            f.left = ret;
            f.state = 2;
            stk[sp + 1] = {f.n - (f.n >> 1), (T)0, 0};
            ++sp;
        } else {
            ret = f.left + ret;
            --sp;
        }
    }
    *out = sizeof(T) == 4 ? (double)sqrtf((float)ret) : sqrt((double)ret);
}

bool on_device(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" qsm_status qsm_norm2_noalloc(qsm_dtype dtype, size_t n, const void *x, const uint8_t *G, double *out,
                                        void *stream)
{
    if (dtype != QSM_F32 && dtype != QSM_F64) return QSM_ERR_DTYPE;
    if (n == 0 || n > kMaxN) return QSM_ERR_DIMS;
    if (!x || !G || !out) return QSM_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return QSM_ERR_CUDA;
    }
    if (!on_device(x) || !on_device(G) || !on_device(out)) return QSM_ERR_ARG;
    double *scratch;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        unsigned long long id = 0;
        if (!current_ctx_id(id)) return QSM_ERR_CUDA;
        ScratchSlot &slot = g_scratch[dev];
        if (id == 0 || slot.ctx_id != id || !slot.ptr) {
            // set-up for this device and context: look the array up (this
            // also creates the context when the runtime has not yet)
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_norm2_leaf_sums) != cudaSuccess || !p) {
                cudaGetLastError();
                return QSM_ERR_CUDA;
            }
            if (!current_ctx_id(id) || id == 0) return QSM_ERR_CUDA;
            slot.ctx_id = id;
            slot.ptr = (double *)p;
        }
        scratch = slot.ptr;
    }
    const cudaStream_t s = (cudaStream_t)stream;
    const size_t nleaf = leaf_count(n);
    const unsigned grid = (unsigned)((nleaf + 255) / 256);
    if (dtype == QSM_F32) {
        leaf_sums_k<float><<<grid, 256, 0, s>>>((float *)scratch, nleaf, n, (const float *)x, G);
        combine_k<float><<<1, 1, 0, s>>>(out, (const float *)scratch, n);
    } else {
        leaf_sums_k<double><<<grid, 256, 0, s>>>(scratch, nleaf, n, (const double *)x, G);
        combine_k<double><<<1, 1, 0, s>>>(out, scratch, n);
    }
    return cudaGetLastError() == cudaSuccess ? QSM_OK : QSM_ERR_CUDA;
}
