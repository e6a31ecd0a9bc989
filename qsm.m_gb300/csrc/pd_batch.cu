// Resident many-volume sessions: batched primal-dual TV/TGV and concurrent
// MG-PCG Poisson solves on one GPU.
//
// The reference solves one volume per MEX call (echo and volume loops are
// serial MATLAB: src/inversion/sstgv.m:68-71, src/bgremove/lbv.m:97-100).
// Here a session keeps every admitted solve's state resident in HBM and
// advances all primal-dual solves together:
//
//   * 30 iterations (the period of the 3-buffer primal / 2-buffer dual
//     rotation and of the every-10th-iteration monitor) are captured once
//     into a CUDA graph and replayed; the graph is re-captured only when the
//     resident set changes.  Kernels read the iteration count from a device
//     counter that the graph advances, so replays need no host work;
//   * a volume large enough to keep part of the GPU busy runs its one-volume
//     fused kernel (pd_fused.cu / pd_stream.cu, tile shape from the
//     autotuner) in its own graph branch; the branches of different volumes
//     overlap on the device;
//   * tiny volumes are packed: one persistent kernel per (tile variant,
//     TV|TGV) chunk and iteration walks a work list of (volume, active tile)
//     items spanning up to 56 volumes, whose descriptors (state pointers of
//     each of the 6 buffer rotations, constants, iteration window, monitor
//     scratch) are one kernel parameter; it runs the same tile / column body
//     (pd_tile.cuh);
//   * either way each volume's chi is bit-identical to its one-volume fused
//     solve;
//   * a volume admitted between replays starts at the session's iteration
//     base (a multiple of 30), so its buffer phase and monitor iterations
//     are the graph's; a volume whose monitors met tol, or that reached its
//     maxiter, does nothing in later launches;
//   * Poisson solves (mgpcg) either stay resident too and advance in the
//     same steps, every kernel of a PCG iteration launched once for all
//     solves of one multigrid shape (mg_pack.cuh), on a stream of their own
//     that runs beside the replays: at least one PCG iteration per 30
//     primal-dual iterations, and more while the replays run -- or, with
//     worker threads, run whole on the workers' streams, concurrently with
//     the replays.
//
// Admission is by device footprint against the session's byte budget.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <chrono>
#include <thread>
#include <vector>

#include "common.cuh"
#include "pd.cuh"
#include "pd_fused.cuh"
#include "pd_tile.cuh"
#include "mg_pack.cuh"

namespace qsm {

constexpr uint32_t kGraphIters = 30;  // lcm(3, 2, 10)
// A volume with at least (SM count) / kSoloDiv active tiles runs its
// one-volume kernel (state pointers as constant operands) in its own graph
// branch; branches overlap, so even a volume of a fraction of a wave keeps
// the GPU busy.  Only tinier volumes are packed into persistent
// multi-volume launches, whose per-item descriptor reads cost more than a
// launch saves above that size (measured on 32 volumes of 0.5-3.8 M
// voxels: branches 0.74 s, persistent packing 1.03 s, one volume after
// another 0.88 s).
constexpr int kSoloDiv = 4;
constexpr int kPhases = 6;            // lcm(3, 2)

// One volume, one buffer rotation (512 bytes).
struct BatchVol {
    FusedArgs a;        // tiles unused; part/count/ctl are the volume's own
    DualC<float> dc;
    PrimalC<float> pc;
    Dims d;
    double tol;
    uint32_t maxiter;   // iterations of this solve
    uint32_t start;     // session iteration at which it started (multiple of kGraphIters)
    uint32_t item0;     // first work item of this volume in its chunk's list
    uint32_t nitems;    // its active tiles
};

// The descriptors of up to kChunkVols volumes travel as one kernel
// parameter (constant bank, read-only: the kernels read state pointers as
// cheaply as the one-volume kernels do); a larger group is split into
// several chunks, each its own persistent launch.
constexpr int kChunkVols = 56;
struct BatchChunk {
    BatchVol v[kChunkVols];
};
static_assert(sizeof(BatchChunk) + 64 <= 32764, "kernel parameter limit");

// Persistent loop over the work items of one chunk: CTA b takes items b,
// b + gridDim.x, ... (items are tiles of equal size, so a static stride
// balances).  items[w] = (volume in the chunk, tile).  Whether a volume is
// past its maxiter or converged is read once when a CTA first meets one of
// its items: `done` cannot change while items of that volume are still
// unprocessed in this launch (the fold that sets it is its last item's).
template <int THREADS, typename Work>
__device__ __forceinline__ void batch_loop(const BatchChunk &P, const uint2 *__restrict__ items, uint32_t nitems,
                                           uint32_t g, bool check, double *red, Work work)
{
    __shared__ int sskip;
    uint32_t loaded = 0xffffffffu;
    for (uint32_t w = blockIdx.x; w < nitems; w += gridDim.x) {
        const uint2 it = __ldg(items + w);
        const BatchVol &v = P.v[it.x];
        __syncthreads();  // the previous item is done with shared memory
        if (it.x != loaded) {
            if (threadIdx.x == 0) sskip = (g - v.start >= v.maxiter) || *(volatile uint32_t *)&v.a.ctl->done;
            loaded = it.x;
            __syncthreads();
        }
        if (sskip) continue;
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        work(v, it.y, acc);
        if (check)
            monitor_fold<THREADS>(v.a.part, v.a.count, v.a.ctl, v.nitems, w - v.item0, red, acc, v.tol,
                                  g - v.start + 1);
    }
}

template <int TX, int TY, int TZ, int MINB, bool TGV, bool CHECK>
__global__ void __launch_bounds__(TX * TY, MINB)
batch_tile_k(const __grid_constant__ BatchChunk P, const uint2 *items, uint32_t nitems, const uint32_t *gbase,
             uint32_t i)
{
    extern __shared__ double smem_raw[];
    const uint32_t g = *gbase + i;
    batch_loop<TX * TY>(P, items, nitems, g, CHECK, smem_raw, [&](const BatchVol &v, unsigned tile, double *acc) {
        if (TGV) tile_tgv<TX, TY, TZ>(v.a, v.dc, v.pc, v.d, tile, CHECK, (float *)smem_raw, acc);
        else tile_tv<TX, TY, TZ>(v.a, v.dc, v.pc, v.d, tile, CHECK, (float *)smem_raw, acc);
    });
}

template <int TX, int TY, bool TGV, bool CHECK>
__global__ void __launch_bounds__((TX + 4) * (TY + 4), TGV ? 1 : 2)
batch_column_k(const __grid_constant__ BatchChunk P, const uint2 *items, uint32_t nitems, const uint32_t *gbase,
               uint32_t i, int cz)
{
    extern __shared__ double smem_raw[];
    const uint32_t g = *gbase + i;
    batch_loop<(TX + 4) * (TY + 4)>(P, items, nitems, g, CHECK, smem_raw,
                                    [&](const BatchVol &v, unsigned tile, double *acc) {
                                        column_pd<TX, TY, TGV>(v.a, v.dc, v.pc, v.d, cz, tile, CHECK,
                                                               (float *)smem_raw, acc);
                                    });
}

__global__ void advance_k(uint32_t *gbase, uint32_t n) { *gbase += n; }

// ---------------------------------------------------------------------------
// kernel table
// ---------------------------------------------------------------------------

struct BatchKernel {
    const void *fn[2];  // [check]
    bool column;
};

template <int TX, int TY, int TZ, int MINB, bool TGV>
static BatchKernel tile_kernel()
{
    return {{(const void *)batch_tile_k<TX, TY, TZ, MINB, TGV, false>, (const void *)batch_tile_k<TX, TY, TZ, MINB, TGV, true>},
            false};
}

template <int TX, int TY, bool TGV>
static BatchKernel column_kernel()
{
    return {{(const void *)batch_column_k<TX, TY, TGV, false>, (const void *)batch_column_k<TX, TY, TGV, true>}, true};
}

// Kernels of variant v (the same tile shapes as the one-volume path).
static BatchKernel batch_kernel(int v, bool tgv)
{
    switch (v) {
    case 0: return tgv ? tile_kernel<32, 8, 4, 4, true>() : tile_kernel<32, 8, 4, 4, false>();
    case 1: return tgv ? tile_kernel<32, 8, 2, 4, true>() : tile_kernel<32, 8, 2, 4, false>();
    case 2: return tgv ? tile_kernel<32, 4, 4, 8, true>() : tile_kernel<32, 4, 4, 8, false>();
    case 3: return tgv ? tile_kernel<32, 16, 2, 2, true>() : tile_kernel<32, 16, 2, 2, false>();
    case 8:
    case 9:
    case 10:  // TMA variants are packed with their register-prefetch stand-in
    case 11:
    case 12: return tgv ? column_kernel<28, 16, true>() : column_kernel<28, 16, false>();
    default: return tgv ? column_kernel<28, 12, true>() : column_kernel<28, 12, false>();
    }
}

}  // namespace qsm

using namespace qsm;

// ---------------------------------------------------------------------------
// session
// ---------------------------------------------------------------------------

namespace {

struct PdJob {
    uint64_t id = 0;
    PdVolume v;
    qsm_dtype dt = QSM_F32;
    double tol = 0.0;
    uint32_t maxiter = 0, start = 0, iters = 0;
    bool finished = false;
    PdCtl ctl{};
    double seconds = 0.0;
    size_t bytes = 0;
    std::vector<unsigned> tiles;  // active tiles of the chosen variant (host copy)
};

struct MgJob {
    uint64_t id = 0;
    Dims d{};
    size_t dims[3] = {0, 0, 0};
    double vsz[3] = {1, 1, 1};
    double tolcg = 0, tolmg = 0;
    int32_t maxitcg = 0, maxitmg = 0, mu = 1, npre = 1, npost = 1, nb = 0, nl = 1;
    bool mixed = true, has_v0 = false;
    void *blk = nullptr;  // device: v0 | f | out | mask
    double *v0 = nullptr, *f = nullptr, *out = nullptr;
    uint8_t *mask = nullptr;
    std::atomic<int> state{0};  // 0 queued, 1 running, 2 finished
    MgPackSolve *ps = nullptr;  // resident solve state (packed sessions)
    qsm_status st = QSM_OK;
    char err[256] = {0};
    qsm_mg_info info{};
    size_t bytes = 0;
};

// Up to kChunkVols volumes of one (tile variant, kind) group: one persistent
// launch per iteration.
struct Chunk {
    int var = 0;
    bool tgv = false;
    std::vector<PdJob *> vols;
    std::vector<uint2> items;
    std::unique_ptr<BatchChunk[]> phase;  // descriptors of each of the kPhases rotations
    uint2 *d_items = nullptr;             // inside the session's item buffer
    unsigned grid = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
};

}  // namespace

struct qsm_session {
    qsm_ctx *ctx = nullptr;
    size_t budget = 0, used = 0;
    uint64_t next_id = 1;
    std::map<uint64_t, std::unique_ptr<PdJob>> pd;
    std::map<uint64_t, std::unique_ptr<MgJob>> mg;

    // iteration base: host mirror and device copy
    uint32_t gbase = 0;
    void *dev_blk = nullptr;  // the device iteration base
    uint32_t *d_gbase = nullptr;

    // batched work of the resident running primal-dual solves
    bool dirty = true;
    bool serial = false;            // chunks one after another on the session stream
    bool one_cta_per_item = false;  // grid = items instead of a persistent grid
    uint32_t solo_tiles = 0;        // volumes with at least this many active tiles run solo
    std::vector<PdJob *> running;
    std::vector<PdJob *> solo;      // one-volume kernels, one graph branch each
    uint2 *d_items = nullptr;
    size_t items_cap = 0;
    std::vector<Chunk> chunks;
    cudaStream_t gstream[2 * kNumVariants] = {};
    cudaEvent_t gdone[2 * kNumVariants] = {};
    cudaEvent_t fork = nullptr, ev0 = nullptr, ev1 = nullptr;
    cudaGraphExec_t exec = nullptr;
    PdCtl *h_ctl = nullptr;  // pinned
    size_t h_ctl_cap = 0;

    // packed Poisson solves: their context (own stream), scratch and the resident solves;
    // a set-up thread with a context of its own prepares admitted solves (submits return at
    // once) and hands them to the steps through `ready`
    qsm_ctx *pctx = nullptr, *sctx = nullptr;
    double *h_res = nullptr;  // pinned
    std::vector<MgJob *> packed;
    std::thread setup;
    std::deque<MgJob *> setup_queue, ready;
    std::condition_variable ready_cv;  // a solve's set-up finished
    int setting_up = 0;                 // submitted solves whose set-up has not finished

    // Poisson workers
    std::vector<std::thread> workers;
    std::vector<qsm_ctx *> wctx;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<MgJob *> queue;
    bool stop = false;
};

namespace {

qsm_status fail(qsm_session *s, qsm_status st, const char *msg)
{
    set_error(s->ctx, "%s", msg);
    return st;
}

size_t mg_footprint(const Dims &d, int nl, bool mixed)
{
    // hierarchy (v, f, r + G, B per level, scratch) + PCG vectors + staged inputs/outputs
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const Dims dp{d.nx + 2, d.ny + 2, d.nz + 2};
    const size_t tm = mixed ? 4 : 8;
    size_t bytes = 0;
    Dims l = dp;
    for (int i = 0; i < nl; ++i) {
        if (i > 0) l = Dims{((l.nx - 2 + 1) >> 1) + 2, ((l.ny - 2 + 1) >> 1) + 2, ((l.nz - 2 + 1) >> 1) + 2};
        bytes += 3 * al(l.n() * tm) + 2 * al(l.n());
    }
    bytes += al(dp.n()) + 256;
    bytes += (mixed ? 4 : 2) * al(dp.n() * 8) + 4096;
    bytes += 3 * al(d.n() * 8) + al(d.n()) + 1024;  // v0, f, out, mask
    return bytes;
}

void worker_main(qsm_session *s, int w)
{
    qsm_ctx *ctx = s->wctx[w];
    cudaSetDevice(ctx->device);
    for (;;) {
        MgJob *j = nullptr;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv.wait(lock, [&] { return s->stop || !s->queue.empty(); });
            if (s->stop && s->queue.empty()) return;
            j = s->queue.front();
            s->queue.pop_front();
        }
        j->state.store(1);
        qsm_status st;
        if (j->mixed)
            st = qsm_mgpcg_mixed(ctx, j->dims, j->has_v0 ? j->v0 : nullptr, j->f, j->mask, j->vsz, j->tolcg,
                                 j->maxitcg, j->tolmg, j->maxitmg, j->mu, j->npre, j->npost, j->nb, j->nl, 0, j->out,
                                 &j->info);
        else
            st = qsm_mgpcg(ctx, QSM_F64, j->dims, j->has_v0 ? j->v0 : nullptr, j->f, j->mask, j->vsz, j->tolcg,
                           j->maxitcg, j->tolmg, j->maxitmg, j->mu, j->npre, j->npost, j->nb, j->nl, 0, j->out,
                           &j->info);
        j->st = st;
        if (st != QSM_OK) snprintf(j->err, sizeof j->err, "%s", qsm_last_error(ctx));
        j->state.store(2);
    }
}

// Sets up admitted Poisson solves of a packed session on its set-up context.
void setup_main(qsm_session *s)
{
    qsm_ctx *ctx = s->sctx;
    cudaSetDevice(ctx->device);
    for (;;) {
        MgJob *j = nullptr;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv.wait(lock, [&] { return s->stop || !s->setup_queue.empty(); });
            if (s->stop) return;  // solves still queued are released with the session
            j = s->setup_queue.front();
            s->setup_queue.pop_front();
        }
        const qsm_status st = mgpack_setup(ctx, j->mixed, j->d, j->has_v0 ? j->v0 : nullptr, j->f, j->mask, j->vsz,
                                           j->tolcg, j->maxitcg, j->tolmg, j->maxitmg, j->mu, j->npre, j->npost, j->nb,
                                           j->nl, &j->ps);
        {
            std::lock_guard<std::mutex> lock(s->mu);
            --s->setting_up;
            if (st != QSM_OK) {
                j->st = st;
                snprintf(j->err, sizeof j->err, "%s", qsm_last_error(ctx));
                j->state.store(2);
            } else {
                s->ready.push_back(j);
            }
        }
        s->ready_cv.notify_all();
    }
}

// Rebuilds the device work lists and re-captures the 30-iteration graph.
qsm_status rebuild(qsm_session *s)
{
    Range nvtx_range("session/rebuild");
    qsm_ctx *ctx = s->ctx;
    s->running.clear();
    for (auto &kv : s->pd)
        if (!kv.second->finished) s->running.push_back(kv.second.get());
    if (s->exec) {
        cudaGraphExecDestroy(s->exec);
        s->exec = nullptr;
    }
    s->chunks.clear();
    s->solo.clear();
    s->dirty = false;
    if (s->running.empty()) return QSM_OK;

    // chunks of one (variant, kind) group, volumes in admission order
    std::map<std::pair<int, int>, size_t> open;  // group -> chunk being filled
    for (PdJob *j : s->running) {
        if (j->tiles.size() >= s->solo_tiles) {
            s->solo.push_back(j);
            continue;
        }
        const auto key = std::make_pair(j->v.var, (int)j->v.tgv);
        auto it = open.find(key);
        if (it == open.end() || s->chunks[it->second].vols.size() == (size_t)kChunkVols) {
            Chunk c;
            c.var = j->v.var;
            c.tgv = j->v.tgv;
            s->chunks.push_back(std::move(c));
            open[key] = s->chunks.size() - 1;
            it = open.find(key);
        }
        s->chunks[it->second].vols.push_back(j);
    }
    size_t nitems = 0;
    for (auto &c : s->chunks) {
        c.phase.reset(new BatchChunk[kPhases]);
        memset(c.phase.get(), 0, kPhases * sizeof(BatchChunk));
        for (size_t k = 0; k < c.vols.size(); ++k) {
            PdJob *j = c.vols[k];
            const uint32_t item0 = (uint32_t)c.items.size();
            for (unsigned t : j->tiles) c.items.push_back(make_uint2((unsigned)k, t));
            for (int p = 0; p < kPhases; ++p) {
                BatchVol &b = c.phase[p].v[k];
                b.a = pd_volume_args(j->v, j->v.var, (uint32_t)p);
                b.a.tiles = nullptr;
                b.dc = j->v.dc;
                b.pc = j->v.pc;
                b.d = j->v.d;
                b.tol = j->tol;
                b.maxiter = j->maxiter;
                b.start = j->start;
                b.item0 = item0;
                b.nitems = (uint32_t)j->tiles.size();
            }
        }
        nitems += c.items.size();
    }
    if (nitems > s->items_cap) {
        if (s->d_items) QSM_TRY(dfree(ctx, s->d_items));
        s->d_items = nullptr;
        s->items_cap = std::max(nitems, 2 * s->items_cap);
        QSM_TRY(dalloc(ctx, (void **)&s->d_items, s->items_cap * sizeof(uint2)));
    }
    size_t off = 0;
    int sm = 0;
    QSM_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, ctx->device));
    for (size_t q = 0; q < s->chunks.size(); ++q) {
        Chunk &c = s->chunks[q];
        c.d_items = s->d_items + off;
        QSM_CUDA(cudaMemcpyAsync(c.d_items, c.items.data(), c.items.size() * sizeof(uint2), cudaMemcpyHostToDevice,
                                 ctx->stream));
        off += c.items.size();
        const BatchKernel bk = batch_kernel(c.var, c.tgv);
        int occ = 0;
        QSM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, bk.fn[0], variant_threads(c.var),
                                                               variant_smem(c.var, c.tgv)));
        occ = std::max(occ, 1);
        c.grid = (unsigned)std::min<size_t>(c.items.size(), (size_t)sm * occ);
        if (s->one_cta_per_item) c.grid = (unsigned)c.items.size();
        c.stream = s->serial ? ctx->stream : s->gstream[q % (2 * kNumVariants)];
        c.done = s->gdone[q % (2 * kNumVariants)];
    }
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));

    // capture kGraphIters iterations: one launch chain per chunk, forked from
    // and joined back into the session stream, then the base advance
    cudaGraph_t graph = nullptr;
    QSM_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaEventRecord(s->fork, ctx->stream);
    for (size_t q = 0; q < s->chunks.size() && ce == cudaSuccess; ++q) {
        Chunk &c = s->chunks[q];
        if (!s->serial && q < (size_t)(2 * kNumVariants)) ce = cudaStreamWaitEvent(c.stream, s->fork, 0);
        const BatchKernel bk = batch_kernel(c.var, c.tgv);
        const int threads = variant_threads(c.var);
        const size_t smem = variant_smem(c.var, c.tgv);
        uint32_t n = (uint32_t)c.items.size();
        for (uint32_t i = 0; i < kGraphIters && ce == cudaSuccess; ++i) {
            const bool chk = ((i + 1) % 10) == 0;
            BatchChunk *P = &c.phase[i % kPhases];
            if (bk.column) {
                int cz = variant(c.var).tz;
                void *args[] = {(void *)P, (void *)&c.d_items, (void *)&n, (void *)&s->d_gbase, (void *)&i,
                                (void *)&cz};
                ce = cudaLaunchKernel(bk.fn[chk], dim3(c.grid), dim3(threads), args, smem, c.stream);
            } else {
                void *args[] = {(void *)P, (void *)&c.d_items, (void *)&n, (void *)&s->d_gbase, (void *)&i};
                ce = cudaLaunchKernel(bk.fn[chk], dim3(c.grid), dim3(threads), args, smem, c.stream);
            }
        }
    }
    // solo volumes: their one-volume kernels, each volume on the next stream
    const size_t nbranch = s->chunks.size() + s->solo.size();
    for (size_t q = 0; q < s->solo.size() && ce == cudaSuccess; ++q) {
        PdJob *j = s->solo[q];
        const size_t slot = s->chunks.size() + q;
        cudaStream_t st = s->serial ? ctx->stream : s->gstream[slot % (2 * kNumVariants)];
        if (!s->serial && slot < (size_t)(2 * kNumVariants)) ce = cudaStreamWaitEvent(st, s->fork, 0);
        for (uint32_t i = 0; i < kGraphIters && ce == cudaSuccess; ++i) {
            FusedArgs a = pd_volume_args(j->v, j->v.var, i % kPhases);
            a.gbase = s->d_gbase;
            a.start = j->start;
            a.maxiter = j->maxiter;
            if (pd_volume_launch(ctx, st, j->v, ((i + 1) % 10) == 0, a, j->tol, i, i % kPhases) != QSM_OK)
                ce = cudaErrorLaunchFailure;
        }
    }
    // join every stream used (branches sharing a stream are already ordered)
    for (size_t q = 0; q < std::min(nbranch, (size_t)(2 * kNumVariants)) && ce == cudaSuccess && !s->serial; ++q) {
        ce = cudaEventRecord(s->gdone[q], s->gstream[q]);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(ctx->stream, s->gdone[q], 0);
    }
    if (ce == cudaSuccess) {
        advance_k<<<1, 1, 0, ctx->stream>>>(s->d_gbase, kGraphIters);
        ce = cudaGetLastError();
    }
    cudaError_t ee = cudaStreamEndCapture(ctx->stream, &graph);
    if (ce != cudaSuccess || ee != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        s->dirty = true;
        set_error(ctx, "graph capture failed: %s", cudaGetErrorString(ce != cudaSuccess ? ce : ee));
        return QSM_ERR_CUDA;
    }
    ce = cudaGraphInstantiate(&s->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
        s->exec = nullptr;
        s->dirty = true;
        set_error(ctx, "graph instantiation failed: %s", cudaGetErrorString(ce));
        return QSM_ERR_CUDA;
    }
    return QSM_OK;
}

qsm_status set_batch_smem(qsm_ctx *ctx)
{
    for (int v = 0; v < kNumVariants; ++v)
        for (int tg = 0; tg < 2; ++tg) {
            if (variant(v).tma) continue;  // never packed (admission switches them to kTmaFallback)
            const BatchKernel bk = batch_kernel(v, tg != 0);
            const int sm = (int)variant_smem(v, tg != 0);
            for (int c = 0; c < 2; ++c)
                QSM_CUDA(cudaFuncSetAttribute(bk.fn[c], cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
        }
    return QSM_OK;
}

void fill_pd_info(const PdJob &j, qsm_pd_info *info)
{
    if (!info) return;
    info->iters = j.iters;
    info->monitor_chi = j.ctl.checks ? j.ctl.n1 : 1.0;
    info->monitor_eta = j.ctl.checks ? j.ctl.n2 : 1.0;
    info->seconds = j.seconds;
    info->active_voxels = j.v.tl[j.v.var].active_vox;
    info->tile[0] = (uint32_t)variant(j.v.var).tx;
    info->tile[1] = (uint32_t)variant(j.v.var).ty;
    info->tile[2] = (uint32_t)variant(j.v.var).tz;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" {

qsm_status qsm_session_create(qsm_ctx *ctx, size_t budget_bytes, int32_t poisson_workers, qsm_session **out)
{
    if (!ctx || !out || poisson_workers < 0 || poisson_workers > 16) return QSM_ERR_ARG;  // 0: packed Poisson solves
    *out = nullptr;
    cudaSetDevice(ctx->device);
    std::unique_ptr<qsm_session> s(new qsm_session());
    s->ctx = ctx;
    s->budget = budget_bytes;
    {
        const char *e = getenv("QSM_BATCH_LAUNCH");  // "serial", "items", "serial,items"
        if (e && strstr(e, "serial")) s->serial = true;
        if (e && strstr(e, "items")) s->one_cta_per_item = true;
        int sm = 0;
        cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, ctx->device);
        s->solo_tiles = (uint32_t)std::max(sm / kSoloDiv, 1);
        const char *t = getenv("QSM_BATCH_SOLO_TILES");
        if (t && *t) s->solo_tiles = (uint32_t)strtoul(t, nullptr, 10);
    }
    QSM_TRY(set_batch_smem(ctx));
    const size_t blk = 256;
    QSM_TRY(dalloc(ctx, &s->dev_blk, blk));
    QSM_CUDA(cudaMemsetAsync(s->dev_blk, 0, blk, ctx->stream));
    s->d_gbase = (uint32_t *)s->dev_blk;
    for (int q = 0; q < 2 * kNumVariants; ++q) {
        QSM_CUDA(cudaStreamCreateWithFlags(&s->gstream[q], cudaStreamNonBlocking));
        QSM_CUDA(cudaEventCreateWithFlags(&s->gdone[q], cudaEventDisableTiming));
    }
    QSM_CUDA(cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming));
    QSM_CUDA(cudaEventCreate(&s->ev0));
    QSM_CUDA(cudaEventCreate(&s->ev1));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int w = 0; w < poisson_workers; ++w) {
        qsm_ctx *wc = nullptr;
        qsm_status st = qsm_ctx_create(ctx->device, &wc);
        if (st != QSM_OK) {
            qsm_session_destroy(s.release());
            return st;
        }
        s->wctx.push_back(wc);
    }
    qsm_session *raw = s.release();
    for (int w = 0; w < poisson_workers; ++w) raw->workers.emplace_back(worker_main, raw, w);
    *out = raw;
    return QSM_OK;
}

qsm_status qsm_session_destroy(qsm_session *s)
{
    if (!s) return QSM_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    for (auto &t : s->workers) t.join();
    if (s->setup.joinable()) s->setup.join();
    for (auto *wc : s->wctx) qsm_ctx_destroy(wc);
    if (s->sctx) cudaStreamSynchronize(s->sctx->stream);
    if (s->pctx) {
        for (auto &kv : s->mg)
            if (kv.second->ps) mgpack_finish(s->pctx, kv.second->ps, nullptr, nullptr);
        cudaStreamSynchronize(s->pctx->stream);
        qsm_ctx_destroy(s->pctx);
    }
    if (s->sctx) qsm_ctx_destroy(s->sctx);
    if (s->h_res) cudaFreeHost(s->h_res);
    qsm_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto &kv : s->pd) pd_volume_free(ctx, &kv.second->v);
    for (auto &kv : s->mg)
        if (kv.second->blk) dfree(ctx, kv.second->blk);
    if (s->exec) cudaGraphExecDestroy(s->exec);
    if (s->d_items) dfree(ctx, s->d_items);
    if (s->dev_blk) dfree(ctx, s->dev_blk);
    for (int q = 0; q < 2 * kNumVariants; ++q) {
        if (s->gstream[q]) cudaStreamDestroy(s->gstream[q]);
        if (s->gdone[q]) cudaEventDestroy(s->gdone[q]);
    }
    if (s->fork) cudaEventDestroy(s->fork);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->h_ctl) cudaFreeHost(s->h_ctl);
    cudaStreamSynchronize(ctx->stream);
    delete s;
    return QSM_OK;
}

size_t qsm_session_footprint(int32_t kind, const size_t dims[3], int32_t nlevels)
{
    if (!dims) return 0;
    const Dims d = make_dims(dims);
    switch (kind) {
    case QSM_JOB_TV: return pd_volume_bytes(false, d);
    case QSM_JOB_TGV: return pd_volume_bytes(true, d);
    case QSM_JOB_MGPCG: return mg_footprint(d, std::max(1, std::min(nlevels, 16)), true);
    case QSM_JOB_MGPCG_F64: return mg_footprint(d, std::max(1, std::min(nlevels, 16)), false);
    default: return 0;
    }
}

size_t qsm_session_bytes_in_use(const qsm_session *s) { return s ? s->used : 0; }

qsm_status qsm_session_submit_pd(qsm_session *s, int32_t tgv, qsm_dtype dt, const size_t dims[3], const void *d2f,
                                 const uint8_t *mask, const double vsz[3], double lam, double alpha, double tol,
                                 uint32_t maxiter, uint64_t *id)
{
    if (!s || !dims || !d2f || !mask || !vsz || !id) return QSM_ERR_ARG;
    if (dt != QSM_F32 && dt != QSM_F64) return QSM_ERR_DTYPE;
    qsm_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    if (d.n() == 0) return fail(s, QSM_ERR_DIMS, "empty volume");
    if (d.n() > 0xffffffffull) return fail(s, QSM_ERR_DIMS, "volume above 2^32 voxels");
    const size_t bytes = pd_volume_bytes(tgv != 0, d);
    if (s->budget && s->used + bytes > s->budget) return fail(s, QSM_ERR_BUSY, "session byte budget exceeded");
    const size_t es = dt == QSM_F32 ? 4 : 8;
    Staged sf, sm;
    QSM_TRY(stage_in(ctx, sf, d2f, d.n() * es, true));
    QSM_TRY(stage_in(ctx, sm, mask, d.n(), true));
    std::unique_ptr<PdJob> j(new PdJob());
    qsm_status st = pd_volume_init(ctx, &j->v, tgv != 0, d, dt, sf.dev, (const uint8_t *)sm.dev, vsz, lam, alpha);
    if (st == QSM_OK) st = pd_volume_tune(ctx, &j->v, maxiter);
    // a volume small enough to be packed runs the packed kernels, which have no TMA form
    if (st == QSM_OK && variant(j->v.var).tma && j->v.tl[j->v.var].nact < s->solo_tiles) j->v.var = kTmaFallback;
    stage_out(ctx, sf, false);
    stage_out(ctx, sm, false);
    if (st != QSM_OK) {
        pd_volume_free(ctx, &j->v);
        return st;
    }
    const TileList &tl = j->v.tl[j->v.var];
    j->tiles.resize(tl.nact);
    if (tl.nact)
        QSM_CUDA(cudaMemcpyAsync(j->tiles.data(), tl.dev, tl.nact * sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    j->id = s->next_id++;
    j->dt = dt;
    j->tol = tol;
    j->maxiter = maxiter;
    j->start = s->gbase;
    j->bytes = bytes;
    if (maxiter == 0 || tl.nact == 0) {
        // nothing to iterate: chi stays 0 (as the one-volume path)
        j->finished = true;
        j->iters = maxiter;
    }
    *id = j->id;
    s->used += bytes;
    s->pd.emplace(j->id, std::move(j));
    s->dirty = true;
    return QSM_OK;
}

qsm_status qsm_session_submit_mgpcg(qsm_session *s, const size_t dims[3], const double *v0, const double *f,
                                    const uint8_t *mask, const double vsz[3], double tolcg, int32_t maxitcg,
                                    double tolmg, int32_t maxitmg, int32_t mu, int32_t npre, int32_t npost,
                                    int32_t nboundary, int32_t nlevels, int32_t mixed, uint64_t *id)
{
    if (!s || !dims || !f || !mask || !vsz || !id) return QSM_ERR_ARG;
    if (nlevels < 1) return QSM_ERR_ARG;
    if (nlevels > 16) return QSM_ERR_DEPTH;
    qsm_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    const Dims d = make_dims(dims);
    if (d.n() == 0) return fail(s, QSM_ERR_DIMS, "empty volume");
    const size_t bytes = mg_footprint(d, nlevels, mixed != 0);
    if (s->budget && s->used + bytes > s->budget) return fail(s, QSM_ERR_BUSY, "session byte budget exceeded");
    std::unique_ptr<MgJob> j(new MgJob());
    const size_t vb = (d.n() * 8 + 255) & ~(size_t)255;
    QSM_TRY(dalloc(ctx, &j->blk, 3 * vb + d.n()));
    char *c = (char *)j->blk;
    j->v0 = (double *)c;
    j->f = (double *)(c + vb);
    j->out = (double *)(c + 2 * vb);
    j->mask = (uint8_t *)(c + 3 * vb);
    if (v0) QSM_CUDA(cudaMemcpyAsync(j->v0, v0, d.n() * 8, cudaMemcpyDefault, ctx->stream));
    QSM_CUDA(cudaMemcpyAsync(j->f, f, d.n() * 8, cudaMemcpyDefault, ctx->stream));
    QSM_CUDA(cudaMemcpyAsync(j->mask, mask, d.n(), cudaMemcpyDefault, ctx->stream));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    j->id = s->next_id++;
    j->d = d;
    for (int q = 0; q < 3; ++q) {
        j->dims[q] = dims[q];
        j->vsz[q] = vsz[q];
    }
    j->tolcg = tolcg;
    j->maxitcg = maxitcg;
    j->tolmg = tolmg;
    j->maxitmg = maxitmg;
    j->mu = mu;
    j->npre = npre;
    j->npost = npost;
    j->nb = nboundary;
    j->nl = nlevels;
    j->mixed = mixed != 0;
    j->has_v0 = v0 != nullptr;
    j->bytes = bytes;
    const bool packed = s->workers.empty();
    if (packed && !s->pctx) {
        // packed: the steps' context, the set-up context and its thread, made on first use
        QSM_TRY(qsm_ctx_create(ctx->device, &s->pctx));
        QSM_TRY(qsm_ctx_create(ctx->device, &s->sctx));
        QSM_CUDA(cudaMallocHost((void **)&s->h_res, 16 * sizeof(double)));
        s->setup = std::thread(setup_main, s);
    }
    *id = j->id;
    s->used += bytes;
    MgJob *raw = j.get();
    s->mg.emplace(j->id, std::move(j));
    if (packed) {
        {
            std::lock_guard<std::mutex> lock(s->mu);
            s->setup_queue.push_back(raw);
            ++s->setting_up;
        }
        s->cv.notify_all();
        return QSM_OK;
    }
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->queue.push_back(raw);
    }
    s->cv.notify_all();
    return QSM_OK;
}

qsm_status qsm_session_step(qsm_session *s, uint32_t iters)
{
    Range nvtx_range("session/step");
    if (!s) return QSM_ERR_ARG;
    qsm_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    if (s->dirty) QSM_TRY(rebuild(s));
    const uint32_t reps = std::max<uint32_t>(1, (iters + kGraphIters - 1) / kGraphIters);
    if (!s->running.empty()) {
        QSM_CUDA(cudaEventRecord(s->ev0, ctx->stream));
        for (uint32_t r = 0; r < reps; ++r) QSM_CUDA(cudaGraphLaunch(s->exec, ctx->stream));
        QSM_CUDA(cudaEventRecord(s->ev1, ctx->stream));
    }
    if (s->pctx) {
        std::unique_lock<std::mutex> lock(s->mu);
        // nothing else to advance while solves are being set up: wait for one (briefly)
        if (s->running.empty() && s->packed.empty() && s->ready.empty() && s->setting_up > 0)
            s->ready_cv.wait_for(lock, std::chrono::milliseconds(2),
                                 [&] { return !s->ready.empty() || s->setting_up == 0; });
        for (MgJob *j : s->ready) {
            j->state.store(1);
            s->packed.push_back(j);
        }
        s->ready.clear();
    }
    // packed Poisson solves, on their own stream while the replays run: at least one PCG
    // iteration per 30 primal-dual iterations, and more for as long as the replays have not
    // finished
    if (!s->packed.empty()) {
        std::vector<MgPackSolve *> ps;
        for (uint32_t r = 0;; ++r) {
            if (r >= reps && (s->running.empty() || cudaEventQuery(s->ev1) != cudaErrorNotReady)) break;
            ps.clear();
            for (MgJob *j : s->packed)
                if (!mgpack_done(j->ps)) ps.push_back(j->ps);
            if (ps.empty()) break;
            const qsm_status st = mgpack_step(s->pctx, ps.data(), (int)ps.size(), s->h_res);
            if (st != QSM_OK) return fail(s, st, qsm_last_error(s->pctx));
        }
        cudaGetLastError();  // a not-ready event query leaves no error behind
        std::vector<MgJob *> keep;
        for (MgJob *j : s->packed) {
            if (!mgpack_done(j->ps)) {
                keep.push_back(j);
                continue;
            }
            j->st = mgpack_finish(s->pctx, j->ps, j->out, &j->info);
            j->ps = nullptr;
            if (j->st != QSM_OK) snprintf(j->err, sizeof j->err, "%s", qsm_last_error(s->pctx));
            j->state.store(2);
        }
        s->packed.swap(keep);
    }
    if (s->running.empty()) return QSM_OK;
    s->gbase += reps * kGraphIters;
    const size_t nv = s->running.size();
    if (nv > s->h_ctl_cap) {
        if (s->h_ctl) cudaFreeHost(s->h_ctl);
        s->h_ctl = nullptr;
        s->h_ctl_cap = std::max(nv, 2 * s->h_ctl_cap);
        QSM_CUDA(cudaMallocHost((void **)&s->h_ctl, s->h_ctl_cap * sizeof(PdCtl)));
    }
    for (size_t k = 0; k < nv; ++k)
        QSM_CUDA(cudaMemcpyAsync(s->h_ctl + k, s->running[k]->v.ctl, sizeof(PdCtl), cudaMemcpyDeviceToHost, ctx->stream));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    for (size_t k = 0; k < nv; ++k) {
        PdJob *j = s->running[k];
        j->ctl = s->h_ctl[k];
        j->seconds += ms * 1e-3;
        const uint32_t done_it = s->gbase - j->start;
        if (j->ctl.stalled) {  // a bounded TMA wait gave up: the job ends with QSM_ERR_TIMEOUT
            j->finished = true;
            j->iters = std::min(done_it, j->maxiter);
        } else if (j->ctl.done) {
            j->finished = true;
            j->iters = j->ctl.iters;
        } else if (done_it >= j->maxiter) {
            j->finished = true;
            j->iters = j->maxiter;
        }
        if (j->finished) s->dirty = true;
    }
    return QSM_OK;
}

qsm_status qsm_session_poll(qsm_session *s, uint64_t id, int32_t *finished, qsm_pd_info *pd_info,
                            qsm_mg_info *mg_info)
{
    if (!s || !finished) return QSM_ERR_ARG;
    auto ip = s->pd.find(id);
    if (ip != s->pd.end()) {
        *finished = ip->second->finished ? 1 : 0;
        fill_pd_info(*ip->second, pd_info);
        if (ip->second->ctl.stalled) return fail(s, QSM_ERR_TIMEOUT, "a bounded wait on a TMA load gave up");
        return QSM_OK;
    }
    auto im = s->mg.find(id);
    if (im != s->mg.end()) {
        MgJob &j = *im->second;
        *finished = j.state.load() == 2 ? 1 : 0;
        if (*finished && mg_info) {
            double *hist = mg_info->resnorm_hist;
            *mg_info = j.info;
            mg_info->resnorm_hist = hist;
        }
        if (*finished && j.st != QSM_OK) return fail(s, j.st, j.err);
        return QSM_OK;
    }
    return fail(s, QSM_ERR_ARG, "unknown session job id");
}

qsm_status qsm_session_fetch(qsm_session *s, uint64_t id, void *out)
{
    if (!s || !out) return QSM_ERR_ARG;
    qsm_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    auto ip = s->pd.find(id);
    if (ip != s->pd.end()) {
        PdJob &j = *ip->second;
        if (!j.finished) return fail(s, QSM_ERR_BUSY, "job still running");
        if (j.ctl.stalled) return fail(s, QSM_ERR_TIMEOUT, "a bounded wait on a TMA load gave up");
        const size_t es = j.dt == QSM_F32 ? 4 : 8;
        Staged so;
        QSM_TRY(stage_in(ctx, so, out, j.v.d.n() * es, false));
        QSM_TRY(pd_volume_result(ctx, j.v, j.iters, j.dt, so.dev));
        QSM_TRY(stage_out(ctx, so, true));
        QSM_CUDA(cudaStreamSynchronize(ctx->stream));
        QSM_TRY(pd_volume_free(ctx, &j.v));
        s->used -= j.bytes;
        s->pd.erase(ip);
        return QSM_OK;
    }
    auto im = s->mg.find(id);
    if (im != s->mg.end()) {
        MgJob &j = *im->second;
        if (j.state.load() != 2) return fail(s, QSM_ERR_BUSY, "job still running");
        qsm_status st = j.st;
        if (st == QSM_OK) {
            QSM_CUDA(cudaMemcpyAsync(out, j.out, j.d.n() * 8, cudaMemcpyDefault, ctx->stream));
            QSM_CUDA(cudaStreamSynchronize(ctx->stream));
        }
        QSM_TRY(dfree(ctx, j.blk));
        s->used -= j.bytes;
        s->mg.erase(im);
        return st;
    }
    return fail(s, QSM_ERR_ARG, "unknown session job id");
}

uint32_t qsm_session_running(const qsm_session *s)
{
    if (!s) return 0;
    uint32_t n = 0;
    for (auto &kv : s->pd) n += kv.second->finished ? 0 : 1;
    for (auto &kv : s->mg) n += kv.second->state.load() == 2 ? 0 : 1;
    return n;
}

static qsm_status pd_batch(qsm_ctx *ctx, bool tgv, qsm_dtype dt, uint32_t count, const size_t *dims,
                           const void *const *d2f, const uint8_t *const *mask, const double vsz[3], double lam,
                           double alpha, double tol, uint32_t maxiter, void *const *chi, qsm_pd_info *info)
{
    if (!ctx || !dims || !d2f || !mask || !vsz || !chi) return QSM_ERR_ARG;
    if (dt != QSM_F32 && dt != QSM_F64) return QSM_ERR_DTYPE;
    qsm_session *s = nullptr;
    QSM_TRY(qsm_session_create(ctx, 0, 0, &s));
    std::vector<uint64_t> ids(count);
    qsm_status st = QSM_OK;
    for (uint32_t b = 0; b < count && st == QSM_OK; ++b)
        st = qsm_session_submit_pd(s, tgv ? 1 : 0, dt, dims + 3 * b, d2f[b], mask[b], vsz, lam, alpha, tol, maxiter,
                                   &ids[b]);
    // advance until every solve stopped (check the monitors every 90 iterations)
    while (st == QSM_OK && qsm_session_running(s) > 0) st = qsm_session_step(s, 3 * kGraphIters);
    for (uint32_t b = 0; b < count && st == QSM_OK; ++b) {
        int32_t fin = 0;
        st = qsm_session_poll(s, ids[b], &fin, info ? info + b : nullptr, nullptr);
        if (st == QSM_OK) st = qsm_session_fetch(s, ids[b], chi[b]);
    }
    if (st != QSM_OK) {
        qsm_session_destroy(s);
        return st;
    }
    return qsm_session_destroy(s);
}

qsm_status qsm_pd_tv_batch(qsm_ctx *ctx, qsm_dtype dt, uint32_t count, const size_t *dims, const void *const *d2f,
                           const uint8_t *const *mask, const double vsz[3], double lam, double tol, uint32_t maxiter,
                           void *const *chi, qsm_pd_info *info)
{
    Range nvtx_range("pd_tv_batch");
    return pd_batch(ctx, false, dt, count, dims, d2f, mask, vsz, lam, 0.0, tol, maxiter, chi, info);
}

qsm_status qsm_pd_tgv_batch(qsm_ctx *ctx, qsm_dtype dt, uint32_t count, const size_t *dims, const void *const *d2f,
                            const uint8_t *const *mask, const double vsz[3], double lam, double alpha, double tol,
                            uint32_t maxiter, void *const *chi, qsm_pd_info *info)
{
    Range nvtx_range("pd_tgv_batch");
    return pd_batch(ctx, true, dt, count, dims, d2f, mask, vsz, lam, alpha, tol, maxiter, chi, info);
}

}  // extern "C"
