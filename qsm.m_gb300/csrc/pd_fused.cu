// Primal-dual TGV / TV inversion, mixed-precision fused path.
//
// One kernel per iteration does the dual update, the primal update and the
// extragradient for a 3-D tile of the interior:
//
//   1. the dual (nu, p, q) is evaluated on the tile plus the one-voxel layer
//      on its low side (which the primal's backward differences read) and
//      nu alone on the high-side faces (the primal's Laplacian reads them),
//      into shared memory; halo points are recomputed by every tile that
//      needs them, with identical arithmetic, instead of synchronising the
//      grid;
//   2. the primal (chi, eta, w) of the tile reads the dual from shared
//      memory and writes the next iterate.
//
// Only tiles holding mask voxels are launched: outside m and mi the
// reference never changes anything, so the primal and the dual stay 0 there
// in every buffer.  Inside a tile, the dual is only read where mi holds (it
// is identically 0 elsewhere).
//
// Storage (all FP32, component-major): the primal family {chi, eta, w1..3}
// is triple-buffered and the extragradient point chi_ = chi^n + (chi^n -
// chi^(n-1)) is formed where it is read, so it is never stored; the dual
// family {nu, p1..3, q1..6} is double-buffered.  Per iteration an active
// voxel reads chi^n, chi^(n-1) (5+5 arrays), the dual (10), f (1) and one
// mask byte, and writes chi^(n+1) (5) and the dual (10): 36 arrays + 1 B =
// 145 B, against 51 arrays + 2 B (206 B) for the reference's two sweeps.
//
// Per voxel the FP32 expressions and their association order are those of
// update_dualf / update_primalf (pd_tgv_mex.c:332-485, :659-812; TV:
// pd_tv_mex.c:314-412, :524-622); the file is built without fused
// multiply-add, so chi is bit-identical to the reference's mx_pdf.
//
// Convergence monitors (every 10th iteration) accumulate in FP64 inside the
// kernel from the old and new chi/eta held in registers: block partials,
// then the last block reduces them in a fixed order (deterministic).
//
// Tile shapes: a few compiled variants; the first solve on a grid size times
// each for a few iterations and keeps the fastest (an in-process table,
// optionally persisted in the file named by QSM_AUTOTUNE_CACHE);
// QSM_FUSED_VARIANT=<index> forces one.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "pd.cuh"
#include "pd_fused.cuh"
#include "pd_tile.cuh"

namespace qsm {

// mask byte: bit 0 = m (primal update), bit 1 = mi (dual update)
__global__ void pack_masks_k(uint8_t *mm, const uint8_t *__restrict__ m, const uint8_t *__restrict__ mi, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        mm[l] = (uint8_t)((m[l] ? 1 : 0) | (mi[l] ? 2 : 0));
}

// A tile is active iff one of its voxels is in m (primal update) or in mi
// (dual update).
__global__ void tile_flags_k(uint8_t *flag, const uint8_t *__restrict__ mm, Dims d, unsigned gx, unsigned gy, int tx,
                             int ty, int tz)
{
    const unsigned t = blockIdx.x;
    const size_t x0 = 1 + (size_t)(t % gx) * tx, y0 = 1 + (size_t)((t / gx) % gy) * ty, z0 = 1 + (size_t)(t / (gx * gy)) * tz;
    int any = 0;
    for (int p = threadIdx.x; p < tx * ty * tz; p += blockDim.x) {
        const size_t x = x0 + p % tx, y = y0 + (p / tx) % ty, z = z0 + p / (tx * ty);
        if (x + 1 < d.nx && y + 1 < d.ny && z + 1 < d.nz && mm[x + d.nx * (y + d.ny * z)]) any = 1;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) flag[t] = (uint8_t)any;
}

// ---------------------------------------------------------------------------
// TGV
// ---------------------------------------------------------------------------

template <int TX, int TY, int TZ, int MINB, bool CHECK>
__global__ void __launch_bounds__(TX * TY, MINB)
tgv_fused_k(FusedArgs s, DualC<float> dc, PrimalC<float> pc, Dims d, double tol, uint32_t it)
{
    extern __shared__ double shd_raw[];  // the dual (reused for the monitor reduction)
    if (s.ctl->done) return;
    const uint32_t itn = launch_iter(s, it);
    if (!itn) return;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    tile_tgv<TX, TY, TZ>(s, dc, pc, d, s.tiles[blockIdx.x], CHECK, (float *)shd_raw, acc);
    if (CHECK) monitor_reduce<TX * TY>(s, shd_raw, acc, tol, itn);
}

// ---------------------------------------------------------------------------
// TV: primal {chi, eta}, dual {nu, p1..3}
// ---------------------------------------------------------------------------

template <int TX, int TY, int TZ, int MINB, bool CHECK>
__global__ void __launch_bounds__(TX * TY, MINB)
tv_fused_k(FusedArgs s, DualC<float> dc, PrimalC<float> pc, Dims d, double tol, uint32_t it)
{
    extern __shared__ double shd_raw[];  // the dual (reused for the monitor reduction)
    if (s.ctl->done) return;
    const uint32_t itn = launch_iter(s, it);
    if (!itn) return;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    tile_tv<TX, TY, TZ>(s, dc, pc, d, s.tiles[blockIdx.x], CHECK, (float *)shd_raw, acc);
    if (CHECK) monitor_reduce<TX * TY>(s, shd_raw, acc, tol, itn);
}

// ---------------------------------------------------------------------------
// variants, launch, autotuning
// ---------------------------------------------------------------------------

// 3-D tiles: threads = tx * ty; streaming: threads = (tx + 4) * (ty + 4);
// 10-12: TMA-staged column kernels (TGV)
static const Variant kVariants[kNumVariants] = {
    {32, 8, 4, false, false},  {32, 8, 2, false, false},  {32, 4, 4, false, false},  {32, 16, 2, false, false},
    {28, 12, 8, true, false},  {28, 12, 16, true, false}, {28, 12, 32, true, false}, {28, 12, 64, true, false},
    {28, 16, 16, true, false}, {28, 16, 32, true, false}, {28, 16, 16, true, true},  {28, 20, 16, true, true},
    {28, 24, 16, true, true}};

const Variant &variant(int v) { return kVariants[v]; }

int variant_threads(int v)
{
    const Variant &x = kVariants[v];
    return x.stream ? (x.tx + 4) * (x.ty + 4) : x.tx * x.ty;
}

size_t variant_smem(int v, bool tgv)
{
    const Variant &x = kVariants[v];
    if (x.tma && tgv) return stream_tma_smem(x.tx, x.ty);
    if (x.stream) return stream_smem(x.tx, x.ty, tgv);
    const size_t bn = (size_t)(x.tx + 2) * (x.ty + 2) * (x.tz + 2);
    const size_t dual = (tgv ? 10 : 4) * bn * sizeof(float);
    const size_t red = 4 * (size_t)x.tx * x.ty * sizeof(double);
    return std::max(dual, red);
}

template <int TX, int TY, int TZ, int MINB>
static void launch_t(cudaStream_t st, bool tgv, bool chk, unsigned nact, const FusedArgs &s, const DualC<float> &dc,
                     const PrimalC<float> &pc, const Dims &d, double tol, uint32_t it, size_t smem)
{
    if (tgv) {
        if (chk) tgv_fused_k<TX, TY, TZ, MINB, true><<<nact, TX * TY, smem, st>>>(s, dc, pc, d, tol, it);
        else tgv_fused_k<TX, TY, TZ, MINB, false><<<nact, TX * TY, smem, st>>>(s, dc, pc, d, tol, it);
    } else {
        if (chk) tv_fused_k<TX, TY, TZ, MINB, true><<<nact, TX * TY, smem, st>>>(s, dc, pc, d, tol, it);
        else tv_fused_k<TX, TY, TZ, MINB, false><<<nact, TX * TY, smem, st>>>(s, dc, pc, d, tol, it);
    }
}

template <int TX, int TY, int TZ, int MINB>
static qsm_status set_smem_t(qsm_ctx *ctx, size_t tgv_smem, size_t tv_smem)
{
    QSM_CUDA(cudaFuncSetAttribute(tgv_fused_k<TX, TY, TZ, MINB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tgv_smem));
    QSM_CUDA(cudaFuncSetAttribute(tgv_fused_k<TX, TY, TZ, MINB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tgv_smem));
    QSM_CUDA(cudaFuncSetAttribute(tv_fused_k<TX, TY, TZ, MINB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tv_smem));
    QSM_CUDA(cudaFuncSetAttribute(tv_fused_k<TX, TY, TZ, MINB, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tv_smem));
    return QSM_OK;
}

bool variant_ok(const PdVolume &v, int var)
{
    return var >= 0 && var < kNumVariants && (!kVariants[var].tma || (v.tgv && !v.maps.empty()));
}

// tm: the volume's TMA maps of this iteration (TMA variants)
static qsm_status launch_variant(qsm_ctx *ctx, cudaStream_t st, int v, bool tgv, bool chk, unsigned nact,
                                 const FusedArgs &s, const DualC<float> &dc, const PrimalC<float> &pc, const Dims &d,
                                 double tol, uint32_t it, const TmaMaps *tm)
{
    const size_t sm = variant_smem(v, tgv);
    if (kVariants[v].tma && !tm) return QSM_ERR_ARG;
    if (kVariants[v].stream)
        return stream_launch(ctx, st, kVariants[v].tx, kVariants[v].ty, kVariants[v].tz, tgv, chk, nact, s, dc, pc, d,
                             tol, it, kVariants[v].tma ? tm : nullptr);
    switch (v) {
    case 0: launch_t<32, 8, 4, 4>(st, tgv, chk, nact, s, dc, pc, d, tol, it, sm); break;
    case 1: launch_t<32, 8, 2, 4>(st, tgv, chk, nact, s, dc, pc, d, tol, it, sm); break;
    case 2: launch_t<32, 4, 4, 8>(st, tgv, chk, nact, s, dc, pc, d, tol, it, sm); break;
    case 3: launch_t<32, 16, 2, 2>(st, tgv, chk, nact, s, dc, pc, d, tol, it, sm); break;
    default: return QSM_ERR_ARG;
    }
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

// the TMA maps of variant var for the iteration whose arguments are pd_volume_args(v, var, rot)
static const TmaMaps *volume_maps(const PdVolume &v, int var, uint32_t rot)
{
    if (!kVariants[var].tma || v.maps.empty()) return nullptr;
    return &v.maps[(size_t)var * 3 + rot % 3];
}

qsm_status pd_volume_launch(qsm_ctx *ctx, cudaStream_t st, const PdVolume &v, bool chk, const FusedArgs &s,
                            double tol, uint32_t it, uint32_t rot)
{
    return launch_variant(ctx, st, v.var, v.tgv, chk, v.tl[v.var].nact, s, v.dc, v.pc, v.d, tol, it,
                          volume_maps(v, v.var, rot));
}

static qsm_status set_all_smem(qsm_ctx *ctx)
{
    QSM_TRY((set_smem_t<32, 8, 4, 4>(ctx, variant_smem(0, true), variant_smem(0, false))));
    QSM_TRY((set_smem_t<32, 8, 2, 4>(ctx, variant_smem(1, true), variant_smem(1, false))));
    QSM_TRY((set_smem_t<32, 4, 4, 8>(ctx, variant_smem(2, true), variant_smem(2, false))));
    QSM_TRY((set_smem_t<32, 16, 2, 2>(ctx, variant_smem(3, true), variant_smem(3, false))));
    return stream_set_smem(ctx);
}

// process-wide tuning table: (tgv, nx, ny, nz) -> variant
using TuneKey = std::tuple<int, size_t, size_t, size_t>;
static std::map<TuneKey, int> g_tuned;
static std::mutex g_tune_mu;
static bool g_tune_loaded = false;

static void tune_load_locked()
{
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char *path = getenv("QSM_AUTOTUNE_CACHE");
    if (!path || !*path) return;
    FILE *fp = fopen(path, "r");
    if (!fp) return;
    int tg, v;
    size_t a, b, c;
    while (fscanf(fp, "%d %zu %zu %zu %d", &tg, &a, &b, &c, &v) == 5)
        if (v >= 0 && v < kNumVariants) g_tuned[TuneKey(tg, a, b, c)] = v;
    fclose(fp);
}

static void tune_store_locked(const TuneKey &k, int v)
{
    g_tuned[k] = v;
    const char *path = getenv("QSM_AUTOTUNE_CACHE");
    if (!path || !*path) return;
    FILE *fp = fopen(path, "a");
    if (!fp) return;
    fprintf(fp, "%d %zu %zu %zu %d\n", std::get<0>(k), std::get<1>(k), std::get<2>(k), std::get<3>(k), v);
    fclose(fp);
}

// ---------------------------------------------------------------------------
// device state of one solve
// ---------------------------------------------------------------------------

namespace {
struct Layout {
    size_t stride, mstride, ntiles_total, nblk_max, bytes;
    size_t pa, pb, da, db, dc;  // bytes of one buffer of each state family
    unsigned gx[kNumVariants], gy[kNumVariants], gz[kNumVariants];
};

Layout layout(bool tgv, const Dims &d)
{
    Layout L;
    const size_t N = d.n();
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    L.stride = al(N * sizeof(float));
    L.pa = al(N * (tgv ? sizeof(float4) : sizeof(float2)));
    L.pb = tgv ? L.stride : 0;
    L.da = al(N * sizeof(float4));
    L.db = tgv ? L.da : 0;
    L.dc = tgv ? al(N * sizeof(float2)) : 0;
    L.mstride = (N + 255) & ~(size_t)255;
    const size_t ix = d.nx > 2 ? d.nx - 2 : 0, iy = d.ny > 2 ? d.ny - 2 : 0, iz = d.nz > 2 ? d.nz - 2 : 0;
    L.ntiles_total = 0;
    L.nblk_max = 0;
    for (int v = 0; v < kNumVariants; ++v) {
        L.gx[v] = (unsigned)((ix + kVariants[v].tx - 1) / kVariants[v].tx);
        L.gy[v] = (unsigned)((iy + kVariants[v].ty - 1) / kVariants[v].ty);
        L.gz[v] = (unsigned)((iz + kVariants[v].tz - 1) / kVariants[v].tz);
        const size_t nb = (size_t)L.gx[v] * L.gy[v] * L.gz[v];
        L.ntiles_total += nb;
        L.nblk_max = std::max(L.nblk_max, nb);
    }
    // 3 primal buffers + 2 dual buffers + f, 3 mask arrays, tile lists, tile flags,
    // monitor partials, counter + control block
    L.bytes = 3 * (L.pa + L.pb) + 2 * (L.da + L.db + L.dc) + L.stride + 3 * L.mstride +
              (L.ntiles_total + 64) * sizeof(unsigned) +
              (L.nblk_max + 64) + 256 + 4 * (L.nblk_max + 1) * sizeof(double) + 1024;
    return L;
}
}  // namespace

size_t pd_volume_bytes(bool tgv, const Dims &d) { return layout(tgv, d).bytes; }

qsm_status pd_volume_init(qsm_ctx *ctx, PdVolume *v, bool tgv, const Dims &d, qsm_dtype dt, const void *d2f,
                          const uint8_t *mask, const double *h, double lam, double alpha)
{
    const Layout L = layout(tgv, d);
    const size_t N = d.n();
    v->tgv = tgv;
    v->d = d;
    v->np = tgv ? 5 : 2;
    v->nd = tgv ? 10 : 4;
    QSM_TRY(dalloc(ctx, &v->blk, L.bytes));
    QSM_CUDA(cudaMemsetAsync(v->blk, 0, L.bytes, ctx->stream));
    char *c = (char *)v->blk;
    for (int b = 0; b < 3; ++b, c += L.pa) v->PA[b] = c;
    for (int b = 0; b < 3; ++b, c += L.pb) v->PB[b] = L.pb ? (float *)c : nullptr;
    for (int b = 0; b < 2; ++b, c += L.da) v->DA[b] = (float4 *)c;
    for (int b = 0; b < 2; ++b, c += L.db) v->DB[b] = L.db ? (float4 *)c : nullptr;
    for (int b = 0; b < 2; ++b, c += L.dc) v->DC[b] = L.dc ? (float2 *)c : nullptr;
    v->f = (float *)c;
    c += L.stride;
    uint8_t *m = (uint8_t *)c, *mi = m + L.mstride;
    v->mm = mi + L.mstride;
    c += 3 * L.mstride;
    unsigned *tiles_base = (unsigned *)c;
    c += (L.ntiles_total + 64) * sizeof(unsigned);
    uint8_t *tflag = (uint8_t *)c;
    c += L.nblk_max + 64;
    c = (char *)(((uintptr_t)c + 255) & ~(uintptr_t)255);
    v->part = (double *)c;
    c += 4 * (L.nblk_max + 1) * sizeof(double);
    c = (char *)(((uintptr_t)c + 255) & ~(uintptr_t)255);
    v->count = (unsigned *)c;
    v->ctl = (PdCtl *)(c + 256);
    v->state_bytes = 3 * (L.pa + L.pb) + 2 * (L.da + L.db + L.dc);

    double tau, sigma;
    pd_steps(h, &tau, &sigma);
    QSM_TRY(set_all_smem(ctx));
    QSM_TRY(launch_masks(ctx, m, mi, mask, d));
    pack_masks_k<<<2048, 256, 0, ctx->stream>>>(v->mm, m, mi, N);
    QSM_CUDA(cudaGetLastError());
    if (dt == QSM_F32)
        QSM_TRY((launch_scale<float, float>(ctx, v->f, (const float *)d2f, sigma, N)));
    else
        QSM_TRY((launch_scale<float, double>(ctx, v->f, (const double *)d2f, sigma, N)));

    // active tiles of every variant, ascending (fixed order of the monitor partials)
    const size_t ix = d.nx > 2 ? d.nx - 2 : 0, iy = d.ny > 2 ? d.ny - 2 : 0, iz = d.nz > 2 ? d.nz - 2 : 0;
    unsigned *tp = tiles_base;
    for (int k = 0; k < kNumVariants; ++k) {
        TileList &tl = v->tl[k];
        tl = TileList();
        tl.gx = L.gx[k];
        tl.gy = L.gy[k];
        tl.gz = L.gz[k];
        const size_t nb = (size_t)tl.gx * tl.gy * tl.gz;
        tl.dev = tp;
        tp += nb;
        if (!nb) continue;
        tile_flags_k<<<(unsigned)nb, 256, 0, ctx->stream>>>(tflag, v->mm, d, tl.gx, tl.gy, kVariants[k].tx,
                                                            kVariants[k].ty, kVariants[k].tz);
        QSM_CUDA(cudaGetLastError());
        std::vector<uint8_t> hf(nb);
        QSM_CUDA(cudaMemcpyAsync(hf.data(), tflag, nb, cudaMemcpyDeviceToHost, ctx->stream));
        QSM_CUDA(cudaStreamSynchronize(ctx->stream));
        std::vector<unsigned> ht;
        ht.reserve(nb);
        for (size_t t = 0; t < nb; ++t) {
            if (!hf[t]) continue;
            ht.push_back((unsigned)t);
            const size_t ttx = t % tl.gx, tty = (t / tl.gx) % tl.gy, ttz = t / ((size_t)tl.gx * tl.gy);
            tl.active_vox += std::min((size_t)kVariants[k].tx, ix - ttx * kVariants[k].tx) *
                             std::min((size_t)kVariants[k].ty, iy - tty * kVariants[k].ty) *
                             std::min((size_t)kVariants[k].tz, iz - ttz * kVariants[k].tz);
        }
        tl.nact = (unsigned)ht.size();
        if (!ht.empty())
            QSM_CUDA(cudaMemcpyAsync(tl.dev, ht.data(), ht.size() * sizeof(unsigned), cudaMemcpyHostToDevice, ctx->stream));
        QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    v->dc = tgv ? make_dual_c<float>(sigma, h, alpha * lam, lam) : make_dual_c<float>(sigma, h, 0.0, lam);
    v->pc = make_primal_c<float>(tau, h);
    v->var = 0;
    // TMA variants: tensor maps of every primal buffer, per tile shape and iterate rotation.
    // Family B's rows must be 16-byte strides: nx a multiple of 4.
    v->maps.clear();
    if (tgv && d.nx % 4 == 0 && d.nx >= 4) {
        std::vector<TmaMaps> maps((size_t)kNumVariants * 3);
        const uint64_t da[3] = {4 * d.nx, d.ny, d.nz}, sa[2] = {16 * d.nx, 16 * d.nx * d.ny};
        const uint64_t db[3] = {d.nx, d.ny, d.nz}, sb[2] = {4 * d.nx, 4 * d.nx * d.ny};
        for (int k = 0; k < kNumVariants; ++k) {
            if (!kVariants[k].tma) continue;
            const uint32_t wx = (uint32_t)kVariants[k].tx + 4, wy = (uint32_t)kVariants[k].ty + 4;
            const uint32_t ba[3] = {4 * wx, wy, 1}, bb[3] = {wx + 4, wy, 1};
            CUtensorMap A[3], Bm[3];
            for (int b = 0; b < 3; ++b) {
                QSM_TRY(tma_encode_3d(ctx, &A[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, v->PA[b], da, sa, ba));
                QSM_TRY(tma_encode_3d(ctx, &Bm[b], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, v->PB[b], db, sb, bb));
            }
            for (uint32_t r = 0; r < 3; ++r) {  // the rotation of pd_volume_args
                TmaMaps &m = maps[(size_t)k * 3 + r];
                m.ac = A[r % 3];
                m.ap = A[(r + 2) % 3];
                m.bc = Bm[r % 3];
                m.bp = Bm[(r + 2) % 3];
            }
        }
        v->maps.swap(maps);
    }
    return QSM_OK;
}

FusedArgs pd_volume_args(const PdVolume &v, int var, uint32_t it)
{
    FusedArgs s;
    memset(&s, 0, sizeof s);
    const int cur = it % 3, prv = (it + 2) % 3, nxt = (it + 1) % 3, dcur = it % 2, dnxt = (it + 1) % 2;
    s.Pc = v.PA[cur];
    s.Pp = v.PA[prv];
    s.Pn = v.PA[nxt];
    s.Pc1 = v.PB[cur];
    s.Pp1 = v.PB[prv];
    s.Pn1 = v.PB[nxt];
    s.Dca = v.DA[dcur];
    s.Dcb = v.DB[dcur];
    s.Dcc = v.DC[dcur];
    s.Dna = v.DA[dnxt];
    s.Dnb = v.DB[dnxt];
    s.Dnc = v.DC[dnxt];
    s.f = v.f;
    s.mm = v.mm;
    s.part = v.part;
    s.count = v.count;
    s.ctl = v.ctl;
    s.tiles = v.tl[var].dev;
    s.gx = v.tl[var].gx;
    s.gy = v.tl[var].gy;
    return s;
}

qsm_status pd_volume_tune(qsm_ctx *ctx, PdVolume *v, uint32_t maxiter)
{
    Range nvtx_range("pd_fused/autotune");
    const char *force = getenv("QSM_FUSED_VARIANT");
    if (force && *force) {
        v->var = std::min(std::max(atoi(force), 0), kNumVariants - 1);
        if (!variant_ok(*v, v->var)) v->var = kTmaFallback;
        return QSM_OK;
    }
    const TuneKey key((int)v->tgv, v->d.nx, v->d.ny, v->d.nz);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        tune_load_locked();
        auto itk = g_tuned.find(key);
        if (itk != g_tuned.end() && variant_ok(*v, itk->second)) {
            v->var = itk->second;
            return QSM_OK;
        }
    }
    v->var = 0;
    if (v->tl[0].nact == 0 || maxiter < 20) return QSM_OK;
    // time each variant over a few iterations on this problem, then reset the state
    cudaEvent_t t0, t1;
    QSM_CUDA(cudaEventCreate(&t0));
    QSM_CUDA(cudaEventCreate(&t1));
    float best = 1e30f;
    for (int k = 0; k < kNumVariants; ++k) {
        if (!variant_ok(*v, k)) continue;
        for (uint32_t it = 0; it < 2; ++it)
            QSM_TRY(launch_variant(ctx, ctx->stream, k, v->tgv, false, v->tl[k].nact, pd_volume_args(*v, k, it),
                                   v->dc, v->pc, v->d, 0.0, it + 1, volume_maps(*v, k, it)));
        QSM_CUDA(cudaEventRecord(t0, ctx->stream));
        for (uint32_t it = 2; it < 8; ++it)
            QSM_TRY(launch_variant(ctx, ctx->stream, k, v->tgv, false, v->tl[k].nact, pd_volume_args(*v, k, it),
                                   v->dc, v->pc, v->d, 0.0, it + 1, volume_maps(*v, k, it)));
        QSM_CUDA(cudaEventRecord(t1, ctx->stream));
        QSM_CUDA(cudaEventSynchronize(t1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, t0, t1);
        if (ms < best) {
            best = ms;
            v->var = k;
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    QSM_CUDA(cudaMemsetAsync(v->PA[0], 0, v->state_bytes, ctx->stream));
    std::lock_guard<std::mutex> lock(g_tune_mu);
    tune_store_locked(key, v->var);
    return QSM_OK;
}

// chi = the first field of primal family A (stride 4 floats for TGV, 2 for TV)
template <typename T>
__global__ void extract_chi_k(T *o, const float *__restrict__ a, int stride, size_t n)
{
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x)
        o[l] = (T)a[l * stride];
}

qsm_status pd_volume_result(qsm_ctx *ctx, const PdVolume &v, uint32_t iters, qsm_dtype dt, void *chi_out)
{
    const float *chi = (const float *)v.PA[iters % 3];
    const size_t N = v.d.n();
    const int stride = v.tgv ? 4 : 2;
    if (N == 0) return QSM_OK;
    const unsigned g = (unsigned)std::min<size_t>((N + 255) / 256, 4096);
    if (dt == QSM_F32)
        extract_chi_k<float><<<g, 256, 0, ctx->stream>>>((float *)chi_out, chi, stride, N);
    else
        extract_chi_k<double><<<g, 256, 0, ctx->stream>>>((double *)chi_out, chi, stride, N);
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

qsm_status pd_volume_free(qsm_ctx *ctx, PdVolume *v)
{
    if (!v->blk) return QSM_OK;
    void *b = v->blk;
    v->blk = nullptr;
    return dfree(ctx, b);
}

// ---------------------------------------------------------------------------
// one-volume driver
// ---------------------------------------------------------------------------

qsm_status pd_fused(qsm_ctx *ctx, bool tgv, const Dims &d, qsm_dtype dt, const void *d2f, const uint8_t *mask,
                    const double *h, double lam, double alpha, double tol, uint32_t maxiter, uint32_t verbose,
                    void *chi_out, qsm_pd_info *info)
{
    Range nvtx_range("pd_fused");
    PdVolume v;
    QSM_TRY(pd_volume_init(ctx, &v, tgv, d, dt, d2f, mask, h, lam, alpha));
    qsm_status st = pd_volume_tune(ctx, &v, maxiter);
    if (st != QSM_OK) {
        pd_volume_free(ctx, &v);
        return st;
    }
    const int var = v.var;
    const unsigned nact = v.tl[var].nact;
    const bool empty = nact == 0;

    cudaEvent_t e0, e1;
    QSM_CUDA(cudaEventCreate(&e0));
    QSM_CUDA(cudaEventCreate(&e1));
    QSM_CUDA(cudaEventRecord(e0, ctx->stream));
    if (verbose) printf("Iter\t\t||delta chi||\t||delta eta||\n");
    const uint32_t pmod = maxiter ? maxiter / (verbose > 4 ? (verbose < maxiter ? verbose : maxiter) : (4 < maxiter ? 4 : maxiter)) : 1;
    PdCtl hctl;
    memset(&hctl, 0, sizeof hctl);
    uint32_t enq = 0;
    for (uint32_t it = 0; it < maxiter; ++it) {
        const bool chk = ((it + 1) % 10) == 0;
        if (!empty)
            QSM_TRY(launch_variant(ctx, ctx->stream, var, tgv, chk, nact, pd_volume_args(v, var, it), v.dc, v.pc, d,
                                   tol, it + 1, volume_maps(v, var, it)));
        enq = it + 1;
        const bool print = verbose && (it == 0 || it == maxiter - 1 || ((it + 1) % pmod) == 0);
        if (print || (chk && ((it + 1) % 100) == 0)) {
            QSM_CUDA(cudaMemcpyAsync(&hctl, v.ctl, sizeof(PdCtl), cudaMemcpyDeviceToHost, ctx->stream));
            QSM_CUDA(cudaStreamSynchronize(ctx->stream));
            if (verbose && (print || hctl.done))
                printf("%5d/%d\t%.3e\t%.3e\n", hctl.done ? hctl.iters : it + 1, maxiter, hctl.checks ? hctl.n1 : 1.0,
                       hctl.checks ? hctl.n2 : 1.0);
            if (hctl.done) break;
        }
    }
    QSM_CUDA(cudaEventRecord(e1, ctx->stream));
    QSM_CUDA(cudaMemcpyAsync(&hctl, v.ctl, sizeof(PdCtl), cudaMemcpyDeviceToHost, ctx->stream));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    const uint32_t iters = hctl.done ? hctl.iters : enq;
    if (hctl.stalled) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        pd_volume_free(ctx, &v);
        set_error(ctx, "fused solve: a bounded wait on a TMA load gave up");
        return QSM_ERR_TIMEOUT;
    }
    QSM_TRY(pd_volume_result(ctx, v, iters, dt, chi_out));
    QSM_CUDA(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (info) {
        info->iters = iters;
        info->monitor_chi = hctl.checks ? hctl.n1 : 1.0;
        info->monitor_eta = hctl.checks ? hctl.n2 : 1.0;
        info->seconds = ms * 1e-3;
        info->active_voxels = v.tl[var].active_vox;
        info->tile[0] = (uint32_t)kVariants[var].tx;
        info->tile[1] = (uint32_t)kVariants[var].ty;
        info->tile[2] = (uint32_t)kVariants[var].tz;
    }
    return pd_volume_free(ctx, &v);
}

}  // namespace qsm
