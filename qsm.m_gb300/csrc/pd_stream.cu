// Primal-dual TGV / TV, mixed-precision fused path: the one-volume
// z-streaming kernels.  A CTA owns a TX x TY column tile of the interior and
// a chunk of planes; the column bodies are column_pd (pd_tile.cuh: register
// prefetch) and column_tma (pd_tma.cuh: TMA-staged primal iterates, TGV).
#include "pd_tile.cuh"
#include "pd_tma.cuh"

namespace qsm {

// TV keeps few enough values in registers for two CTAs per SM
template <int TX, int TY, bool TGV, bool CHECK>
__global__ void __launch_bounds__((TX + 4) * (TY + 4), TGV ? 1 : 2)
stream_k(FusedArgs s, DualC<float> dc, PrimalC<float> pc, Dims d, int cz, double tol, uint32_t it)
{
    extern __shared__ double smem_raw[];
    if (s.ctl->done) return;
    const uint32_t itn = launch_iter(s, it);
    if (!itn) return;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    column_pd<TX, TY, TGV>(s, dc, pc, d, cz, s.tiles[blockIdx.x], CHECK, (float *)smem_raw, acc);
    if (CHECK) monitor_reduce<(TX + 4) * (TY + 4)>(s, smem_raw, acc, tol, itn);
}

template <int TX, int TY, bool CHECK>
__global__ void __launch_bounds__((TX + 4) * (TY + 4), 1)
stream_tma_k(const __grid_constant__ TmaMaps tm, FusedArgs s, DualC<float> dc, PrimalC<float> pc, Dims d, int cz,
             double tol, uint32_t it)
{
    extern __shared__ __align__(16) unsigned char smem_tma[];
    if (s.ctl->done) return;
    const uint32_t itn = launch_iter(s, it);
    if (!itn) return;
    char *base = tma_smem_base(smem_tma);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    column_tma<TX, TY>(tm, s, dc, pc, d, cz, s.tiles[blockIdx.x], CHECK, base, acc);
    // the monitor fold reuses shared memory past the plane barriers
    if (CHECK) monitor_reduce<(TX + 4) * (TY + 4)>(s, (double *)(base + 128), acc, tol, itn);
}

size_t stream_smem(int tx, int ty, bool tgv)
{
    const size_t nt = (size_t)(tx + 4) * (ty + 4);
    // exchange planes of (extragradient, dual): three and three step barriers for TGV, two
    // for TV (column_pd)
    const size_t planes = tgv ? 3 * (5 + 10) * nt * sizeof(float) + 3 * sizeof(uint64_t)
                              : 2 * (2 + 4) * nt * sizeof(float);
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

size_t stream_tma_smem(int tx, int ty)
{
    if (tx == 28 && ty == 16) return TmaLayout<28, 16>::REQUEST;
    if (tx == 28 && ty == 20) return TmaLayout<28, 20>::REQUEST;
    if (tx == 28 && ty == 24) return TmaLayout<28, 24>::REQUEST;
    return 0;
}

template <int TX, int TY>
static qsm_status set_tma_t(qsm_ctx *ctx)
{
    const int b = (int)TmaLayout<TX, TY>::REQUEST;
    QSM_CUDA(cudaFuncSetAttribute(stream_tma_k<TX, TY, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    QSM_CUDA(cudaFuncSetAttribute(stream_tma_k<TX, TY, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    return QSM_OK;
}

qsm_status stream_set_smem(qsm_ctx *ctx)
{
    QSM_TRY((set_t<28, 12>(ctx)));
    QSM_TRY((set_t<28, 16>(ctx)));
    QSM_TRY((set_tma_t<28, 16>(ctx)));
    QSM_TRY((set_tma_t<28, 20>(ctx)));
    QSM_TRY((set_tma_t<28, 24>(ctx)));
    return QSM_OK;
}

template <int TX, int TY>
static void launch_tma_t(cudaStream_t st, bool chk, unsigned nact, const TmaMaps &tm, const FusedArgs &s,
                         const DualC<float> &dc, const PrimalC<float> &pc, const Dims &d, int cz, double tol,
                         uint32_t it)
{
    const size_t sm = TmaLayout<TX, TY>::REQUEST;
    const int nt = (TX + 4) * (TY + 4);
    if (chk) stream_tma_k<TX, TY, true><<<nact, nt, sm, st>>>(tm, s, dc, pc, d, cz, tol, it);
    else stream_tma_k<TX, TY, false><<<nact, nt, sm, st>>>(tm, s, dc, pc, d, cz, tol, it);
}

template <int TX, int TY>
static void launch_t(cudaStream_t st, bool tgv, bool chk, unsigned nact, const FusedArgs &s, const DualC<float> &dc,
                     const PrimalC<float> &pc, const Dims &d, int cz, double tol, uint32_t it)
{
    const size_t sm = stream_smem(TX, TY, tgv);
    const int nt = (TX + 4) * (TY + 4);
    if (tgv) {
        if (chk) stream_k<TX, TY, true, true><<<nact, nt, sm, st>>>(s, dc, pc, d, cz, tol, it);
        else stream_k<TX, TY, true, false><<<nact, nt, sm, st>>>(s, dc, pc, d, cz, tol, it);
    } else {
        if (chk) stream_k<TX, TY, false, true><<<nact, nt, sm, st>>>(s, dc, pc, d, cz, tol, it);
        else stream_k<TX, TY, false, false><<<nact, nt, sm, st>>>(s, dc, pc, d, cz, tol, it);
    }
}

qsm_status stream_launch(qsm_ctx *ctx, cudaStream_t st, int tx, int ty, int cz, bool tgv, bool chk, unsigned nact,
                         const FusedArgs &s, const DualC<float> &dc, const PrimalC<float> &pc, const Dims &d,
                         double tol, uint32_t it, const TmaMaps *tm)
{
    if (tm) {
        if (!tgv) return QSM_ERR_ARG;
        if (tx == 28 && ty == 16) launch_tma_t<28, 16>(st, chk, nact, *tm, s, dc, pc, d, cz, tol, it);
        else if (tx == 28 && ty == 20) launch_tma_t<28, 20>(st, chk, nact, *tm, s, dc, pc, d, cz, tol, it);
        else if (tx == 28 && ty == 24) launch_tma_t<28, 24>(st, chk, nact, *tm, s, dc, pc, d, cz, tol, it);
        else return QSM_ERR_ARG;
        QSM_CUDA(cudaGetLastError());
        return QSM_OK;
    }
    if (tx == 28 && ty == 12) launch_t<28, 12>(st, tgv, chk, nact, s, dc, pc, d, cz, tol, it);
    else if (tx == 28 && ty == 16) launch_t<28, 16>(st, tgv, chk, nact, s, dc, pc, d, cz, tol, it);
    else return QSM_ERR_ARG;
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

}  // namespace qsm
