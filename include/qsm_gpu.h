/*
 * qsm_gpu.h -- C ABI of the GB300 (sm_103a) QSM library.
 *
 * One entry point per QSM.m C-MEX gateway on the hot path, with the MEX
 * gateway's argument order and meaning, so a thin MEX shim (see
 * qsm.m_gb300/mex/) can forward mxGetData() pointers unchanged:
 *
 *   - arrays are MATLAB column-major, x fastest: l = i + nx*j + nx*ny*k;
 *     vector fields are component-major (component c at offset c*N);
 *   - masks are uint8 0/1 (MATLAB logical);
 *   - vsz is double[3] (voxel size);
 *   - dtype selects float32 or float64, as mxIsSingle(prhs[0]) does;
 *   - every array pointer may be HOST or DEVICE memory (detected per
 *     pointer).  Host arrays are copied to the device and results copied
 *     back inside the call; device arrays are used in place with no copy;
 *   - "in-place" operator gateways write into their first array argument(s)
 *     exactly where the MEX file writes (masked variants only where G), so
 *     other elements keep the caller's contents;
 *   - solver gateways never modify their inputs and write a separate output.
 *
 * Every call is enqueued on the context's stream and returns after the
 * result is complete (host outputs are copied back; device outputs are
 * synchronised).  Errors are status codes instead of mexErrMsgTxt; the
 * message of the last failure is available from qsm_last_error().
 *
 * Citations name the reference gateway each function replaces, as
 * path:line within kamesy/QSM.m.
 */
#ifndef QSM_GPU_H
#define QSM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QSM_GPU_ABI_VERSION 2

/* Number of blocks of the lane-order reduction (lanes = 256 * QSM_RED_NBLK). */
#define QSM_RED_NBLK 1024

typedef enum {
    QSM_OK = 0,
    QSM_ERR_ARG = 1,        /* null pointer, bad scalar */
    QSM_ERR_DIMS = 2,       /* unsupported or inconsistent dimensions */
    QSM_ERR_DTYPE = 3,      /* unsupported dtype */
    QSM_ERR_NOMEM = 4,      /* device allocation failed */
    QSM_ERR_CUDA = 5,       /* CUDA runtime error (see qsm_last_error) */
    QSM_ERR_NONFINITE = 6,  /* a convergence monitor became NaN/Inf */
    QSM_ERR_DEPTH = 7,      /* nlevels > 16 ("nlevels too large. Increase MAX_DEPTH.") */
    QSM_ERR_BUSY = 8,       /* session has no free slot / over budget */
    QSM_ERR_TIMEOUT = 9     /* a bounded device wait gave up */
} qsm_status;

typedef enum { QSM_F64 = 0, QSM_F32 = 1 } qsm_dtype;

typedef struct qsm_ctx qsm_ctx;

/* ---------------- context ---------------- */

/* Test hook (no counterpart in the reference).  QSM_DEBUG_GRID_BARRIER_TIMEOUT
 * makes every grid barrier of the whole-GPU multigrid kernels (the coarsest
 * solve and list sweeps on cooperative launches) wait for one arrival more
 * than the grid makes, with a short poll limit, so that their bounded wait
 * runs out: the solve then returns QSM_ERR_TIMEOUT and the context stays
 * usable.  flags = 0 restores normal operation. */
#define QSM_DEBUG_GRID_BARRIER_TIMEOUT 1u
qsm_status qsm_ctx_set_debug(qsm_ctx *ctx, uint32_t flags);

/* Creates a context on `device` with its own non-blocking stream and a
 * stream-ordered memory pool. */
qsm_status qsm_ctx_create(int device, qsm_ctx **ctx);
qsm_status qsm_ctx_destroy(qsm_ctx *ctx);
/* Use a caller-owned cudaStream_t (passed as void*) instead of the context's. */
qsm_status qsm_ctx_set_stream(qsm_ctx *ctx, void *cuda_stream);
void *qsm_ctx_get_stream(qsm_ctx *ctx);
qsm_status qsm_ctx_set_verbose(qsm_ctx *ctx, int verbose);
const char *qsm_last_error(const qsm_ctx *ctx);
const char *qsm_status_string(qsm_status s);
int qsm_abi_version(void);

/* ---------------- primal-dual inversions ---------------- */

typedef struct {
    uint32_t iters;        /* iterations run */
    double monitor_chi;    /* ||chi - chi0|| / ||chi|| at the last check */
    double monitor_eta;    /* ||eta - eta0|| / ||eta|| at the last check */
    double seconds;        /* device time of the iteration loop */
    uint64_t active_voxels;/* voxels the iteration kernels visit: the interior for the
                              plain path, the interior of the tiles holding mask voxels
                              for the fused path (outside them nothing changes) */
    uint32_t tile[3];      /* fused path: the tile shape used (x, y, z); 0 for the plain path */
} qsm_pd_info;

/* chi = pd_tgv_mex(d2f, mask, vsz, lam, alpha, tol, maxiter, verbose)
 * Replaces src/inversion/mex/pd_tgv_mex.c:104-135 (mexFunction) with
 * mx_pdd/mx_pdf :139-323.  Plain path: one kernel per reference loop nest
 * (dual, primal, monitor copy, monitor check), no fused multiply-add;
 * bit-exact with the reference in FP64 and FP32.  info may be NULL. */
qsm_status qsm_pd_tgv(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                      const void *d2f, const uint8_t *mask, const double vsz[3],
                      double lam, double alpha, double tol, uint32_t maxiter,
                      uint32_t verbose, void *chi, qsm_pd_info *info);

/* chi = pd_tv_mex(d2f, mask, vsz, lam, tol, maxiter, verbose)
 * Replaces src/inversion/mex/pd_tv_mex.c:100-130 with mx_pdd/mx_pdf :134-306. */
qsm_status qsm_pd_tv(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                     const void *d2f, const uint8_t *mask, const double vsz[3],
                     double lam, double tol, uint32_t maxiter, uint32_t verbose,
                     void *chi, qsm_pd_info *info);

/* Mixed-precision fused variants of the two gateways above (same arguments
 * and meaning).  The stencil arithmetic runs in FP32 inside one fused
 * dual+primal(+extragradient) kernel per iteration; the convergence
 * monitors' per-voxel terms are summed per thread in compensated FP32 and
 * across threads in FP64.  Per voxel it evaluates the reference's FP32
 * expressions (pd_tgv_mex.c:332-485, :659-812) without fused multiply-add,
 * so chi equals the reference's own single-precision result (mx_pdf).
 * dtype gives the type of d2f/chi in memory (F64 inputs are rounded to
 * FP32 on the device, the result widened back). */
qsm_status qsm_pd_tgv_fused(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                            const void *d2f, const uint8_t *mask, const double vsz[3],
                            double lam, double alpha, double tol, uint32_t maxiter,
                            uint32_t verbose, void *chi, qsm_pd_info *info);
qsm_status qsm_pd_tv_fused(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                           const void *d2f, const uint8_t *mask, const double vsz[3],
                           double lam, double tol, uint32_t maxiter, uint32_t verbose,
                           void *chi, qsm_pd_info *info);

/* ---------------- FFT total-variation inversion (ADMM) ---------------- */

typedef struct {
    uint32_t iters;        /* ADMM iterations run */
    double rho;            /* final penalty parameter */
    double nr, eps_pri;    /* primal residual and its tolerance at the last iteration */
    double ns, eps_dual;   /* dual residual and its tolerance */
    double seconds;        /* device time of the iterations */
} qsm_tv_info;

/* x = tv(f, mask, vsz, bdir, opts) for one 3-D volume:
 * src/inversion/tv.m:101-277 (tv_), dipole kernel dipoleKernel.m:56-65, Laplace
 * symbol laplaceKernel.m / tv.m:140-142; opts as tv.m:38-82 (defaults mu 7.5e3,
 * tv 1 anisotropic | 2 isotropic, rtol 0.1, atol 1e-4, maxit 20, rho 9, alpha 1.5,
 * rtau 0.7, stau 100, gamma 3).  Arithmetic in dtype (FP64 as MATLAB's default
 * class), reductions in FP64; cuFFT R2C/C2R with a fused k-space multiply.
 * Every dimension must be >= 3.  info may be NULL. */
qsm_status qsm_tv_admm(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3], const void *f,
                       const uint8_t *mask, const double vsz[3], const double bdir[3], double mu,
                       int32_t tv, double rtol, double atol, int32_t maxit, double rho,
                       double alpha, double rtau, double stau, double gamma, int32_t verbose,
                       void *x, qsm_tv_info *info);

/* ---------------- finite-difference operators (in place) ---------------- */

/* gradf_mex(dx, dy, dz, u, h): src/utils/fd/mex/gradf_mex.c:13-47 */
qsm_status qsm_gradf(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                     void *dx, void *dy, void *dz, const void *u, const double vsz[3]);
/* gradb_mex: src/utils/fd/mex/gradb_mex.c:13-47 */
qsm_status qsm_gradb(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                     void *dx, void *dy, void *dz, const void *u, const double vsz[3]);
/* gradc_mex: src/utils/fd/mex/gradc_mex.c:13-47 */
qsm_status qsm_gradc(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                     void *dx, void *dy, void *dz, const void *u, const double vsz[3]);
/* gradfm_mex(dx, dy, dz, u, G, h): src/utils/fd/mex/gradfm_mex.c:15-50 */
qsm_status qsm_gradfm(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                      void *dx, void *dy, void *dz, const void *u, const uint8_t *G,
                      const double vsz[3]);
/* gradbm_mex: src/utils/fd/mex/gradbm_mex.c:15-50 */
qsm_status qsm_gradbm(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                      void *dx, void *dy, void *dz, const void *u, const uint8_t *G,
                      const double vsz[3]);
/* gradcm_mex: src/utils/fd/mex/gradcm_mex.c:15-50 */
qsm_status qsm_gradcm(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                      void *dx, void *dy, void *dz, const void *u, const uint8_t *G,
                      const double vsz[3]);
/* gradf_adj_mex(du, x, y, z, h): src/utils/fd/mex/gradf_adj_mex.c:15-49 */
qsm_status qsm_gradf_adj(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                         void *du, const void *x, const void *y, const void *z,
                         const double vsz[3]);
/* gradb_adj_mex: src/utils/fd/mex/gradb_adj_mex.c:15-49 */
qsm_status qsm_gradb_adj(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                         void *du, const void *x, const void *y, const void *z,
                         const double vsz[3]);
/* gradfm_adj_mex(du, x, y, z, G, h): src/utils/fd/mex/gradfm_adj_mex.c:15-50 */
qsm_status qsm_gradfm_adj(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                          void *du, const void *x, const void *y, const void *z,
                          const uint8_t *G, const double vsz[3]);
/* gradbm_adj_mex: src/utils/fd/mex/gradbm_adj_mex.c:15-50 */
qsm_status qsm_gradbm_adj(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                          void *du, const void *x, const void *y, const void *z,
                          const uint8_t *G, const double vsz[3]);
/* gradfp_mex(dx, dy, dz, u, h): src/inversion/mex/gradfp_mex.c:13-47 */
qsm_status qsm_gradfp(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                      void *dx, void *dy, void *dz, const void *u, const double vsz[3]);
/* gradfp_adj_mex(du, x, y, z, h): src/inversion/mex/gradfp_adj_mex.c:15-49 */
qsm_status qsm_gradfp_adj(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                          void *du, const void *x, const void *y, const void *z,
                          const double vsz[3]);
/* lap1_mex(d2u, u, G, h) ("lap_mex" in its usage string):
 * src/utils/fd/mex/lap1_mex.c:29-60 */
qsm_status qsm_lap1(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                    void *d2u, const void *u, const uint8_t *G, const double vsz[3]);
/* lapw_mex(d2u, u, h): src/unwrap/mex/lapw_mex.c:21-51 */
qsm_status qsm_lapw(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                    void *d2u, const void *u, const double vsz[3]);

/* ---------------- multigrid pieces (in place) ---------------- */

/* gauss_seidel_mex(v, f, G, h, iter, reverse), red-black build:
 * src/utils/poisson_solver/mex/gauss_seidel_mex.c:19-49 (+ gauss_seideld :196-311) */
qsm_status qsm_gauss_seidel(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                            void *v, const void *f, const uint8_t *G, const double vsz[3],
                            int32_t iter, int32_t reverse);
/* residual_mex(r, f, x, G, h): src/utils/poisson_solver/mex/residual_mex.c:17-49 (+ residuald :82-165) */
qsm_status qsm_residual(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                        void *r, const void *f, const void *x, const uint8_t *G,
                        const double vsz[3]);
/* lapmg_mex(d2u, u, G, h): src/utils/poisson_solver/mex/lapmg_mex.c:17-45 (+ lapmgd :73-154) */
qsm_status qsm_lapmg(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                     void *d2u, const void *u, const uint8_t *G, const double vsz[3]);
/* restrict_mex(x2, x, G2): src/utils/poisson_solver/mex/restrict_mex.c:17-45 (+ restrictd :200-332).
 * dims2 = size of x2 and G2, dims = size of x. */
qsm_status qsm_restrict(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims2[3], void *x2,
                        const size_t dims[3], const void *x, const uint8_t *G2);
/* prolong_mex(x, x2, G): src/utils/poisson_solver/mex/prolong_mex.c:17-45 (+ prolongd :180-304) */
qsm_status qsm_prolong(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3], void *x,
                       const size_t dims2[3], const void *x2, const uint8_t *G);
/* correct_mex(x, x2, G): src/utils/poisson_solver/mex/correct_mex.c:17-45 (+ correctd :180-304) */
qsm_status qsm_correct(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3], void *x,
                       const size_t dims2[3], const void *x2, const uint8_t *G);
/* coarsen_grid_mex(G2, G): src/utils/poisson_solver/mex/coarsen_grid_mex.c:12-33 (+ coarsen_grid :52-125) */
qsm_status qsm_coarsen_grid(qsm_ctx *ctx, const size_t dims2[3], uint8_t *G2,
                            const size_t dims[3], const uint8_t *G);
/* boundary_mask_mex(B, G): src/utils/poisson_solver/mex/boundary_mask_mex.c:11-29 (+ boundary_mask :46-132) */
qsm_status qsm_boundary_mask(qsm_ctx *ctx, const size_t dims[3], uint8_t *B, const uint8_t *G);
/* boundary_mask_l1_mex(B, G, l1): src/utils/poisson_solver/mex/boundary_mask_l1_mex.c:12-32 (+ boundary_mask_l1 :49-117) */
qsm_status qsm_boundary_mask_l1(qsm_ctx *ctx, const size_t dims[3], uint8_t *B,
                                const uint8_t *G, uint8_t l1);
/* p = norm2_mex(x, G): src/utils/poisson_solver/mex/norm2_mex.c:21-51 (+ norm22d :113-131).
 * Masked 2-norm; *out receives it (as double; FP32 result widened). */
qsm_status qsm_norm2(qsm_ctx *ctx, qsm_dtype dtype, size_t n, const void *x,
                     const uint8_t *G, double *out);

/* Largest n accepted by qsm_norm2_noalloc (2^25 elements). */
#define QSM_NORM2_NOALLOC_MAX_N ((size_t)1 << 25)

/* Masked pairwise 2-norm of qsm_norm2 that allocates no memory.  No
 * counterpart in the reference: it exists for callers that cannot let a
 * library allocate device memory (a MATLAB session that hands MEX files its
 * own gpuArray memory; pipelines that allocate everything once at start-up,
 * since cudaMalloc/cudaFree synchronise the device mid-run).
 *   - x (n values of dtype), G (n bytes) and out (one double) are DEVICE
 *     pointers; the work is enqueued on `stream` (a cudaStream_t, NULL for
 *     the default stream) and *out is written when it completes;
 *   - no context is needed; scratch is a fixed device array inside the
 *     library (4 MiB per GPU that loads it, held until exit), so n must be
 *     1..QSM_NORM2_NOALLOC_MAX_N, otherwise QSM_ERR_DIMS;
 *   - all calls share that array: calls that overlap on the GPU race;
 *   - the first call on each device looks up the array's address with that
 *     device current; make that first call before any stream capture;
 *   - a device reset (cudaDeviceReset; MATLAB's reset(gpuDevice)) replaces
 *     the device's context and unloads the array: the next call notices the
 *     new context and looks the address up again, so it is a first call
 *     too and also belongs before any stream capture. */
qsm_status qsm_norm2_noalloc(qsm_dtype dtype, size_t n, const void *x, const uint8_t *G,
                             double *out, void *stream);

/* ---------------- Poisson solvers ---------------- */

typedef struct {
    int32_t iters;          /* PCG iterations (mgpcg) or cycles run */
    double resnorm;         /* final ||r||_2 (padded array, as the reference) */
    double seconds;         /* device time */
    double *resnorm_hist;   /* optional, caller-owned, >= maxitcg doubles */
    int32_t coarse_ctas;    /* coarsest-level solver: 0 host-driven loop, 1 one CTA,
                               > 1 a thread-block cluster of that many CTAs, < 0 a
                               cooperative launch of -coarse_ctas CTAs (one per SM) */
    int32_t coarse_outer;   /* outer iterations (256 sweeps each) it ran in total */
} qsm_mg_info;

/* v = mgpcg_mex(v, f, mask, vsz, tolcg, maxitcg, tolmg, maxitmg, mu, npre,
 *               npost, nboundary, nlevels, verbose)
 * Replaces src/utils/poisson_solver/mex/mgpcg_mex.c:73-123 (mx_pcg :126-216,
 * mx_mg :219-239, mx_cycle :242-279, mx_init :282-332).  Plain path: PCG and
 * V-cycle in dtype; inner products in lane order (bit-exact with the oracle
 * built on the project's BLAS shim).  v0 is the initial guess; v_out gets
 * the solution. */
qsm_status qsm_mgpcg(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                     const void *v0, const void *f, const uint8_t *mask, const double vsz[3],
                     double tolcg, int32_t maxitcg, double tolmg, int32_t maxitmg,
                     int32_t mu, int32_t npre, int32_t npost, int32_t nboundary,
                     int32_t nlevels, int32_t verbose, void *v_out, qsm_mg_info *info);

/* Mixed-precision variant: FP64 PCG recurrence (residual update, inner
 * products, step lengths) preconditioned by an FP32 V-cycle (FP32 smoother,
 * residual, transfer operators, coarse solve with the reference's FP32
 * coarse tolerance 1e-4).  The recurrence's multiply-adds are FP64 fused
 * multiply-adds (one rounding each), so its result is not bit-identical to
 * the FP64 solve's; it is reproducible run to run.  v0/f/v_out are FP64.
 * Same arguments otherwise. */
qsm_status qsm_mgpcg_mixed(qsm_ctx *ctx, const size_t dims[3],
                           const double *v0, const double *f, const uint8_t *mask,
                           const double vsz[3], double tolcg, int32_t maxitcg, double tolmg,
                           int32_t maxitmg, int32_t mu, int32_t npre, int32_t npost,
                           int32_t nboundary, int32_t nlevels, int32_t verbose,
                           double *v_out, qsm_mg_info *info);

/* Packed Poisson solves (no reference counterpart: the reference solves one
 * volume per mgpcg_mex call): `count` solves with shared options, volume b of
 * size dims[3b..3b+2] with FP64 arrays f[b], mask[b], v_out[b] (host or
 * device) and initial guess v0[b] (v0 or v0[b] NULL: zeros).  mixed selects the
 * FP32 V-cycle of qsm_mgpcg_mixed, else all FP64 as qsm_mgpcg.  Solves with a
 * fixed number of V-cycles (tolmg <= 0, as lbv.m's options), voxel lists on
 * every level and a coarsest grid one CTA holds advance together, up to 16 at
 * a time: each PCG iteration launches each of its kernels once for all of
 * them.  Any other solve runs by itself.  Every v_out[b] equals the solve
 * alone bit for bit.  info: NULL or `count` entries. */
qsm_status qsm_mgpcg_batch(qsm_ctx *ctx, int32_t mixed, uint32_t count, const size_t *dims,
                           const double *const *v0, const double *const *f,
                           const uint8_t *const *mask, const double vsz[3], double tolcg,
                           int32_t maxitcg, double tolmg, int32_t maxitmg, int32_t mu,
                           int32_t npre, int32_t npost, int32_t nboundary, int32_t nlevels,
                           double *const *v_out, qsm_mg_info *info);

/* v = mg_mex(v, f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels)
 * Replaces src/utils/poisson_solver/mex/mg_mex.c:55-91. */
qsm_status qsm_mg(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                  const void *v0, const void *f, const uint8_t *mask, const double vsz[3],
                  double tol, int32_t maxit, int32_t mu, int32_t npre, int32_t npost,
                  int32_t nboundary, int32_t nlevels, void *v_out, qsm_mg_info *info);

/* v = fmg_mex(f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels)
 * Replaces src/utils/poisson_solver/mex/fmg_mex.c:54-90. */
qsm_status qsm_fmg(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[3],
                   const void *f, const uint8_t *mask, const double vsz[3],
                   double tol, int32_t maxit, int32_t mu, int32_t npre, int32_t npost,
                   int32_t nboundary, int32_t nlevels, void *v_out, qsm_mg_info *info);

/* ---------------- many-volume batches and resident sessions ----------------
 *
 * No counterpart in the reference: QSM.m solves one volume per MEX call and
 * loops over echoes/volumes in MATLAB (src/inversion/sstgv.m:68-71,
 * src/bgremove/lbv.m:97-100).  These entry points keep many solves resident
 * on one GPU and advance them together.
 */

/* Batched fused primal-dual solves: `count` volumes, volume b of size
 * dims[3b..3b+2] with arrays d2f[b], mask[b] and output chi[b] (host or
 * device, dtype as in qsm_pd_tv_fused).  vsz, lam, alpha, tol and maxiter
 * are shared.  All volumes advance in one persistent launch per tile shape
 * and iteration, replayed from a captured CUDA graph; each chi[b] equals
 * qsm_pd_tv_fused / qsm_pd_tgv_fused of that volume alone.  info may be
 * NULL or hold `count` entries (seconds = device time of the whole batch). */
qsm_status qsm_pd_tv_batch(qsm_ctx *ctx, qsm_dtype dtype, uint32_t count, const size_t *dims,
                           const void *const *d2f, const uint8_t *const *mask, const double vsz[3],
                           double lam, double tol, uint32_t maxiter, void *const *chi,
                           qsm_pd_info *info);
qsm_status qsm_pd_tgv_batch(qsm_ctx *ctx, qsm_dtype dtype, uint32_t count, const size_t *dims,
                            const void *const *d2f, const uint8_t *const *mask, const double vsz[3],
                            double lam, double alpha, double tol, uint32_t maxiter,
                            void *const *chi, qsm_pd_info *info);

/* A session holds admitted solves resident in device memory until their
 * results are fetched.  Primal-dual solves advance together in
 * qsm_session_step (the batched launches above).  Poisson solves: with
 * poisson_workers = 0 they stay resident too and advance in the same steps,
 * packed as in qsm_mgpcg_batch, on a stream of their own beside the replays:
 * at least one PCG iteration per 30 primal-dual iterations, and more while
 * the step's replays are still running; with
 * poisson_workers > 0 each runs whole on one of that many host threads, each
 * with its own stream, concurrently with the steps.  Admission: a submit whose footprint
 * (qsm_session_footprint) does not fit in budget_bytes minus the bytes in
 * use fails with QSM_ERR_BUSY and changes nothing (budget 0 = no limit).
 * A session is driven from one host thread. */
typedef struct qsm_session qsm_session;
typedef enum {
    QSM_JOB_TV = 0,        /* pd_tv (fused, FP32 state) */
    QSM_JOB_TGV = 1,       /* pd_tgv (fused, FP32 state) */
    QSM_JOB_MGPCG = 2,     /* mgpcg, FP64 PCG + FP32 V-cycle */
    QSM_JOB_MGPCG_F64 = 3  /* mgpcg, FP64 throughout */
} qsm_job_kind;

qsm_status qsm_session_create(qsm_ctx *ctx, size_t budget_bytes, int32_t poisson_workers,
                              qsm_session **session);
qsm_status qsm_session_destroy(qsm_session *session);
/* Device bytes a job of this kind and size holds while resident. */
size_t qsm_session_footprint(int32_t kind, const size_t dims[3], int32_t nlevels);
size_t qsm_session_bytes_in_use(const qsm_session *session);
/* Admits a TV (tgv = 0, alpha unused) or TGV solve with pd_tv_mex /
 * pd_tgv_mex arguments.  Inputs are copied; the call returns once the
 * solve's state is initialised (and, for a new grid size, its tile shape
 * tuned). */
qsm_status qsm_session_submit_pd(qsm_session *session, int32_t tgv, qsm_dtype dtype,
                                 const size_t dims[3], const void *d2f, const uint8_t *mask,
                                 const double vsz[3], double lam, double alpha, double tol,
                                 uint32_t maxiter, uint64_t *id);
/* Admits an mgpcg_mex solve (FP64 arrays; v0 may be NULL for zeros; mixed
 * selects the FP32 V-cycle).  Inputs are copied.  It runs on the next free
 * Poisson worker, or, without workers, is set up on the session's set-up
 * thread (the call returns at once) and advances in the steps from then on. */
qsm_status qsm_session_submit_mgpcg(qsm_session *session, const size_t dims[3], const double *v0,
                                    const double *f, const uint8_t *mask, const double vsz[3],
                                    double tolcg, int32_t maxitcg, double tolmg, int32_t maxitmg,
                                    int32_t mu, int32_t npre, int32_t npost, int32_t nboundary,
                                    int32_t nlevels, int32_t mixed, uint64_t *id);
/* Advances every running primal-dual solve by `iters` iterations (rounded up
 * to a multiple of 30; solves stop at their own maxiter or tolerance), and
 * every resident Poisson solve by at least one PCG iteration per 30 of them
 * (more while they run), and returns when they are done. */
qsm_status qsm_session_step(qsm_session *session, uint32_t iters);
/* *finished = 1 once the job's result can be fetched.  pd_info / mg_info
 * (either may be NULL) receive the job's statistics. */
qsm_status qsm_session_poll(qsm_session *session, uint64_t id, int32_t *finished,
                            qsm_pd_info *pd_info, qsm_mg_info *mg_info);
/* Copies a finished job's result (chi in the submit dtype, or the FP64
 * Poisson solution) to `out` (host or device) and releases its state. */
qsm_status qsm_session_fetch(qsm_session *session, uint64_t id, void *out);
/* Jobs admitted and not yet finished. */
uint32_t qsm_session_running(const qsm_session *session);

/* ---------------- MATLAB-level pipelines (crop, echo loop, solve) ----------------
 *
 * The wrappers' own steps on the device: crop to the mask's bounding box
 * (src/utils/cropIndices.m) grown by a margin and clamped, the per-echo
 * Laplacian and solve, and the scatter back into a zero array of the input's
 * size.  dims[4] = {nx, ny, nz, echoes}; echo t starts at t*nx*ny*nz.  An
 * empty mask is QSM_ERR_ARG (the MATLAB code indexes an empty array). */

/* x = sstgv(phas, mask, vsz, lambda, alpha, tol, maxit, verbose):
 * src/inversion/sstgv.m:1-87 (crop margin 2, d2u = lapw(u), pd_tgv_mex(-d2u, ...),
 * or pd_tv_mex when alpha <= eps).  fused = 0: the plain path (bit-exact with the
 * reference); fused != 0: the mixed-precision fused path, all echoes advanced
 * together.  info: NULL or one entry per echo. */
qsm_status qsm_sstgv(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[4], const void *phas,
                     const uint8_t *mask, const double vsz[3], double lambda, double alpha,
                     double tol, uint32_t maxit, uint32_t verbose, int32_t fused, void *x,
                     qsm_pd_info *info);

/* fl = lbv(f, mask, vsz, tol, maxit, mgopts, verbose): src/bgremove/lbv.m:1-113
 * (crop margin 1, d2u = lap(u, m), mgpcg(-d2u, m, ...) with mgopts.maxit/npre/npost/
 * nboundary, mu 1, tolmg -1, nlevels = max(1, floor(log2(min(size))) - 3) of the
 * cropped grid).  maxit <= 0: ceil(sqrt(numel(mask))).  mixed != 0 (FP64 only): the
 * FP32 V-cycle preconditioner.  info: NULL or one entry per echo (resnorm_hist is
 * not filled). */
qsm_status qsm_lbv(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[4], const void *f,
                   const uint8_t *mask, const double vsz[3], double tol, int32_t maxit,
                   int32_t mg_maxit, int32_t npre, int32_t npost, int32_t nboundary,
                   int32_t verbose, int32_t mixed, void *fl, qsm_mg_info *info);

/* [uphas, d2phas] = unwrapLaplacian(phas, mask, vsz): src/unwrap/unwrapLaplacian.m:1-87
 * (crop margin 1, d2u = lapw(u), mgpcg(-m.*d2u, m, h, 1e-8, ceil(sqrt(numel(m))),
 * mg maxit 2, npre = npost = 2, nboundary 2)).  d2phas may be NULL. */
qsm_status qsm_unwrap_laplacian(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[4],
                                const void *phas, const uint8_t *mask, const double vsz[3],
                                int32_t mixed, void *uphas, void *d2phas);

/* ---------------- FFT background-field removal ----------------
 *
 * f and mask are cropped to cropIndices(mask), zero-padded to a 7-smooth size
 * (padfastfft.m, third_party/nextfastfft.m) and convolved with spherical-mean-
 * value kernels (smvKernel.m) by cuFFT; fl is zero outside the crop.  Eroded
 * masks are real(ifft3(H .* fft3(single(mask)))) > 0.999 in FP32, as the MATLAB
 * code computes them; the field arithmetic is in dtype.  dims[4] = {nx, ny, nz,
 * echoes}.  mask_out (NULL allowed) receives the eroded mask the function
 * returns as its second output.  An empty mask is QSM_ERR_ARG. */

/* [fl, mask] = sharp(f, mask, vsz, r, thr): src/bgremove/sharp.m:1-84 (r 9, thr 0.05) */
qsm_status qsm_sharp(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[4], const void *f,
                     const uint8_t *mask, const double vsz[3], double r, double thr, void *fl,
                     uint8_t *mask_out);

/* [fl, mask] = vsharp(f, mask, vsz, rs, thr): src/bgremove/vsharp.m:1-153.
 * nradii <= 0: rs = 9 : -2*max(vsz) : 2*max(vsz).  At least two radii. */
qsm_status qsm_vsharp(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[4], const void *f,
                      const uint8_t *mask, const double vsz[3], const double *radii,
                      int32_t nradii, double thr, void *fl, uint8_t *mask_out);

/* [fl, mask] = resharp(f, mask, vsz, r, lambda, tol, maxit): src/bgremove/resharp.m:1-88
 * (r 3, lambda 1e-2, tol < 0: sqrt(eps(class)), maxit <= 0: ceil(sqrt(numel(mask)))).
 * MATLAB's cgs is replaced by the published CGS iteration (x0 = 0, no preconditioner,
 * stop when the updated residual is <= tol*||b||); iters (NULL allowed) per echo. */
qsm_status qsm_resharp(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[4], const void *f,
                       const uint8_t *mask, const double vsz[3], double r, double lambda, double tol,
                       int32_t maxit, int32_t verbose, void *fl, uint8_t *mask_out, int32_t *iters);

/* fl = pdf(f, mask, vsz, w, bdir, lambda, tol, maxit, verbose): src/bgremove/pdf.m:1-86
 * (w NULL: the mask; bdir [0 0 1]; lambda 0; tol < 0: 1e-5; maxit <= 0:
 * ceil(sqrt(numel(mask)))).  The least-squares problem is solved by LSMR (Fong &
 * Saunders 2011; atol = btol = tol, conlim 1e8, no reorthogonalisation) on the full
 * grid; the dipole kernel is psf2otf of the image-space kernel (dipoleKernel.m 'i').
 * w has the dtype of f.  iters (NULL allowed) per echo. */
qsm_status qsm_pdf(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[4], const void *f,
                   const uint8_t *mask, const void *w, const double vsz[3], const double bdir[3],
                   double lambda, double tol, int32_t maxit, int32_t verbose, void *fl,
                   int32_t *iters);

/* [fl, mask] = ismv(f, mask, vsz, r, tol, maxit, verbose): src/bgremove/ismv.m:1-112
 * (r 3, tol < 0: sqrt(eps(class)), maxit 500).  iters (NULL allowed) receives the
 * iterations of each echo. */
qsm_status qsm_ismv(qsm_ctx *ctx, qsm_dtype dtype, const size_t dims[4], const void *f,
                    const uint8_t *mask, const double vsz[3], double r, double tol, int32_t maxit,
                    int32_t verbose, void *fl, uint8_t *mask_out, int32_t *iters);

/* ---------------- NIfTI-1 (src/io/loadNii.m, saveNii.m) ----------------
 *
 * loadNii(filename) = third_party/NIfTI/load_nii.m: the header (either byte
 * order), the image as stored, then xform_nii.m: scl_slope / scl_inter applied
 * to real images (the result single, or double for a double image), and the
 * sform (else qform) affine, which must be a generalized permutation matrix
 * once entries below tolerance x the smallest of its three largest are
 * cleared, turned into axis flips and a permutation to x, y, z order; voxel
 * sizes from the affine, in millimetres.  saveNii(filename, img, vsz) =
 * make_nii(img, vsz) + save_nii: a 352-byte 'n+1' header (sform_code 1 from
 * vsz) and the image in its own class.  File access and gzip are the
 * caller's. */
typedef struct {
    /* as stored */
    int32_t filetype;            /* 2: 'n+1' single file, 1: 'ni1' .hdr/.img pair, 0: Analyze 7.5 */
    int32_t big_endian;
    int32_t stored_datatype;
    int32_t bitpix;              /* of the stored datatype */
    int64_t stored_dim[8];       /* dim, entries < 1 read as 1 */
    int64_t vox_offset;          /* first voxel byte in an 'n+1' file; 0 for a separate .img */
    double vox_offset_stored;
    double scl_slope, scl_inter;
    double quatern[3], qoffset[3], srow[12];
    /* the loaded image */
    int32_t datatype;            /* 16 or 64 after scaling, else as stored */
    int32_t scaled;              /* load_nii applied scl_slope / scl_inter */
    int64_t dim[8];              /* spatial sizes in loaded axis order */
    double pixdim[8];            /* abs, millimetres, loaded axis order (as stored for Analyze) */
    double originator[5];
    int32_t perm[3];             /* loaded axis j is stored axis perm[j] (0-based) */
    int32_t flip[3];             /* loaded axis j runs backwards through that stored axis */
    int32_t reoriented;          /* perm / flip is not the identity */
    int32_t qform_code, sform_code;  /* 0 once the affine was applied */
    int32_t xyzt_units;          /* spatial unit set to mm when it was m or um */
    char data_type[11], db_name[19], descrip[81], aux_file[25], intent_name[17], magic[5];
    char error[160];             /* message of a failed parse */
} qsm_nifti_hdr;

/* Parse the first nbytes (>= 348) of a .nii file or a .hdr file: load_nii_hdr.m
 * and the header side of load_nii_img.m / xform_nii.m.  tolerance <= 0 means eps
 * (load_nii's default is 0.1); preferred_form 's', 'q', 'S' or 'Q' as in
 * load_nii.m ('s': sform, else qform).  Host only; no context.  A bad header
 * returns QSM_ERR_ARG or QSM_ERR_DTYPE with hdr->error set; images over 2^40
 * elements are QSM_ERR_DIMS. */
qsm_status qsm_nifti_parse(const void *header, size_t nbytes, double tolerance, char preferred_form,
                           qsm_nifti_hdr *hdr);
/* Bytes of the stored image: prod(stored_dim[1..7]) * bitpix / 8. */
size_t qsm_nifti_payload_bytes(const qsm_nifti_hdr *hdr);
/* img (host or device, prod(dim[1..7]) elements, MATLAB order of hdr->dim) = the
 * loaded image of the stored bytes `payload` (host or device, starting at the first
 * voxel, at least qsm_nifti_payload_bytes(hdr) bytes; device buffers aligned to
 * their element sizes): byte order, scaling, flips and permutation in one device
 * pass.
 * out_datatype 0 gives the loaded class (hdr->datatype); 16 / 64 convert to
 * single / double.  Bit, complex and RGB datatypes are QSM_ERR_DTYPE. */
qsm_status qsm_nifti_decode(qsm_ctx *ctx, const qsm_nifti_hdr *hdr, const void *payload,
                            int32_t out_datatype, void *img);
/* The header saveNii writes for img (host or device) of NIfTI `datatype` (the
 * class of img: 2, 4, 8, 16, 64, 256, 512, 768) with MATLAB size
 * size[0..ndims-1] and voxel size vsz: filetype 2, 352 bytes of a single .nii
 * (the image bytes follow unchanged); filetype 1, the 348 bytes of a .hdr whose
 * image goes to the .img (save_nii.m).  glmax / glmin are rounded from img. */
qsm_status qsm_nifti_make_header(qsm_ctx *ctx, int32_t datatype, int32_t ndims, const int64_t *size,
                                 const double vsz[3], int32_t filetype, const void *img,
                                 uint8_t *hdr_out);

/* ---------------- lane-order inner product (BLAS-1 replacement) ---------------- */

/* *out = x . y in the library's documented lane order (mx_dot,
 * src/utils/poisson_solver/mex/mx_blas.c:108-131 over MATLAB's ddot/sdot). */
qsm_status qsm_dot(qsm_ctx *ctx, qsm_dtype dtype, size_t n, const void *x, const void *y,
                   double *out);

/* ---------------- diagnostics ---------------- */

/* *ops_per_s = the device's throughput of separate multiplies and adds in
 * dtype (the instructions the exact kernels issue; no fused multiply-add):
 * every SM fully occupied, eight independent x = x * m + c chains per thread,
 * timed with events on the context's stream (best of three launches).  The
 * FP64 figure is the roofline of the bit-exact FP64 solvers. */
qsm_status qsm_fp_pipe_rate(qsm_ctx *ctx, qsm_dtype dtype, double *ops_per_s);

/* *mismatches = the number of inputs on which the library's integer-arithmetic
 * FP32 <-> FP64 conversions (the mixed-precision PCG's, which keep them off the
 * FP64 pipe) differ from the device's own conversions: all 2^32 floats, and
 * 2^30 doubles, most aimed at rounding ties, subnormal and overflowing float
 * results.  0 on every correct build. */
qsm_status qsm_fp_convert_check(qsm_ctx *ctx, unsigned long long *mismatches);

#ifdef __cplusplus
}
#endif

#endif /* QSM_GPU_H */
