// Packed Poisson solves for resident sessions (pd_batch.cu): a session that
// keeps MG-PCG solves resident advances them together, one PCG iteration per
// step, each kernel of the iteration launched once for every solve of the
// same multigrid shape (mg.cu:pcg_pack_iter).  Results are those of the
// solves alone, bit for bit.
#pragma once

#include "common.cuh"

namespace qsm {

struct MgPackSolve;

// Sets up one solve (FP64 device arrays of an unpadded grid d; v0 may be null)
// on ctx's stream: everything mgpcg does before its first iteration.
qsm_status mgpack_setup(qsm_ctx *ctx, bool mixed, const Dims &d, const double *v0, const double *f,
                        const uint8_t *mask, const double vsz[3], double tolcg, int32_t maxitcg, double tolmg,
                        int32_t maxitmg, int32_t mu, int32_t npre, int32_t npost, int32_t nb, int32_t nl,
                        MgPackSolve **out);
// Whether the solve met its tolerance or maxit.
bool mgpack_done(const MgPackSolve *s);
// One PCG iteration of every solve in s[0..n) that is not done: packed where
// solves share a shape (up to 16 per launch), else one by one.  h_res: 16
// pinned doubles of scratch.
qsm_status mgpack_step(qsm_ctx *ctx, MgPackSolve *const *s, int n, double *h_res);
// Writes the solution (device, unpadded) and the statistics, and frees the solve.
qsm_status mgpack_finish(qsm_ctx *ctx, MgPackSolve *s, double *vout, qsm_mg_info *info);

}  // namespace qsm
