"""GPU multigrid pieces and Poisson solvers against the reference's golden
outputs and the oracle: bit-for-bit (inner products follow the documented
lane order on both sides).  The mixed-precision PCG (FP64 recurrence, FP32
V-cycle) is checked for its error against the FP64 oracle."""
import numpy as np
import pytest

from conftest import bits_equal, first_diff

pytestmark = pytest.mark.gpu


def _z(shape, dt):
    return np.zeros(shape, dtype=dt, order="F")


@pytest.mark.parametrize("dt", ("float64", "float32"))
def test_mg_pieces_golden(gpu_ctx, qsm, golden, dt):
    g = golden("mg_ops")
    h = g["h"]
    for si in range(3):
        tag = f"s{si}_{dt}"
        v, f, x, G, G2, c2 = (g[f"{tag}_{k}"] for k in ("v", "f", "x", "G", "G2", "c2"))
        shape, sz2 = v.shape, c2.shape
        for rev in (0, 1):
            vv = v.copy(order="F")
            qsm.gauss_seidel_mex(vv, f, G, h, 3, rev)
            assert bits_equal(vv, g[f"{tag}_gs{rev}"]), f"gs{rev} {shape} {first_diff(vv, g[f'{tag}_gs{rev}'])}"
        r = _z(shape, dt)
        qsm.residual_mex(r, f, x, G, h)
        assert bits_equal(r, g[f"{tag}_residual"])
        r = _z(shape, dt)
        qsm.lapmg_mex(r, x, G, h)
        assert bits_equal(r, g[f"{tag}_lapmg"])
        r2 = _z(sz2, dt)
        qsm.restrict_mex(r2, x, G2)
        assert bits_equal(r2, g[f"{tag}_restrict"]), first_diff(r2, g[f"{tag}_restrict"])
        r = v.copy(order="F")
        qsm.prolong_mex(r, c2, G)
        assert bits_equal(r, g[f"{tag}_prolong"]), first_diff(r, g[f"{tag}_prolong"])
        r = v.copy(order="F")
        qsm.correct_mex(r, c2, G)
        assert bits_equal(r, g[f"{tag}_correct"])


def test_masks_norm_golden(gpu_ctx, qsm, golden):
    g = golden("mg_ops")
    for si in range(3):
        Gb = g[f"s{si}_Gb"]
        g2 = np.zeros(g[f"s{si}_coarsen"].shape, np.uint8, order="F")
        qsm.coarsen_grid_mex(g2, Gb)
        assert bits_equal(g2, g[f"s{si}_coarsen"])
        B = np.zeros(Gb.shape, np.uint8, order="F")
        qsm.boundary_mask_mex(B, Gb)
        assert bits_equal(B, g[f"s{si}_bmask"])
        for l1 in (1, 2, 3):
            B = np.zeros(Gb.shape, np.uint8, order="F")
            qsm.boundary_mask_l1_mex(B, Gb, l1)
            assert bits_equal(B, g[f"s{si}_bmask_l1_{l1}"]), f"l1={l1}"
        assert qsm.norm2_mex(g[f"s{si}_xn"], Gb) == float(g[f"s{si}_norm2"])


@pytest.mark.parametrize("dt", ("float64", "float32"))
def test_solvers_golden(gpu_ctx, qsm, golden, dt):
    g = golden("solvers")
    for ci, levels in ((0, (1, 2, 3)), (1, (3,))):
        tag = f"c{ci}_{dt}"
        f, m = g[f"{tag}_f"], g[f"{tag}_mask"]
        v0 = np.zeros(f.shape, dtype=dt, order="F")
        for nl in levels:
            a = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 40, -1.0, 1, 1, 1, 1, 2, nl)
            assert bits_equal(a, g[f"{tag}_mgpcg{nl}"]), f"mgpcg nl={nl} {first_diff(a, g[f'{tag}_mgpcg{nl}'])}"
            a = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 40, 1e-3, 3, 1, 2, 2, 2, nl)
            assert bits_equal(a, g[f"{tag}_mgpcg_mg{nl}"]), f"mgpcg(mg tol) nl={nl}"
            a = qsm.mg_mex(v0, f, m, [1, 1, 1], 1e-6, 4, 1, 2, 2, 2, nl)
            assert bits_equal(a, g[f"{tag}_mg{nl}"]), f"mg nl={nl}"
            a = qsm.fmg_mex(f, m, [1, 1, 1], -1.0, 2, 1, 2, 2, 2, nl)
            assert bits_equal(a, g[f"{tag}_fmg{nl}"]), f"fmg nl={nl}"


def test_lane_dot(gpu_ctx, qsm, port):
    rng = np.random.default_rng(11)
    for n in (1, 1000, 262144, 262145, 3_000_001):
        x, y = rng.standard_normal(n), rng.standard_normal(n)
        assert qsm.lane_dot(x, y) == port.lane_dot(x, y)
        xf, yf = x.astype(np.float32), y.astype(np.float32)
        assert qsm.lane_dot(xf, yf) == port.lane_dot(xf, yf)


def test_mgpcg_lbv_options_vs_oracle(gpu_ctx, qsm, port):
    """LBV's options (mg maxit 2, npre = npost = 2, 5 levels) on a 62^3 problem."""
    import qsm_gb300.synthetic as S

    f, m, _ = S.poisson_case((62, 62, 62), 4, semi=(20.0, 28.0))
    v0 = np.zeros(f.shape, order="F")
    oi, gi = {}, {}
    b = port.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 100, -1.0, 2, 1, 2, 2, 2, 4, info=oi)
    a = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 100, -1.0, 2, 1, 2, 2, 2, 4, info=gi)
    assert gi["iters"] == oi["iters"]
    assert bits_equal(a, b), first_diff(a, b)
    # mixed: FP64 PCG + FP32 V-cycle, same stopping rule
    mi = {}
    c = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 100, -1.0, 2, 1, 2, 2, 2, 4, mixed=True, info=mi)
    rel = np.linalg.norm(c - b) / np.linalg.norm(b)
    assert rel < 1e-6, rel
    assert mi["iters"] <= oi["iters"] + 3


@pytest.mark.parametrize("dt", ("float64", "float32"))
@pytest.mark.parametrize("shape,nl", [((62, 62, 62), 2), ((62, 62, 62), 3), ((40, 36, 45), 2), ((30, 26, 12), 2),
                                      ((28, 24, 16), 1), ((26, 22, 13), 1)])
def test_coarse_levels_vs_oracle(gpu_ctx, qsm, port, dt, shape, nl):
    """Coarsest grids from 5 to 31 interior planes: solved on a thread-block
    cluster (one slab of planes per CTA, uneven slabs included) in FP64, and
    in FP32 on one CTA from colour lists where its shared memory holds the
    grid, else on the cluster; the boundary-band sweeps run from voxel lists.
    Bit-for-bit against the oracle for the PCG, the plain V-cycle iteration
    and FMG."""
    import qsm_gb300.synthetic as S

    f, m, _ = S.poisson_case(shape, 7 + nl, semi=(8.0, 30.0))
    f = f.astype(dt)
    v0 = np.zeros(shape, dtype=dt, order="F")
    oi, gi = {}, {}
    b = port.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 30, -1.0, 2, 1, 2, 2, 2, nl, info=oi)
    a = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 30, -1.0, 2, 1, 2, 2, 2, nl, info=gi)
    assert gi["iters"] == oi["iters"]
    assert gi["coarse_ctas"] >= (1 if dt == "float32" else 2), gi  # one CTA (FP32) or the cluster
    assert bits_equal(a, b), first_diff(a, b)
    a = qsm.mg_mex(v0, f, m, [1, 1, 1], 1e-6, 3, 1, 2, 2, 2, nl)
    assert bits_equal(a, port.mg_mex(v0, f, m, [1, 1, 1], 1e-6, 3, 1, 2, 2, 2, nl))
    a = qsm.fmg_mex(f, m, [1, 0.9, 1.2], -1.0, 2, 1, 2, 2, 2, nl)
    assert bits_equal(a, port.fmg_mex(f, m, [1, 0.9, 1.2], -1.0, 2, 1, 2, 2, 2, nl))


@pytest.mark.parametrize("dt", ("float64", "float32"))
def test_coarse_grid_solver_vs_oracle(gpu_ctx, qsm, port, dt):
    """A shallow hierarchy (2 levels) whose coarsest colour passes hold ~9.5k
    voxels: the coarsest solve runs over the whole GPU (one CTA per SM, grid
    barrier per pass).  Bit-for-bit against the oracle."""
    import qsm_gb300.synthetic as S

    f, m, _ = S.poisson_case((96, 88, 80), 9, semi=(30.0, 40.0))
    f = f.astype(dt)
    v0 = np.zeros(f.shape, dtype=dt, order="F")
    oi, gi = {}, {}
    b = port.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 30, -1.0, 1, 1, 2, 2, 2, 2, info=oi)
    a = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 30, -1.0, 1, 1, 2, 2, 2, 2, info=gi)
    assert gi["coarse_ctas"] < 0, gi  # the whole-GPU solver ran
    assert gi["iters"] == oi["iters"] and gi["coarse_outer"] > 0
    assert bits_equal(a, b), first_diff(a, b)
    gm = {}
    a = qsm.mg_mex(v0, f, m, [1, 1, 1], 1e-6, 2, 1, 2, 2, 2, 2, info=gm)
    assert gm["coarse_ctas"] < 0
    assert bits_equal(a, port.mg_mex(v0, f, m, [1, 1, 1], 1e-6, 2, 1, 2, 2, 2, 2))


@pytest.mark.parametrize("outside", ["zero", "f_nonzero", "f_negzero", "v0"])
@pytest.mark.parametrize("dt", ("float64", "float32"))
def test_mgpcg_masked_steps_bitexact(gpu_ctx, qsm, port, outside, dt):
    """The PCG vector steps skip the voxels outside the mask when f and the
    initial guess are +0 there, and run over the whole array otherwise (f with
    values or -0 outside the mask, an initial guess everywhere): both forms
    bit-identical to the oracle, FP64 and FP32, and the mixed FP32-V-cycle
    solve within 1e-10 of the FP64 one."""
    import qsm_gb300.synthetic as S

    f, m, _ = S.poisson_case((70, 64, 52), 11, semi=(18.0, 26.0))
    rng = np.random.default_rng(12)
    v0 = np.zeros(f.shape, order="F")
    if outside == "f_nonzero":
        f = np.asfortranarray(np.where(m != 0, f, 0.1 * rng.standard_normal(f.shape)))
    elif outside == "f_negzero":
        f = np.asfortranarray(np.where(m != 0, f, -0.0))
    elif outside == "v0":
        v0 = np.asfortranarray(0.01 * rng.standard_normal(f.shape))
    f = np.asfortranarray(f.astype(dt))
    v0 = np.asfortranarray(v0.astype(dt))
    # values outside the mask stay in the residual, so the relative tolerance is
    # never met there: a few iterations (many more break the reference down in FP32)
    maxit = 6 if outside == "f_nonzero" else 60
    oi, gi = {}, {}
    b = port.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, maxit, -1.0, 2, 1, 2, 2, 2, 4, info=oi)
    a = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, maxit, -1.0, 2, 1, 2, 2, 2, 4, info=gi)
    assert gi["iters"] == oi["iters"]
    assert bits_equal(a, b), first_diff(a, b)
    if dt == "float64" and outside != "f_nonzero":
        c = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, maxit, -1.0, 2, 1, 2, 2, 2, 4, mixed=True)
        assert np.linalg.norm(c - a) <= 1e-10 * np.linalg.norm(a)


def test_coarsest_idle_solve_bitexact(gpu_ctx, qsm, port):
    """A thin volume with five levels leaves a coarsest grid whose mask and
    right-hand side are empty: the reference's coarsest loop cannot meet
    tol * ||f|| = 0 and runs all 1024 outer iterations without changing a
    value.  The one-CTA FP32 solver stops after the first with the same
    result, still reports the 1024 outer iterations of each call, and the
    whole solve stays bit-identical to the oracle (which takes ~20 s here)."""
    import qsm_gb300.synthetic as S

    f, m, _ = S.poisson_case((48, 48, 16), 3, semi=(6.0, 20.0))
    f = np.asfortranarray(f.astype(np.float32))
    v0 = np.zeros(f.shape, dtype=np.float32, order="F")
    oi, gi = {}, {}
    b = port.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 3, -1.0, 2, 1, 2, 2, 2, 5, info=oi)
    a = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 3, -1.0, 2, 1, 2, 2, 2, 5, info=gi)
    assert gi["iters"] == oi["iters"]
    assert bits_equal(a, b), first_diff(a, b)
    assert gi["coarse_ctas"] == 1
    assert gi["coarse_outer"] == 1024 * 2 * gi["iters"]  # every call idle, counted as the reference runs it
    assert gi["seconds"] < 0.5, gi["seconds"]


def test_coarsest_idle_cluster_solve_bitexact(gpu_ctx, qsm, port):
    """The same idle coarsest loop in FP64 on the thread-block cluster: a mask
    a few planes thick in a 64 x 64 x 40 grid leaves the 6 x 6 x 4 coarsest
    grid without mask voxels; the cluster solver stops each idle call after
    one outer iteration, reports 1024, and matches the oracle bit for bit."""
    import qsm_gb300.synthetic as S

    rng = np.random.default_rng(8)
    shape = (64, 64, 40)
    m = S.ellipsoid_mask(shape, (24.0, 20.0, 3.0))
    u = np.asfortranarray(rng.standard_normal(shape))
    f = np.asfortranarray(-S.lap7(u, m, (1.0, 1.0, 1.0)))
    v0 = np.zeros(shape, order="F")
    oi, gi = {}, {}
    b = port.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 3, -1.0, 2, 1, 2, 2, 2, 5, info=oi)
    a = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 3, -1.0, 2, 1, 2, 2, 2, 5, info=gi)
    assert gi["iters"] == oi["iters"]
    assert bits_equal(a, b), first_diff(a, b)
    assert gi["coarse_ctas"] >= 2  # the cluster solver
    assert gi["coarse_outer"] == 1024 * 2 * gi["iters"]
    assert gi["seconds"] < 0.5, gi["seconds"]


def test_grid_barrier_wait_runs_out(gpu_ctx, qsm, port):
    """The grid barrier of the whole-GPU multigrid kernels waits a bounded
    number of polls.  With the context's test hook every barrier waits for
    one arrival more than the grid makes, so each wait runs out: the solve
    must return QSM_ERR_TIMEOUT within seconds (no hang), and the same
    context must then solve normally, bit for bit against the oracle."""
    import time

    import qsm_gb300._lib as _lib
    import qsm_gb300.synthetic as S

    f, m, _ = S.poisson_case((96, 88, 80), 9, semi=(30.0, 40.0))
    v0 = np.zeros(f.shape, dtype=f.dtype, order="F")
    L = _lib.lib()
    assert L.qsm_ctx_set_debug(gpu_ctx.handle, 1) == 0
    try:
        t0 = time.perf_counter()
        gi = {}
        with pytest.raises(_lib.QsmError) as ei:
            qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 30, -1.0, 1, 1, 2, 2, 2, 2, info=gi, ctx=gpu_ctx)
        assert ei.value.status == 9  # QSM_ERR_TIMEOUT
        assert time.perf_counter() - t0 < 60
        with pytest.raises(_lib.QsmError) as ei:
            qsm.mg_mex(v0, f, m, [1, 1, 1], 1e-6, 2, 1, 2, 2, 2, 2, ctx=gpu_ctx)
        assert ei.value.status == 9
    finally:
        assert L.qsm_ctx_set_debug(gpu_ctx.handle, 0) == 0
    assert L.qsm_ctx_set_debug(gpu_ctx.handle, 2) == 1  # unknown flags are refused (QSM_ERR_ARG)
    oi, gi = {}, {}
    b = port.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 30, -1.0, 1, 1, 2, 2, 2, 2, info=oi)
    a = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 30, -1.0, 1, 1, 2, 2, 2, 2, info=gi, ctx=gpu_ctx)
    assert gi["coarse_ctas"] < 0  # the whole-GPU solver ran again, its barriers completing
    assert gi["iters"] == oi["iters"]
    assert bits_equal(a, b), first_diff(a, b)


@pytest.mark.parametrize("dt", ("float64", "float32"))
def test_mgpcg_256_lbv_options_bitexact(gpu_ctx, qsm, port, dt):
    """The benchmark's Poisson problem at full size (256^3, LBV options, 5
    levels: 16-CTA cluster coarsest solve in FP64, one CTA in FP32, list passes, fused PCG steps):
    bit-for-bit against the oracle, same iteration count."""
    import qsm_gb300.synthetic as S

    f, m, _ = S.config1(seed=1)
    f = f.astype(dt)
    v0 = np.zeros(f.shape, dtype=dt, order="F")
    oi, gi = {}, {}
    b = port.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 40, -1.0, 2, 1, 2, 2, 2, 5, info=oi)
    a = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 40, -1.0, 2, 1, 2, 2, 2, 5, info=gi)
    assert gi["iters"] == oi["iters"] == 10
    assert gi["coarse_ctas"] == (1 if dt == "float32" else 16)
    assert bits_equal(a, b), first_diff(a, b)


def test_mixed_pcg_cluster_coarse(gpu_ctx, qsm, port):
    """FP64 PCG with the FP32 V-cycle (FP32 coarsest solve on one CTA from
    colour lists): same stopping rule, error against the FP64 oracle."""
    import qsm_gb300.synthetic as S

    f, m, _ = S.poisson_case((70, 64, 58), 5, semi=(20.0, 30.0))
    v0 = np.zeros(f.shape, order="F")
    oi, mi = {}, {}
    b = port.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 100, -1.0, 2, 1, 2, 2, 2, 3, info=oi)
    c = qsm.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 100, -1.0, 2, 1, 2, 2, 2, 3, mixed=True, info=mi)
    assert mi["coarse_ctas"] >= 1, mi
    assert np.linalg.norm(c - b) / np.linalg.norm(b) < 1e-6
    assert mi["iters"] <= oi["iters"] + 3


def test_mg_errors(gpu_ctx, qsm):
    f = np.zeros((8, 8, 8), order="F")
    with pytest.raises(qsm.QsmError, match="DEPTH"):
        qsm.mgpcg_mex(f, f, np.ones((8, 8, 8), np.uint8), [1, 1, 1], 1e-8, 5, -1.0, 1, 1, 1, 1, 2, 17)
    with pytest.raises(qsm.QsmError, match="DIMS"):
        qsm.restrict_mex(np.zeros((9, 9, 9), order="F"), np.zeros((8, 8, 8), order="F"), np.ones((9, 9, 9), np.uint8))


def test_fp_convert_exact(gpu_ctx, qsm):
    """The mixed solver's integer-arithmetic FP32 <-> FP64 conversions give
    the device's own conversion bits on every float and on 2^30 doubles aimed
    at rounding ties, subnormal and overflowing results."""
    assert qsm.fp_convert_check(ctx=gpu_ctx) == 0


@pytest.mark.parametrize("mixed", [True, False])
def test_mgpcg_batch_bitexact(gpu_ctx, qsm, mixed):
    """Packed Poisson solves: volumes of different sizes (different
    hierarchies and iteration counts; one with an initial guess that is -0
    or nonzero outside the mask, so its PCG steps run over the whole array)
    advance together, each kernel of a PCG iteration launched once for all.
    Each result equals the same solve alone bit for bit."""
    import qsm_gb300.synthetic as S

    shapes = [(40, 36, 34), (58, 50, 44), (33, 61, 29), (70, 40, 52), (96, 88, 80)]
    cases = [S.poisson_case(sh, 800 + k, semi=(10.0, 30.0))[:2] for k, sh in enumerate(shapes)]
    fs = [c[0] for c in cases]
    ms = [c[1] for c in cases]
    v0s = [None] * len(cases)
    v0s[1] = np.asfortranarray(0.01 * fs[1] - 0.0)
    args = ([1, 1, 1], 1e-8, 60, -1.0, 2, 1, 2, 2, 2, 4)
    infos = []
    outs = qsm.mgpcg_batch(v0s, fs, ms, *args, mixed=mixed, infos=infos)
    for b in range(len(cases)):
        info = {}
        ref = qsm.mgpcg_mex(v0s[b], fs[b], ms[b], *args, mixed=mixed, info=info)
        assert infos[b]["iters"] == info["iters"], (b, infos[b], info)
        assert infos[b]["coarse_ctas"] == 1  # one CTA per solve in the packed launches
        assert np.array_equal(infos[b]["resnorm_hist"], info["resnorm_hist"])
        assert bits_equal(outs[b], ref), (b, first_diff(outs[b], ref))


def test_mgpcg_batch_groups(gpu_ctx, qsm):
    """More solves than one packed launch takes (16): 18 small volumes in two
    groups, each equal to its solve alone."""
    import qsm_gb300.synthetic as S

    rng = np.random.default_rng(5)
    shapes = [tuple(int(x) for x in rng.integers(18, 34, 3)) for _ in range(18)]
    cases = [S.poisson_case(sh, 900 + k, semi=(5.0, 14.0))[:2] for k, sh in enumerate(shapes)]
    args = ([1, 1, 1], 1e-8, 40, -1.0, 2, 1, 2, 2, 2, 3)
    outs = qsm.mgpcg_batch(None, [c[0] for c in cases], [c[1] for c in cases], *args, mixed=True)
    for (f, m), out in zip(cases, outs):
        ref = qsm.mgpcg_mex(None, f, m, *args, mixed=True)
        assert bits_equal(out, ref), first_diff(out, ref)


@pytest.mark.parametrize("dt_mixed", [False, True])
def test_mgpcg_batch_tiny_grids_vs_oracle(gpu_ctx, qsm, port, dt_mixed):
    """Packed solves of tiny grids (3 to 9 voxels per axis, odd and even, masks
    filling the box or touching its faces, a single voxel): FP64 solves
    against the oracle bit for bit; the FP32 V-cycle ones against their solves
    alone."""
    rng = np.random.default_rng(21)
    shapes = [(3, 3, 3), (4, 5, 3), (7, 6, 9), (8, 8, 8), (9, 4, 6), (5, 9, 7)]
    fs, ms = [], []
    for k, sh in enumerate(shapes):
        f = np.asfortranarray(rng.standard_normal(sh))
        m = np.ones(sh, np.uint8, order="F") if k % 2 == 0 else np.asfortranarray(
            (rng.random(sh) > 0.3).astype(np.uint8))
        if k == 4:
            m[:] = 0
            m[2, 1, 3] = 1  # a single voxel
        fs.append(np.asfortranarray(f * m))
        ms.append(m)
    args = ([1, 1, 1], 1e-8, 30, -1.0, 2, 1, 2, 2, 2, 2)
    outs = qsm.mgpcg_batch(None, fs, ms, *args, mixed=dt_mixed)
    for f, m, out in zip(fs, ms, outs):
        if dt_mixed:
            ref = qsm.mgpcg_mex(None, f, m, *args, mixed=True)
        else:
            ref = port.mgpcg_mex(np.zeros_like(f, order="F"), f, m, *args)
        assert bits_equal(out, ref), (f.shape, first_diff(out, ref))
