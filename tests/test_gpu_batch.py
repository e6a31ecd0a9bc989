"""Many-volume batches and resident sessions on the GPU.

Every volume of a batch, and every job of a session, must give exactly the
result it gives alone: chi bit-identical to the one-volume fused path and to
the reference's FP32 algorithm (the oracle), whatever the other volumes'
sizes, kinds, admission times and iteration counts."""
import numpy as np
import pytest

from conftest import bits_equal, first_diff

pytestmark = pytest.mark.gpu

SHAPES = [(41, 35, 29), (56, 44, 31), (37, 52, 45)]


def _case(shape, seed, dtype=np.float32, fill=0.42):
    rng = np.random.default_rng(seed)
    d2f = np.asfortranarray((rng.standard_normal(shape) * 0.05).astype(dtype))
    g = np.indices(shape).astype(float)
    c = [(n - 1) / 2 + rng.uniform(-2, 2) for n in shape]
    q = sum(((g[i] - c[i]) / (fill * shape[i])) ** 2 for i in range(3))
    return d2f, np.asfortranarray((q <= 1).astype(np.uint8))


LAUNCH = {"packed": "4294967295", "solo": "0"}  # QSM_BATCH_SOLO_TILES


@pytest.mark.parametrize("launch", ["packed", "solo"])
@pytest.mark.parametrize("variant", list(range(13)))
def test_batch_matches_oracle_every_variant(gpu_ctx, qsm, port, variant, launch, monkeypatch):
    """Uneven volumes, 40 iterations (not a multiple of the 30-iteration
    graph), packed into persistent launches or each in its own graph branch:
    each chi equals the oracle's FP32 chi."""
    monkeypatch.setenv("QSM_FUSED_VARIANT", str(variant))
    monkeypatch.setenv("QSM_BATCH_SOLO_TILES", LAUNCH[launch])
    cases = [_case(s, 100 + k) for k, s in enumerate(SHAPES)]
    infos = []
    out = qsm.pd_tv_batch([c[0] for c in cases], [c[1] for c in cases], [1, 1, 1], 0.003, 0.0, 40, infos=infos)
    for (d2f, m), chi, inf in zip(cases, out, infos):
        ref = port.pd_tv_mex(d2f, m, [1, 1, 1], 0.003, 0.0, 40)
        assert bits_equal(chi, ref), first_diff(chi, ref)
        assert inf["iters"] == 40
    out = qsm.pd_tgv_batch([c[0] for c in cases], [c[1] for c in cases], [1, 0.9, 1.2], 0.003, 2.0, 0.0, 40,
                           infos=infos)
    for (d2f, m), chi, inf in zip(cases, out, infos):
        ref = port.pd_tgv_mex(d2f, m, [1, 0.9, 1.2], 0.003, 2.0, 0.0, 40)
        assert bits_equal(chi, ref), first_diff(chi, ref)
        assert inf["iters"] == 40


def test_batch_c3_sized_volume_vs_oracle(gpu_ctx, qsm, port, monkeypatch):
    """A volume at the batched configuration's sizes (240 x 240 x 128, tile
    shapes from the autotuner, its own graph branch) batched with a small
    one: TV and TGV chi bit-identical to the oracle's FP32 result."""
    monkeypatch.delenv("QSM_FUSED_VARIANT", raising=False)
    monkeypatch.delenv("QSM_BATCH_SOLO_TILES", raising=False)
    cases = [_case((240, 240, 128), 300), _case((56, 44, 31), 301)]
    out = qsm.pd_tv_batch([c[0] for c in cases], [c[1] for c in cases], [1, 1, 1], 1e-3, 0.0, 40)
    for (d2f, m), chi in zip(cases, out):
        ref = port.pd_tv_mex(d2f, m, [1, 1, 1], 1e-3, 0.0, 40)
        assert bits_equal(chi, ref), first_diff(chi, ref)
    out = qsm.pd_tgv_batch([c[0] for c in cases], [c[1] for c in cases], [1, 1, 1], 0.003, 2.0, 0.0, 40)
    for (d2f, m), chi in zip(cases, out):
        ref = port.pd_tgv_mex(d2f, m, [1, 1, 1], 0.003, 2.0, 0.0, 40)
        assert bits_equal(chi, ref), first_diff(chi, ref)


def test_batch_equals_alone_autotuned(gpu_ctx, qsm, monkeypatch):
    """Tile shapes from the autotuner (tuned per grid size at admission): each
    volume's chi and monitors equal its one-volume fused solve."""
    monkeypatch.delenv("QSM_FUSED_VARIANT", raising=False)
    shapes = [(61, 39, 33), (45, 58, 27), (50, 50, 50), (33, 29, 64)]
    cases = [_case(s, 200 + k) for k, s in enumerate(shapes)]
    infos = []
    out = qsm.pd_tgv_batch([c[0] for c in cases], [c[1] for c in cases], [1, 1, 1], 0.003, 2.0, 0.0, 70,
                           infos=infos)
    for (d2f, m), chi, inf in zip(cases, out, infos):
        alone = {}
        ref = qsm.pd_tgv_mex(d2f, m, [1, 1, 1], 0.003, 2.0, 0.0, 70, fused=True, info=alone)
        assert bits_equal(chi, ref), first_diff(chi, ref)
        assert inf["tile"] == alone["tile"]
        assert inf["monitors"] == alone["monitors"]
        assert inf["active_voxels"] == alone["active_voxels"]


def test_batch_fp64_io_and_empty_volume(gpu_ctx, qsm):
    """FP64 arrays are rounded in and widened out as in the one-volume call; a
    volume with an empty mask returns zeros without disturbing the rest."""
    a = _case((40, 36, 30), 300, np.float64)
    b = _case((48, 40, 34), 301, np.float64)
    empty = (np.asfortranarray(np.ones((20, 20, 20))), np.zeros((20, 20, 20), np.uint8, order="F"))
    out = qsm.pd_tv_batch([a[0], empty[0], b[0]], [a[1], empty[1], b[1]], [1, 1, 1], 0.003, 0.0, 35)
    assert out[0].dtype == np.float64
    for (d2f, m), chi in zip([a, b], [out[0], out[2]]):
        ref = qsm.pd_tv_mex(d2f, m, [1, 1, 1], 0.003, 0.0, 35, fused=True)
        assert bits_equal(chi, ref), first_diff(chi, ref)
    assert not np.any(out[1])


@pytest.mark.parametrize("launch", ["packed", "solo"])
def test_batch_stopping_rule(gpu_ctx, qsm, launch, monkeypatch):
    """tol > 0: each volume stops at its own one-volume iteration count."""
    monkeypatch.setenv("QSM_BATCH_SOLO_TILES", LAUNCH[launch])
    cases = [_case((30, 28, 26), 400, fill=0.3), _case((44, 40, 36), 401, fill=0.45)]
    infos = []
    out = qsm.pd_tgv_batch([c[0] for c in cases], [c[1] for c in cases], [1, 1, 1], 0.003, 2.0, 5e-3, 3000,
                           infos=infos)
    for (d2f, m), chi, inf in zip(cases, out, infos):
        alone = {}
        ref = qsm.pd_tgv_mex(d2f, m, [1, 1, 1], 0.003, 2.0, 5e-3, 3000, fused=True, info=alone)
        assert inf["iters"] == alone["iters"] < 3000
        assert bits_equal(chi, ref), first_diff(chi, ref)


def _poisson(shape, seed):
    from qsm_gb300 import synthetic

    f, m, _ = synthetic.poisson_case(shape, seed, semi=(0.3 * min(shape), 0.45 * min(shape)), jitter=2.0,
                                     sigma=(3.0, 8.0))
    return f, m


MG_ARGS = (1e-8, 200, -1.0, 2, 1, 2, 2, 2, 3)  # tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nb, nlevels


@pytest.mark.parametrize("launch", ["packed", "solo", "hybrid"])
def test_session_result_same_alone_and_in_mix(gpu_ctx, qsm, launch, monkeypatch):
    """A TGV job alone, then the same job admitted into a running mix of TV,
    TGV and Poisson jobs (admitted at different times, different sizes and
    iteration counts): chi is bit-identical.  The Poisson job equals the
    stand-alone mixed-precision mgpcg."""
    monkeypatch.setenv("QSM_BATCH_SOLO_TILES", {"hybrid": "60", **LAUNCH}[launch])
    ja = _case((46, 42, 38), 500)
    with qsm.Session(poisson_workers=2) as s:
        ia = s.submit_pd(ja[0], ja[1], [1, 1, 1], 0.003, 2.0, 0.0, 100, tgv=True)
        while s.running():
            s.step(30)
        alone = s.fetch(ia)
        assert s.bytes_in_use() == 0

    jb = _case((60, 38, 44), 501)
    jc = _case((35, 47, 31), 502)
    pf, pm = _poisson((40, 36, 34), 503)
    with qsm.Session(poisson_workers=2) as s:
        ib = s.submit_pd(jb[0], jb[1], [1, 1, 1], 0.003, 0.0, 0.0, 170, tgv=False)
        s.step(30)
        ip = s.submit_mgpcg(None, pf, pm, [1, 1, 1], *MG_ARGS, mixed=True)
        ia = s.submit_pd(ja[0], ja[1], [1, 1, 1], 0.003, 2.0, 0.0, 100, tgv=True)
        s.step(60)
        ic = s.submit_pd(jc[0], jc[1], [1, 1, 1], 0.002, 2.0, 0.0, 50, tgv=True)
        while s.running():
            s.step(30)
        mixed = s.fetch(ia)
        fin, inf = s.poll(ib)
        assert fin and inf["iters"] == 170
        chib = s.fetch(ib)
        chic = s.fetch(ic)
        vp = s.fetch(ip)
        assert s.bytes_in_use() == 0
    assert bits_equal(mixed, alone), first_diff(mixed, alone)
    refb = qsm.pd_tv_mex(jb[0], jb[1], [1, 1, 1], 0.003, 0.0, 170, fused=True)
    assert bits_equal(chib, refb), first_diff(chib, refb)
    refc = qsm.pd_tgv_mex(jc[0], jc[1], [1, 1, 1], 0.002, 2.0, 0.0, 50, fused=True)
    assert bits_equal(chic, refc), first_diff(chic, refc)
    refp = qsm.mgpcg_mex(None, pf, pm, [1, 1, 1], *MG_ARGS, mixed=True)
    assert bits_equal(vp, refp), first_diff(vp, refp)


def test_session_admission_budget(gpu_ctx, qsm):
    """A submit that does not fit in the byte budget is refused with
    QSM_ERR_BUSY and changes nothing; fetching frees the bytes."""
    a = _case((40, 40, 40), 600)
    b = _case((50, 44, 40), 601)
    fa = qsm.footprint("tgv", a[0].shape)
    fb = qsm.footprint("tv", b[0].shape)
    with qsm.Session(budget_bytes=fa + fb - 1, poisson_workers=0) as s:
        ia = s.submit_pd(a[0], a[1], [1, 1, 1], 0.003, 2.0, 0.0, 30, tgv=True)
        assert s.bytes_in_use() == fa
        with pytest.raises(qsm.QsmError, match="BUSY"):
            s.submit_pd(b[0], b[1], [1, 1, 1], 0.003, 0.0, 0.0, 30, tgv=False)
        assert s.bytes_in_use() == fa
        with pytest.raises(qsm.QsmError, match="BUSY"):
            s.fetch(ia)  # still running
        s.step(30)
        s.fetch(ia)
        assert s.bytes_in_use() == 0
        ib = s.submit_pd(b[0], b[1], [1, 1, 1], 0.003, 0.0, 0.0, 30, tgv=False)
        s.step(30)
        chi = s.fetch(ib)
        with pytest.raises(qsm.QsmError, match="ARG"):
            s.fetch(ib)  # already released
    ref = qsm.pd_tv_mex(b[0], b[1], [1, 1, 1], 0.003, 0.0, 30, fused=True)
    assert bits_equal(chi, ref)


def test_session_packed_poisson_in_mix(gpu_ctx, qsm):
    """Packed Poisson solves (no worker threads): solves of different sizes
    and both V-cycle precisions, admitted at different steps, are set up on
    the session's set-up thread, stay resident and advance at least one PCG
    iteration per 30 primal-dual iterations beside a TV solve, each PCG kernel
    launched once for all solves of one shape.  Each result equals its solve
    alone bit for bit, and so does the TV solve."""
    cases = [_poisson(s, 1000 + k) for k, s in enumerate([(40, 36, 34), (58, 50, 44), (33, 61, 29), (70, 40, 52)])]
    mixed = (True, False, True, True)
    jb = _case((60, 38, 44), 501)
    with qsm.Session(poisson_workers=0) as s:
        ids = [s.submit_mgpcg(None, f, m, [1, 1, 1], *MG_ARGS, mixed=mx) for (f, m), mx in zip(cases[:2], mixed[:2])]
        ib = s.submit_pd(jb[0], jb[1], [1, 1, 1], 0.003, 0.0, 0.0, 170, tgv=False)
        s.step(30)
        ids += [s.submit_mgpcg(None, f, m, [1, 1, 1], *MG_ARGS, mixed=mx) for (f, m), mx in zip(cases[2:], mixed[2:])]
        steps = 1
        while s.running():
            s.step(30)
            steps += 1
        infos = []
        for i in ids:
            fin, inf = s.poll(i)
            assert fin
            infos.append(inf)
        outs = [s.fetch(i) for i in ids]
        chib = s.fetch(ib)
        assert s.bytes_in_use() == 0
    for (f, m), mx, out, inf in zip(cases, mixed, outs, infos):
        info = {}
        ref = qsm.mgpcg_mex(None, f, m, [1, 1, 1], *MG_ARGS, mixed=mx, info=info)
        assert inf["iters"] == info["iters"]
        assert bits_equal(out, ref), first_diff(out, ref)
    refb = qsm.pd_tv_mex(jb[0], jb[1], [1, 1, 1], 0.003, 0.0, 170, fused=True)
    assert bits_equal(chib, refb), first_diff(chib, refb)


def test_session_concurrent_poisson_sizes(gpu_ctx, qsm):
    """Several Poisson solves of different sizes (different coarse grids) run
    at once on the worker streams; each equals its stand-alone solve."""
    cases = [_poisson(s, 700 + k) for k, s in enumerate([(40, 36, 34), (58, 50, 44), (33, 61, 29), (70, 40, 52)])]
    with qsm.Session(poisson_workers=3) as s:
        ids = [s.submit_mgpcg(None, f, m, [1, 1, 1], *MG_ARGS, mixed=mixed)
               for (f, m), mixed in zip(cases, (True, False, True, True))]
        while s.running():
            s.step(30)
        outs = [s.fetch(i) for i in ids]
    for (f, m), mixed, out in zip(cases, (True, False, True, True), outs):
        ref = qsm.mgpcg_mex(None, f, m, [1, 1, 1], *MG_ARGS, mixed=mixed)
        assert bits_equal(out, ref), first_diff(out, ref)


def test_session_packed_destroy_while_resident(gpu_ctx, qsm):
    """A packed session destroyed with Poisson solves still queued for set-up
    or resident mid-solve releases them; a new session then solves as
    before, bit for bit against the solve alone."""
    cases = [_poisson(s, 1100 + k) for k, s in enumerate([(40, 36, 34), (33, 41, 29), (48, 30, 36)])]
    with qsm.Session(poisson_workers=0) as s:
        for f, m in cases:
            s.submit_mgpcg(None, f, m, [1, 1, 1], *MG_ARGS, mixed=True)
        s.step(30)
    f, m = cases[1]
    with qsm.Session(poisson_workers=0) as s:
        i = s.submit_mgpcg(None, f, m, [1, 1, 1], *MG_ARGS, mixed=True)
        while s.running():
            s.step(30)
        out = s.fetch(i)
        assert s.bytes_in_use() == 0
    ref = qsm.mgpcg_mex(None, f, m, [1, 1, 1], *MG_ARGS, mixed=True)
    assert bits_equal(out, ref), first_diff(out, ref)
