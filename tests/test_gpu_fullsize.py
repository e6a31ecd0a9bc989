"""The benchmark's volume (224 x 224 x 128) against the oracle.

The headline TGV inversion (the brain phantom of the benchmark): the plain
FP64 path and the fused FP32 path (the autotuned kernel and the TMA kernels)
bit for bit over 40 iterations, and the benchmark's own 1000-iteration mixed
inversion within 1e-4 relative L2 of the FP64 oracle.

The widened rows on the field of the next-rows arm, with the bars of their
small-size tests: lbv bit-for-bit (its 3-level hierarchy runs the coarsest
solve over the whole GPU), V-SHARP <= 1e-9 with identical eroded masks, TV
ADMM and PDF <= 1e-9 in FP64 over the first iterations (the FFT libraries
round differently), TV ADMM FP32 <= 1e-4."""
import numpy as np
import pytest

from conftest import bits_equal, first_diff

pytestmark = pytest.mark.gpu

SHAPE = (224, 224, 128)


@pytest.fixture(scope="module")
def field():
    import qsm_gb300.synthetic as S

    f, _, m = S.field_case(SHAPE, 7, echoes=1)
    return f, m


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def headline():
    import qsm_gb300.synthetic as S

    d2f, mask, _ = S.config2()
    return d2f, mask


LAM, ALPHA = 0.003, 2.0


def test_tgv_headline_plain_fp64_bitexact(gpu_ctx, qsm, port, headline):
    d2f, m = headline
    a = qsm.pd_tgv_mex(d2f, m, [1, 1, 1], LAM, ALPHA, 0.0, 40)
    b = port.pd_tgv_mex(d2f, m, [1, 1, 1], LAM, ALPHA, 0.0, 40)
    assert bits_equal(a, b), first_diff(a, b)


@pytest.mark.parametrize("variant", [None, 8, 10, 11])
def test_tgv_headline_fused_fp32_bitexact(gpu_ctx, qsm, port, headline, variant, monkeypatch):
    """The fused kernels on the headline grid against the reference's FP32
    algorithm (mx_pdf): the autotuner's pick (None), the register-prefetch
    column kernel and the TMA-staged ones."""
    d2f, m = headline
    if variant is None:
        monkeypatch.delenv("QSM_FUSED_VARIANT", raising=False)
    else:
        monkeypatch.setenv("QSM_FUSED_VARIANT", str(variant))
    d32 = np.asfortranarray(d2f.astype(np.float32))
    a = qsm.pd_tgv_mex(d32, m, [1, 1, 1], LAM, ALPHA, 0.0, 40, fused=True)
    b = port.pd_tgv_mex(d32, m, [1, 1, 1], LAM, ALPHA, 0.0, 40)
    assert bits_equal(a, b), first_diff(a, b)


def test_tgv_headline_1000_iterations_vs_fp64_oracle(gpu_ctx, qsm, port, headline, monkeypatch):
    """The benchmark's inversion (1000 iterations, tol 0) through the mixed
    fused path stays within 1e-4 relative L2 of the FP64 oracle (OpenMP on the
    host cores, about 15 s)."""
    monkeypatch.delenv("QSM_FUSED_VARIANT", raising=False)
    d2f, m = headline
    a = qsm.pd_tgv_mex(d2f, m, [1, 1, 1], LAM, ALPHA, 0.0, 1000, fused=True)
    b = port.pd_tgv_mex(d2f, m, [1, 1, 1], LAM, ALPHA, 0.0, 1000)
    rel = _rel(a, b)
    assert rel <= 1e-4, rel


def test_lbv_fullsize_bitexact(gpu_ctx, qsm, port, field):
    import pipelines

    f, m = field
    infos = []
    fl = qsm.lbv(f, m, [1, 1, 1], infos=infos)
    ref = pipelines.lbv(f, m, [1, 1, 1])
    assert infos[0]["coarse_ctas"] < 0  # the whole-GPU coarsest solver
    assert bits_equal(fl, ref), first_diff(fl, ref)


def test_vsharp_fullsize(gpu_ctx, qsm, port, field):
    import bgremove

    f, m = field
    fl, mo = qsm.vsharp(f, m, [1, 1, 1])
    rfl, rmo = bgremove.vsharp(f, m, [1, 1, 1])
    assert np.array_equal(mo, rmo)
    assert _rel(fl, rfl) <= 1e-9


def test_tv_admm_fullsize(gpu_ctx, qsm, port, field):
    import tv_admm

    f, m = field
    fm = np.asfortranarray(f * m)
    opts = dict(maxit=2)
    trace, info = [], {}
    ref = tv_admm.tv(fm, m, [1, 1, 1], opts=opts, trace=trace)
    x = qsm.tv(fm, m, [1, 1, 1], opts=opts, info=info)
    assert info["iters"] == len(trace) and info["rho"] == trace[-1]["rho"]
    assert _rel(x, ref) <= 1e-9
    x32 = qsm.tv(fm.astype(np.float32), m, [1, 1, 1], opts=opts)
    assert _rel(x32, ref) <= 1e-4


def test_pdf_fullsize(gpu_ctx, qsm, port, field):
    import bgremove

    f, m = field
    info, rinfo = {}, {}
    fl = qsm.pdf(f, m, [1, 1, 1], None, (0.0, 0.0, 1.0), 0.0, 1e-5, 2, info=info)
    rfl = bgremove.pdf(f, m, [1, 1, 1], None, (0.0, 0.0, 1.0), 0.0, 1e-5, 2, info=rinfo)
    assert info["iters"] == rinfo["iters"]
    assert _rel(fl, rfl) <= 1e-9
