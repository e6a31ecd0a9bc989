"""The widened rows at the benchmark's volume (224 x 224 x 128, the field of
the next-rows arm) against the oracle, with the bars of their small-size
tests: lbv bit-for-bit (its 3-level hierarchy runs the coarsest solve over the
whole GPU), V-SHARP <= 1e-9 with identical eroded masks, TV ADMM and PDF
<= 1e-9 in FP64 over the first iterations (the FFT libraries round
differently), TV ADMM FP32 <= 1e-4."""
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
