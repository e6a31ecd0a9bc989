"""GPU pipelines of the MATLAB wrappers (sstgv.m, lbv.m, unwrapLaplacian.m:
crop to the mask, echo loop, Laplacian, solve, scatter) against their CPU
restatement over the oracle's MEX steps.  The plain paths are bit-exact; the
fused sstgv is bit-exact with the reference's FP32 algorithm; the mixed
Poisson solve is within 1e-6 relative L2 of the FP64 one."""
import numpy as np
import pytest

from conftest import bits_equal, first_diff

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pip(port):
    import pipelines
    return pipelines


def _case(shape, echoes, seed, dtype=np.float64, centre=None):
    from qsm_gb300 import synthetic
    rng = np.random.default_rng(seed)
    c = centre or tuple(n / 2 for n in shape)
    m = synthetic.ellipsoid_mask(shape, [0.3 * n for n in shape], centre=c)
    g = np.indices(shape).astype(float)
    base = sum(np.sin(0.3 * (a + 1) * g[a]) for a in range(3))
    ph = np.stack([base * (0.2 + 0.1 * t) + rng.normal(0, 0.01, shape) for t in range(echoes)], axis=3)
    ph = np.asfortranarray(ph.astype(dtype))
    return (np.asfortranarray(ph[..., 0]) if echoes == 1 else ph), m


@pytest.mark.parametrize("dt", (np.float64, np.float32))
@pytest.mark.parametrize("echoes", (1, 2))
def test_sstgv_plain_bitexact(gpu_ctx, qsm, pip, dt, echoes):
    # mask near the low corner: the crop box is clamped there
    ph, m = _case((30, 26, 22), echoes, 1, dt, centre=(8.0, 13.0, 11.0))
    x = qsm.sstgv(ph, m, [1, 0.9, 1.1], 1e-3, 2.0, 0.0, 30, fused=False)
    ref = pip.sstgv(ph, m, [1, 0.9, 1.1], 1e-3, 2.0, 0.0, 30)
    assert bits_equal(x, ref), first_diff(x, ref)


@pytest.mark.parametrize("alpha", (2.0, 0.0))
def test_sstgv_fused_echoes_batched(gpu_ctx, qsm, pip, alpha):
    """Three echoes through the batched fused path equal the FP32 reference
    algorithm (alpha = 0 takes the TV branch, sstgv.m:83-87)."""
    ph, m = _case((34, 30, 26), 3, 2, np.float32)
    infos = []
    x = qsm.sstgv(ph, m, [1, 1, 1], 1e-3, alpha, 0.0, 40, fused=True, infos=infos)
    ref = pip.sstgv(ph, m, [1, 1, 1], 1e-3, alpha, 0.0, 40)
    assert bits_equal(x, ref), first_diff(x, ref)
    assert [i["iters"] for i in infos] == [40, 40, 40]


@pytest.mark.parametrize("dt", (np.float64, np.float32))
def test_lbv_bitexact(gpu_ctx, qsm, pip, dt):
    ph, m = _case((34, 30, 28), 2, 3, dt)
    fl = qsm.lbv(ph, m, [1, 1, 1])
    ref = pip.lbv(ph, m, [1, 1, 1])
    assert bits_equal(fl, ref), first_diff(fl, ref)


def test_lbv_mixed_vcycle(gpu_ctx, qsm, pip):
    ph, m = _case((34, 30, 28), 1, 4)
    fl = qsm.lbv(ph, m, [1, 1, 1], mixed=True)
    ref = pip.lbv(ph, m, [1, 1, 1])
    assert np.linalg.norm(fl - ref) <= 1e-6 * np.linalg.norm(ref)


def test_unwrap_laplacian_bitexact(gpu_ctx, qsm, pip):
    ph, m = _case((32, 28, 24), 2, 5)
    up, d2 = qsm.unwrap_laplacian(ph, m, [1, 1, 1])
    rup, rd2 = pip.unwrap_laplacian(ph, m, [1, 1, 1])
    assert bits_equal(d2, rd2), first_diff(d2, rd2)
    assert bits_equal(up, rup), first_diff(up, rup)


def test_pipelines_reject_empty_mask(gpu_ctx, qsm):
    z = np.zeros((8, 8, 8), order="F")
    m = np.zeros((8, 8, 8), np.uint8, order="F")
    for fn in (lambda: qsm.sstgv(z, m, [1, 1, 1], maxit=5), lambda: qsm.lbv(z, m, [1, 1, 1]),
               lambda: qsm.unwrap_laplacian(z, m, [1, 1, 1])):
        with pytest.raises(qsm.QsmError, match="ARG"):
            fn()
