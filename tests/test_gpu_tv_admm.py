"""GPU FFT total-variation inversion (tv.m ADMM, cuFFT) against the CPU
restatement (oracle/tv_admm.py: numpy FFTs, the oracle's gradfp MEX pieces).

FP64: the same ADMM iterations (count and rho schedule) and relative L2
difference <= 1e-9 (the two FFT libraries round differently).  FP32 stencils
and FFTs with FP64 reductions: relative L2 <= 1e-4 against the FP64 oracle."""
import numpy as np
import pytest

from conftest import first_diff

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tvo(port):
    import tv_admm
    return tv_admm


def _case(shape, seed, bdir=(0.0, 0.0, 1.0), vsz=(1.0, 1.0, 1.0)):
    from qsm_gb300 import synthetic
    rng = np.random.default_rng(seed)
    m = synthetic.ellipsoid_mask(shape, [0.4 * n for n in shape])
    chi = synthetic.ellipsoid_phantom(shape, 6, rng, m, semi=(2.0, 6.0), chi=(-0.1, 0.1))
    D = synthetic.dipole_kernel(shape, vsz, bdir)
    f = np.real(np.fft.ifftn(D * np.fft.fftn(chi))) + rng.normal(0, 0.002, shape)
    return np.asfortranarray(f * m), m


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("shape", [(32, 28, 24), (31, 27, 25)])
@pytest.mark.parametrize("mode", [1, 2])
def test_tv_fp64_matches_oracle(gpu_ctx, qsm, tvo, shape, mode):
    f, m = _case(shape, 11)
    opts = dict(maxit=12, tv=mode)
    trace, info = [], {}
    ref = tvo.tv(f, m, [1, 1, 1], opts=opts, trace=trace)
    x = qsm.tv(f, m, [1, 1, 1], opts=opts, info=info)
    assert info["iters"] == len(trace)
    assert abs(info["nr"] - trace[-1]["nr"]) <= 1e-9 * trace[-1]["nr"]
    assert _rel(x, ref) <= 1e-9, first_diff(x, ref)
    assert np.all(x[m == 0] == 0)


def test_tv_oblique_field_even_sizes(gpu_ctx, qsm, tvo):
    """Oblique B0 on even sizes: the half-spectrum multiply must reproduce
    real(ifft3(...)) on the Nyquist planes."""
    b = np.array([0.3, 0.2, 0.9])
    b = b / np.linalg.norm(b)
    f, m = _case((30, 26, 22), 12, bdir=b, vsz=(1.0, 0.9, 1.2))
    opts = dict(maxit=10)
    ref = tvo.tv(f, m, [1, 0.9, 1.2], b, opts=opts)
    x = qsm.tv(f, m, [1, 0.9, 1.2], b, opts=opts)
    assert _rel(x, ref) <= 1e-9, first_diff(x, ref)


@pytest.mark.parametrize("rtol", [0.5, 0.2, 0.1, 0.05])
def test_tv_stops_on_tolerance(gpu_ctx, qsm, tvo, rtol):
    """Loose tolerances: both stop at the same iteration before maxit, with the
    same final rho and residuals.  The stopping test runs on the device and the
    host looks every eighth iteration, so the tolerances put the stop at
    several positions within those groups: the reported iterate is the
    converged one, not a later queued one."""
    f, m = _case((28, 28, 28), 13)
    opts = dict(maxit=200, rtol=rtol, atol=1e-2)
    trace, info = [], {}
    ref = tvo.tv(f, m, [1, 1, 1], opts=opts, trace=trace)
    x = qsm.tv(f, m, [1, 1, 1], opts=opts, info=info)
    assert info["iters"] == len(trace) < 200
    assert info["rho"] == trace[-1]["rho"]
    assert abs(info["nr"] - trace[-1]["nr"]) <= 1e-9 * trace[-1]["nr"]
    assert _rel(x, ref) <= 1e-9
    x32 = qsm.tv(f.astype(np.float32), m, [1, 1, 1], opts=opts, info=info)
    assert _rel(x32, ref) <= 1e-4 or info["iters"] != len(trace)


@pytest.mark.parametrize("mode", [1, 2])
def test_tv_fp32(gpu_ctx, qsm, tvo, mode):
    """FP32: anisotropic TV runs the fused shrinkage + norm pass, isotropic the
    two-kernel path."""
    f, m = _case((40, 36, 32), 14)
    opts = dict(maxit=12, tv=mode)
    ref = tvo.tv(f, m, [1, 1, 1], opts=opts)
    x = qsm.tv(f.astype(np.float32), m, [1, 1, 1], opts=opts)
    assert x.dtype == np.float32
    assert _rel(x, ref) <= 1e-4


def test_tv_echoes_and_device_tensors(gpu_ctx, qsm, tvo):
    torch = pytest.importorskip("torch")
    f1, m = _case((24, 22, 20), 15)
    f2, _ = _case((24, 22, 20), 16)
    f4 = np.asfortranarray(np.stack([f1, f2], axis=3))
    opts = dict(maxit=6)
    x = qsm.tv(f4, m, [1, 1, 1], opts=opts)
    ref = tvo.tv(f4, m, [1, 1, 1], opts=opts)
    assert _rel(x, ref) <= 1e-9
    fd = torch.from_numpy(np.ascontiguousarray(f1.transpose(2, 1, 0))).cuda()
    md = torch.from_numpy(np.ascontiguousarray(m.transpose(2, 1, 0))).cuda()
    xd = qsm.tv(fd, md, [1, 1, 1], opts=opts)
    assert _rel(xd.cpu().numpy().transpose(2, 1, 0), ref[..., 0]) <= 1e-9


def test_tv_errors(gpu_ctx, qsm):
    with pytest.raises(qsm.QsmError, match="DIMS"):
        qsm.tv(np.zeros((8, 8, 2)), np.ones((8, 8, 2), np.uint8), [1, 1, 1])
    with pytest.raises(qsm.QsmError, match="ARG"):
        qsm.tv(np.zeros((8, 8, 8)), np.ones((8, 8, 8), np.uint8), [1, 1, 1], opts=dict(tv=3))
