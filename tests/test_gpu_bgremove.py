"""GPU FFT background removal (sharp.m, vsharp.m, ismv.m, resharp.m, pdf.m on
cuFFT) against the CPU restatement (oracle/bgremove.py, numpy FFTs).  FP64
fields: relative L2 difference <= 1e-9 (the FFT libraries round differently;
iterative methods a looser bar where stated); eroded masks identical;
iterative methods stop at the same iteration.  FP32 fields: <= 1e-4 against
the FP64 restatement (PDF: 1e-3)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg(port):
    import bgremove
    return bgremove


def _case(shape, seed, echoes=1):
    """A local field inside an ellipsoidal mask plus a smooth background from
    sources outside it."""
    from qsm_gb300 import synthetic
    rng = np.random.default_rng(seed)
    m = synthetic.ellipsoid_mask(shape, [0.36 * n for n in shape], centre=[n / 2 + 0.7 for n in shape])
    g = np.indices(shape).astype(float)
    out = []
    for t in range(echoes):
        chi = synthetic.ellipsoid_phantom(shape, 5, rng, m, semi=(2.0, 5.0), chi=(-0.1, 0.1))
        loc = np.real(np.fft.ifftn(synthetic.dipole_kernel(shape) * np.fft.fftn(chi)))
        src = [(-8.0, 0.3 * shape[1], 0.5 * shape[2]), (shape[0] + 6.0, 0.6 * shape[1], 0.2 * shape[2])]
        bgf = sum(((g[0] - c[0]) ** 2 + (g[1] - c[1]) ** 2 + (g[2] - c[2]) ** 2) ** -0.5 for c in src)
        out.append((loc + (1 + t) * 20.0 * bgf) * m)
    f = out[0] if echoes == 1 else np.stack(out, axis=3)
    return np.asfortranarray(f), m


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("shape,vsz", [((40, 36, 32), (1.0, 1.0, 1.0)), ((37, 41, 29), (1.0, 0.9, 1.2))])
def test_sharp(gpu_ctx, qsm, bg, shape, vsz):
    f, m = _case(shape, 1)
    fl, mo = qsm.sharp(f, m, vsz, 4.0, 0.05)
    rfl, rmo = bg.sharp(f, m, vsz, 4.0, 0.05)
    assert np.array_equal(mo, rmo)
    assert _rel(fl, rfl) <= 1e-9


@pytest.mark.parametrize("rs", [None, [6.0, 4.0, 3.0], [5.0, 3.0]])
def test_vsharp(gpu_ctx, qsm, bg, rs):
    f, m = _case((44, 40, 36), 2, echoes=2)
    fl, mo = qsm.vsharp(f, m, [1, 1, 1], rs, 0.05)
    rfl, rmo = bg.vsharp(f, m, [1, 1, 1], rs, 0.05)
    assert np.array_equal(mo, rmo)
    assert _rel(fl, rfl) <= 1e-9


def test_ismv(gpu_ctx, qsm, bg):
    f, m = _case((40, 38, 34), 3)
    info, rinfo = {}, {}
    fl, mo = qsm.ismv(f, m, [1, 1, 1], 3.0, 1e-6, 200, info=info)
    rfl, rmo = bg.ismv(f, m, [1, 1, 1], 3.0, 1e-6, 200, info=rinfo)
    assert np.array_equal(mo, rmo)
    assert info["iters"] == rinfo["iters"] and 0 < info["iters"][0] < 200
    assert _rel(fl, rfl) <= 1e-8


def test_fp32(gpu_ctx, qsm, bg):
    f, m = _case((40, 36, 32), 4)
    rfl, _ = bg.sharp(f, m, [1, 1, 1], 4.0, 0.05)
    fl, _ = qsm.sharp(f.astype(np.float32), m, [1, 1, 1], 4.0, 0.05)
    assert fl.dtype == np.float32 and _rel(fl, rfl) <= 1e-4
    rfl, _ = bg.vsharp(f, m, [1, 1, 1], [5.0, 3.0], 0.05)
    fl, _ = qsm.vsharp(f.astype(np.float32), m, [1, 1, 1], [5.0, 3.0], 0.05)
    assert _rel(fl, rfl) <= 1e-4


def test_errors(gpu_ctx, qsm):
    z = np.zeros((10, 10, 10), order="F")
    with pytest.raises(qsm.QsmError, match="ARG"):
        qsm.sharp(z, np.zeros((10, 10, 10), np.uint8), [1, 1, 1])
    with pytest.raises(qsm.QsmError, match="ARG"):
        qsm.vsharp(z, np.ones((10, 10, 10), np.uint8), [1, 1, 1], [4.0])


def test_resharp(gpu_ctx, qsm, bg):
    f, m = _case((40, 36, 32), 5, echoes=2)
    info, rinfo = {}, {}
    fl, mo = qsm.resharp(f, m, [1, 1, 1], 3.0, 1e-2, 1e-6, 100, info=info)
    rfl, rmo = bg.resharp(f, m, [1, 1, 1], 3.0, 1e-2, 1e-6, 100, info=rinfo)
    assert np.array_equal(mo, rmo)
    assert info["iters"] == rinfo["iters"] and 0 < info["iters"][0] < 100
    assert _rel(fl, rfl) <= 1e-8


@pytest.mark.parametrize("vsz,bdir,lam,weighted", [
    ((1.0, 1.0, 1.0), (0.0, 0.0, 1.0), 0.0, False),
    ((1.0, 0.9, 1.1), (0.1, 0.2, 0.95), 0.0, True),
    ((1.0, 1.0, 1.2), (0.0, 0.0, 2.0), 1e-3, False),
])
def test_pdf(gpu_ctx, qsm, bg, vsz, bdir, lam, weighted):
    """30 LSMR iterations.  The GPU's reductions and cuFFT round differently from
    numpy, and LSMR without reorthogonalisation amplifies such differences as the
    iteration goes on: with a real-to-complex FFT in place of fftn, the oracle
    moves by 1e-14 after 30 iterations but by 5e-9 after 60 on the weighted
    oblique case.  So 30 iterations and 1e-9."""
    f, m = _case((40, 36, 32), 6, echoes=2)
    w = None
    if weighted:
        w = np.asfortranarray(m * (0.5 + np.random.default_rng(1).random(m.shape)))
    info, rinfo = {}, {}
    fl = qsm.pdf(f, m, vsz, w, bdir, lam, 1e-5, 30, info=info)
    rfl = bg.pdf(f, m, vsz, w, bdir, lam, 1e-5, 30, info=rinfo)
    assert info["iters"] == rinfo["iters"]
    assert _rel(fl, rfl) <= 1e-9


def test_pdf_defaults(gpu_ctx, qsm, bg):
    """Default tol and maxit (ceil(sqrt(numel(mask))) = 215 here, where LSMR stops):
    past ~120 iterations the reference's own iteration amplifies rounding
    differences to ~1e-4 of the local field (the oracle against itself with a
    real-to-complex FFT: 2e-4), so the bar here is the iteration count and 1e-2."""
    f, m = _case((40, 36, 32), 6)
    info, rinfo = {}, {}
    fl = qsm.pdf(f, m, [1, 1, 1], info=info)
    rfl = bg.pdf(f, m, [1, 1, 1], info=rinfo)
    assert info["iters"] == rinfo["iters"] == [215]
    assert _rel(fl, rfl) <= 1e-2
    # w all zero is the mask (pdf.m:50-52)
    fz = qsm.pdf(f, m, [1, 1, 1], np.zeros(m.shape), maxit=40)
    fm = qsm.pdf(f, m, [1, 1, 1], None, maxit=40)
    assert np.array_equal(fz, fm)


def test_pdf_fp32(gpu_ctx, qsm, bg):
    f, m = _case((40, 36, 32), 7)
    rfl = bg.pdf(f, m, [1, 1, 1], maxit=40)
    fl = qsm.pdf(f.astype(np.float32), m, [1, 1, 1], maxit=40)
    assert fl.dtype == np.float32 and _rel(fl, rfl) <= 1e-3


def test_krylov_fp32(gpu_ctx, qsm, bg):
    """FP32 iSMV and RESHARP (per-thread compensated FP32 sums, FP64 across threads)
    against the FP64 restatement."""
    f, m = _case((40, 36, 32), 8)
    f32 = f.astype(np.float32)
    rfl, rmo = bg.ismv(f, m, [1, 1, 1], 3.0, 1e-4, 100)
    fl, mo = qsm.ismv(f32, m, [1, 1, 1], 3.0, 1e-4, 100)
    assert fl.dtype == np.float32 and np.array_equal(mo, rmo) and _rel(fl, rfl) <= 1e-3
    rfl, rmo = bg.resharp(f, m, [1, 1, 1], 3.0, 1e-2, 1e-4, 50)
    fl, mo = qsm.resharp(f32, m, [1, 1, 1], 3.0, 1e-2, 1e-4, 50)
    assert np.array_equal(mo, rmo) and _rel(fl, rfl) <= 1e-3


def test_device_tensors_4d(gpu_ctx, qsm, bg):
    """Echoes as a CUDA tensor (torch shape = MATLAB size reversed) give the host result."""
    torch = pytest.importorskip("torch")
    f, m = _case((36, 32, 28), 9, echoes=2)
    fd = torch.from_numpy(np.ascontiguousarray(np.transpose(f, (3, 2, 1, 0)))).cuda()
    md = torch.from_numpy(np.ascontiguousarray(m.T)).cuda()
    fl, mo = qsm.vsharp(fd, md, [1, 1, 1], [5.0, 3.0], 0.05)
    hfl, hmo = qsm.vsharp(f, m, [1, 1, 1], [5.0, 3.0], 0.05)
    assert np.array_equal(fl.cpu().numpy().transpose(3, 2, 1, 0), hfl)
    assert np.array_equal(mo.cpu().numpy().T, hmo)
    pl = qsm.pdf(fd, md, [1, 1, 1], maxit=10)
    assert np.array_equal(pl.cpu().numpy().transpose(3, 2, 1, 0), qsm.pdf(f, m, [1, 1, 1], maxit=10))


def test_pdf_errors(gpu_ctx, qsm):
    f = np.zeros((10, 10, 10), order="F")
    m = np.ones((10, 10, 10), np.uint8)
    with pytest.raises(qsm.QsmError, match="ARG"):
        qsm.pdf(f, m, [1, 1, 1], bdir=[0, 0, 0])
    with pytest.raises(qsm.QsmError, match="ARG"):
        qsm.pdf(f, m, [1, 0, 1])
    with pytest.raises(ValueError):
        qsm.pdf(f, m, [1, 1, 1], w=np.ones((5, 5, 5)))
