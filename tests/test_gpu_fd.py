"""GPU finite-difference operators against the oracle and the reference's
golden outputs: bit-for-bit, FP64 and FP32, host and device arrays."""
import numpy as np
import pytest

from conftest import bits_equal, first_diff

pytestmark = pytest.mark.gpu

GRADS = ("gradf", "gradb", "gradc", "gradfp")
GRADMS = ("gradfm", "gradbm", "gradcm")
ADJS = ("gradf_adj", "gradb_adj", "gradfp_adj")
ADJMS = ("gradfm_adj", "gradbm_adj")


def _z(shape, dt):
    return np.zeros(shape, dtype=dt, order="F")


@pytest.mark.parametrize("dt", ("float64", "float32"))
def test_fd_golden(gpu_ctx, qsm, golden, dt):
    g = golden("fd_ops")
    h = g["h"]
    for si in range(int(g["nshapes"])):
        tag = f"s{si}_{dt}"
        u, x, y, w, G, uw = (g[f"{tag}_{k}"] for k in ("u", "x", "y", "z", "G", "uw"))
        shape = u.shape
        for nm in GRADS + GRADMS:
            r = [_z(shape, dt) for _ in range(3)]
            args = (u, G, h) if nm in GRADMS else (u, h)
            getattr(qsm, nm + "_mex")(*r, *args)
            ref = g[f"{tag}_{nm}"]
            for c in range(3):
                assert bits_equal(r[c], np.asfortranarray(ref[..., c])), f"{nm}{shape}[{c}] {first_diff(r[c], ref[..., c])}"
        for nm in ADJS + ADJMS:
            r = _z(shape, dt)
            args = (x, y, w, G, h) if nm in ADJMS else (x, y, w, h)
            getattr(qsm, nm + "_mex")(r, *args)
            assert bits_equal(r, g[f"{tag}_{nm}"]), f"{nm}{shape} {first_diff(r, g[f'{tag}_{nm}'])}"
        r = _z(shape, dt)
        qsm.lap1_mex(r, u, G, h)
        assert bits_equal(r, g[f"{tag}_lap1"]), f"lap1{shape} {first_diff(r, g[f'{tag}_lap1'])}"
        r = _z(shape, dt)
        qsm.lapw_mex(r, uw, h)
        assert bits_equal(r, g[f"{tag}_lapw"]), f"lapw{shape}"


@pytest.mark.parametrize("shape", [(64, 48, 40), (129, 67, 33), (31, 200, 9)])
@pytest.mark.parametrize("dt", ("float64", "float32"))
def test_fd_vs_oracle_larger(gpu_ctx, qsm, port, shape, dt):
    """Sizes beyond the fixtures (partial tiles, odd extents) against the oracle."""
    rng = np.random.default_rng(hash((shape, dt)) % 2**32)
    u = np.asfortranarray(rng.standard_normal(shape).astype(dt))
    x, y, w = (np.asfortranarray(rng.standard_normal(shape).astype(dt)) for _ in range(3))
    G = np.asfortranarray((rng.random(shape) > 0.2).astype(np.uint8))
    h = [0.8, 1.0, 1.1]
    for nm in GRADS + GRADMS:
        a = [_z(shape, dt) for _ in range(3)]
        b = [_z(shape, dt) for _ in range(3)]
        args = (u, G, h) if nm in GRADMS else (u, h)
        getattr(qsm, nm + "_mex")(*a, *args)
        getattr(port, nm + "_mex")(*b, *args)
        for c in range(3):
            assert bits_equal(a[c], b[c]), f"{nm}[{c}] {first_diff(a[c], b[c])}"
    for nm in ADJS + ADJMS:
        a, b = _z(shape, dt), _z(shape, dt)
        args = (x, y, w, G, h) if nm in ADJMS else (x, y, w, h)
        getattr(qsm, nm + "_mex")(a, *args)
        getattr(port, nm + "_mex")(b, *args)
        assert bits_equal(a, b), f"{nm} {first_diff(a, b)}"
    a, b = _z(shape, dt), _z(shape, dt)
    qsm.lap1_mex(a, u, G, h)
    port.lap1_mex(b, u, G, h)
    assert bits_equal(a, b)
    uw = np.asfortranarray((rng.standard_normal(shape) * 5).astype(dt))
    a, b = _z(shape, dt), _z(shape, dt)
    qsm.lapw_mex(a, uw, h)
    port.lapw_mex(b, uw, h)
    assert bits_equal(a, b)


def test_fd_device_tensors(gpu_ctx, qsm, port):
    """torch CUDA tensors are used in place (C-order (nz,ny,nx) == MATLAB x-fastest)."""
    torch = pytest.importorskip("torch")
    shape = (40, 33, 21)
    rng = np.random.default_rng(5)
    u = np.asfortranarray(rng.standard_normal(shape))
    ut = torch.from_numpy(np.ascontiguousarray(u.transpose(2, 1, 0))).cuda()
    d = [torch.zeros_like(ut) for _ in range(3)]
    qsm.gradc_mex(*d, ut, [1, 1, 1])
    ref = [_z(shape, "float64") for _ in range(3)]
    port.gradc_mex(*ref, u, [1, 1, 1])
    for c in range(3):
        got = d[c].cpu().numpy().transpose(2, 1, 0)
        assert bits_equal(np.asfortranarray(got), ref[c])


def test_masked_leaves_untouched(gpu_ctx, qsm):
    """Masked operators only write where G (the rest keeps the caller's data)."""
    shape = (10, 9, 8)
    u = np.asfortranarray(np.random.default_rng(1).standard_normal(shape))
    G = np.zeros(shape, np.uint8, order="F")
    G[2:7, 2:6, 2:5] = 1
    sentinel = 7.25
    d = [np.full(shape, sentinel, order="F") for _ in range(3)]
    qsm.gradcm_mex(*d, u, G, [1, 1, 1])
    for c in range(3):
        assert np.all(d[c][G == 0] == sentinel)


def test_fd_errors(gpu_ctx, qsm):
    a = np.zeros((1, 4, 4), order="F")
    with pytest.raises(qsm.QsmError, match="DIMS"):
        qsm.gradf_mex(a.copy(order="F"), a.copy(order="F"), a.copy(order="F"), a, [1, 1, 1])
    b = np.zeros((4, 4, 4), np.float32, order="F")
    with pytest.raises(TypeError):
        qsm.gradf_mex(b, b.copy(order="F"), b.copy(order="F"), np.zeros((4, 4, 4), order="F"), [1, 1, 1])
