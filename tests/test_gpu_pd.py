"""GPU primal-dual TGV / TV against the oracle and the reference's golden
outputs.  The plain path is bit-exact in FP64 and FP32; the fused
mixed-precision path is bit-exact with the reference's FP32 result, and its
error against the FP64 oracle is within the stated 1e-4 relative L2."""
import hashlib

import numpy as np
import pytest

from conftest import bits_equal, first_diff

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt", ("float64", "float32"))
@pytest.mark.parametrize("case", [0, 1, 2])
def test_pd_golden_plain(gpu_ctx, qsm, golden, dt, case):
    g = golden("pd")
    tag = f"c{case}_{dt}"
    d2f, m, h = g[f"{tag}_d2f"], g[f"{tag}_mask"], g[f"{tag}_h"]
    lam, alpha, tol, iters = g[f"{tag}_args"]
    chi = qsm.pd_tgv_mex(d2f, m, h, lam, alpha, tol, int(iters))
    assert bits_equal(chi, g[f"{tag}_tgv"]), first_diff(chi, g[f"{tag}_tgv"])
    chi = qsm.pd_tv_mex(d2f, m, h, lam, tol, int(iters))
    assert bits_equal(chi, g[f"{tag}_tv"]), first_diff(chi, g[f"{tag}_tv"])


@pytest.mark.parametrize("case", [0, 1, 2])
def test_pd_golden_fused_fp32(gpu_ctx, qsm, golden, case):
    """The fused kernel reproduces the reference's single-precision chi."""
    g = golden("pd")
    tag = f"c{case}_float32"
    d2f, m, h = g[f"{tag}_d2f"], g[f"{tag}_mask"], g[f"{tag}_h"]
    lam, alpha, tol, iters = g[f"{tag}_args"]
    chi = qsm.pd_tgv_mex(d2f, m, h, lam, alpha, tol, int(iters), fused=True)
    assert bits_equal(chi, g[f"{tag}_tgv"]), first_diff(chi, g[f"{tag}_tgv"])
    chi = qsm.pd_tv_mex(d2f, m, h, lam, tol, int(iters), fused=True)
    assert bits_equal(chi, g[f"{tag}_tv"]), first_diff(chi, g[f"{tag}_tv"])


def test_config0_fp64_bitexact(gpu_ctx, qsm, golden):
    """64^3, 1000 iterations, FP64 plain path == reference (SHA-256)."""
    g = golden("config0_tgv")
    lam, alpha, tol, iters = g["args"]
    info = {}
    chi = qsm.pd_tgv_mex(g["d2f"], g["mask"], [1, 1, 1], lam, alpha, tol, int(iters), info=info)
    assert info["iters"] == 1000
    digest = np.frombuffer(hashlib.sha256(np.asfortranarray(chi).tobytes(order="F")).digest(), dtype=np.uint8)
    assert np.array_equal(digest, g["chi_sha256"]), first_diff(chi[::7, ::5, ::3], g["chi_samples"])


def test_config0_fused_error(gpu_ctx, qsm, port, golden):
    """Mixed path (FP32 fused, FP64 input/output) vs the FP64 oracle: rel-L2 <= 1e-4,
    and bit-identical to the FP32 oracle."""
    g = golden("config0_tgv")
    lam, alpha, tol, iters = g["args"]
    d2f, m = g["d2f"], g["mask"]
    chi_mixed = qsm.pd_tgv_mex(d2f, m, [1, 1, 1], lam, alpha, tol, int(iters), fused=True)
    chi64 = port.pd_tgv_mex(d2f, m, [1, 1, 1], lam, alpha, tol, int(iters))
    rel = np.linalg.norm(chi_mixed - chi64) / np.linalg.norm(chi64)
    assert rel <= 1e-4, rel
    chi32 = port.pd_tgv_mex(np.asfortranarray(d2f.astype(np.float32)), m, [1, 1, 1], lam, alpha, tol, int(iters))
    assert bits_equal(chi_mixed.astype(np.float32), chi32)


@pytest.mark.parametrize("shape", [(37, 70, 19), (3, 3, 3), (5, 4, 130)])
@pytest.mark.parametrize("dt", ("float64", "float32"))
def test_pd_vs_oracle_shapes(gpu_ctx, qsm, port, shape, dt):
    rng = np.random.default_rng(7)
    d2f = np.asfortranarray((rng.standard_normal(shape) * 0.05).astype(dt))
    m = np.asfortranarray((rng.random(shape) > 0.15).astype(np.uint8))
    h = [1.0, 0.9, 1.2]
    for fused in (False, True):
        if fused and dt == "float64":
            continue
        a = qsm.pd_tgv_mex(d2f, m, h, 0.003, 2.0, 0.0, 30, fused=fused)
        b = port.pd_tgv_mex(d2f, m, h, 0.003, 2.0, 0.0, 30)
        assert bits_equal(a, b), f"tgv fused={fused} {first_diff(a, b)}"
        a = qsm.pd_tv_mex(d2f, m, h, 0.003, 0.0, 30, fused=fused)
        b = port.pd_tv_mex(d2f, m, h, 0.003, 0.0, 30)
        assert bits_equal(a, b), f"tv fused={fused} {first_diff(a, b)}"


def test_pd_stopping_rule(gpu_ctx, qsm, port):
    """tol > 0: both paths stop at the oracle's iteration (checked every 10)."""
    rng = np.random.default_rng(3)
    shape = (24, 22, 20)
    d2f = np.asfortranarray(rng.standard_normal(shape) * 0.01)
    g = np.indices(shape).astype(float)
    m = np.asfortranarray((sum((g[i] - 11) ** 2 for i in range(3)) < 64).astype(np.uint8))
    oi, pi_, fi = {}, {}, {}
    b = port.pd_tgv_mex(d2f, m, [1, 1, 1], 0.003, 2.0, 5e-3, 2000, info=oi)
    a = qsm.pd_tgv_mex(d2f, m, [1, 1, 1], 0.003, 2.0, 5e-3, 2000, info=pi_)
    assert oi["iters"] < 2000 and oi["iters"] % 10 == 0
    assert pi_["iters"] == oi["iters"]
    assert bits_equal(a, b)
    assert pi_["monitors"] == oi["monitors"]  # lane-order monitors are bit-identical
    b32 = port.pd_tgv_mex(d2f.astype(np.float32), m, [1, 1, 1], 0.003, 2.0, 5e-3, 2000, info=oi)
    a32 = qsm.pd_tgv_mex(d2f.astype(np.float32), m, [1, 1, 1], 0.003, 2.0, 5e-3, 2000, fused=True, info=fi)
    assert fi["iters"] == oi["iters"]
    assert bits_equal(a32, b32)


def test_pd_empty_mask_and_device_tensors(gpu_ctx, qsm):
    torch = pytest.importorskip("torch")
    shape = (16, 12, 10)
    d2f = torch.randn(shape[::-1], dtype=torch.float64, device="cuda")
    m = torch.zeros(shape[::-1], dtype=torch.uint8, device="cuda")
    chi = qsm.pd_tgv_mex(d2f, m, [1, 1, 1], 0.003, 2.0, 0.0, 20)
    assert chi.is_cuda and float(chi.abs().max()) == 0.0
    chi = qsm.pd_tv_mex(d2f.float(), m, [1, 1, 1], 0.003, 0.0, 20, fused=True)
    assert float(chi.abs().max()) == 0.0


def test_pd_errors(gpu_ctx, qsm):
    a = np.zeros((0, 4, 4), order="F")
    with pytest.raises(qsm.QsmError, match="DIMS"):
        qsm.pd_tgv_mex(a, np.zeros((0, 4, 4), np.uint8), [1, 1, 1], 0.003, 2.0, 0.0, 5)
    with pytest.raises(TypeError):
        qsm.pd_tgv_mex(np.zeros((4, 4, 4), np.int32), np.ones((4, 4, 4), np.uint8), [1, 1, 1], 0.003, 2.0, 0.0, 5)


def _active_voxels(m, tile):
    """Interior voxels of the tiles that hold a voxel of m or of the dual mask
    mi (all six neighbours in m), each tile clipped to the interior."""
    mm = m != 0
    mi = np.zeros_like(mm)
    mi[1:-1, 1:-1, 1:-1] = (mm[:-2, 1:-1, 1:-1] & mm[2:, 1:-1, 1:-1] & mm[1:-1, :-2, 1:-1] & mm[1:-1, 2:, 1:-1] &
                            mm[1:-1, 1:-1, :-2] & mm[1:-1, 1:-1, 2:])
    act = (mm | mi)[1:-1, 1:-1, 1:-1]
    tx, ty, tz = tile
    tot = 0
    for a in range(0, act.shape[0], tx):
        for b in range(0, act.shape[1], ty):
            for c in range(0, act.shape[2], tz):
                blk = act[a:a + tx, b:b + ty, c:c + tz]
                tot += blk.size if blk.any() else 0
    return tot


@pytest.mark.parametrize("shape", [(77, 41, 23), (70, 30, 75)])
@pytest.mark.parametrize("variant", list(range(13)))
def test_fused_tile_variants_bitexact(gpu_ctx, qsm, port, variant, shape, monkeypatch):
    """Every tile variant (3-D tiles 0-3, z-streaming column tiles 4-9, TMA
    column tiles 10-12, which stand down to variant 8 where nx is not a
    multiple of 4 and for TV) gives the reference's FP32 result (partial
    tiles and chunks, odd extents, a mask that leaves whole tiles inactive)."""
    monkeypatch.setenv("QSM_FUSED_VARIANT", str(variant))
    rng = np.random.default_rng(40 + variant)
    d2f = np.asfortranarray((rng.standard_normal(shape) * 0.05).astype(np.float32))
    g = np.indices(shape).astype(float)
    c = [(n - 1) / 2 for n in shape]
    m = np.asfortranarray(((((g[0] - c[0]) / (0.42 * shape[0])) ** 2 + ((g[1] - c[1]) / (0.42 * shape[1])) ** 2 +
                            ((g[2] - c[2]) / (0.42 * shape[2])) ** 2) <= 1).astype(np.uint8))
    info = {}
    a = qsm.pd_tgv_mex(d2f, m, [1, 1, 1], 0.003, 2.0, 0.0, 30, fused=True, info=info)
    b = port.pd_tgv_mex(d2f, m, [1, 1, 1], 0.003, 2.0, 0.0, 30)
    assert bits_equal(a, b), first_diff(a, b)
    # tiles that miss the mask are skipped: the launched voxels are exactly those of the active tiles
    assert info["active_voxels"] == _active_voxels(m, tuple(info["tile"]))
    a = qsm.pd_tv_mex(d2f, m, [1, 1, 1], 0.003, 0.0, 30, fused=True)
    b = port.pd_tv_mex(d2f, m, [1, 1, 1], 0.003, 0.0, 30)
    assert bits_equal(a, b), first_diff(a, b)


TMA_TILES = {10: (28, 16, 16), 11: (28, 20, 16), 12: (28, 24, 16)}


def _ellipsoid_case(shape, seed, fill=0.42):
    rng = np.random.default_rng(seed)
    d2f = np.asfortranarray((rng.standard_normal(shape) * 0.05).astype(np.float32))
    g = np.indices(shape).astype(float)
    c = [(n - 1) / 2 for n in shape]
    q = sum(((g[i] - c[i]) / (fill * shape[i])) ** 2 for i in range(3))
    return d2f, np.asfortranarray((q <= 1).astype(np.uint8))


@pytest.mark.parametrize("shape", [(76, 41, 23), (72, 30, 75), (60, 64, 40), (32, 24, 18)])
@pytest.mark.parametrize("variant", [10, 11, 12])
def test_fused_tma_variants_bitexact(gpu_ctx, qsm, port, variant, shape, monkeypatch):
    """The TMA-staged column kernels (nx a multiple of 4) give the reference's
    FP32 TGV result bit for bit: partial tiles and z-chunks, plane boxes that
    reach outside the volume on every side (read as the TMA's zero fill), a
    grid smaller than one tile, anisotropic voxels."""
    monkeypatch.setenv("QSM_FUSED_VARIANT", str(variant))
    d2f, m = _ellipsoid_case(shape, 70 + variant)
    for vsz in ([1, 1, 1], [1, 0.9, 1.2]):
        info = {}
        a = qsm.pd_tgv_mex(d2f, m, vsz, 0.003, 2.0, 0.0, 30, fused=True, info=info)
        assert tuple(info["tile"]) == TMA_TILES[variant]
        b = port.pd_tgv_mex(d2f, m, vsz, 0.003, 2.0, 0.0, 30)
        assert bits_equal(a, b), first_diff(a, b)
        assert info["active_voxels"] == _active_voxels(m, tuple(info["tile"]))


def test_fused_tma_monitors_equal_register_path(gpu_ctx, qsm, monkeypatch):
    """Same tile (28 x 16): the TMA kernel's in-kernel monitors and stopping
    iteration equal the register-prefetch kernel's (every thread sums the
    same voxels in the same order)."""
    rng = np.random.default_rng(3)
    shape = (24, 22, 20)  # the stopping-rule case above (nx a multiple of 4)
    d2f = np.asfortranarray((rng.standard_normal(shape) * 0.01).astype(np.float32))
    g = np.indices(shape).astype(float)
    m = np.asfortranarray((sum((g[i] - 11) ** 2 for i in range(3)) < 64).astype(np.uint8))
    out = {}
    for variant in (8, 10):
        monkeypatch.setenv("QSM_FUSED_VARIANT", str(variant))
        info = {}
        chi = qsm.pd_tgv_mex(d2f, m, [1, 1, 1], 0.003, 2.0, 5e-3, 2000, fused=True, info=info)
        out[variant] = (chi, info)
    (c8, i8), (c10, i10) = out[8], out[10]
    assert i8["iters"] == i10["iters"] < 2000
    assert i8["monitors"] == i10["monitors"]
    assert bits_equal(c8, c10), first_diff(c8, c10)


def test_autotuned_solve_is_reset(gpu_ctx, qsm, port, monkeypatch):
    """The first solve on a new grid size times the tile variants on the live
    state and then restarts from zero: the result is unchanged."""
    monkeypatch.delenv("QSM_FUSED_VARIANT", raising=False)
    rng = np.random.default_rng(9)
    shape = (53, 47, 29)  # a size no other test uses, so tuning runs here
    d2f = np.asfortranarray((rng.standard_normal(shape) * 0.05).astype(np.float32))
    m = np.asfortranarray((rng.random(shape) > 0.1).astype(np.uint8))
    info = {}
    a = qsm.pd_tgv_mex(d2f, m, [1, 1, 1], 0.003, 2.0, 0.0, 40, fused=True, info=info)
    b = port.pd_tgv_mex(d2f, m, [1, 1, 1], 0.003, 2.0, 0.0, 40)
    assert bits_equal(a, b), first_diff(a, b)
    assert tuple(info["tile"]) in {(32, 8, 4), (32, 8, 2), (32, 4, 4), (32, 16, 2), (28, 12, 8), (28, 12, 16),
                                   (28, 12, 32), (28, 12, 64)}


@pytest.mark.parametrize("h", ([1.0, 0.9, 1.1], [0.7, 1.3, 0.9], [1.2, 0.8, 0.5]))
def test_pd_anisotropic_voxels(gpu_ctx, qsm, port, h):
    """Step sizes and stencil weights come from 1/h^2 sums computed on the
    host; with two or more non-unit voxel sizes an FMA-contracting host
    compiler rounds them differently from the reference, so every path is
    checked bit for bit on such sizes."""
    rng = np.random.default_rng(11)
    shape = (26, 22, 18)
    m = np.asfortranarray((rng.random(shape) > 0.2).astype(np.uint8))
    for dt in ("float64", "float32"):
        d2f = np.asfortranarray((rng.standard_normal(shape) * 0.05).astype(dt))
        for fused in ((False, True) if dt == "float32" else (False,)):
            a = qsm.pd_tgv_mex(d2f, m, h, 0.003, 2.0, 0.0, 20, fused=fused)
            b = port.pd_tgv_mex(d2f, m, h, 0.003, 2.0, 0.0, 20)
            assert bits_equal(a, b), f"tgv {dt} fused={fused} {first_diff(a, b)}"
            a = qsm.pd_tv_mex(d2f, m, h, 0.003, 0.0, 20, fused=fused)
            b = port.pd_tv_mex(d2f, m, h, 0.003, 0.0, 20)
            assert bits_equal(a, b), f"tv {dt} fused={fused} {first_diff(a, b)}"


def test_fused_large_volume_matches_plain(gpu_ctx, qsm):
    """384x384x256 (37.7 M voxels, about 9 GB of solver state): the fused FP32 solve
    equals the plain FP32 solve (the reference's loop structure) bit for bit, so
    offsets past 2^31 bytes and tile counts past 65535 index correctly."""
    torch = pytest.importorskip("torch")
    shape = (384, 384, 256)
    g = torch.Generator(device="cuda").manual_seed(5)
    d2f = (torch.randn(tuple(reversed(shape)), generator=g, device="cuda", dtype=torch.float32) * 0.05)
    z, y, x = torch.meshgrid(*[torch.arange(n, device="cuda", dtype=torch.float32) for n in reversed(shape)],
                             indexing="ij")
    r2 = ((x - 191.5) / 170) ** 2 + ((y - 191.5) / 170) ** 2 + ((z - 127.5) / 110) ** 2
    mask = (r2 <= 1).to(torch.uint8)
    info = {}
    a = qsm.pd_tgv_mex(d2f, mask, [1, 1, 1], 0.003, 2.0, 0.0, 12, fused=True, info=info)
    b = qsm.pd_tgv_mex(d2f, mask, [1, 1, 1], 0.003, 2.0, 0.0, 12)
    assert torch.equal(a, b)
    a = qsm.pd_tv_mex(d2f, mask, [1, 1, 1], 0.003, 0.0, 12, fused=True)
    b = qsm.pd_tv_mex(d2f, mask, [1, 1, 1], 0.003, 0.0, 12)
    assert torch.equal(a, b)
