"""The CPU oracle (oracle/qsm_oracle.c) against golden outputs of QSM.m's own
C-MEX sources (tests/golden/*.npz, made by tests/golden/gen_golden.py):
bit-for-bit, in FP64 and FP32, for every hot-path gateway."""
import hashlib

import numpy as np
import pytest

from conftest import bits_equal, first_diff

DTYPES = ("float64", "float32")


def _z(shape, dt):
    return np.zeros(shape, dtype=dt, order="F")


@pytest.mark.parametrize("dt", DTYPES)
def test_fd_operators(port, golden, dt):
    g = golden("fd_ops")
    h = g["h"]
    for si in range(int(g["nshapes"])):
        tag = f"s{si}_{dt}"
        u, x, y, w, G, uw = (g[f"{tag}_{k}"] for k in ("u", "x", "y", "z", "G", "uw"))
        shape = u.shape
        for nm in ("gradf", "gradb", "gradc", "gradfp", "gradfm", "gradbm", "gradcm"):
            r = [_z(shape, dt) for _ in range(3)]
            args = (u, G, h) if nm.endswith("m") else (u, h)
            getattr(port, nm + "_mex")(*r, *args)
            ref = g[f"{tag}_{nm}"]
            for c in range(3):
                assert bits_equal(r[c], np.asfortranarray(ref[..., c])), f"{nm}{shape}[{c}] {first_diff(r[c], ref[..., c])}"
        for nm in ("gradf_adj", "gradb_adj", "gradfp_adj", "gradfm_adj", "gradbm_adj"):
            r = _z(shape, dt)
            args = (x, y, w, G, h) if "m_adj" in nm else (x, y, w, h)
            getattr(port, nm + "_mex")(r, *args)
            assert bits_equal(r, g[f"{tag}_{nm}"]), f"{nm}{shape} {first_diff(r, g[f'{tag}_{nm}'])}"
        r = _z(shape, dt)
        port.lap1_mex(r, u, G, h)
        assert bits_equal(r, g[f"{tag}_lap1"]), f"lap1{shape}"
        r = _z(shape, dt)
        port.lapw_mex(r, uw, h)
        assert bits_equal(r, g[f"{tag}_lapw"]), f"lapw{shape}"


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("case", [0, 1, 2])
def test_pd_solvers(port, golden, dt, case):
    g = golden("pd")
    tag = f"c{case}_{dt}"
    d2f, m, h = g[f"{tag}_d2f"], g[f"{tag}_mask"], g[f"{tag}_h"]
    lam, alpha, tol, iters = g[f"{tag}_args"]
    chi = port.pd_tgv_mex(d2f, m, h, lam, alpha, tol, int(iters))
    assert bits_equal(chi, g[f"{tag}_tgv"]), first_diff(chi, g[f"{tag}_tgv"])
    chi = port.pd_tv_mex(d2f, m, h, lam, tol, int(iters))
    assert bits_equal(chi, g[f"{tag}_tv"]), first_diff(chi, g[f"{tag}_tv"])


def test_config0_tgv_1000_iterations(port, golden):
    """64^3 TGV, 1000 iterations, FP64: the reference's chi, by SHA-256."""
    g = golden("config0_tgv")
    lam, alpha, tol, iters = g["args"]
    chi = port.pd_tgv_mex(g["d2f"], g["mask"], [1, 1, 1], lam, alpha, tol, int(iters))
    assert bits_equal(chi[::7, ::5, ::3], g["chi_samples"])
    digest = np.frombuffer(hashlib.sha256(np.asfortranarray(chi).tobytes(order="F")).digest(), dtype=np.uint8)
    assert np.array_equal(digest, g["chi_sha256"])


@pytest.mark.parametrize("dt", DTYPES)
def test_multigrid_pieces(port, golden, dt):
    g = golden("mg_ops")
    h = g["h"]
    for si in range(3):
        tag = f"s{si}_{dt}"
        v, f, x, G, G2, c2 = (g[f"{tag}_{k}"] for k in ("v", "f", "x", "G", "G2", "c2"))
        shape, sz2 = v.shape, c2.shape
        for rev in (0, 1):
            vv = v.copy(order="F")
            port.gauss_seidel_mex(vv, f, G, h, 3, rev)
            assert bits_equal(vv, g[f"{tag}_gs{rev}"]), f"gs rev={rev} {shape} {first_diff(vv, g[f'{tag}_gs{rev}'])}"
        r = _z(shape, dt)
        port.residual_mex(r, f, x, G, h)
        assert bits_equal(r, g[f"{tag}_residual"])
        r = _z(shape, dt)
        port.lapmg_mex(r, x, G, h)
        assert bits_equal(r, g[f"{tag}_lapmg"])
        r2 = _z(sz2, dt)
        port.restrict_mex(r2, x, G2)
        assert bits_equal(r2, g[f"{tag}_restrict"])
        r = v.copy(order="F")
        port.prolong_mex(r, c2, G)
        assert bits_equal(r, g[f"{tag}_prolong"])
        r = v.copy(order="F")
        port.correct_mex(r, c2, G)
        assert bits_equal(r, g[f"{tag}_correct"])


def test_masks_and_norm(port, golden):
    g = golden("mg_ops")
    for si in range(3):
        Gb = g[f"s{si}_Gb"]
        sz2 = g[f"s{si}_coarsen"].shape
        g2 = np.zeros(sz2, np.uint8, order="F")
        port.coarsen_grid_mex(g2, Gb)
        assert bits_equal(g2, g[f"s{si}_coarsen"])
        B = np.zeros(Gb.shape, np.uint8, order="F")
        port.boundary_mask_mex(B, Gb)
        assert bits_equal(B, g[f"s{si}_bmask"])
        for l1 in (1, 2, 3):
            B = np.zeros(Gb.shape, np.uint8, order="F")
            port.boundary_mask_l1_mex(B, Gb, l1)
            assert bits_equal(B, g[f"s{si}_bmask_l1_{l1}"])
        assert port.norm2_mex(g[f"s{si}_xn"], Gb) == float(g[f"s{si}_norm2"])


@pytest.mark.parametrize("dt", DTYPES)
def test_poisson_solvers(port, golden, dt):
    g = golden("solvers")
    for ci, levels in ((0, (1, 2, 3)), (1, (3,))):
        tag = f"c{ci}_{dt}"
        f, m = g[f"{tag}_f"], g[f"{tag}_mask"]
        v0 = np.zeros(f.shape, dtype=dt, order="F")
        for nl in levels:
            a = port.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 40, -1.0, 1, 1, 1, 1, 2, nl)
            assert bits_equal(a, g[f"{tag}_mgpcg{nl}"]), f"mgpcg nl={nl}"
            a = port.mgpcg_mex(v0, f, m, [1, 1, 1], 1e-8, 40, 1e-3, 3, 1, 2, 2, 2, nl)
            assert bits_equal(a, g[f"{tag}_mgpcg_mg{nl}"]), f"mgpcg(mg tol) nl={nl}"
            a = port.mg_mex(v0, f, m, [1, 1, 1], 1e-6, 4, 1, 2, 2, 2, nl)
            assert bits_equal(a, g[f"{tag}_mg{nl}"]), f"mg nl={nl}"
            a = port.fmg_mex(f, m, [1, 1, 1], -1.0, 2, 1, 2, 2, 2, nl)
            assert bits_equal(a, g[f"{tag}_fmg{nl}"]), f"fmg nl={nl}"


def test_nlevels_limit(port):
    f = np.zeros((8, 8, 8), order="F")
    with pytest.raises(ValueError, match="MAX_DEPTH"):
        port.mgpcg_mex(f, f, np.ones((8, 8, 8), np.uint8), [1, 1, 1], 1e-8, 5, -1.0, 1, 1, 1, 1, 2, 17)
