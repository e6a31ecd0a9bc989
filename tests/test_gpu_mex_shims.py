"""The MEX shims (qsm.m_gb300/mex/qsm_mex.c) run on the GPU: each gateway is
compiled against the project's mxArray runtime (oracle/ref/mexshim) and the
library, then called with MATLAB-style arguments exactly as the reference's
gateways are called.  The reference's 29 gateways must reproduce the golden
outputs of the reference's own MEX files bit for bit; the whole-function
gateways must equal the Python API's results (the same library calls)."""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from conftest import ROOT, bits_equal, first_diff
from test_mex_shims import GATEWAYS

pytestmark = pytest.mark.gpu

NAMES = {"UNWRAP_LAPLACIAN": "unwrapLaplacian", "SSTGV": "sstgv", "LBV": "lbv", "SHARP": "sharp",
         "VSHARP": "vsharp", "RESHARP": "resharp", "ISMV": "ismv", "PDF": "pdf"}


@pytest.fixture(scope="module")
def mex(qsm, tmp_path_factory):
    import refmex
    out = tmp_path_factory.mktemp("mex")
    libdir = os.path.join(ROOT, "qsm.m_gb300")
    shim = os.path.join(ROOT, "oracle", "ref", "mexshim")
    src = os.path.join(ROOT, "qsm.m_gb300", "mex", "qsm_mex.c")

    def build(gw):
        name = NAMES.get(gw, gw.lower() + "_mex")
        so = str(out / f"{name}.so")
        cmd = ["gcc", "-std=c11", "-O2", "-shared", "-fPIC", f"-DQSM_MEX_{gw}", "-I", shim, "-I",
               os.path.join(ROOT, "include"), src, os.path.join(shim, "mxruntime.c"), "-L", libdir, "-lqsm_gb300",
               f"-Wl,-rpath,{libdir}", "-o", so]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        return name, so

    with ThreadPoolExecutor(8) as ex:
        paths = dict(ex.map(build, GATEWAYS))

    def call(name, *args, nlhs=1):
        return refmex.call(name, *args, nlhs=nlhs, path=paths[name])

    return call


def _z(shape, dt):
    return np.zeros(shape, dtype=dt, order="F")


@pytest.mark.parametrize("dt", ("float64", "float32"))
def test_fd_gateways(gpu_ctx, mex, golden, dt):
    g = golden("fd_ops")
    h = g["h"]
    tag = f"s0_{dt}"
    u, x, y, w, G, uw = (g[f"{tag}_{k}"] for k in ("u", "x", "y", "z", "G", "uw"))
    for nm in ("gradf", "gradb", "gradc", "gradfp", "gradfm", "gradbm", "gradcm"):
        r = [_z(u.shape, dt) for _ in range(3)]
        args = (u, G, h) if nm.endswith("m") else (u, h)
        mex(nm + "_mex", *r, *args, nlhs=0)
        ref = g[f"{tag}_{nm}"]
        for c in range(3):
            assert bits_equal(r[c], np.asfortranarray(ref[..., c])), f"{nm}[{c}] {first_diff(r[c], ref[..., c])}"
    for nm in ("gradf_adj", "gradb_adj", "gradfp_adj", "gradfm_adj", "gradbm_adj"):
        r = _z(u.shape, dt)
        args = (x, y, w, G, h) if nm.startswith(("gradfm", "gradbm")) else (x, y, w, h)
        mex(nm + "_mex", r, *args, nlhs=0)
        assert bits_equal(r, g[f"{tag}_{nm}"]), nm
    r = _z(u.shape, dt)
    mex("lap1_mex", r, u, G, h, nlhs=0)
    assert bits_equal(r, g[f"{tag}_lap1"])
    r = _z(u.shape, dt)
    mex("lapw_mex", r, uw, h, nlhs=0)
    assert bits_equal(r, g[f"{tag}_lapw"])


@pytest.mark.parametrize("dt", ("float64", "float32"))
def test_pd_gateways(gpu_ctx, mex, golden, dt):
    g = golden("pd")
    tag = f"c0_{dt}"
    d2f, m, h = g[f"{tag}_d2f"], g[f"{tag}_mask"], g[f"{tag}_h"]
    lam, alpha, tol, iters = g[f"{tag}_args"]
    chi = mex("pd_tgv_mex", d2f, m, h, lam, alpha, tol, float(iters), 0.0)
    assert chi.dtype == d2f.dtype and bits_equal(chi, g[f"{tag}_tgv"]), first_diff(chi, g[f"{tag}_tgv"])
    chi = mex("pd_tv_mex", d2f, m, h, lam, tol, float(iters), 0.0)
    assert bits_equal(chi, g[f"{tag}_tv"]), first_diff(chi, g[f"{tag}_tv"])


@pytest.mark.parametrize("dt", ("float64", "float32"))
def test_mg_gateways(gpu_ctx, mex, golden, dt):
    g = golden("mg_ops")
    h = g["h"]
    tag = f"s0_{dt}"
    v, f, x, G, G2, c2 = (g[f"{tag}_{k}"] for k in ("v", "f", "x", "G", "G2", "c2"))
    for rev in (0, 1):
        vv = v.copy(order="F")
        mex("gauss_seidel_mex", vv, f, G, h, 3.0, float(rev), nlhs=0)
        assert bits_equal(vv, g[f"{tag}_gs{rev}"]), f"gs{rev}"
    r = _z(v.shape, dt)
    mex("residual_mex", r, f, x, G, h, nlhs=0)
    assert bits_equal(r, g[f"{tag}_residual"])
    r = _z(v.shape, dt)
    mex("lapmg_mex", r, x, G, h, nlhs=0)
    assert bits_equal(r, g[f"{tag}_lapmg"])
    r2 = _z(c2.shape, dt)
    mex("restrict_mex", r2, x, G2, nlhs=0)
    assert bits_equal(r2, g[f"{tag}_restrict"])
    for nm in ("prolong", "correct"):
        r = v.copy(order="F")
        mex(nm + "_mex", r, c2, G, nlhs=0)
        assert bits_equal(r, g[f"{tag}_{nm}"]), nm


def test_mask_gateways(gpu_ctx, mex, golden):
    g = golden("mg_ops")
    Gb = g["s0_Gb"]
    g2 = np.zeros(g["s0_coarsen"].shape, np.uint8, order="F")
    mex("coarsen_grid_mex", g2, Gb, nlhs=0)
    assert bits_equal(g2, g["s0_coarsen"])
    B = np.zeros(Gb.shape, np.uint8, order="F")
    mex("boundary_mask_mex", B, Gb, nlhs=0)
    assert bits_equal(B, g["s0_bmask"])
    for l1 in (1, 2, 3):
        B = np.zeros(Gb.shape, np.uint8, order="F")
        mex("boundary_mask_l1_mex", B, Gb, float(l1), nlhs=0)
        assert bits_equal(B, g[f"s0_bmask_l1_{l1}"]), l1
    p = mex("norm2_mex", g["s0_xn"], Gb)
    assert p.dtype == g["s0_xn"].dtype and float(p.ravel()[0]) == float(g["s0_norm2"])


@pytest.mark.parametrize("dt", ("float64", "float32"))
def test_solver_gateways(gpu_ctx, mex, golden, dt):
    g = golden("solvers")
    tag = f"c0_{dt}"
    f, m = g[f"{tag}_f"], g[f"{tag}_mask"]
    v0 = np.zeros(f.shape, dtype=dt, order="F")
    h = np.array([1.0, 1.0, 1.0])
    nl = 2.0
    a = mex("mgpcg_mex", v0, f, m, h, 1e-8, 40.0, -1.0, 1.0, 1.0, 1.0, 1.0, 2.0, nl, 0.0)
    assert bits_equal(a, g[f"{tag}_mgpcg2"]), first_diff(a, g[f"{tag}_mgpcg2"])
    a = mex("mg_mex", v0, f, m, h, 1e-6, 4.0, 1.0, 2.0, 2.0, 2.0, nl)
    assert bits_equal(a, g[f"{tag}_mg2"])
    a = mex("fmg_mex", f, m, h, -1.0, 2.0, 1.0, 2.0, 2.0, 2.0, nl)
    assert bits_equal(a, g[f"{tag}_fmg2"])


def _field(shape, echoes, seed, dt=np.float64):
    from qsm_gb300 import synthetic
    rng = np.random.default_rng(seed)
    m = synthetic.ellipsoid_mask(shape, [0.33 * n for n in shape], centre=[n / 2 + 0.4 for n in shape])
    gi = np.indices(shape).astype(float)
    base = sum(np.sin(0.25 * (a + 1) * gi[a]) for a in range(3))
    f = np.stack([(base * (0.3 + 0.1 * t) + rng.normal(0, 0.01, shape)) * m for t in range(echoes)], axis=3)
    f = np.asfortranarray(f.astype(dt))
    return (np.asfortranarray(f[..., 0]) if echoes == 1 else f), m


def test_wrapper_gateways(gpu_ctx, mex, qsm):
    """The whole MATLAB functions: masks passed as double arrays, vsz as a scalar,
    defaults from omitted and empty arguments, 4-D fields."""
    f, m = _field((30, 28, 24), 2, 1)
    md = m.astype(np.float64)
    empty = np.zeros((0, 0))
    # sstgv: double runs the plain FP64 path, single the fused FP32 path
    x = mex("sstgv", f, md, 1.0, 1e-3, 2.0, 0.0, 20.0, 0.0)
    assert bits_equal(x, qsm.sstgv(f, m, [1, 1, 1], 1e-3, 2.0, 0.0, 20, fused=False))
    fs = f.astype(np.float32)
    x = mex("sstgv", fs, m.astype(bool), [1.0, 1.0, 1.0], 1e-3, 2.0, 0.0, 20.0, 0.0)
    assert x.dtype == np.float32 and bits_equal(x, qsm.sstgv(fs, m, [1, 1, 1], 1e-3, 2.0, 0.0, 20, fused=True))
    fl = mex("lbv", f, md, 1.0, 1e-8, empty, np.array([3.0, 2.0, 2.0, 2.0]))
    assert bits_equal(fl, qsm.lbv(f, m, [1, 1, 1], 1e-8, None, dict(maxit=3)))
    up, d2 = mex("unwrapLaplacian", f, md, 1.0, nlhs=2)
    rup, rd2 = qsm.unwrap_laplacian(f, m, [1, 1, 1])
    assert bits_equal(up, rup) and bits_equal(d2, rd2)
    fl, mo = mex("sharp", f, md, 1.0, 4.0, nlhs=2)
    rfl, rmo = qsm.sharp(f, m, [1, 1, 1], 4.0, 0.05)
    assert bits_equal(fl, rfl) and np.array_equal(mo, rmo)
    fl, mo = mex("vsharp", f, md, 1.0, np.array([5.0, 3.0]), nlhs=2)
    rfl, rmo = qsm.vsharp(f, m, [1, 1, 1], [5.0, 3.0], 0.05)
    assert bits_equal(fl, rfl) and np.array_equal(mo, rmo)
    fl, mo = mex("resharp", f, md, 1.0, 3.0, 1e-2, 1e-6, 30.0, nlhs=2)
    rfl, rmo = qsm.resharp(f, m, [1, 1, 1], 3.0, 1e-2, 1e-6, 30)
    assert bits_equal(fl, rfl) and np.array_equal(mo, rmo)
    fl, mo = mex("ismv", f, md, 1.0, empty, 1e-6, 50.0, nlhs=2)
    rfl, rmo = qsm.ismv(f, m, [1, 1, 1], 3.0, 1e-6, 50)
    assert bits_equal(fl, rfl) and np.array_equal(mo, rmo)
    w = m * 0.5 + 0.5
    fl = mex("pdf", fs, md, 1.0, w, np.array([0.0, 0.1, 1.0]), 0.0, 1e-5, 20.0)
    rfl = qsm.pdf(fs, m, [1, 1, 1], w.astype(np.float32), [0.0, 0.1, 1.0], 0.0, 1e-5, 20)
    assert fl.dtype == np.float32 and bits_equal(fl, rfl)


def test_gateway_errors(gpu_ctx, mex):
    f, m = _field((12, 12, 12), 1, 2)
    with pytest.raises(RuntimeError, match="Usage"):
        mex("pd_tgv_mex", f, m, [1.0, 1.0, 1.0])
    with pytest.raises(RuntimeError, match="Usage"):
        mex("sharp", f)
    with pytest.raises(RuntimeError, match="mgopts"):
        mex("lbv", f, m, 1.0, 1e-8, 10.0, np.array([1.0, 2.0]))
    with pytest.raises(RuntimeError):
        mex("sharp", f, np.zeros((12, 12, 12)), 1.0)  # empty mask: status message
