"""Generates the golden fixtures in this directory by running QSM.m's own
C-MEX sources (built by ``make -C oracle/ref REF=<QSM.m checkout>`` into
oracle/_ref/) through oracle/refmex.py.

Each fixture stores the inputs and the reference's outputs, so tests need
neither the reference nor a particular numpy RNG/FFT build to replay them.

    python tests/golden/gen_golden.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import refmex  # noqa: E402

F = np.asfortranarray
H = np.array([1.0, 0.7, 1.3])
FD_SHAPES = [(7, 6, 5), (12, 9, 10), (2, 3, 4), (3, 3, 3), (5, 2, 6)]


def z(shape, dt):
    return np.zeros(shape, dtype=dt, order="F")


def ball(shape, r):
    g = np.indices(shape).astype(np.float64)
    c = [(s - 1) / 2 for s in shape]
    return F((sum((g[i] - c[i]) ** 2 for i in range(3)) <= r * r).astype(np.uint8))


def gen_fd(rng):
    out = {}
    for si, shape in enumerate(FD_SHAPES):
        for dt in (np.float64, np.float32):
            tag = f"s{si}_{np.dtype(dt).name}"
            u = F(rng.standard_normal(shape).astype(dt))
            x, y, w = (F(rng.standard_normal(shape).astype(dt)) for _ in range(3))
            G = F((rng.random(shape) > 0.3).astype(np.uint8))
            uw = F((rng.standard_normal(shape) * 4).astype(dt))
            out[f"{tag}_u"], out[f"{tag}_x"], out[f"{tag}_y"], out[f"{tag}_z"] = u, x, y, w
            out[f"{tag}_G"], out[f"{tag}_uw"] = G, uw
            for nm in ("gradf", "gradb", "gradc", "gradfp"):
                r = [z(shape, dt) for _ in range(3)]
                refmex.call(nm + "_mex", *r, u, H, nlhs=0)
                out[f"{tag}_{nm}"] = np.stack(r, axis=-1)
            for nm in ("gradfm", "gradbm", "gradcm"):
                r = [z(shape, dt) for _ in range(3)]
                refmex.call(nm + "_mex", *r, u, G, H, nlhs=0)
                out[f"{tag}_{nm}"] = np.stack(r, axis=-1)
            for nm in ("gradf_adj", "gradb_adj", "gradfp_adj"):
                r = z(shape, dt)
                refmex.call(nm + "_mex", r, x, y, w, H, nlhs=0)
                out[f"{tag}_{nm}"] = r
            for nm in ("gradfm_adj", "gradbm_adj"):
                r = z(shape, dt)
                refmex.call(nm + "_mex", r, x, y, w, G, H, nlhs=0)
                out[f"{tag}_{nm}"] = r
            r = z(shape, dt)
            refmex.call("lap1_mex", r, u, G, H, nlhs=0)
            out[f"{tag}_lap1"] = r
            r = z(shape, dt)
            refmex.call("lapw_mex", r, uw, H, nlhs=0)
            out[f"{tag}_lapw"] = r
    out["h"] = H
    out["nshapes"] = np.array(len(FD_SHAPES))
    return out


def gen_pd(rng):
    out = {}
    cases = [((16, 14, 12), 5.0, 40, 0.0), ((9, 8, 7), 3.0, 25, 0.0), ((18, 16, 15), 6.5, 300, 2e-3)]
    for ci, (shape, r, iters, tol) in enumerate(cases):
        m = ball(shape, r)
        for dt in (np.float64, np.float32):
            tag = f"c{ci}_{np.dtype(dt).name}"
            d2f = F((rng.standard_normal(shape) * 0.05).astype(dt))
            h = np.array([1.0, 1.0, 1.0]) if ci != 1 else np.array([0.9, 1.0, 1.2])
            out[f"{tag}_d2f"], out[f"{tag}_mask"], out[f"{tag}_h"] = d2f, m, h
            out[f"{tag}_args"] = np.array([0.003, 2.0, tol, iters], dtype=np.float64)
            out[f"{tag}_tgv"] = refmex.call("pd_tgv_mex", d2f, m, h, 0.003, 2.0, tol, float(iters), 0.0)
            out[f"{tag}_tv"] = refmex.call("pd_tv_mex", d2f, m, h, 0.003, tol, float(iters), 0.0)
    return out


def gen_config0():
    import qsm_gb300.synthetic as S  # noqa: E402

    d2f, mask, _ = S.config0(seed=0)
    chi = refmex.call("pd_tgv_mex", d2f, mask, np.array([1.0, 1.0, 1.0]), 0.003, 2.0, 0.0, 1000.0, 0.0)
    return {
        "d2f": d2f, "mask": mask, "chi_sha256": np.frombuffer(hashlib.sha256(F(chi).tobytes(order="F")).digest(), dtype=np.uint8),
        "chi_samples": chi[::7, ::5, ::3].copy(order="F"), "args": np.array([0.003, 2.0, 0.0, 1000.0]),
    }


def gen_mg(rng):
    out = {}
    for si, shape in enumerate([(12, 11, 10), (9, 8, 7), (6, 5, 7)]):
        sz2 = tuple(((s - 2 + 1) >> 1) + 2 for s in shape)
        for dt in (np.float64, np.float32):
            tag = f"s{si}_{np.dtype(dt).name}"
            v = F(rng.standard_normal(shape).astype(dt))
            f = F(rng.standard_normal(shape).astype(dt))
            x = F(rng.standard_normal(shape).astype(dt))
            G = F((rng.random(shape) > 0.25).astype(np.uint8))
            G2 = F((rng.random(sz2) > 0.25).astype(np.uint8))
            c2 = F(rng.standard_normal(sz2).astype(dt))
            for k, a in dict(v=v, f=f, x=x, G=G, G2=G2, c2=c2).items():
                out[f"{tag}_{k}"] = a
            for rev in (0, 1):
                vv = v.copy(order="F")
                refmex.call("gauss_seidel_mex", vv, f, G, H, 3.0, float(rev), nlhs=0)
                out[f"{tag}_gs{rev}"] = vv
            r = z(shape, dt)
            refmex.call("residual_mex", r, f, x, G, H, nlhs=0)
            out[f"{tag}_residual"] = r
            r = z(shape, dt)
            refmex.call("lapmg_mex", r, x, G, H, nlhs=0)
            out[f"{tag}_lapmg"] = r
            r2 = z(sz2, dt)
            refmex.call("restrict_mex", r2, x, G2, nlhs=0)
            out[f"{tag}_restrict"] = r2
            r = v.copy(order="F")
            refmex.call("prolong_mex", r, c2, G, nlhs=0)
            out[f"{tag}_prolong"] = r
            r = v.copy(order="F")
            refmex.call("correct_mex", r, c2, G, nlhs=0)
            out[f"{tag}_correct"] = r
        Gb = F((rng.random(shape) > 0.15).astype(np.uint8))
        out[f"s{si}_Gb"] = Gb
        g2 = np.zeros(sz2, np.uint8, order="F")
        refmex.call("coarsen_grid_mex", g2, Gb, nlhs=0)
        out[f"s{si}_coarsen"] = g2
        B = np.zeros(shape, np.uint8, order="F")
        refmex.call("boundary_mask_mex", B, Gb, nlhs=0)
        out[f"s{si}_bmask"] = B
        for l1 in (1, 2, 3):
            B = np.zeros(shape, np.uint8, order="F")
            refmex.call("boundary_mask_l1_mex", B, Gb, float(l1), nlhs=0)
            out[f"s{si}_bmask_l1_{l1}"] = B
        xn = F(rng.standard_normal(shape))
        out[f"s{si}_xn"] = xn
        out[f"s{si}_norm2"] = np.asarray(refmex.call("norm2_mex", xn, Gb)).reshape(())
    out["h"] = H
    return out


def gen_solvers(rng):
    out = {}
    cases = [((20, 18, 16), (1, 2, 3)), ((34, 30, 28), (3,))]
    for ci, (shape, levels) in enumerate(cases):
        m = ball(shape, min(shape) / 2 - 2)
        u = F(rng.standard_normal(shape))
        f = z(shape, np.float64)
        refmex.call("lapmg_mex", f, u, m, np.array([1.0, 1.0, 1.0]), nlhs=0)
        f = F(-f)
        for dt in (np.float64, np.float32):
            tag = f"c{ci}_{np.dtype(dt).name}"
            fd = F(f.astype(dt))
            v0 = z(shape, dt)
            out[f"{tag}_f"], out[f"{tag}_mask"] = fd, m
            for nl in levels:
                out[f"{tag}_mgpcg{nl}"] = refmex.call("mgpcg_mex", v0, fd, m.astype(bool), np.array([1.0, 1, 1]), 1e-8,
                                                     40.0, -1.0, 1.0, 1.0, 1.0, 1.0, 2.0, float(nl), 0.0)
                out[f"{tag}_mgpcg_mg{nl}"] = refmex.call("mgpcg_mex", v0, fd, m.astype(bool), np.array([1.0, 1, 1]),
                                                        1e-8, 40.0, 1e-3, 3.0, 1.0, 2.0, 2.0, 2.0, float(nl), 0.0)
                out[f"{tag}_mg{nl}"] = refmex.call("mg_mex", v0, fd, m.astype(bool), np.array([1.0, 1, 1]), 1e-6, 4.0,
                                                  1.0, 2.0, 2.0, 2.0, float(nl))
                out[f"{tag}_fmg{nl}"] = refmex.call("fmg_mex", fd, m.astype(bool), np.array([1.0, 1, 1]), -1.0, 2.0,
                                                   1.0, 2.0, 2.0, 2.0, float(nl))
    return out


def main():
    rng = np.random.default_rng(20261203)
    np.savez_compressed(os.path.join(HERE, "fd_ops.npz"), **gen_fd(rng))
    np.savez_compressed(os.path.join(HERE, "pd.npz"), **gen_pd(rng))
    np.savez_compressed(os.path.join(HERE, "mg_ops.npz"), **gen_mg(rng))
    np.savez_compressed(os.path.join(HERE, "solvers.npz"), **gen_solvers(rng))
    np.savez_compressed(os.path.join(HERE, "config0_tgv.npz"), **gen_config0())
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
