"""CPU restatement of QSM.m's MATLAB-level wrappers around the MEX gateways.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the oracle of the GPU
pipelines; the product never imports it.

Follows src/utils/cropIndices.m, src/inversion/sstgv.m:1-87,
src/bgremove/lbv.m:1-113, src/unwrap/unwrapLaplacian.m:1-87 and the option
defaults of src/utils/poisson_solver/mgpcg.m:1-40: numpy slicing for the crop
and the echo loop, and the oracle library's bit-exact restatements of
lapw_mex, lap1_mex, pd_tgv_mex, pd_tv_mex and mgpcg_mex for every numeric
step.  The wrappers themselves are MATLAB and cannot run here; the MEX steps
they call are pinned against the reference build.
"""
from __future__ import annotations

import math

import numpy as np

import port


def crop_indices(mask):
    """cropIndices(x): 0-based index ranges of the x-, y-, z-slices that hold
    mask voxels."""
    m = np.asarray(mask) != 0
    ix = np.flatnonzero(m.any(axis=(1, 2)))
    iy = np.flatnonzero(m.any(axis=(0, 2)))
    iz = np.flatnonzero(m.any(axis=(0, 1)))
    return ix, iy, iz


def crop_box(mask, pad):
    """The wrappers' box: first-pad .. last+pad per axis, clamped (sstgv.m:57-63)."""
    ix, iy, iz = crop_indices(mask)
    if ix.size == 0:
        raise ValueError("empty mask")
    n = mask.shape
    return tuple(slice(max(0, r[0] - pad), min(n[a] - 1, r[-1] + pad) + 1) for a, r in enumerate((ix, iy, iz)))


def _echoes(a):
    a = np.asarray(a)
    return [a] if a.ndim == 3 else [a[..., t] for t in range(a.shape[3])]


def _levels(shape):
    # mgpcg.m:33-35
    return max(1, int(math.floor(math.log2(min(shape)))) - 3)


def sstgv(phas, mask, vsz, lam=1e-4, alpha=3.0, tol=3e-4, maxit=5000):
    """sstgv.m:1-87: crop (margin 2), d2u = lapw(u), pd_tgv_mex(-d2u, ...)
    (pd_tv_mex when alpha <= eps), scatter into zeros."""
    b = crop_box(mask, 2)
    m = np.asfortranarray(np.asarray(mask)[b]).astype(np.uint8)
    out = np.zeros(np.shape(phas), dtype=np.asarray(phas).dtype, order="F")
    res = []
    for u in _echoes(phas):
        uc = np.asfortranarray(u[b])
        d2u = np.zeros_like(uc, order="F")
        port.lapw_mex(d2u, uc, vsz)
        if alpha > np.finfo(np.float64).eps:
            x = port.pd_tgv_mex(-d2u, m, vsz, lam, alpha, tol, maxit)
        else:
            x = port.pd_tv_mex(-d2u, m, vsz, lam, tol, maxit)
        res.append(x)
    if out.ndim == 3:
        out[b] = res[0]
    else:
        for t, x in enumerate(res):
            out[b + (t,)] = x
    return out


def _poisson(f_in, mask, vsz, unwrap, tol, maxit, mgopts):
    b = crop_box(mask, 1)
    m = np.asfortranarray(np.asarray(mask)[b]).astype(np.uint8)
    out = np.zeros(np.shape(f_in), dtype=np.asarray(f_in).dtype, order="F")
    d2out = np.zeros_like(out, order="F")
    nl = _levels(m.shape)
    mx = int(math.ceil(math.sqrt(m.size))) if unwrap else maxit
    for t, u in enumerate(_echoes(f_in)):
        uc = np.asfortranarray(u[b])
        d2u = np.zeros_like(uc, order="F")
        if unwrap:
            port.lapw_mex(d2u, uc, vsz)
            f = -(m.astype(uc.dtype) * d2u)
        else:
            port.lap1_mex(d2u, uc, m, vsz)
            f = -d2u
        v = port.mgpcg_mex(np.zeros_like(uc, order="F"), np.asfortranarray(f), m.astype(bool), vsz, tol, mx, -1.0,
                           mgopts["maxit"], 1, mgopts["npre"], mgopts["npost"], mgopts["nboundary"], nl)
        idx = b if out.ndim == 3 else b + (t,)
        out[idx] = v
        d2out[idx] = d2u
    return out, d2out


def lbv(f, mask, vsz, tol=1e-8, maxit=None, mgopts=None):
    """lbv.m:1-113: crop (margin 1), d2u = lap(u, m), mgpcg(-d2u, m, ...)."""
    o = dict(maxit=2, npre=2, npost=2, nboundary=2)
    o.update(mgopts or {})
    if not maxit:
        maxit = int(math.ceil(math.sqrt(np.asarray(mask).size)))
    return _poisson(f, mask, vsz, False, tol, maxit, o)[0]


def unwrap_laplacian(phas, mask, vsz):
    """unwrapLaplacian.m:1-87: crop (margin 1), d2u = lapw(u),
    mgpcg(-m.*d2u, m, h, 1e-8, ceil(sqrt(numel(m))), LBV options)."""
    return _poisson(phas, mask, vsz, True, 1e-8, 0, dict(maxit=2, npre=2, npost=2, nboundary=2))
