"""GB300-native QSM hot path: Python mirror of QSM.m's C-MEX gateways.

Each function has the name, argument order and meaning of the MEX gateway it
replaces (``pd_tgv_mex(d2f, mask, vsz, lam, alpha, tol, maxiter, verbose)``,
``gradf_mex(dx, dy, dz, u, h)`` ...) and forwards to the CUDA library
``libqsm_gb300.so`` through its C ABI (include/qsm_gpu.h).  There is no CPU
fallback: if the library cannot be loaded, every call raises.

Arrays follow MATLAB's layout (x fastest, l = i + nx*j + nx*ny*k):

* numpy arrays of shape ``(nx, ny, nz)`` in Fortran order live in host
  memory; the library copies them to the GPU and results back inside the
  call;
* torch CUDA tensors are used in place on the device; a tensor whose strides
  are Fortran-ordered has dims = shape, a C-contiguous tensor of shape
  ``(nz, ny, nx)`` has dims = reversed shape.

Masks are uint8/bool 0/1.  In-place gateways write into their first
argument(s) where the MEX file writes; solvers return a new array of the
input's kind.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import MgInfo, PdInfo, QsmError, QsmLibraryError, TvInfo, context, lib
from . import nifti  # noqa: E402  (loadNii / saveNii)

__all__ = [
    "pd_tgv_mex", "pd_tv_mex", "gradf_mex", "gradb_mex", "gradc_mex", "gradfm_mex", "gradbm_mex", "gradcm_mex",
    "gradf_adj_mex", "gradb_adj_mex", "gradfm_adj_mex", "gradbm_adj_mex", "gradfp_mex", "gradfp_adj_mex",
    "lap1_mex", "lapw_mex", "gauss_seidel_mex", "residual_mex", "lapmg_mex", "restrict_mex", "prolong_mex",
    "correct_mex", "coarsen_grid_mex", "boundary_mask_mex", "boundary_mask_l1_mex", "norm2_mex", "mgpcg_mex",
    "mg_mex", "fmg_mex", "lane_dot", "fp_pipe_rate", "tv", "sstgv", "lbv", "unwrap_laplacian", "sharp", "vsharp", "ismv", "resharp", "pdf", "nifti",
    "pd_tv_batch", "pd_tgv_batch", "Session", "footprint", "QsmError",
    "QsmLibraryError", "context", "lib",
]

try:  # torch is optional (device-resident callers)
    import torch as _torch
except Exception:  # pragma: no cover
    _torch = None


def _is_torch(a) -> bool:
    return _torch is not None and isinstance(a, _torch.Tensor)


_NP_DT = {np.dtype(np.float64): _lib.QSM_F64, np.dtype(np.float32): _lib.QSM_F32}


class _Arr:
    """Pointer, MATLAB dims and dtype code of one argument."""

    def __init__(self, a, *, writable=False, mask=False, ref=None):
        self.obj = a
        if _is_torch(a):
            if not a.is_cuda:
                raise ValueError("torch tensors must be CUDA tensors (use numpy for host arrays)")
            if mask and a.dtype == _torch.bool:
                a = a.to(_torch.uint8)
                self.obj = a
            n = a.dim()
            shp = tuple(a.shape)
            if a.is_contiguous():
                self.dims = tuple(reversed(shp))[:3] if n >= 3 else tuple(reversed(shp)) + (1,) * (3 - n)
            else:
                st = a.stride()
                exp, acc = [], 1
                for s in shp:
                    exp.append(acc)
                    acc *= s
                if list(st) != exp:
                    raise ValueError("tensor must be contiguous in C or Fortran order")
                self.dims = shp[:3] + (1,) * (3 - min(3, n))
            self.ptr = ctypes.c_void_p(a.data_ptr())
            self.numel = a.numel()
            if mask:
                if a.dtype != _torch.uint8:
                    raise TypeError("masks must be uint8 or bool")
                self.dt = None
            else:
                if a.dtype == _torch.float64:
                    self.dt = _lib.QSM_F64
                elif a.dtype == _torch.float32:
                    self.dt = _lib.QSM_F32
                else:
                    raise TypeError(f"unsupported dtype {a.dtype}")
        else:
            a = np.asarray(a)
            if mask:
                if a.dtype != np.uint8:
                    a = (a != 0).astype(np.uint8)
            elif a.dtype not in _NP_DT:
                raise TypeError(f"unsupported dtype {a.dtype}")
            if not a.flags.f_contiguous:
                if writable:
                    raise ValueError("in-place arguments must be Fortran-ordered numpy arrays")
                a = np.asfortranarray(a)
            if writable and not a.flags.writeable:
                raise ValueError("in-place argument is read-only")
            self.obj = a
            self.dims = tuple(a.shape[:3]) + (1,) * (3 - min(3, a.ndim))
            self.ptr = ctypes.c_void_p(a.ctypes.data)
            self.numel = a.size
            self.dt = None if mask else _NP_DT[a.dtype]

    def dims_c(self):
        return (ctypes.c_size_t * 3)(*self.dims)


def _h(vsz):
    h = np.ascontiguousarray(np.asarray(vsz, dtype=np.float64).reshape(-1))
    if h.size == 1:
        h = np.repeat(h, 3)
    if h.size != 3:
        raise ValueError("vsz must have 3 entries")
    return (ctypes.c_double * 3)(*h)


def _sync_torch(*arrs):
    if _torch is not None and any(_is_torch(a.obj) for a in arrs):
        _torch.cuda.current_stream().synchronize()


def _same(arrs):
    dt = arrs[0].dt
    for a in arrs[1:]:
        if a.dt is not None and a.dt != dt:
            raise TypeError("all floating-point arrays must share one dtype")
    return dt


def _zeros_like(a: _Arr):
    if _is_torch(a.obj):
        return _torch.zeros_like(a.obj)
    return np.zeros(a.obj.shape, dtype=a.obj.dtype, order="F")


def _ctx(ctx):
    return ctx if ctx is not None else context(0)


# ---------------------------------------------------------------------------
# primal-dual inversions (pd_tgv_mex.c, pd_tv_mex.c)
# ---------------------------------------------------------------------------

def pd_tgv_mex(d2f, mask, vsz, lam, alpha, tol, maxiter, verbose=0, *, fused=False, info=None, ctx=None, out=None):
    """chi = pd_tgv_mex(d2f, mask, vsz, lam, alpha, tol, maxiter, verbose).

    fused=False: plain path, bit-identical to the reference in d2f's dtype.
    fused=True: mixed-precision fused FP32 kernel, monitors folded in FP64 (chi
    equals the reference's FP32 result; FP64 input is rounded, output widened).
    out: optional preallocated result (same kind, shape and dtype as d2f).
    """
    f, m = _Arr(d2f), _Arr(mask, mask=True)
    out = _zeros_like(f) if out is None else out
    o = _Arr(out, writable=True)
    pi = PdInfo()
    _sync_torch(f, m, o)
    _ctx(ctx).call("qsm_pd_tgv_fused" if fused else "qsm_pd_tgv", f.dt, f.dims_c(), f.ptr, m.ptr, _h(vsz),
                   float(lam), float(alpha), float(tol), int(maxiter), int(verbose), o.ptr, ctypes.byref(pi))
    if info is not None:
        info.update(iters=pi.iters, monitors=(pi.monitor_chi, pi.monitor_eta), seconds=pi.seconds,
                    active_voxels=pi.active_voxels, tile=tuple(pi.tile))
    return out


def pd_tv_mex(d2f, mask, vsz, lam, tol, maxiter, verbose=0, *, fused=False, info=None, ctx=None, out=None):
    """chi = pd_tv_mex(d2f, mask, vsz, lam, tol, maxiter, verbose)."""
    f, m = _Arr(d2f), _Arr(mask, mask=True)
    out = _zeros_like(f) if out is None else out
    o = _Arr(out, writable=True)
    pi = PdInfo()
    _sync_torch(f, m, o)
    _ctx(ctx).call("qsm_pd_tv_fused" if fused else "qsm_pd_tv", f.dt, f.dims_c(), f.ptr, m.ptr, _h(vsz),
                   float(lam), float(tol), int(maxiter), int(verbose), o.ptr, ctypes.byref(pi))
    if info is not None:
        info.update(iters=pi.iters, monitors=(pi.monitor_chi, pi.monitor_eta), seconds=pi.seconds,
                    active_voxels=pi.active_voxels, tile=tuple(pi.tile))
    return out


# ---------------------------------------------------------------------------
# finite-difference operators (in place)
# ---------------------------------------------------------------------------

def _grad(name, dx, dy, dz, u, h, G=None, ctx=None):
    a = [_Arr(dx, writable=True), _Arr(dy, writable=True), _Arr(dz, writable=True), _Arr(u)]
    dt = _same(a)
    args = [dt, a[3].dims_c(), a[0].ptr, a[1].ptr, a[2].ptr, a[3].ptr]
    g = None
    if G is not None:
        g = _Arr(G, mask=True)
        args.append(g.ptr)
    _sync_torch(*a)
    _ctx(ctx).call(name, *args, _h(h))


def gradf_mex(dx, dy, dz, u, h, *, ctx=None): _grad("qsm_gradf", dx, dy, dz, u, h, ctx=ctx)
def gradb_mex(dx, dy, dz, u, h, *, ctx=None): _grad("qsm_gradb", dx, dy, dz, u, h, ctx=ctx)
def gradc_mex(dx, dy, dz, u, h, *, ctx=None): _grad("qsm_gradc", dx, dy, dz, u, h, ctx=ctx)
def gradfp_mex(dx, dy, dz, u, h, *, ctx=None): _grad("qsm_gradfp", dx, dy, dz, u, h, ctx=ctx)
def gradfm_mex(dx, dy, dz, u, G, h, *, ctx=None): _grad("qsm_gradfm", dx, dy, dz, u, h, G, ctx=ctx)
def gradbm_mex(dx, dy, dz, u, G, h, *, ctx=None): _grad("qsm_gradbm", dx, dy, dz, u, h, G, ctx=ctx)
def gradcm_mex(dx, dy, dz, u, G, h, *, ctx=None): _grad("qsm_gradcm", dx, dy, dz, u, h, G, ctx=ctx)


def _adj(name, du, x, y, z, h, G=None, ctx=None):
    a = [_Arr(du, writable=True), _Arr(x), _Arr(y), _Arr(z)]
    dt = _same(a)
    args = [dt, a[0].dims_c(), a[0].ptr, a[1].ptr, a[2].ptr, a[3].ptr]
    if G is not None:
        args.append(_Arr(G, mask=True).ptr)
    _sync_torch(*a)
    _ctx(ctx).call(name, *args, _h(h))


def gradf_adj_mex(du, x, y, z, h, *, ctx=None): _adj("qsm_gradf_adj", du, x, y, z, h, ctx=ctx)
def gradb_adj_mex(du, x, y, z, h, *, ctx=None): _adj("qsm_gradb_adj", du, x, y, z, h, ctx=ctx)
def gradfp_adj_mex(du, x, y, z, h, *, ctx=None): _adj("qsm_gradfp_adj", du, x, y, z, h, ctx=ctx)
def gradfm_adj_mex(du, x, y, z, G, h, *, ctx=None): _adj("qsm_gradfm_adj", du, x, y, z, h, G, ctx=ctx)
def gradbm_adj_mex(du, x, y, z, G, h, *, ctx=None): _adj("qsm_gradbm_adj", du, x, y, z, h, G, ctx=ctx)


def lap1_mex(d2u, u, G, h, *, ctx=None):
    o, a, g = _Arr(d2u, writable=True), _Arr(u), _Arr(G, mask=True)
    _sync_torch(o, a)
    _ctx(ctx).call("qsm_lap1", _same([o, a]), a.dims_c(), o.ptr, a.ptr, g.ptr, _h(h))


def lapw_mex(d2u, u, h, *, ctx=None):
    o, a = _Arr(d2u, writable=True), _Arr(u)
    _sync_torch(o, a)
    _ctx(ctx).call("qsm_lapw", _same([o, a]), a.dims_c(), o.ptr, a.ptr, _h(h))


# ---------------------------------------------------------------------------
# multigrid pieces (in place)
# ---------------------------------------------------------------------------

def gauss_seidel_mex(v, f, G, h, iters, reverse, *, ctx=None):
    a, b, g = _Arr(v, writable=True), _Arr(f), _Arr(G, mask=True)
    _sync_torch(a, b)
    _ctx(ctx).call("qsm_gauss_seidel", _same([a, b]), a.dims_c(), a.ptr, b.ptr, g.ptr, _h(h), int(iters), int(reverse))


def residual_mex(r, f, x, G, h, *, ctx=None):
    a, b, c, g = _Arr(r, writable=True), _Arr(f), _Arr(x), _Arr(G, mask=True)
    _sync_torch(a, b, c)
    _ctx(ctx).call("qsm_residual", _same([a, b, c]), a.dims_c(), a.ptr, b.ptr, c.ptr, g.ptr, _h(h))


def lapmg_mex(d2u, u, G, h, *, ctx=None):
    a, b, g = _Arr(d2u, writable=True), _Arr(u), _Arr(G, mask=True)
    _sync_torch(a, b)
    _ctx(ctx).call("qsm_lapmg", _same([a, b]), a.dims_c(), a.ptr, b.ptr, g.ptr, _h(h))


def restrict_mex(x2, x, G2, *, ctx=None):
    a, b, g = _Arr(x2, writable=True), _Arr(x), _Arr(G2, mask=True)
    _sync_torch(a, b)
    _ctx(ctx).call("qsm_restrict", _same([a, b]), a.dims_c(), a.ptr, b.dims_c(), b.ptr, g.ptr)


def prolong_mex(x, x2, G, *, ctx=None):
    a, b, g = _Arr(x, writable=True), _Arr(x2), _Arr(G, mask=True)
    _sync_torch(a, b)
    _ctx(ctx).call("qsm_prolong", _same([a, b]), a.dims_c(), a.ptr, b.dims_c(), b.ptr, g.ptr)


def correct_mex(x, x2, G, *, ctx=None):
    a, b, g = _Arr(x, writable=True), _Arr(x2), _Arr(G, mask=True)
    _sync_torch(a, b)
    _ctx(ctx).call("qsm_correct", _same([a, b]), a.dims_c(), a.ptr, b.dims_c(), b.ptr, g.ptr)


def coarsen_grid_mex(G2, G, *, ctx=None):
    a, b = _Arr(G2, writable=True, mask=True), _Arr(G, mask=True)
    _ctx(ctx).call("qsm_coarsen_grid", a.dims_c(), a.ptr, b.dims_c(), b.ptr)
    _writeback_mask(G2, a)


def boundary_mask_mex(B, G, *, ctx=None):
    a, b = _Arr(B, writable=True, mask=True), _Arr(G, mask=True)
    _ctx(ctx).call("qsm_boundary_mask", b.dims_c(), a.ptr, b.ptr)
    _writeback_mask(B, a)


def boundary_mask_l1_mex(B, G, l1, *, ctx=None):
    a, b = _Arr(B, writable=True, mask=True), _Arr(G, mask=True)
    _ctx(ctx).call("qsm_boundary_mask_l1", b.dims_c(), a.ptr, b.ptr, int(l1) & 0xFF)
    _writeback_mask(B, a)


def _writeback_mask(orig, a: _Arr):
    # bool outputs were converted to a uint8 copy; copy the result back
    if a.obj is not orig:
        if _is_torch(orig):
            orig.copy_(a.obj.to(orig.dtype))
        else:
            orig[...] = a.obj.astype(orig.dtype)


def norm2_mex(x, G, *, ctx=None):
    a, g = _Arr(x), _Arr(G, mask=True)
    out = ctypes.c_double(0.0)
    _sync_torch(a)
    _ctx(ctx).call("qsm_norm2", a.dt, a.numel, a.ptr, g.ptr, ctypes.byref(out))
    return out.value


def lane_dot(x, y, *, ctx=None):
    """x . y in the library's lane order (the BLAS-1 dot of the PCG)."""
    a, b = _Arr(x), _Arr(y)
    out = ctypes.c_double(0.0)
    _sync_torch(a, b)
    _ctx(ctx).call("qsm_dot", _same([a, b]), a.numel, a.ptr, b.ptr, ctypes.byref(out))
    return out.value


def fp_pipe_rate(dtype="float64", *, ctx=None) -> float:
    """Measured multiply/add throughput (operations per second) of the device
    in dtype: the roofline of the bit-exact FP64 solvers."""
    out = ctypes.c_double(0.0)
    dt = _lib.QSM_F64 if np.dtype(dtype) == np.float64 else _lib.QSM_F32
    _ctx(ctx).call("qsm_fp_pipe_rate", dt, ctypes.byref(out))
    return out.value


def fp_convert_check(*, ctx=None) -> int:
    """Inputs on which the library's integer FP32 <-> FP64 conversions differ
    from the device's (all floats, 2^30 chosen doubles): 0 on a correct build."""
    out = ctypes.c_ulonglong(0)
    _ctx(ctx).call("qsm_fp_convert_check", ctypes.byref(out))
    return out.value


# ---------------------------------------------------------------------------
# Poisson solvers
# ---------------------------------------------------------------------------

def mgpcg_mex(v, f, mask, vsz, tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nboundary, nlevels, verbose=0,
              *, mixed=False, info=None, ctx=None):
    """v = mgpcg_mex(v, f, mask, vsz, tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nboundary, nlevels, verbose).

    mixed=True runs the FP64 PCG recurrence with an FP32 V-cycle (FP64 arrays only).
    """
    fa, m = _Arr(f), _Arr(mask, mask=True)
    va = _Arr(v) if v is not None else None
    out = _zeros_like(fa)
    o = _Arr(out, writable=True)
    hist = np.zeros(max(1, int(maxitcg)), dtype=np.float64)
    mi = MgInfo()
    mi.resnorm_hist = hist.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    _sync_torch(fa, m, o)
    vp = va.ptr if va is not None else None
    if mixed:
        if fa.dt != _lib.QSM_F64:
            raise TypeError("the mixed-precision solver takes FP64 arrays")
        _ctx(ctx).call("qsm_mgpcg_mixed", fa.dims_c(), vp, fa.ptr, m.ptr, _h(vsz), float(tolcg), int(maxitcg),
                       float(tolmg), int(maxitmg), int(mu), int(npre), int(npost), int(nboundary), int(nlevels),
                       int(verbose), o.ptr, ctypes.byref(mi))
    else:
        _ctx(ctx).call("qsm_mgpcg", fa.dt, fa.dims_c(), vp, fa.ptr, m.ptr, _h(vsz), float(tolcg), int(maxitcg),
                       float(tolmg), int(maxitmg), int(mu), int(npre), int(npost), int(nboundary), int(nlevels),
                       int(verbose), o.ptr, ctypes.byref(mi))
    if info is not None:
        info.update(iters=mi.iters, resnorm=mi.resnorm, seconds=mi.seconds, resnorm_hist=hist[: mi.iters].copy(),
                    coarse_ctas=mi.coarse_ctas, coarse_outer=mi.coarse_outer)
    return out


def mg_mex(v, f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels, *, info=None, ctx=None):
    """v = mg_mex(v, f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels)."""
    fa, m = _Arr(f), _Arr(mask, mask=True)
    va = _Arr(v) if v is not None else None
    out = _zeros_like(fa)
    o = _Arr(out, writable=True)
    mi = MgInfo()
    _sync_torch(fa, m, o)
    _ctx(ctx).call("qsm_mg", fa.dt, fa.dims_c(), va.ptr if va is not None else None, fa.ptr, m.ptr, _h(vsz),
                   float(tol), int(maxit), int(mu), int(npre), int(npost), int(nboundary), int(nlevels), o.ptr,
                   ctypes.byref(mi))
    if info is not None:
        info.update(cycles=mi.iters, seconds=mi.seconds, coarse_ctas=mi.coarse_ctas, coarse_outer=mi.coarse_outer)
    return out


def fmg_mex(f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels, *, info=None, ctx=None):
    """v = fmg_mex(f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels)."""
    fa, m = _Arr(f), _Arr(mask, mask=True)
    out = _zeros_like(fa)
    o = _Arr(out, writable=True)
    mi = MgInfo()
    _sync_torch(fa, m, o)
    _ctx(ctx).call("qsm_fmg", fa.dt, fa.dims_c(), fa.ptr, m.ptr, _h(vsz), float(tol), int(maxit), int(mu),
                   int(npre), int(npost), int(nboundary), int(nlevels), o.ptr, ctypes.byref(mi))
    if info is not None:
        info.update(cycles=mi.iters, seconds=mi.seconds, coarse_ctas=mi.coarse_ctas, coarse_outer=mi.coarse_outer)
    return out


# ---------------------------------------------------------------------------
# FFT total-variation inversion (src/inversion/tv.m)
# ---------------------------------------------------------------------------

TV_DEFAULTS = dict(mu=7.5e3, tv=1, rtol=1e-1, atol=1e-4, maxit=20, verbose=0, rho=9.0, alpha=1.5, rtau=0.7,
                   stau=1e2, gamma=3.0)  # tv.m:38-82


def tv(f, mask, vsz, bdir=(0.0, 0.0, 1.0), opts=None, *, info=None, ctx=None):
    """x = tv(f, mask, vsz, bdir, opts): ADMM total-variation dipole inversion
    with the k-space data term (tv.m).  f is 3-D, or 4-D with echoes along the
    last axis (each echo solved in turn, tv.m:87-95).  Computes in f's dtype."""
    o = dict(TV_DEFAULTS)
    if opts:
        o.update({k: v for k, v in dict(opts).items() if v is not None})
    b = np.asarray(bdir, dtype=np.float64).reshape(3)
    bd = (ctypes.c_double * 3)(*b)
    if not _is_torch(f) and np.ndim(f) == 4:
        f4 = np.asarray(f)
        out = np.zeros(f4.shape, dtype=f4.dtype, order="F")
        infos = []
        for t in range(f4.shape[3]):
            it = {}
            out[..., t] = tv(np.asfortranarray(f4[..., t]), mask, vsz, bdir, o, info=it, ctx=ctx)
            infos.append(it)
        if info is not None:
            info.update(echoes=infos)
        return out
    fa, m = _Arr(f), _Arr(mask, mask=True)
    out = _zeros_like(fa)
    oa = _Arr(out, writable=True)
    ti = TvInfo()
    _sync_torch(fa, m, oa)
    _ctx(ctx).call("qsm_tv_admm", fa.dt, fa.dims_c(), fa.ptr, m.ptr, _h(vsz), bd, float(o["mu"]), int(o["tv"]),
                   float(o["rtol"]), float(o["atol"]), int(o["maxit"]), float(o["rho"]), float(o["alpha"]),
                   float(o["rtau"]), float(o["stau"]), float(o["gamma"]), int(o["verbose"]), oa.ptr, ctypes.byref(ti))
    if info is not None:
        info.update(iters=ti.iters, rho=ti.rho, nr=ti.nr, eps_pri=ti.eps_pri, ns=ti.ns, eps_dual=ti.eps_dual,
                    seconds=ti.seconds)
    return out


# ---------------------------------------------------------------------------
# MATLAB-level pipelines: crop to the mask, echo loop, solve (sstgv.m, lbv.m,
# unwrapLaplacian.m)
# ---------------------------------------------------------------------------

def _dims4(a: _Arr):
    n3 = a.dims[0] * a.dims[1] * a.dims[2]
    ne = a.numel // n3 if n3 else 0
    return (ctypes.c_size_t * 4)(a.dims[0], a.dims[1], a.dims[2], ne), ne


def sstgv(phas, mask, vsz, lambda_=1e-4, alpha=3.0, tol=3e-4, maxit=5000, verbose=0, *, fused=True, infos=None,
          ctx=None):
    """x = sstgv(phas, mask, vsz, lambda, alpha, tol, maxit, verbose) (sstgv.m defaults).
    phas is 3-D or 4-D (echoes last).  fused=False runs the plain path (bit-exact with the
    reference MEX), fused=True the mixed-precision path with the echoes batched."""
    a, m = _Arr(phas), _Arr(mask, mask=True)
    out = _zeros_like(a)
    o = _Arr(out, writable=True)
    d4, ne = _dims4(a)
    pis = (PdInfo * max(ne, 1))()
    _sync_torch(a, m, o)
    _ctx(ctx).call("qsm_sstgv", a.dt, d4, a.ptr, m.ptr, _h(vsz), float(lambda_), float(alpha), float(tol), int(maxit),
                   int(verbose), 1 if fused else 0, o.ptr, pis)
    if infos is not None:
        infos[:] = [_pd_info_dict(pis[t]) for t in range(ne)]
    return out


def lbv(f, mask, vsz, tol=1e-8, maxit=None, mgopts=None, verbose=0, *, mixed=False, infos=None, ctx=None):
    """fl = lbv(f, mask, vsz, tol, maxit, mgopts, verbose) (lbv.m defaults: maxit
    ceil(sqrt(numel(mask))), mgopts maxit 2, npre 2, npost 2, nboundary 2)."""
    o_ = dict(maxit=2, npre=2, npost=2, nboundary=2)
    if mgopts:
        o_.update({k: v for k, v in dict(mgopts).items() if v is not None})
    a, m = _Arr(f), _Arr(mask, mask=True)
    out = _zeros_like(a)
    o = _Arr(out, writable=True)
    d4, ne = _dims4(a)
    mis = (MgInfo * max(ne, 1))()
    _sync_torch(a, m, o)
    _ctx(ctx).call("qsm_lbv", a.dt, d4, a.ptr, m.ptr, _h(vsz), float(tol), int(maxit or 0), int(o_["maxit"]),
                   int(o_["npre"]), int(o_["npost"]), int(o_["nboundary"]), int(verbose), 1 if mixed else 0, o.ptr,
                   mis)
    if infos is not None:
        infos[:] = [dict(iters=mis[t].iters, resnorm=mis[t].resnorm, seconds=mis[t].seconds,
                         coarse_ctas=mis[t].coarse_ctas, coarse_outer=mis[t].coarse_outer) for t in range(ne)]
    return out


def unwrap_laplacian(phas, mask, vsz, *, mixed=False, ctx=None):
    """[uphas, d2phas] = unwrapLaplacian(phas, mask, vsz)."""
    a, m = _Arr(phas), _Arr(mask, mask=True)
    up, d2 = _zeros_like(a), _zeros_like(a)
    o1, o2 = _Arr(up, writable=True), _Arr(d2, writable=True)
    d4, _ = _dims4(a)
    _sync_torch(a, m, o1, o2)
    _ctx(ctx).call("qsm_unwrap_laplacian", a.dt, d4, a.ptr, m.ptr, _h(vsz), 1 if mixed else 0, o1.ptr, o2.ptr)
    return up, d2


# ---------------------------------------------------------------------------
# FFT background-field removal (sharp.m, vsharp.m, ismv.m)
# ---------------------------------------------------------------------------

def _mask_like(m: _Arr):
    if _is_torch(m.obj):
        return _torch.zeros_like(m.obj, dtype=_torch.uint8)
    return np.zeros(m.obj.shape, dtype=np.uint8, order="F")


def sharp(f, mask, vsz, r=9.0, thr=0.05, *, ctx=None):
    """[fl, mask] = sharp(f, mask, vsz, r, thr)."""
    a, m = _Arr(f), _Arr(mask, mask=True)
    fl, mo = _zeros_like(a), _mask_like(m)
    o, om = _Arr(fl, writable=True), _Arr(mo, writable=True, mask=True)
    d4, _ = _dims4(a)
    _sync_torch(a, m, o, om)
    _ctx(ctx).call("qsm_sharp", a.dt, d4, a.ptr, m.ptr, _h(vsz), float(r), float(thr), o.ptr, om.ptr)
    return fl, mo


def vsharp(f, mask, vsz, rs=None, thr=0.05, *, ctx=None):
    """[fl, mask] = vsharp(f, mask, vsz, rs, thr); rs None: 9 : -2*max(vsz) : 2*max(vsz)."""
    a, m = _Arr(f), _Arr(mask, mask=True)
    fl, mo = _zeros_like(a), _mask_like(m)
    o, om = _Arr(fl, writable=True), _Arr(mo, writable=True, mask=True)
    d4, _ = _dims4(a)
    r = np.ascontiguousarray(np.asarray(rs if rs is not None else [], dtype=np.float64).reshape(-1))
    _sync_torch(a, m, o, om)
    _ctx(ctx).call("qsm_vsharp", a.dt, d4, a.ptr, m.ptr, _h(vsz), r.ctypes.data if r.size else None, int(r.size),
                   float(thr), o.ptr, om.ptr)
    return fl, mo


def resharp(f, mask, vsz, r=3.0, lambda_=1e-2, tol=None, maxit=None, verbose=0, *, info=None, ctx=None):
    """[fl, mask] = resharp(f, mask, vsz, r, lambda, tol, maxit); the Tikhonov system is
    solved by CGS (x0 = 0); tol None: sqrt(eps(class(f))); maxit None: ceil(sqrt(numel(mask)))."""
    a, m = _Arr(f), _Arr(mask, mask=True)
    fl, mo = _zeros_like(a), _mask_like(m)
    o, om = _Arr(fl, writable=True), _Arr(mo, writable=True, mask=True)
    d4, ne = _dims4(a)
    its = (ctypes.c_int32 * max(ne, 1))()
    _sync_torch(a, m, o, om)
    _ctx(ctx).call("qsm_resharp", a.dt, d4, a.ptr, m.ptr, _h(vsz), float(r), float(lambda_),
                   -1.0 if tol is None else float(tol), int(maxit or 0), int(verbose), o.ptr, om.ptr, its)
    if info is not None:
        info.update(iters=[int(its[t]) for t in range(ne)])
    return fl, mo


def pdf(f, mask, vsz, w=None, bdir=(0.0, 0.0, 1.0), lambda_=0.0, tol=1e-5, maxit=None, verbose=0, *,
        info=None, ctx=None):
    """fl = pdf(f, mask, vsz, w, bdir, lambda, tol, maxit, verbose): projection onto dipole
    fields solved by LSMR on the full grid; w None (or all zero): the mask; maxit None:
    ceil(sqrt(numel(mask)))."""
    a, m = _Arr(f), _Arr(mask, mask=True)
    wa = None
    if w is not None:
        single = a.dt == _lib.QSM_F32
        if _is_torch(w):
            wa = _Arr(w.to(_torch.float32 if single else _torch.float64))
        else:
            wa = _Arr(np.asarray(w, dtype=np.float32 if single else np.float64))
        if wa.dims != m.dims:
            raise ValueError("w must have the mask's size")
    fl = _zeros_like(a)
    o = _Arr(fl, writable=True)
    d4, ne = _dims4(a)
    its = (ctypes.c_int32 * max(ne, 1))()
    _sync_torch(*(x for x in (a, m, wa, o) if x is not None))
    _ctx(ctx).call("qsm_pdf", a.dt, d4, a.ptr, m.ptr, None if wa is None else wa.ptr, _h(vsz), _h(bdir),
                   float(lambda_), -1.0 if tol is None else float(tol), int(maxit or 0), int(verbose), o.ptr, its)
    if info is not None:
        info.update(iters=[int(its[t]) for t in range(ne)])
    return fl


def ismv(f, mask, vsz, r=3.0, tol=None, maxit=500, verbose=0, *, info=None, ctx=None):
    """[fl, mask] = ismv(f, mask, vsz, r, tol, maxit, verbose); tol None: sqrt(eps(class(f)))."""
    a, m = _Arr(f), _Arr(mask, mask=True)
    fl, mo = _zeros_like(a), _mask_like(m)
    o, om = _Arr(fl, writable=True), _Arr(mo, writable=True, mask=True)
    d4, ne = _dims4(a)
    its = (ctypes.c_int32 * max(ne, 1))()
    _sync_torch(a, m, o, om)
    _ctx(ctx).call("qsm_ismv", a.dt, d4, a.ptr, m.ptr, _h(vsz), float(r), -1.0 if tol is None else float(tol),
                   int(maxit), int(verbose), o.ptr, om.ptr, its)
    if info is not None:
        info.update(iters=[int(its[t]) for t in range(ne)])
    return fl, mo


# ---------------------------------------------------------------------------
# many-volume batches and resident sessions (no reference counterpart: QSM.m
# loops over volumes in MATLAB, src/inversion/sstgv.m:68-71)
# ---------------------------------------------------------------------------

def _pd_info_dict(pi: PdInfo) -> dict:
    return dict(iters=pi.iters, monitors=(pi.monitor_chi, pi.monitor_eta), seconds=pi.seconds,
                active_voxels=pi.active_voxels, tile=tuple(pi.tile))


def _pd_batch(name, d2fs, masks, vsz, scalars, *, infos, ctx, outs):
    fs = [_Arr(a) for a in d2fs]
    ms = [_Arr(a, mask=True) for a in masks]
    if len(fs) != len(ms):
        raise ValueError("one mask per volume")
    dt = _same(fs) if fs else _lib.QSM_F32
    outs = [_zeros_like(f) for f in fs] if outs is None else list(outs)
    os_ = [_Arr(o, writable=True) for o in outs]
    n = len(fs)
    dims = (ctypes.c_size_t * (3 * max(n, 1)))(*[x for f in fs for x in f.dims])
    pf = (ctypes.c_void_p * max(n, 1))(*[f.ptr.value for f in fs])
    pm = (ctypes.c_void_p * max(n, 1))(*[m.ptr.value for m in ms])
    po = (ctypes.c_void_p * max(n, 1))(*[o.ptr.value for o in os_])
    pis = (PdInfo * max(n, 1))()
    _sync_torch(*(fs + ms + os_))
    _ctx(ctx).call(name, dt, n, dims, pf, pm, _h(vsz), *scalars[:-1], int(scalars[-1]), po, pis)
    if infos is not None:
        infos[:] = [_pd_info_dict(pis[b]) for b in range(n)]
    return outs


def pd_tv_batch(d2fs, masks, vsz, lam, tol, maxiter, *, infos=None, ctx=None, outs=None):
    """[chi_b] = pd_tv_mex(d2f_b, mask_b, vsz, lam, tol, maxiter) for every volume b, advanced together
    (fused FP32 path, one persistent launch per tile shape and iteration, CUDA-graph replays)."""
    return _pd_batch("qsm_pd_tv_batch", d2fs, masks, vsz, (float(lam), float(tol), maxiter), infos=infos, ctx=ctx,
                     outs=outs)


def pd_tgv_batch(d2fs, masks, vsz, lam, alpha, tol, maxiter, *, infos=None, ctx=None, outs=None):
    """[chi_b] = pd_tgv_mex(d2f_b, mask_b, vsz, lam, alpha, tol, maxiter) for every volume b, advanced together."""
    return _pd_batch("qsm_pd_tgv_batch", d2fs, masks, vsz, (float(lam), float(alpha), float(tol), maxiter),
                     infos=infos, ctx=ctx, outs=outs)


def mgpcg_batch(v0s, fs, masks, vsz, tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nboundary, nlevels, *,
                mixed=True, infos=None, ctx=None, outs=None):
    """[v_b] = mgpcg_mex(v0_b, f_b, mask_b, vsz, ...) for every volume b (FP64 arrays; v0s None or entries None
    for zeros), packed: solves with tolmg <= 0 advance together, each kernel of a PCG iteration launched once
    for up to 16 of them.  Each v_b equals the solve alone bit for bit; mixed selects the FP32 V-cycle."""
    fa = [_Arr(a) for a in fs]
    ms = [_Arr(a, mask=True) for a in masks]
    if len(fa) != len(ms):
        raise ValueError("one mask per volume")
    if any(a.dt != _lib.QSM_F64 for a in fa):
        raise TypeError("mgpcg_batch takes FP64 arrays")
    n = len(fa)
    v0a = [None if (v0s is None or v0s[b] is None) else _Arr(v0s[b]) for b in range(n)]
    outs = [_zeros_like(a) for a in fa] if outs is None else list(outs)
    oa = [_Arr(o, writable=True) for o in outs]
    dims = (ctypes.c_size_t * (3 * max(n, 1)))(*[x for a in fa for x in a.dims])
    p0 = (ctypes.c_void_p * max(n, 1))(*[(v.ptr.value if v is not None else None) for v in v0a])
    pf = (ctypes.c_void_p * max(n, 1))(*[a.ptr.value for a in fa])
    pm = (ctypes.c_void_p * max(n, 1))(*[m.ptr.value for m in ms])
    po = (ctypes.c_void_p * max(n, 1))(*[o.ptr.value for o in oa])
    mis = (MgInfo * max(n, 1))()
    hists = [np.zeros(max(1, int(maxitcg)), dtype=np.float64) for _ in range(n)]
    for b in range(n):
        mis[b].resnorm_hist = hists[b].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    _sync_torch(*(fa + ms + oa + [v for v in v0a if v is not None]))
    _ctx(ctx).call("qsm_mgpcg_batch", int(bool(mixed)), n, dims, p0, pf, pm, _h(vsz), float(tolcg), int(maxitcg),
                   float(tolmg), int(maxitmg), int(mu), int(npre), int(npost), int(nboundary), int(nlevels), po, mis)
    if infos is not None:
        infos[:] = [dict(iters=mis[b].iters, resnorm=mis[b].resnorm, seconds=mis[b].seconds,
                         resnorm_hist=hists[b][: mis[b].iters].copy(), coarse_ctas=mis[b].coarse_ctas,
                         coarse_outer=mis[b].coarse_outer) for b in range(n)]
    return outs


def footprint(kind: str, dims, nlevels: int = 5) -> int:
    """Device bytes a resident job holds: kind in {"tv", "tgv", "mgpcg", "mgpcg_f64"}."""
    k = {"tv": _lib.QSM_JOB_TV, "tgv": _lib.QSM_JOB_TGV, "mgpcg": _lib.QSM_JOB_MGPCG,
         "mgpcg_f64": _lib.QSM_JOB_MGPCG_F64}[kind]
    return int(lib().qsm_session_footprint(k, (ctypes.c_size_t * 3)(*dims), int(nlevels)))


class Session:
    """Resident solves on one GPU (qsm_session_* in include/qsm_gpu.h).

    Primal-dual solves advance together in :meth:`step`.  Poisson solves
    stay resident and advance in :meth:`step` too (``poisson_workers=0``, the
    default: packed launches, at least one PCG iteration per 30 primal-dual
    iterations, more while the step's replays run), or run whole on
    ``poisson_workers`` worker streams concurrently.  A submit that does
    not fit in ``budget_bytes`` raises :class:`QsmError` with status
    QSM_ERR_BUSY and leaves the session unchanged.
    """

    def __init__(self, budget_bytes: int = 0, poisson_workers: int = 0, *, ctx=None):
        self.ctx = _ctx(ctx)
        h = _lib.SES()
        self._check(lib().qsm_session_create(self.ctx.handle, int(budget_bytes), int(poisson_workers),
                                             ctypes.byref(h)), "qsm_session_create")
        self.handle = h
        self._meta = {}
        self.poisson_workers = int(poisson_workers)  # 0: Poisson solves advance in step()

    def _check(self, st, name):
        if st != 0:
            msg = lib().qsm_last_error(self.ctx.handle) or b""
            raise QsmError(st, f"{name}: {msg.decode(errors='replace')}")

    def submit_pd(self, d2f, mask, vsz, lam, alpha, tol, maxiter, *, tgv=True) -> int:
        f, m = _Arr(d2f), _Arr(mask, mask=True)
        _sync_torch(f, m)
        jid = ctypes.c_uint64()
        self._check(lib().qsm_session_submit_pd(self.handle, 1 if tgv else 0, f.dt, f.dims_c(), f.ptr, m.ptr,
                                                _h(vsz), float(lam), float(alpha), float(tol), int(maxiter),
                                                ctypes.byref(jid)), "qsm_session_submit_pd")
        self._meta[jid.value] = ("pd", f)
        return jid.value

    def submit_mgpcg(self, v, f, mask, vsz, tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nboundary, nlevels,
                     *, mixed=True) -> int:
        fa, m = _Arr(f), _Arr(mask, mask=True)
        if fa.dt != _lib.QSM_F64:
            raise TypeError("session Poisson solves take FP64 arrays")
        va = _Arr(v) if v is not None else None
        _sync_torch(fa, m)
        jid = ctypes.c_uint64()
        self._check(lib().qsm_session_submit_mgpcg(
            self.handle, fa.dims_c(), va.ptr if va is not None else None, fa.ptr, m.ptr, _h(vsz), float(tolcg),
            int(maxitcg), float(tolmg), int(maxitmg), int(mu), int(npre), int(npost), int(nboundary), int(nlevels),
            1 if mixed else 0, ctypes.byref(jid)), "qsm_session_submit_mgpcg")
        self._meta[jid.value] = ("mg", fa)
        return jid.value

    def step(self, iters: int = 30):
        self._check(lib().qsm_session_step(self.handle, int(iters)), "qsm_session_step")

    def poll(self, jid: int):
        """(finished, info dict)"""
        fin = ctypes.c_int32()
        pi, mi = PdInfo(), MgInfo()
        self._check(lib().qsm_session_poll(self.handle, int(jid), ctypes.byref(fin), ctypes.byref(pi),
                                           ctypes.byref(mi)), "qsm_session_poll")
        kind = self._meta[jid][0] if jid in self._meta else "pd"
        if kind == "pd":
            return bool(fin.value), _pd_info_dict(pi)
        return bool(fin.value), dict(iters=mi.iters, resnorm=mi.resnorm, seconds=mi.seconds)

    def fetch(self, jid: int, out=None):
        if jid not in self._meta:
            raise QsmError(1, f"qsm_session_fetch: unknown session job id {jid}")
        kind, a = self._meta[jid]
        out = _zeros_like(a) if out is None else out
        o = _Arr(out, writable=True)
        _sync_torch(o)
        self._check(lib().qsm_session_fetch(self.handle, int(jid), o.ptr), "qsm_session_fetch")
        del self._meta[jid]
        return out

    def running(self) -> int:
        return int(lib().qsm_session_running(self.handle))

    def bytes_in_use(self) -> int:
        return int(lib().qsm_session_bytes_in_use(self.handle))

    def close(self):
        if getattr(self, "handle", None):
            lib().qsm_session_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
