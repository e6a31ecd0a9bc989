"""numpy front end of the CPU oracle (``oracle/liborc.so``, built from
``oracle/qsm_oracle.c`` by ``make -C oracle``).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()``
and bench.py's CPU-baseline leg as the oracle the library is compared
against.  The product never imports it.

Function names and argument order follow the QSM.m MEX gateways they
restate (``pd_tgv_mex(d2f, mask, vsz, lam, alpha, tol, maxiter, verbose)``
and so on).  Arrays use MATLAB's layout: volumes are numpy arrays of shape
``(nx, ny, nz)`` in Fortran order (x fastest); vector fields carry a trailing
component axis; masks are uint8 0/1.  The in-place operator gateways
(``gradf_mex(dx, dy, dz, u, h)`` ...) write into the arrays passed, like the
MEX files; the solver gateways return a new array.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_DIR = os.path.dirname(os.path.abspath(__file__))
# QSM_ORACLE_LIB: another build of the same sources (the sanitizer build of
# tests/test_oracle_sanitized.py)
LIB_PATH = os.environ.get("QSM_ORACLE_LIB") or os.path.join(_DIR, "liborc.so")
_lib = None

_P = ctypes.c_void_p
_SZ = ctypes.POINTER(ctypes.c_size_t)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} missing: run `make -C oracle`")
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.orc_lane_dot.restype = ctypes.c_double
        _lib.orc_lane_dot.argtypes = [_P, _P, ctypes.c_size_t, ctypes.c_int]
        _lib.orc_lane_nrm2.restype = ctypes.c_double
        _lib.orc_lane_nrm2.argtypes = [_P, ctypes.c_size_t, ctypes.c_int]
        for s in ("d", "f"):
            getattr(_lib, f"orc_norm2_{s}").restype = ctypes.c_double if s == "d" else ctypes.c_float
    return _lib


def _sfx(a: np.ndarray) -> str:
    if a.dtype == np.float64:
        return "d"
    if a.dtype == np.float32:
        return "f"
    raise TypeError(f"expected float32/float64, got {a.dtype}")


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def _chk(a: np.ndarray, dtype=None) -> np.ndarray:
    if not a.flags.f_contiguous:
        raise ValueError("arrays must be Fortran-ordered (x fastest)")
    if dtype is not None and a.dtype != dtype:
        raise TypeError(f"expected {dtype}, got {a.dtype}")
    return a


def _dims(a: np.ndarray):
    s = a.shape[:3] + (1,) * (3 - min(3, a.ndim))
    return (ctypes.c_size_t * 3)(*s)


def _h(vsz) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(vsz, dtype=np.float64).reshape(3))


def _mask(m) -> np.ndarray:
    return np.asfortranarray(np.asarray(m) != 0).astype(np.uint8, order="F")


# ---------------- finite-difference operators (in place) ----------------

def _grad(name, dx, dy, dz, u, h, G=None):
    s = _sfx(u)
    for a in (dx, dy, dz, u):
        _chk(a, u.dtype)
    hh = _h(h)
    f = getattr(lib(), f"orc_{name}_{s}")
    if G is None:
        f(_ptr(dx), _ptr(dy), _ptr(dz), _ptr(u), _ptr(hh), _dims(u))
    else:
        g = _mask(G)
        f(_ptr(dx), _ptr(dy), _ptr(dz), _ptr(u), _ptr(g), _ptr(hh), _dims(u))


def gradf_mex(dx, dy, dz, u, h): _grad("gradf", dx, dy, dz, u, h)
def gradb_mex(dx, dy, dz, u, h): _grad("gradb", dx, dy, dz, u, h)
def gradc_mex(dx, dy, dz, u, h): _grad("gradc", dx, dy, dz, u, h)
def gradfp_mex(dx, dy, dz, u, h): _grad("gradfp", dx, dy, dz, u, h)
def gradfm_mex(dx, dy, dz, u, G, h): _grad("gradfm", dx, dy, dz, u, h, G)
def gradbm_mex(dx, dy, dz, u, G, h): _grad("gradbm", dx, dy, dz, u, h, G)
def gradcm_mex(dx, dy, dz, u, G, h): _grad("gradcm", dx, dy, dz, u, h, G)


def _adj(name, du, x, y, z, h, G=None):
    s = _sfx(du)
    for a in (du, x, y, z):
        _chk(a, du.dtype)
    hh = _h(h)
    f = getattr(lib(), f"orc_{name}_{s}")
    if G is None:
        f(_ptr(du), _ptr(x), _ptr(y), _ptr(z), _ptr(hh), _dims(du))
    else:
        g = _mask(G)
        f(_ptr(du), _ptr(x), _ptr(y), _ptr(z), _ptr(g), _ptr(hh), _dims(du))


def gradf_adj_mex(du, x, y, z, h): _adj("gradf_adj", du, x, y, z, h)
def gradb_adj_mex(du, x, y, z, h): _adj("gradb_adj", du, x, y, z, h)
def gradfp_adj_mex(du, x, y, z, h): _adj("gradfp_adj", du, x, y, z, h)
def gradfm_adj_mex(du, x, y, z, G, h): _adj("gradfm_adj", du, x, y, z, h, G)
def gradbm_adj_mex(du, x, y, z, G, h): _adj("gradbm_adj", du, x, y, z, h, G)


def lap1_mex(d2u, u, G, h):
    s = _sfx(u)
    _chk(d2u, u.dtype); _chk(u)
    g = _mask(G)
    hh = _h(h)
    getattr(lib(), f"orc_lap1_{s}")(_ptr(d2u), _ptr(u), _ptr(g), _ptr(hh), _dims(u))


def lapw_mex(d2u, u, h):
    s = _sfx(u)
    _chk(d2u, u.dtype); _chk(u)
    hh = _h(h)
    getattr(lib(), f"orc_lapw_{s}")(_ptr(d2u), _ptr(u), _ptr(hh), _dims(u))


# ---------------- primal-dual solvers ----------------

def pd_tgv_mex(d2f, mask, vsz, lam, alpha, tol, maxiter, verbose=0, info=None):
    d2f = np.asfortranarray(d2f)
    s = _sfx(d2f)
    m = _mask(mask)
    chi = np.zeros(d2f.shape, dtype=d2f.dtype, order="F")
    it = ctypes.c_uint32(0)
    mon = (ctypes.c_double * 2)()
    fn = getattr(lib(), f"orc_pd_tgv_{s}")
    fn.restype = ctypes.c_int
    fn.argtypes = [_P, _P, _P, _P, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_uint32, _SZ,
                   ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_double)]
    hh = _h(vsz)
    rc = fn(_ptr(chi), _ptr(d2f), _ptr(m), _ptr(hh), lam, alpha, tol, int(maxiter), _dims(d2f), ctypes.byref(it), mon)
    if rc:
        raise MemoryError("orc_pd_tgv failed")
    if info is not None:
        info.update(iters=it.value, monitors=(mon[0], mon[1]))
    return chi


def pd_tv_mex(d2f, mask, vsz, lam, tol, maxiter, verbose=0, info=None):
    d2f = np.asfortranarray(d2f)
    s = _sfx(d2f)
    m = _mask(mask)
    chi = np.zeros(d2f.shape, dtype=d2f.dtype, order="F")
    it = ctypes.c_uint32(0)
    mon = (ctypes.c_double * 2)()
    fn = getattr(lib(), f"orc_pd_tv_{s}")
    fn.restype = ctypes.c_int
    fn.argtypes = [_P, _P, _P, _P, ctypes.c_double, ctypes.c_double, ctypes.c_uint32, _SZ,
                   ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_double)]
    hh = _h(vsz)
    rc = fn(_ptr(chi), _ptr(d2f), _ptr(m), _ptr(hh), lam, tol, int(maxiter), _dims(d2f), ctypes.byref(it), mon)
    if rc:
        raise MemoryError("orc_pd_tv failed")
    if info is not None:
        info.update(iters=it.value, monitors=(mon[0], mon[1]))
    return chi


# ---------------- multigrid pieces (in place) ----------------

def gauss_seidel_mex(v, f, G, h, iters, reverse):
    s = _sfx(v)
    g = _mask(G)
    fn = getattr(lib(), f"orc_gauss_seidel_{s}")
    fn.argtypes = [_P, _P, _P, _P, _SZ, ctypes.c_int32, ctypes.c_int]
    fn(_ptr(_chk(v)), _ptr(_chk(f, v.dtype)), _ptr(g), _ptr(_h(h)), _dims(v), int(iters), int(bool(reverse)))


def residual_mex(r, f, x, G, h):
    s = _sfx(r)
    g = _mask(G)
    getattr(lib(), f"orc_residual_{s}")(_ptr(_chk(r)), _ptr(_chk(f, r.dtype)), _ptr(_chk(x, r.dtype)), _ptr(g), _ptr(_h(h)), _dims(r))


def lapmg_mex(d2u, u, G, h):
    s = _sfx(u)
    g = _mask(G)
    getattr(lib(), f"orc_lapmg_{s}")(_ptr(_chk(d2u, u.dtype)), _ptr(_chk(u)), _ptr(g), _ptr(_h(h)), _dims(u))


def restrict_mex(x2, x, G2):
    s = _sfx(x)
    g = _mask(G2)
    getattr(lib(), f"orc_restrict_{s}")(_ptr(_chk(x2, x.dtype)), _ptr(_chk(x)), _ptr(g), _dims(x2), _dims(x))


def _pc(x, x2, G, add):
    s = _sfx(x)
    g = _mask(G)
    fn = getattr(lib(), f"orc_prolong_correct_{s}")
    fn.argtypes = [_P, _P, _P, _SZ, _SZ, ctypes.c_int]
    fn(_ptr(_chk(x)), _ptr(_chk(x2, x.dtype)), _ptr(g), _dims(x), _dims(x2), add)


def prolong_mex(x, x2, G): _pc(x, x2, G, 0)
def correct_mex(x, x2, G): _pc(x, x2, G, 1)


def coarsen_grid_mex(G2, G):
    assert G2.dtype == np.uint8 and G.dtype == np.uint8
    lib().orc_coarsen_grid(_ptr(_chk(G2)), _ptr(_chk(G)), _dims(G2), _dims(G))


def boundary_mask_mex(B, G):
    assert B.dtype == np.uint8 and G.dtype == np.uint8
    lib().orc_boundary_mask(_ptr(_chk(B)), _ptr(_chk(G)), _dims(G))


def boundary_mask_l1_mex(B, G, l1):
    assert B.dtype == np.uint8 and G.dtype == np.uint8
    fn = lib().orc_boundary_mask_l1
    fn.argtypes = [_P, _P, _SZ, ctypes.c_uint8]
    fn(_ptr(_chk(B)), _ptr(_chk(G)), _dims(G), int(l1) & 0xFF)


def norm2_mex(x, G):
    x = np.asfortranarray(x)
    g = _mask(G)
    s = _sfx(x)
    fn = getattr(lib(), f"orc_norm2_{s}")
    fn.argtypes = [_P, _P, ctypes.c_size_t]
    return fn(_ptr(x), _ptr(g), x.size)


def lane_dot(x, y):
    x = np.ascontiguousarray(x).ravel(order="K")
    y = np.ascontiguousarray(y).ravel(order="K")
    return lib().orc_lane_dot(_ptr(x), _ptr(y), x.size, int(x.dtype == np.float32))


def lane_nrm2(x):
    x = np.ascontiguousarray(x).ravel(order="K")
    return lib().orc_lane_nrm2(_ptr(x), x.size, int(x.dtype == np.float32))


# ---------------- solver drivers ----------------

def mgpcg_mex(v, f, mask, vsz, tolcg, maxitcg, tolmg, maxitmg, mu, npre, npost, nboundary, nlevels,
              verbose=0, info=None):
    f = np.asfortranarray(f)
    s = _sfx(f)
    v = np.asfortranarray(v, dtype=f.dtype)
    m = _mask(mask)
    out = np.zeros(f.shape, dtype=f.dtype, order="F")
    it = ctypes.c_int32(0)
    res = np.zeros(max(1, int(maxitcg)), dtype=np.float64)
    fn = getattr(lib(), f"orc_mgpcg_{s}")
    fn.restype = ctypes.c_int
    fn.argtypes = [_P, _P, _P, _P, _P, _SZ, ctypes.c_double, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
                   ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                   ctypes.POINTER(ctypes.c_int32), _P]
    rc = fn(_ptr(out), _ptr(v), _ptr(f), _ptr(m), _ptr(_h(vsz)), _dims(f), tolcg, int(maxitcg), tolmg, int(maxitmg),
            int(mu), int(npre), int(npost), int(nboundary), int(nlevels), ctypes.byref(it), _ptr(res))
    if rc == -2:
        raise ValueError("nlevels too large. Increase MAX_DEPTH.")
    if rc:
        raise MemoryError("orc_mgpcg failed")
    if info is not None:
        info.update(iters=it.value, resnorm=res[: it.value].copy())
    return out


def mg_mex(v, f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels):
    f = np.asfortranarray(f)
    s = _sfx(f)
    v = np.asfortranarray(v, dtype=f.dtype)
    m = _mask(mask)
    out = np.zeros(f.shape, dtype=f.dtype, order="F")
    fn = getattr(lib(), f"orc_mg_{s}")
    fn.restype = ctypes.c_int
    fn.argtypes = [_P, _P, _P, _P, _P, _SZ, ctypes.c_double] + [ctypes.c_int32] * 6
    rc = fn(_ptr(out), _ptr(v), _ptr(f), _ptr(m), _ptr(_h(vsz)), _dims(f), tol, int(maxit), int(mu), int(npre),
            int(npost), int(nboundary), int(nlevels))
    if rc == -2:
        raise ValueError("nlevels too large. Increase MAX_DEPTH.")
    if rc:
        raise MemoryError("orc_mg failed")
    return out


def fmg_mex(f, mask, vsz, tol, maxit, mu, npre, npost, nboundary, nlevels):
    f = np.asfortranarray(f)
    s = _sfx(f)
    m = _mask(mask)
    out = np.zeros(f.shape, dtype=f.dtype, order="F")
    fn = getattr(lib(), f"orc_fmg_{s}")
    fn.restype = ctypes.c_int
    fn.argtypes = [_P, _P, _P, _P, _SZ, ctypes.c_double] + [ctypes.c_int32] * 6
    rc = fn(_ptr(out), _ptr(f), _ptr(m), _ptr(_h(vsz)), _dims(f), tol, int(maxit), int(mu), int(npre),
            int(npost), int(nboundary), int(nlevels))
    if rc == -2:
        raise ValueError("nlevels too large. Increase MAX_DEPTH.")
    if rc:
        raise MemoryError("orc_fmg failed")
    return out
