"""Run QSM.m's own C-MEX gateways (compiled by ``oracle/ref/Makefile`` into
``oracle/_ref/*.so``) from numpy, through the project-written mxArray runtime.

TEST INFRASTRUCTURE ONLY.  It pins the C restatement in ``oracle/qsm_oracle.c``,
generates the golden fixtures under ``tests/golden/`` and runs the library's own
MEX shims in the tests.  The product never imports it.

Arrays follow MATLAB's layout: a volume is a numpy array of shape
``(nx, ny, nz)`` in Fortran order (x fastest), vector fields have a trailing
component axis, masks are ``uint8``/``bool``.  Python scalars become 1x1
double arrays, as MATLAB passes them.  Every argument is copied into a fresh
mxArray; after the call, arguments that the gateway wrote in place (the
operator MEX files write into ``prhs[0]``) are copied back into the caller's
numpy arrays, so ``call('gradf_mex', dx, dy, dz, u, h)`` updates ``dx, dy, dz``
exactly as MATLAB's in-place MEX convention does.  Logical outputs come back
as uint8.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

REF_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref")

_CLASS = {
    np.dtype(np.float64): 6,   # mxDOUBLE_CLASS
    np.dtype(np.float32): 7,   # mxSINGLE_CLASS
    np.dtype(np.bool_): 3,     # mxLOGICAL_CLASS
    np.dtype(np.uint8): 9,     # mxUINT8_CLASS
    np.dtype(np.int32): 12,
    np.dtype(np.uint32): 13,
}
_DTYPE = {6: np.float64, 7: np.float32, 3: np.uint8, 9: np.uint8, 12: np.int32, 13: np.uint32}

_libs: dict[str, ctypes.CDLL] = {}


def available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "pd_tgv_mex.so"))


def _lib(name: str, path: str | None = None) -> ctypes.CDLL:
    key = path or name
    if key not in _libs:
        path = path or os.path.join(REF_DIR, name + ".so")
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} missing: run `make -C oracle/ref`")
        lib = ctypes.CDLL(path, mode=os.RTLD_LOCAL | os.RTLD_NOW)
        lib.mxCreateNumericArray.restype = ctypes.c_void_p
        lib.mxCreateNumericArray.argtypes = [ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t), ctypes.c_int, ctypes.c_int]
        lib.mxGetData.restype = ctypes.c_void_p
        lib.mxGetData.argtypes = [ctypes.c_void_p]
        lib.mxGetNumberOfElements.restype = ctypes.c_size_t
        lib.mxGetNumberOfElements.argtypes = [ctypes.c_void_p]
        lib.mxGetNumberOfDimensions.restype = ctypes.c_size_t
        lib.mxGetNumberOfDimensions.argtypes = [ctypes.c_void_p]
        lib.mxGetDimensions.restype = ctypes.POINTER(ctypes.c_size_t)
        lib.mxGetDimensions.argtypes = [ctypes.c_void_p]
        lib.mxGetClassID.restype = ctypes.c_int
        lib.mxGetClassID.argtypes = [ctypes.c_void_p]
        lib.mxDestroyArray.argtypes = [ctypes.c_void_p]
        lib.shim_call.restype = ctypes.c_int
        lib.shim_call.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        lib.shim_last_error.restype = ctypes.c_char_p
        _libs[key] = lib
    return _libs[key]


def _to_mx(lib, a):
    if not isinstance(a, np.ndarray):
        a = np.asarray(a, dtype=np.float64)
    if a.dtype not in _CLASS:
        raise TypeError(f"unsupported dtype {a.dtype}")
    shape = a.shape if a.ndim >= 2 else ((1, 1) if a.ndim == 0 else (1, a.shape[0]))
    dims = (ctypes.c_size_t * len(shape))(*shape)
    mx = lib.mxCreateNumericArray(len(shape), dims, _CLASS[a.dtype], 0)
    flat = np.asarray(a, dtype=np.uint8 if a.dtype == np.bool_ else a.dtype).ravel(order="F")
    if flat.size:
        ctypes.memmove(lib.mxGetData(mx), flat.ctypes.data, flat.nbytes)
    return mx


def _from_mx(lib, mx):
    cls = lib.mxGetClassID(mx)
    nd = lib.mxGetNumberOfDimensions(mx)
    dp = lib.mxGetDimensions(mx)
    shape = tuple(dp[i] for i in range(nd))
    n = lib.mxGetNumberOfElements(mx)
    dt = np.dtype(_DTYPE[cls])
    buf = (ctypes.c_char * (n * dt.itemsize)).from_address(lib.mxGetData(mx))
    out = np.frombuffer(bytes(buf), dtype=dt).reshape(shape, order="F")
    return out.copy(order="F")


def call(name: str, *args, nlhs: int = 1, verbose: bool = False, path: str | None = None):
    """Call gateway ``name`` (e.g. ``'pd_tgv_mex'``) with MATLAB-style args.

    Returns the first output (or a tuple when ``nlhs > 1``, or None when
    ``nlhs == 0``).  Raises RuntimeError with the gateway's mexErrMsgTxt text.
    ``path`` names another gateway library linked with the same runtime (the
    tests run the library's own MEX shims this way).
    """
    lib = _lib(name, path)
    mxs = [_to_mx(lib, a) for a in args]
    prhs = (ctypes.c_void_p * max(1, len(mxs)))(*mxs)
    plhs = (ctypes.c_void_p * max(1, nlhs))()
    rc = lib.shim_call(nlhs, plhs, len(mxs), prhs, 1 if verbose else 0)
    if rc != 0:
        msg = lib.shim_last_error().decode()
        for m in mxs:
            lib.mxDestroyArray(m)
        raise RuntimeError(f"{name}: {msg}")
    # in-place writes: copy back into numpy arguments
    for a, m in zip(args, mxs):
        if isinstance(a, np.ndarray) and a.flags.writeable and a.size:
            back = _from_mx(lib, m).reshape(a.shape, order="F")
            a[...] = back.astype(a.dtype, copy=False)
    outs = []
    for i in range(nlhs):
        if plhs[i]:
            outs.append(_from_mx(lib, plhs[i]))
            lib.mxDestroyArray(plhs[i])
        else:
            outs.append(None)
    for m in mxs:
        lib.mxDestroyArray(m)
    if nlhs == 0:
        return None
    return outs[0] if nlhs == 1 else tuple(outs)
