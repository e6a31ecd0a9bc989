"""ctypes binding of ``libqsm_gb300.so`` (the C ABI in include/qsm_gpu.h).

The library is the product: there is no fallback.  If the shared object is
missing or cannot be loaded, :func:`lib` raises :class:`QsmLibraryError`;
build it with ``python qsm.m_gb300/build.py`` (or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqsm_gb300.so")

P = ctypes.c_void_p
SZ3 = ctypes.POINTER(ctypes.c_size_t)
D3 = ctypes.POINTER(ctypes.c_double)
U8 = ctypes.c_void_p
I32 = ctypes.c_int32
U32 = ctypes.c_uint32
DBL = ctypes.c_double
CTX = ctypes.c_void_p
STATUS = ctypes.c_int

QSM_F64, QSM_F32 = 0, 1

# QSM_GPU_ABI_VERSION these bindings are written for (struct layouts included)
ABI_VERSION = 2

STATUS_NAMES = {
    0: "QSM_OK", 1: "QSM_ERR_ARG", 2: "QSM_ERR_DIMS", 3: "QSM_ERR_DTYPE", 4: "QSM_ERR_NOMEM",
    5: "QSM_ERR_CUDA", 6: "QSM_ERR_NONFINITE", 7: "QSM_ERR_DEPTH", 8: "QSM_ERR_BUSY", 9: "QSM_ERR_TIMEOUT",
}


class QsmLibraryError(RuntimeError):
    pass


class QsmError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class PdInfo(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_uint32), ("monitor_chi", ctypes.c_double),
                ("monitor_eta", ctypes.c_double), ("seconds", ctypes.c_double),
                ("active_voxels", ctypes.c_uint64), ("tile", ctypes.c_uint32 * 3)]


class TvInfo(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_uint32), ("rho", ctypes.c_double), ("nr", ctypes.c_double),
                ("eps_pri", ctypes.c_double), ("ns", ctypes.c_double), ("eps_dual", ctypes.c_double),
                ("seconds", ctypes.c_double)]


class MgInfo(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int32), ("resnorm", ctypes.c_double), ("seconds", ctypes.c_double),
                ("resnorm_hist", ctypes.POINTER(ctypes.c_double)), ("coarse_ctas", ctypes.c_int32),
                ("coarse_outer", ctypes.c_int32)]


class NiftiHdr(ctypes.Structure):
    """qsm_nifti_hdr (include/qsm_gpu.h)."""
    _fields_ = [("filetype", ctypes.c_int32), ("big_endian", ctypes.c_int32),
                ("stored_datatype", ctypes.c_int32), ("bitpix", ctypes.c_int32),
                ("stored_dim", ctypes.c_int64 * 8), ("vox_offset", ctypes.c_int64),
                ("vox_offset_stored", ctypes.c_double), ("scl_slope", ctypes.c_double), ("scl_inter", ctypes.c_double),
                ("quatern", ctypes.c_double * 3), ("qoffset", ctypes.c_double * 3), ("srow", ctypes.c_double * 12),
                ("datatype", ctypes.c_int32), ("scaled", ctypes.c_int32), ("dim", ctypes.c_int64 * 8),
                ("pixdim", ctypes.c_double * 8), ("originator", ctypes.c_double * 5),
                ("perm", ctypes.c_int32 * 3), ("flip", ctypes.c_int32 * 3), ("reoriented", ctypes.c_int32),
                ("qform_code", ctypes.c_int32), ("sform_code", ctypes.c_int32), ("xyzt_units", ctypes.c_int32),
                ("data_type", ctypes.c_char * 11), ("db_name", ctypes.c_char * 19), ("descrip", ctypes.c_char * 81),
                ("aux_file", ctypes.c_char * 25), ("intent_name", ctypes.c_char * 17), ("magic", ctypes.c_char * 5),
                ("error", ctypes.c_char * 160)]


# name -> argtypes (after ctx); every function returns qsm_status
_GRAD = [I32, SZ3, P, P, P, P, D3]
_GRADM = [I32, SZ3, P, P, P, P, U8, D3]
_ADJ = [I32, SZ3, P, P, P, P, D3]
_ADJM = [I32, SZ3, P, P, P, P, U8, D3]
SIGNATURES = {
    "qsm_pd_tgv": [I32, SZ3, P, U8, D3, DBL, DBL, DBL, U32, U32, P, ctypes.POINTER(PdInfo)],
    "qsm_pd_tv": [I32, SZ3, P, U8, D3, DBL, DBL, U32, U32, P, ctypes.POINTER(PdInfo)],
    "qsm_pd_tgv_fused": [I32, SZ3, P, U8, D3, DBL, DBL, DBL, U32, U32, P, ctypes.POINTER(PdInfo)],
    "qsm_pd_tv_fused": [I32, SZ3, P, U8, D3, DBL, DBL, U32, U32, P, ctypes.POINTER(PdInfo)],
    "qsm_gradf": _GRAD, "qsm_gradb": _GRAD, "qsm_gradc": _GRAD, "qsm_gradfp": _GRAD,
    "qsm_gradfm": _GRADM, "qsm_gradbm": _GRADM, "qsm_gradcm": _GRADM,
    "qsm_gradf_adj": _ADJ, "qsm_gradb_adj": _ADJ, "qsm_gradfp_adj": _ADJ,
    "qsm_gradfm_adj": _ADJM, "qsm_gradbm_adj": _ADJM,
    "qsm_lap1": [I32, SZ3, P, P, U8, D3],
    "qsm_lapw": [I32, SZ3, P, P, D3],
    "qsm_gauss_seidel": [I32, SZ3, P, P, U8, D3, I32, I32],
    "qsm_residual": [I32, SZ3, P, P, P, U8, D3],
    "qsm_lapmg": [I32, SZ3, P, P, U8, D3],
    "qsm_restrict": [I32, SZ3, P, SZ3, P, U8],
    "qsm_prolong": [I32, SZ3, P, SZ3, P, U8],
    "qsm_correct": [I32, SZ3, P, SZ3, P, U8],
    "qsm_coarsen_grid": [SZ3, U8, SZ3, U8],
    "qsm_boundary_mask": [SZ3, U8, U8],
    "qsm_boundary_mask_l1": [SZ3, U8, U8, ctypes.c_uint8],
    "qsm_norm2": [I32, ctypes.c_size_t, P, U8, D3],
    "qsm_dot": [I32, ctypes.c_size_t, P, P, D3],
    "qsm_mgpcg": [I32, SZ3, P, P, U8, D3, DBL, I32, DBL, I32, I32, I32, I32, I32, I32, I32, P, ctypes.POINTER(MgInfo)],
    "qsm_mgpcg_mixed": [SZ3, P, P, U8, D3, DBL, I32, DBL, I32, I32, I32, I32, I32, I32, I32, P, ctypes.POINTER(MgInfo)],
    "qsm_mgpcg_batch": [I32, U32, P, P, P, P, D3, DBL, I32, DBL, I32, I32, I32, I32, I32, I32, P, P],
    "qsm_mg": [I32, SZ3, P, P, U8, D3, DBL, I32, I32, I32, I32, I32, I32, P, ctypes.POINTER(MgInfo)],
    "qsm_fmg": [I32, SZ3, P, U8, D3, DBL, I32, I32, I32, I32, I32, I32, P, ctypes.POINTER(MgInfo)],
    "qsm_tv_admm": [I32, SZ3, P, U8, D3, D3, DBL, I32, DBL, DBL, I32, DBL, DBL, DBL, DBL, DBL, I32, P,
                    ctypes.POINTER(TvInfo)],
    "qsm_sstgv": [I32, SZ3, P, U8, D3, DBL, DBL, DBL, U32, U32, I32, P, P],
    "qsm_lbv": [I32, SZ3, P, U8, D3, DBL, I32, I32, I32, I32, I32, I32, I32, P, P],
    "qsm_unwrap_laplacian": [I32, SZ3, P, U8, D3, I32, P, P],
    "qsm_sharp": [I32, SZ3, P, U8, D3, DBL, DBL, P, P],
    "qsm_vsharp": [I32, SZ3, P, U8, D3, P, I32, DBL, P, P],
    "qsm_ismv": [I32, SZ3, P, U8, D3, DBL, DBL, I32, I32, P, P, P],
    "qsm_resharp": [I32, SZ3, P, U8, D3, DBL, DBL, DBL, I32, I32, P, P, P],
    "qsm_pdf": [I32, SZ3, P, U8, P, D3, D3, DBL, DBL, I32, I32, P, P],
    "qsm_nifti_decode": [ctypes.POINTER(NiftiHdr), P, I32, P],
    "qsm_nifti_make_header": [I32, I32, ctypes.POINTER(ctypes.c_int64), D3, I32, P, P],
    # count volumes: dims (size_t[3*count]), arrays of d2f / mask / chi pointers
    "qsm_pd_tv_batch": [I32, U32, P, P, P, D3, DBL, DBL, U32, P, P],
    "qsm_pd_tgv_batch": [I32, U32, P, P, P, D3, DBL, DBL, DBL, U32, P, P],
}

SES = ctypes.c_void_p
U64P = ctypes.POINTER(ctypes.c_uint64)
# session functions: name -> (argtypes, restype)
SESSION_SIGNATURES = {
    "qsm_session_create": ([CTX, ctypes.c_size_t, I32, ctypes.POINTER(SES)], STATUS),
    "qsm_session_destroy": ([SES], STATUS),
    "qsm_session_footprint": ([I32, SZ3, I32], ctypes.c_size_t),
    "qsm_session_bytes_in_use": ([SES], ctypes.c_size_t),
    "qsm_session_submit_pd": ([SES, I32, I32, SZ3, P, U8, D3, DBL, DBL, DBL, U32, U64P], STATUS),
    "qsm_session_submit_mgpcg": ([SES, SZ3, P, P, U8, D3, DBL, I32, DBL, I32, I32, I32, I32, I32, I32, I32, U64P],
                                 STATUS),
    "qsm_session_step": ([SES, U32], STATUS),
    "qsm_session_poll": ([SES, ctypes.c_uint64, ctypes.POINTER(I32), ctypes.POINTER(PdInfo), ctypes.POINTER(MgInfo)],
                         STATUS),
    "qsm_session_fetch": ([SES, ctypes.c_uint64, P], STATUS),
    "qsm_session_running": ([SES], U32),
}

# host-only functions without a context: name -> (argtypes, restype)
HOST_SIGNATURES = {
    "qsm_nifti_parse": ([P, ctypes.c_size_t, DBL, ctypes.c_char, ctypes.POINTER(NiftiHdr)], STATUS),
    "qsm_nifti_payload_bytes": ([ctypes.POINTER(NiftiHdr)], ctypes.c_size_t),
}

QSM_JOB_TV, QSM_JOB_TGV, QSM_JOB_MGPCG, QSM_JOB_MGPCG_F64 = 0, 1, 2, 3

_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise QsmLibraryError(f"{LIB_PATH} is missing; build it with `python qsm.m_gb300/build.py`")
    try:
        L = ctypes.CDLL(LIB_PATH)
    except OSError as e:
        raise QsmLibraryError(f"cannot load {LIB_PATH}: {e}") from e
    L.qsm_ctx_create.argtypes = [ctypes.c_int, ctypes.POINTER(CTX)]
    L.qsm_ctx_create.restype = STATUS
    L.qsm_ctx_destroy.argtypes = [CTX]
    L.qsm_ctx_destroy.restype = STATUS
    L.qsm_ctx_set_stream.argtypes = [CTX, P]
    L.qsm_ctx_set_stream.restype = STATUS
    L.qsm_ctx_get_stream.argtypes = [CTX]
    L.qsm_ctx_get_stream.restype = P
    L.qsm_ctx_set_verbose.argtypes = [CTX, ctypes.c_int]
    L.qsm_ctx_set_verbose.restype = STATUS
    L.qsm_ctx_set_debug.argtypes = [CTX, ctypes.c_uint32]
    L.qsm_ctx_set_debug.restype = STATUS
    L.qsm_last_error.argtypes = [CTX]
    L.qsm_last_error.restype = ctypes.c_char_p
    L.qsm_status_string.argtypes = [ctypes.c_int]
    L.qsm_status_string.restype = ctypes.c_char_p
    L.qsm_abi_version.argtypes = []
    L.qsm_abi_version.restype = ctypes.c_int
    if L.qsm_abi_version() != ABI_VERSION:
        raise QsmLibraryError(f"{LIB_PATH} has ABI {L.qsm_abi_version()}, these bindings need {ABI_VERSION}; "
                              "rebuild it with `python qsm.m_gb300/build.py`")
    L.qsm_fp_pipe_rate.argtypes = [CTX, I32, ctypes.POINTER(DBL)]
    L.qsm_fp_pipe_rate.restype = STATUS
    L.qsm_fp_convert_check.argtypes = [CTX, ctypes.POINTER(ctypes.c_ulonglong)]
    L.qsm_fp_convert_check.restype = STATUS
    L.qsm_norm2_noalloc.argtypes = [I32, ctypes.c_size_t, P, U8, P, P]
    L.qsm_norm2_noalloc.restype = STATUS
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = [CTX] + args
        fn.restype = STATUS
    for name, (args, res) in list(SESSION_SIGNATURES.items()) + list(HOST_SIGNATURES.items()):
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def exported_symbols() -> list[str]:
    """Names of every function include/qsm_gpu.h declares."""
    return sorted(list(SIGNATURES) + list(SESSION_SIGNATURES) + list(HOST_SIGNATURES) + ["qsm_ctx_create", "qsm_ctx_destroy", "qsm_ctx_set_stream",
                                      "qsm_ctx_get_stream", "qsm_ctx_set_verbose", "qsm_ctx_set_debug", "qsm_last_error",
                                      "qsm_status_string", "qsm_abi_version", "qsm_norm2_noalloc",
                                      "qsm_fp_pipe_rate", "qsm_fp_convert_check"])


class Context:
    """A library context: one device, one stream, one memory pool."""

    def __init__(self, device: int = 0):
        self.device = device
        h = CTX()
        st = lib().qsm_ctx_create(device, ctypes.byref(h))
        if st != 0:
            raise QsmError(st, "qsm_ctx_create failed (is a CUDA device present?)")
        self.handle = h

    def call(self, name: str, *args):
        st = getattr(lib(), name)(self.handle, *args)
        if st != 0:
            msg = lib().qsm_last_error(self.handle) or b""
            raise QsmError(st, f"{name}: {msg.decode(errors='replace')}")
        return st

    def close(self):
        if getattr(self, "handle", None):
            lib().qsm_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_ctx: dict[int, Context] = {}


def context(device: int = 0) -> Context:
    if device not in _ctx:
        _ctx[device] = Context(device)
    return _ctx[device]
