"""NIfTI-1 files the way QSM.m reads and writes them: ``loadNii`` / ``saveNii``
(src/io/loadNii.m, saveNii.m) over ``load_nii`` / ``save_nii`` (third_party/NIfTI).

The header logic and the voxel pass are the library's (``qsm_nifti_parse``,
``qsm_nifti_decode``, ``qsm_nifti_make_header``): a loaded image arrives in
HBM (``device=True``: a CUDA tensor) or in host memory already byte-swapped,
scaled and reoriented as load_nii returns it.  This module only opens files
and runs gzip, as the MATLAB code leaves those to fopen / gunzip.
"""
from __future__ import annotations

import ctypes
import gzip
import os

import numpy as np

from . import _lib

_NP = {2: np.uint8, 4: np.int16, 8: np.int32, 16: np.float32, 64: np.float64, 256: np.int8, 512: np.uint16,
       768: np.uint32, 1024: np.int64, 1280: np.uint64}
_CLASS = {np.dtype(v): k for k, v in _NP.items()}


class Nii:
    """The struct load_nii returns: ``img``, ``hdr`` (a dict of the loaded header),
    ``filetype`` (2 'n+1', 1 'ni1', 0 Analyze), ``machine``, ``fileprefix``."""

    def __init__(self, img, hdr, filetype, machine, fileprefix):
        self.img, self.hdr, self.filetype, self.machine, self.fileprefix = img, hdr, filetype, machine, fileprefix


def _read(path):
    with open(path, "rb") as fh:
        data = fh.read()
    return gzip.decompress(data) if path.endswith(".gz") else data


def parse_header(header: bytes, tolerance=0.1, preferred_form="s") -> _lib.NiftiHdr:
    """qsm_nifti_parse on header bytes (host only)."""
    h = _lib.NiftiHdr()
    buf = ctypes.create_string_buffer(bytes(header), len(header))
    st = _lib.lib().qsm_nifti_parse(buf, len(header), float(tolerance), preferred_form.encode()[:1],
                                   ctypes.byref(h))
    if st != 0:
        raise _lib.QsmError(st, h.error.decode(errors="replace"))
    return h


def _hdr_dict(h: _lib.NiftiHdr) -> dict:
    nd = 8
    return dict(dim=[int(h.dim[i]) for i in range(nd)], datatype=int(h.datatype), bitpix=8 * _itemsize(h.datatype),
                pixdim=[float(h.pixdim[i]) for i in range(nd)], scl_slope=float(h.scl_slope),
                scl_inter=float(h.scl_inter), originator=[float(h.originator[i]) for i in range(5)],
                qform_code=int(h.qform_code), sform_code=int(h.sform_code), xyzt_units=int(h.xyzt_units),
                descrip=h.descrip.decode(errors="replace"), aux_file=h.aux_file.decode(errors="replace"),
                magic=h.magic.decode(errors="replace"), scaled=bool(h.scaled),
                rot_orient=[int(h.perm[i]) + 1 for i in range(3)] if h.reoriented else [],
                flip_orient=[int(h.flip[i]) for i in range(3)] if h.reoriented else [],
                stored_datatype=int(h.stored_datatype), stored_dim=[int(h.stored_dim[i]) for i in range(nd)])


def _itemsize(dt):
    return np.dtype(_NP[dt]).itemsize if dt in _NP else 0


def decode(header: bytes, payload, *, tolerance=0.1, preferred_form="s", device=False, out_dtype=None, ctx=None):
    """(img, hdr) of load_nii from the header bytes and the stored image bytes
    (from the first voxel; bytes, a numpy uint8 array or a CUDA uint8 tensor).
    ``out_dtype`` (float32 / float64) converts; default: load_nii's class.
    ``device`` returns a CUDA tensor (torch shape = MATLAB size reversed)."""
    h = parse_header(header[:348], tolerance, preferred_form)
    need = _lib.lib().qsm_nifti_payload_bytes(ctypes.byref(h))
    if hasattr(payload, "data_ptr"):
        if payload.numel() * payload.element_size() < need:
            raise ValueError(f"the image needs {need} bytes, the payload holds fewer")
        src_ptr, keep = ctypes.c_void_p(payload.data_ptr()), payload
    else:
        src = np.frombuffer(payload, dtype=np.uint8) if not isinstance(payload, np.ndarray) else payload
        if src.nbytes < need:
            raise ValueError(f"the image needs {need} bytes, the payload holds {src.nbytes}")
        src = np.ascontiguousarray(src)
        src_ptr, keep = ctypes.c_void_p(src.ctypes.data), src
    odt = 0 if out_dtype is None else _CLASS[np.dtype(out_dtype)]
    cls = _NP.get(int(h.datatype) if odt == 0 else odt)
    if cls is None:
        raise _lib.QsmError(3, f"datatype {h.stored_datatype} (bit, complex or RGB) is not decoded")
    shape = [int(h.dim[i]) for i in range(1, 8)]
    while len(shape) > 3 and shape[-1] == 1:  # MATLAB drops trailing singleton dimensions
        shape.pop()
    ctx = ctx or _lib.context(0)
    if device:
        import torch

        tdt = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
               np.dtype(np.uint8): torch.uint8, np.dtype(np.int8): torch.int8, np.dtype(np.int16): torch.int16,
               np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64}
        if np.dtype(cls) not in tdt:
            raise TypeError(f"no torch dtype for {np.dtype(cls)}; pass out_dtype")
        img = torch.empty(tuple(reversed(shape)), dtype=tdt[np.dtype(cls)], device=f"cuda:{ctx.device}")
        torch.cuda.current_stream().synchronize()
        ptr = ctypes.c_void_p(img.data_ptr())
    else:
        img = np.empty(shape, dtype=cls, order="F")
        ptr = ctypes.c_void_p(img.ctypes.data)
    ctx.call("qsm_nifti_decode", ctypes.byref(h), src_ptr, int(odt), ptr)
    del keep
    return img, h


def load_nii(filename, *, tolerance=0.1, preferred_form="s", device=False, out_dtype=None, ctx=None) -> Nii:
    """load_nii(filename, [], [], [], [], [], tolerance, preferred_form) for .nii,
    .nii.gz and .hdr/.img (optionally .gz) files; see decode() for the options."""
    fn = os.fspath(filename)
    if fn.endswith(".gz") and not fn.endswith((".nii.gz", ".hdr.gz", ".img.gz")):
        raise ValueError("Please check filename.")
    base = fn[:-3] if fn.endswith(".gz") else fn
    gz = ".gz" if fn.endswith(".gz") else ""
    if base.endswith(".nii"):
        data = _read(fn)
        h = parse_header(data[:348], tolerance, preferred_form)
        off = int(h.vox_offset)
        hdr_bytes, payload = data[:348], memoryview(data)[off:]
        prefix = base[:-4]
    else:
        prefix = base[:-4] if base.endswith((".hdr", ".img")) else base
        hdr_bytes = _read(prefix + ".hdr" + gz)[:348]
        payload = _read(prefix + ".img" + gz)
    img, h = decode(hdr_bytes, payload, tolerance=tolerance, preferred_form=preferred_form, device=device,
                    out_dtype=out_dtype, ctx=ctx)
    return Nii(img, _hdr_dict(h), int(h.filetype), "ieee-be" if h.big_endian else "ieee-le", prefix)


def loadNii(filename, **kw) -> Nii:  # noqa: N802 (the MATLAB name)
    """loadNii.m: a .nii or .nii.gz file, else an error."""
    fn = os.fspath(filename)
    if not os.path.isfile(fn):
        raise FileNotFoundError(f"file {fn} does not exist")
    ext = os.path.splitext(fn)[1].lower()
    if ext not in (".gz", ".nii"):
        raise ValueError(f"wrong file extension {fn}")
    return load_nii(fn, **kw)


def _torch_layout(img):
    """MATLAB size of a CUDA tensor that is C-contiguous (torch shape = MATLAB size
    reversed) or F-contiguous (torch shape = MATLAB size), as the rest of the
    package reads tensors; either way its memory is in MATLAB order."""
    shp = tuple(img.shape)
    if img.is_contiguous():
        return list(reversed(shp))
    exp, acc = [], 1
    for n in shp:
        exp.append(acc)
        acc *= n
    if list(img.stride()) != exp:
        raise ValueError("tensor must be contiguous in C or Fortran order")
    return list(shp)


def header_bytes(img, vsz=(1.0, 1.0, 1.0), filetype=2, *, ctx=None) -> bytes:
    """The header save_nii writes for make_nii(img, vsz) (img: numpy or CUDA tensor)."""
    if hasattr(img, "data_ptr"):
        import torch

        tdt = {torch.float32: np.float32, torch.float64: np.float64, torch.uint8: np.uint8, torch.int8: np.int8,
               torch.int16: np.int16, torch.int32: np.int32}
        if img.dtype not in tdt:
            raise TypeError("Datatype is not supported by make_nii.")
        dt = _CLASS[np.dtype(tdt[img.dtype])]
        size = _torch_layout(img)
        ptr = ctypes.c_void_p(img.data_ptr())
        torch.cuda.current_stream().synchronize()
    else:
        img = np.asarray(img)
        if img.dtype not in _CLASS:
            raise TypeError("Datatype is not supported by make_nii.")
        dt = _CLASS[img.dtype]
        size = list(img.shape) if img.ndim >= 2 else ([1, 1] if img.ndim == 0 else [img.shape[0], 1])
        img = np.asfortranarray(img)
        ptr = ctypes.c_void_p(img.ctypes.data)
    sz = (ctypes.c_int64 * max(1, len(size)))(*size)
    h = np.asarray(vsz, dtype=np.float64).reshape(-1)
    if h.size == 1:
        h = np.repeat(h, 3)
    vs = (ctypes.c_double * 3)(*[float(v) for v in h[:3]])
    out = (ctypes.c_uint8 * 352)()
    (ctx or _lib.context(0)).call("qsm_nifti_make_header", dt, len(size), sz, vs, int(filetype), ptr, out)
    return bytes(out)[:352 if filetype == 2 else 348]


def save_nii(img, filename, vsz=(1.0, 1.0, 1.0), *, ctx=None):
    """save_nii(make_nii(img, vsz), filename): .nii, .nii.gz, or a .hdr/.img pair
    (optionally gzipped).  The SPM .mat file save_nii adds beside a pair is not
    written."""
    fn = os.fspath(filename)
    gz = fn.endswith(".gz")
    if gz and not fn.endswith((".nii.gz", ".hdr.gz", ".img.gz")):
        raise ValueError("Please check filename.")
    base = fn[:-3] if gz else fn
    if hasattr(img, "data_ptr"):
        body_src = img
        arr = None
    else:
        arr = np.asfortranarray(np.asarray(img))
        body_src = arr
    pair = not base.endswith(".nii")
    hdr = header_bytes(body_src, vsz, 1 if pair else 2, ctx=ctx)
    if arr is None:
        _torch_layout(img)  # C- or F-contiguous: either way its memory order is MATLAB order
        body = img.detach().cpu().numpy().tobytes(order="A")
    else:
        body = arr.tobytes(order="F")
    w = (lambda p, b: open(p, "wb").write(gzip.compress(b))) if gz else (lambda p, b: open(p, "wb").write(b))
    if pair:
        prefix = base[:-4] if base.endswith((".hdr", ".img")) else base
        ext = ".gz" if gz else ""
        w(prefix + ".hdr" + ext, hdr)
        w(prefix + ".img" + ext, body)
    else:
        w(fn, hdr + body)


def saveNii(filename, img, vsz=(1.0, 1.0, 1.0), **kw):  # noqa: N802 (the MATLAB name)
    """saveNii.m: make the parent directory, then save_nii(make_nii(img, vsz), filename)."""
    d = os.path.dirname(os.fspath(filename))
    if d and not os.path.isdir(d):
        os.makedirs(d)
    save_nii(img, filename, vsz, **kw)
