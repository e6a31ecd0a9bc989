"""CPU restatement of QSM.m's NIfTI reading and writing.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the oracle of the library's
NIfTI path; the product never imports it.

Follows src/io/loadNii.m and saveNii.m over the NIfTI toolbox in
third_party/NIfTI: load_nii_hdr.m (header fields at their NIfTI-1 offsets,
little-endian first, then big-endian), load_nii_img.m:read_image (the stored
class; dims below 1 read as 1), xform_nii.m (scl_slope / scl_inter; change_hdr
with the sform preferred, small affine entries cleared, generalized
permutation check, voxel size, originator and get_orient; get_units; flips and
permute), make_nii.m + save_nii.m + save_nii_hdr.m (the 352-byte 'n+1'
header, sform_code 1 from pixdim, glmax / glmin rounded).  Written in numpy
with struct; the reference is MATLAB code that cannot run here and ships no
NIfTI file, so parity of the restatement itself is unpinned.
"""
from __future__ import annotations

import math
import struct

import numpy as np

DT = {2: np.uint8, 4: np.int16, 8: np.int32, 16: np.float32, 64: np.float64, 256: np.int8, 512: np.uint16,
      768: np.uint32, 1024: np.int64, 1280: np.uint64}
CLASS = {np.dtype(v): k for k, v in DT.items()}
BITPIX = {1: 1, 2: 8, 4: 16, 8: 32, 16: 32, 32: 64, 64: 64, 128: 24, 256: 8, 511: 96, 512: 16, 768: 32, 1024: 64,
          1280: 64, 1792: 128}


def _deblank(b: bytes) -> str:
    s = b.decode("latin-1")
    return s.rstrip(" \t\n\r\v\f\x00")


def read_header(b: bytes) -> dict:
    """load_nii_hdr.m: the fields, with the byte order that makes sizeof_hdr 348."""
    if len(b) < 348:
        raise ValueError("short header")
    e = "<"
    if struct.unpack("<i", b[:4])[0] != 348:
        e = ">"
        if struct.unpack(">i", b[:4])[0] != 348:
            raise ValueError("file is corrupted")
    u = lambda fmt, off: struct.unpack_from(e + fmt, b, off)  # noqa: E731
    h = {"machine": "ieee-le" if e == "<" else "ieee-be"}
    h["data_type"] = _deblank(b[4:14])
    h["db_name"] = _deblank(b[14:32])
    h["dim"] = list(u("8h", 40))
    h["datatype"] = u("h", 70)[0]
    h["bitpix"] = u("h", 72)[0]
    h["pixdim"] = [float(x) for x in u("8f", 76)]
    h["vox_offset"] = float(u("f", 108)[0])
    h["scl_slope"] = float(u("f", 112)[0])
    h["scl_inter"] = float(u("f", 116)[0])
    h["xyzt_units"] = b[123]
    h["glmax"], h["glmin"] = u("2i", 140)
    h["descrip"] = _deblank(b[148:228])
    h["aux_file"] = _deblank(b[228:252])
    h["qform_code"], h["sform_code"] = u("2h", 252)
    h["quatern"] = [float(x) for x in u("3f", 256)]
    h["qoffset"] = [float(x) for x in u("3f", 268)]
    h["srow"] = [[float(x) for x in u("4f", 280 + 16 * r)] for r in range(3)]
    h["intent_name"] = _deblank(b[328:344])
    h["magic"] = _deblank(b[344:348])
    h["originator"] = [float(x) for x in u("5h", 253)]
    if h["magic"] not in ("n+1", "ni1"):
        h["qform_code"] = h["sform_code"] = 0
    h["filetype"] = 2 if h["magic"] == "n+1" else 1 if h["magic"] == "ni1" else 0
    return h


def _gen_perm(R):
    if np.linalg.det(R) == 0:
        return False
    f = R.flatten(order="F")
    nz = f[f != 0]
    return nz.size == 3 and np.array_equal(nz, R.sum(axis=0))


def _change_hdr(h, tolerance, form):
    """xform_nii.m:change_hdr -> (orient, voxel sizes set in h)."""
    use = None
    if form == "S":
        if h["sform_code"] == 0:
            raise ValueError("User requires sform, sform not set in header")
        use = "s"
    elif form == "Q":
        if h["qform_code"] == 0:
            raise ValueError("User requires qform, qform not set in header")
        use = "q"
    elif form == "q":
        use = "q" if h["qform_code"] > 0 else "s" if h["sform_code"] > 0 else None
    else:
        use = "s" if h["sform_code"] > 0 else "q" if h["qform_code"] > 0 else None
    orient = [1, 2, 3]
    R = None
    if use == "s":
        R = np.array([r[:3] for r in h["srow"]], dtype=np.float64)
        T = np.array([r[3] for r in h["srow"]], dtype=np.float64)
        if not _gen_perm(R):
            rs = np.sort(np.abs(R.flatten(order="F")))
            R[np.abs(R) < tolerance * rs[-3:].min()] = 0
            if not _gen_perm(R):
                raise ValueError("Non-orthogonal rotation or shearing found inside the affine matrix")
    elif use == "q":
        b, c, d = h["quatern"]
        if 1.0 - (b * b + c * c + d * d) < 0:
            if abs(1.0 - (b * b + c * c + d * d)) < 1e-5:
                a = 0.0
            else:
                raise ValueError("Incorrect quaternion values in this NIFTI data.")
        else:
            a = math.sqrt(1.0 - (b * b + c * c + d * d))
        qfac = h["pixdim"][0] or 1.0
        S = np.diag([h["pixdim"][1], h["pixdim"][2], qfac * h["pixdim"][3]])
        R = np.array([[a * a + b * b - c * c - d * d, 2 * b * c - 2 * a * d, 2 * b * d + 2 * a * c],
                      [2 * b * c + 2 * a * d, a * a + c * c - b * b - d * d, 2 * c * d - 2 * a * b],
                      [2 * b * d - 2 * a * c, 2 * c * d + 2 * a * b, a * a + d * d - c * c - b * b]])
        T = np.array(h["qoffset"], dtype=np.float64)
        if not _gen_perm(R):
            rs = np.sort(np.abs(R.flatten(order="F")))
            R[np.abs(R) < tolerance * rs[-3:].min()] = 0
            R = R @ S
            if not _gen_perm(R):
                raise ValueError("Non-orthogonal rotation or shearing found inside the affine matrix")
        else:
            R = R @ S
    if R is not None:
        vox = np.abs(R.sum(axis=0))
        invR = np.linalg.inv(R)
        org = invR @ (-T) + 1
        orient = []
        for i in range(3):
            col = int(np.flatnonzero(invR[i])[0]) + 1
            orient.append(col if invR[i].sum() > 0 else col + 3)
        h["pixdim"][1:4] = [float(v) for v in vox]
        h["originator"][0:3] = [float(v) for v in org]
        h["qform_code"] = h["sform_code"] = 0
    su = h["xyzt_units"] & 7
    unit = 1e3 if su == 1 else 1e-3 if su == 3 else 1.0
    if unit != 1.0:
        h["pixdim"][1:4] = [p * unit for p in h["pixdim"][1:4]]
        h["xyzt_units"] = (h["xyzt_units"] & ~7) | 2
    h["pixdim"] = [abs(p) for p in h["pixdim"]]
    return orient


def load_nii(header: bytes, payload: bytes, tolerance=0.1, preferred_form="s"):
    """load_nii.m on the bytes of a header and of the stored image (from the first
    voxel).  Returns (img, hdr): img in the loaded class and MATLAB order."""
    h = read_header(header)
    dt = h["datatype"]
    if dt not in DT:
        raise ValueError(f"datatype {dt} not handled here")
    h["bitpix"] = BITPIX[dt]
    dim = [d if d >= 1 else 1 for d in h["dim"]]
    h["dim"] = dim
    n = int(np.prod(dim[1:8]))
    e = "<" if h["machine"] == "ieee-le" else ">"
    img = np.frombuffer(payload, dtype=np.dtype(DT[dt]).newbyteorder(e), count=n).astype(DT[dt])
    shape = list(dim[1:8])
    while len(shape) > 3 and shape[-1] == 1:  # MATLAB drops trailing singleton dimensions
        shape.pop()
    img = img.reshape(shape, order="F")
    h["scaled"] = False
    if (h["scl_slope"] != 0 and dt in (2, 4, 8, 16, 64, 256, 512, 768)
            and (h["scl_slope"] != 1 or h["scl_inter"] != 0)):
        img = h["scl_slope"] * img.astype(np.float64) + h["scl_inter"]
        if dt != 64:
            img = img.astype(np.float32)
            h["datatype"] = 16
        h["scaled"] = True
    h["perm"], h["flip"] = [0, 1, 2], [0, 0, 0]
    if h["filetype"] == 0:
        return img, h
    orient = _change_hdr(h, tolerance if tolerance > 0 else np.finfo(float).eps, preferred_form)
    if orient != [1, 2, 3]:
        rot = [(o + 2) % 3 + 1 for o in orient]
        flip = [o - r for o, r in zip(orient, rot)]
        for i in range(3):
            if flip[i]:
                img = np.flip(img, axis=i)
        order = sorted(range(3), key=lambda i: rot[i])
        new_dim = [dim[1 + i] for i in order]
        h["dim"][1:4] = new_dim
        h["pixdim"][1:4] = [h["pixdim"][1 + i] for i in order]
        org = [h["originator"][i] for i in order]
        flip = [flip[i] for i in order]
        for i in range(3):
            if flip[i] and org[i] != 0:
                org[i] = new_dim[i] - org[i] + 1
        h["originator"][0:3] = org
        img = np.transpose(img, order + list(range(3, img.ndim)))
        h["perm"], h["flip"] = order, [1 if f else 0 for f in flip]
    return np.asfortranarray(img), h


def _round(v):
    return math.floor(v + 0.5) if v >= 0 else -math.floor(-v + 0.5)


def make_header(img, vsz=(1.0, 1.0, 1.0), filetype=2) -> bytes:
    """make_nii(img, vsz) + save_nii's header (352 bytes for 'n+1', 348 for 'ni1')."""
    img = np.asarray(img)
    if img.dtype not in CLASS or CLASS[img.dtype] in (1024, 1280):
        raise ValueError("Datatype is not supported by make_nii.")
    dt = CLASS[img.dtype]
    size = list(img.shape) if img.ndim >= 2 else ([1, 1] if img.ndim == 0 else [img.shape[0], 1])
    while len(size) > 2 and size[-1] == 1:
        size.pop()
    if len(size) > 7:
        raise ValueError("NIfTI only allows a maximum of 7 Dimension matrix.")
    dims = [len(size)] + size + [1] * 7
    dims = [max(-32768, min(32767, int(v))) for v in dims[:8]]
    pix = [0.0, float(vsz[0]), float(vsz[1]), float(vsz[2]), 1.0, 1.0, 1.0, 1.0]
    a = img.astype(np.float64).ravel()
    a = a[~np.isnan(a)]

    def i32(v):
        v = _round(v)
        return int(max(-2147483648, min(2147483647, v)))

    glmax, glmin = (i32(a.max()), i32(a.min())) if a.size else (0, 0)
    b = bytearray(352 if filetype == 2 else 348)
    struct.pack_into("<i", b, 0, 348)
    b[38] = ord("r")
    struct.pack_into("<8h", b, 40, *dims)
    struct.pack_into("<hhh", b, 70, dt, BITPIX[dt], 0)
    struct.pack_into("<8f", b, 76, *pix)
    struct.pack_into("<f", b, 108, 352.0 if filetype == 2 else 0.0)
    struct.pack_into("<ii", b, 140, glmax, glmin)
    b[228:232] = b"none"
    struct.pack_into("<hh", b, 252, 0, 1)
    srow = [pix[1], 0, 0, (1 - 0) * pix[1], 0, pix[2], 0, (1 - 0) * pix[2], 0, 0, pix[3], (1 - 0) * pix[3]]
    struct.pack_into("<12f", b, 280, *srow)
    b[344:347] = b"n+1" if filetype == 2 else b"ni1"
    return bytes(b)


def save_bytes(img, vsz=(1.0, 1.0, 1.0)) -> bytes:
    """The bytes of the .nii that saveNii writes."""
    img = np.asarray(img)
    return make_header(img, vsz) + np.asfortranarray(img).tobytes(order="F")
