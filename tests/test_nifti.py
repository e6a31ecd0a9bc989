"""NIfTI header logic on the CPU: the library's parser (qsm_nifti_parse, host
code) against the numpy restatement (oracle/nifti.py) on hand-built headers
(orientations from sform and qform, byte orders, scaling, units, Analyze and
pair files, errors), and the restatement's own round trip and byte layout."""
import math
import struct

import numpy as np
import pytest


@pytest.fixture(scope="module")
def nio(port):
    import nifti
    return nifti


@pytest.fixture(scope="module")
def qn():
    from qsm_gb300 import nifti
    return nifti


def build_header(e="<", dim=(3, 6, 5, 4, 1, 1, 1, 1), datatype=16, pixdim=(1, 1, 1, 1, 1, 1, 1, 1), slope=0.0,
                 inter=0.0, qform=0, sform=0, quatern=(0, 0, 0), qoffset=(0, 0, 0), srow=None, xyzt=0, magic=b"n+1",
                 vox_offset=352.0, originator=None):
    from nifti import BITPIX
    b = bytearray(352)
    struct.pack_into(e + "i", b, 0, 348)
    b[38] = ord("r")
    struct.pack_into(e + "8h", b, 40, *dim)
    struct.pack_into(e + "hh", b, 70, datatype, BITPIX[datatype])
    struct.pack_into(e + "8f", b, 76, *pixdim)
    struct.pack_into(e + "3f", b, 108, vox_offset, slope, inter)
    b[123] = xyzt
    struct.pack_into(e + "hh", b, 252, qform, sform)
    struct.pack_into(e + "3f", b, 256, *quatern)
    struct.pack_into(e + "3f", b, 268, *qoffset)
    if srow is not None:
        struct.pack_into(e + "12f", b, 280, *[v for r in srow for v in r])
    b[344:348] = magic.ljust(4, b"\0")
    if originator is not None:
        struct.pack_into(e + "5h", b, 253, *originator)
    return bytes(b)


S45 = math.sin(math.pi / 4)
CASES = {
    "identity_sform": dict(sform=1, srow=[[1, 0, 0, 1], [0, 1, 0, 1], [0, 0, 1, 1]]),
    "lps_sform": dict(sform=1, srow=[[-1, 0, 0, 30], [0, -1, 0, 20], [0, 0, 1, -5]]),
    "permuted_sform": dict(sform=2, pixdim=(1, 1.5, 2, 0.5, 1, 1, 1, 1),
                           srow=[[0, 0, 0.5, -10], [1.5, 0, 0, 4], [0, -2, 0, 7]]),
    "small_shear": dict(sform=1, srow=[[1, 0.01, 0, 0], [0, 1, 0, 0], [0.02, 0, -1, 3]]),
    "qform_rot90_qfac": dict(qform=1, pixdim=(-1, 0.9, 1.1, 1.3, 1, 1, 1, 1), quatern=(0, 0, S45),
                             qoffset=(5, -3, 2)),
    "sform_over_qform": dict(qform=1, sform=1, quatern=(0, 0, S45), srow=[[2, 0, 0, 0], [0, 2, 0, 0], [0, 0, 2, 0]]),
    "metres": dict(sform=1, xyzt=1, pixdim=(1, 0.001, 0.001, 0.002, 1, 1, 1, 1),
                   srow=[[0.001, 0, 0, 0], [0, 0.001, 0, 0], [0, 0, 0.002, 0]]),
    "micrometres": dict(sform=1, xyzt=3, srow=[[-500, 0, 0, 0], [0, 500, 0, 0], [0, 0, 800, 0]]),
    "no_affine": dict(pixdim=(1, -1.2, 0.8, 1.0, 1, 1, 1, 1)),
    "analyze": dict(magic=b"", pixdim=(1, -1.2, 0.8, 1.0, 1, 1, 1, 1), sform=1, originator=(3, 2, 1, 0, 0),
                    srow=[[-1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]]),
    "pair_ni1": dict(magic=b"ni1", vox_offset=0.0, sform=1, srow=[[0, 1, 0, 0], [1, 0, 0, 0], [0, 0, -1, 0]]),
    "scaled_int16": dict(datatype=4, slope=2.0, inter=-1.0, sform=1, srow=[[-1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]]),
    "unit_slope": dict(datatype=16, slope=1.0, inter=0.0),
    "scaled_double": dict(datatype=64, slope=0.5, inter=3.0),
    "four_d": dict(dim=(4, 6, 5, 4, 3, 1, 1, 1), datatype=8, sform=1,
                   srow=[[0, 0, 1, 0], [0, -1, 0, 0], [1, 0, 0, 0]]),
}


@pytest.mark.parametrize("endian", ["<", ">"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_parse_matches_restatement(nio, qn, case, endian):
    hb = build_header(endian, **CASES[case])
    h = qn.parse_header(hb)
    n = int(np.prod([max(1, d) for d in CASES[case].get("dim", (3, 6, 5, 4, 1, 1, 1, 1))][1:]))
    dt = CASES[case].get("datatype", 16)
    payload = np.arange(n, dtype=nio.DT[dt]).astype(np.dtype(nio.DT[dt]).newbyteorder(endian)).tobytes()
    img, r = nio.load_nii(hb, payload)
    d = qn._hdr_dict(h)
    assert d["dim"] == r["dim"]
    assert d["datatype"] == (16 if r["scaled"] and dt != 64 else dt)
    assert d["scaled"] == r["scaled"]
    np.testing.assert_allclose(d["pixdim"], r["pixdim"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(d["originator"], r["originator"], rtol=1e-12, atol=1e-12)
    assert [d["qform_code"], d["sform_code"]] == [r["qform_code"], r["sform_code"]]
    assert d["xyzt_units"] == r["xyzt_units"]
    perm = [p - 1 for p in d["rot_orient"]] if d["rot_orient"] else [0, 1, 2]
    flip = d["flip_orient"] if d["flip_orient"] else [0, 0, 0]
    assert perm == r["perm"] and flip == r["flip"]
    assert h.big_endian == (endian == ">")
    assert list(img.shape[:3]) == d["dim"][1:4]


def test_orientation_examples(nio):
    """Closed forms: an LPS sform flips x and y; a permuted sform sorts the stored
    axes into x, y, z and flips the one that runs backwards."""
    hb = build_header("<", dim=(3, 4, 3, 2, 1, 1, 1, 1), **{k: v for k, v in CASES["lps_sform"].items()})
    a = np.arange(24, dtype=np.float32)
    img, h = nio.load_nii(hb, a.tobytes())
    ref = a.reshape((4, 3, 2), order="F")[::-1, ::-1, :]
    assert np.array_equal(img, ref) and h["flip"] == [1, 1, 0]
    hb = build_header("<", dim=(3, 4, 3, 2, 1, 1, 1, 1), **{k: v for k, v in CASES["permuted_sform"].items()})
    img, h = nio.load_nii(hb, a.tobytes())
    # stored axis 0 -> world y, axis 1 -> -z, axis 2 -> x
    ref = np.transpose(a.reshape((4, 3, 2), order="F")[:, ::-1, :], (2, 0, 1))
    assert np.array_equal(img, ref) and h["dim"][1:4] == [2, 4, 3]
    assert h["pixdim"][1:4] == [0.5, 1.5, 2.0]


def test_errors(nio, qn):
    from qsm_gb300 import _lib
    with pytest.raises(_lib.QsmError, match="348"):
        qn.parse_header(b"\0" * 100)
    bad = bytearray(build_header("<"))
    struct.pack_into("<i", bad, 0, 12)
    with pytest.raises(_lib.QsmError, match="corrupted"):
        qn.parse_header(bytes(bad))
    shear = build_header("<", sform=1, srow=[[1, 0.5, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]])
    with pytest.raises(_lib.QsmError, match="Non-orthogonal"):
        qn.parse_header(shear)
    with pytest.raises(ValueError, match="Non-orthogonal"):
        nio.load_nii(shear, np.zeros(120, np.float32).tobytes())
    # the same shear passes with a looser tolerance (entries below 0.6 x 1 are cleared)
    assert qn.parse_header(shear, tolerance=0.6).reoriented == 0
    badq = build_header("<", qform=1, quatern=(0.9, 0.9, 0.0))
    with pytest.raises(_lib.QsmError, match="quaternion"):
        qn.parse_header(badq)
    with pytest.raises(_lib.QsmError, match="sform not set"):
        qn.parse_header(build_header("<", qform=1, quatern=(0, 0, 0)), preferred_form="S")


def test_restatement_round_trip_and_layout(nio):
    rng = np.random.default_rng(0)
    for dt in (np.float64, np.float32, np.int16, np.uint8):
        img = np.asfortranarray((rng.standard_normal((7, 6, 5)) * 50).astype(dt))
        raw = nio.save_bytes(img, (0.9, 1.0, 1.2))
        assert len(raw) == 352 + img.nbytes and raw[344:348] == b"n+1\0"
        assert struct.unpack_from("<i", raw, 0)[0] == 348 and struct.unpack_from("<f", raw, 108)[0] == 352.0
        out, h = nio.load_nii(raw[:352], raw[352:])
        assert out.dtype == img.dtype and np.array_equal(out, img)
        np.testing.assert_allclose(h["pixdim"][1:4], [0.9, 1.0, 1.2], rtol=1e-7)
        assert max(abs(v) for v in h["originator"][:3]) < 1e-12  # (1/a) * -a + 1
        assert struct.unpack_from("<ii", raw, 140) == (round(float(img.max())), round(float(img.min())))
    # MATLAB size() drops trailing singletons: a 4-D array with one echo is 3-D
    raw = nio.make_header(np.zeros((4, 3, 2, 1), np.float32))
    assert struct.unpack_from("<8h", raw, 40) == (3, 4, 3, 2, 1, 1, 1, 1)
    with pytest.raises(ValueError):
        nio.make_header(np.zeros((2, 2, 2), bool))


def test_oversized_dims_are_refused(qn):
    from qsm_gb300 import _lib
    hb = build_header("<", dim=(7, 32767, 32767, 32767, 32767, 2, 2, 2))
    with pytest.raises(_lib.QsmError, match="too large"):
        qn.parse_header(hb)
