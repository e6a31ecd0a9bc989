"""NIfTI on the GPU: the library's device decode (byte order, scaling,
reorientation) and header writer against the numpy restatement
(oracle/nifti.py), bit for bit, and file round trips through loadNii /
saveNii (.nii, .nii.gz, .hdr/.img pairs) with host and device images."""
import numpy as np
import pytest

from test_nifti import CASES, build_header

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nio(port):
    import nifti
    return nifti


@pytest.fixture(scope="module")
def qn(gpu_ctx):
    from qsm_gb300 import nifti
    return nifti


def _payload(nio, dt, n, endian, seed):
    rng = np.random.default_rng(seed)
    t = np.dtype(nio.DT[dt])
    if t.kind == "f":
        a = (rng.standard_normal(n) * 100).astype(t)
    else:
        info = np.iinfo(t)
        a = rng.integers(max(info.min, -(1 << 40)), min(info.max, 1 << 40), n, dtype=t, endpoint=True)
    return a.astype(t.newbyteorder(endian)).tobytes()


@pytest.mark.parametrize("dt", [2, 4, 8, 16, 64, 256, 512, 768, 1024, 1280])
@pytest.mark.parametrize("case", ["identity_sform", "permuted_sform", "qform_rot90_qfac", "four_d", "analyze"])
@pytest.mark.parametrize("endian", ["<", ">"])
def test_decode_bitexact(qn, nio, dt, case, endian):
    kw = dict(CASES[case])
    kw["datatype"] = dt
    if dt in (2, 4, 256, 512) and case == "identity_sform":
        kw.update(slope=0.25, inter=-3.0)  # load_nii scales these to single
    if dt == 64 and case == "permuted_sform":
        kw.update(slope=1.5, inter=2.0)    # a scaled double stays double
    hb = build_header(endian, **kw)
    dim = kw.get("dim", (3, 6, 5, 4, 1, 1, 1, 1))
    n = int(np.prod(dim[1:]))
    pl = _payload(nio, dt, n, endian, dt + len(case))
    ref, rh = nio.load_nii(hb, pl)
    img, h = qn.decode(hb, pl)
    assert img.dtype == ref.dtype and img.shape == ref.shape
    assert np.array_equal(img, ref)
    for odt in (np.float32, np.float64):
        out, _ = qn.decode(hb, pl, out_dtype=odt)
        assert out.dtype == odt and np.array_equal(out, ref.astype(odt))


def test_decode_to_device(qn, nio):
    torch = pytest.importorskip("torch")
    kw = dict(CASES["permuted_sform"], datatype=4, slope=0.5, inter=1.0, dim=(4, 20, 18, 16, 3, 1, 1, 1))
    hb = build_header("<", **kw)
    pl = _payload(nio, 4, 20 * 18 * 16 * 3, "<", 7)
    ref, _ = nio.load_nii(hb, pl)
    d, _ = qn.decode(hb, pl, device=True)
    assert d.is_cuda and d.dtype == torch.float32
    assert np.array_equal(d.cpu().numpy().transpose(3, 2, 1, 0), ref)
    # stored bytes already in HBM
    dp = torch.from_numpy(np.frombuffer(pl, np.uint8).copy()).cuda()
    d2, _ = qn.decode(hb, dp, device=True, out_dtype=np.float64)
    assert np.array_equal(d2.cpu().numpy().transpose(3, 2, 1, 0), ref.astype(np.float64))


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int16, np.uint8, np.int32, np.uint16, np.int8,
                                   np.uint32])
def test_header_bitexact(qn, nio, dtype):
    rng = np.random.default_rng(3)
    img = np.asfortranarray((rng.standard_normal((9, 8, 7, 2)) * 60).astype(dtype))
    if np.dtype(dtype).kind == "f":
        img[0, 0, 0, 0] = np.nan  # ignored by max / min
    assert qn.header_bytes(img, (0.9, 1.1, 1.3)) == nio.make_header(img, (0.9, 1.1, 1.3))
    assert qn.header_bytes(img, (1, 1, 1), filetype=1) == nio.make_header(img, (1, 1, 1), filetype=1)


def test_file_round_trips(qn, nio, tmp_path):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    chi = np.asfortranarray(rng.standard_normal((24, 20, 16)))
    for name in ("chi.nii", "sub/chi.nii.gz", "pair/chi.hdr", "pairgz/chi.img.gz"):
        fn = str(tmp_path / name)
        qn.saveNii(fn, chi, [1.0, 0.9, 1.1])  # makes the directory, as saveNii.m does
        nii = qn.load_nii(fn)
        assert nii.img.dtype == np.float64 and np.array_equal(nii.img, chi)
        np.testing.assert_allclose(nii.hdr["pixdim"][1:4], [1.0, 0.9, 1.1], rtol=1e-7)
    raw = open(tmp_path / "chi.nii", "rb").read()
    assert raw == nio.save_bytes(chi, [1.0, 0.9, 1.1])
    ref, _ = nio.load_nii(raw[:352], raw[352:])
    assert np.array_equal(qn.loadNii(str(tmp_path / "chi.nii")).img, ref)
    # a device image saved and read back to the device
    dev = torch.from_numpy(np.ascontiguousarray(chi.astype(np.float32).T)).cuda()
    qn.saveNii(str(tmp_path / "dev.nii.gz"), dev, [1, 1, 1])
    back = qn.loadNii(str(tmp_path / "dev.nii.gz"), device=True)
    assert torch.equal(back.img, dev)
    with pytest.raises(ValueError, match="extension"):
        qn.loadNii(str(tmp_path / "pair" / "chi.hdr"))


def test_misaligned_device_payload_is_rejected(qn, nio):
    """Whole-word loads need an aligned payload: a device buffer at an odd byte
    offset is refused before any launch."""
    torch = pytest.importorskip("torch")
    from qsm_gb300 import _lib
    hb = build_header("<", datatype=4)
    pl = _payload(nio, 4, 6 * 5 * 4, "<", 1)
    buf = torch.zeros(len(pl) + 1, dtype=torch.uint8, device="cuda")
    buf[1:] = torch.from_numpy(np.frombuffer(pl, np.uint8).copy()).cuda()
    with pytest.raises(_lib.QsmError, match="aligned"):
        qn.decode(hb, buf[1:])
    img, _ = qn.decode(hb, buf[1:].clone())
    ref, _ = nio.load_nii(hb, pl)
    assert np.array_equal(img, ref)


def test_fortran_ordered_tensor_saves_in_matlab_order(qn, nio, tmp_path):
    torch = pytest.importorskip("torch")
    chi = np.asfortranarray(np.random.default_rng(8).standard_normal((12, 10, 8)).astype(np.float32))
    f_tensor = torch.from_numpy(np.ascontiguousarray(chi.T)).cuda().permute(2, 1, 0)  # F-contiguous, MATLAB size
    c_tensor = torch.from_numpy(np.ascontiguousarray(chi.T)).cuda()     # C-contiguous, shape reversed
    for t, name in ((f_tensor, "f.nii"), (c_tensor, "c.nii")):
        qn.saveNii(str(tmp_path / name), t, [1, 1, 1])
        assert open(tmp_path / name, "rb").read() == nio.save_bytes(chi, [1, 1, 1])
    with pytest.raises(ValueError, match="contiguous"):
        qn.header_bytes(torch.zeros((6, 6, 6), device="cuda")[:, ::2, :])
