"""The C-ABI library builds, loads without a GPU, and exports every entry
point include/qsm_gpu.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "qsm_gpu.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qsm_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def built():
    import qsm_gb300.build as b

    return b.build()


def test_header_declares_boundary():
    names = declared()
    for must in ("qsm_pd_tgv", "qsm_pd_tv", "qsm_mgpcg", "qsm_gradf", "qsm_lap1", "qsm_lapw", "qsm_gauss_seidel"):
        assert must in names


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(built):
    from qsm_gb300 import _lib

    assert sorted(_lib.exported_symbols()) == declared()
    L = _lib.lib()
    assert L.qsm_abi_version() == _lib.ABI_VERSION == 2
    assert L.qsm_status_string(7) == b"nlevels too large. Increase MAX_DEPTH."


def test_context_fails_cleanly_without_gpu(built):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from qsm_gb300 import _lib

    with pytest.raises(_lib.QsmError):
        _lib.Context(0)


def test_ops_fail_loudly_without_library(monkeypatch, tmp_path):
    from qsm_gb300 import _lib

    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(_lib.QsmLibraryError):
        _lib.lib()


def test_build_flags_pin_arch_and_no_fma():
    import qsm_gb300.build as b

    flags = " ".join(b.NVCC_FLAGS)
    assert "arch=compute_103a,code=sm_103a" in flags
    assert "-fmad=false" in flags
    assert "-ffp-contract=off" in flags  # host-side constants, contracted by default on aarch64
    assert "use_fast_math" not in flags
