"""The thin C-MEX shims over the C ABI (qsm.m_gb300/mex/qsm_mex.c) compile for
every gateway with warnings as errors (types checked against the C ABI header
and a MATLAB-API header; MATLAB itself is not available to link them).  The
GPU test tests/test_gpu_mex_shims.py runs them."""
import os
import subprocess

import pytest

from conftest import ROOT

# the reference's 29 MEX gateways, then the whole MATLAB functions
GATEWAYS = ["PD_TGV", "PD_TV", "GRADF", "GRADB", "GRADC", "GRADFM", "GRADBM", "GRADCM", "GRADF_ADJ", "GRADB_ADJ",
            "GRADFM_ADJ", "GRADBM_ADJ", "GRADFP", "GRADFP_ADJ", "LAP1", "LAPW", "MGPCG", "MG", "FMG",
            "GAUSS_SEIDEL", "RESIDUAL", "LAPMG", "RESTRICT", "PROLONG", "CORRECT", "COARSEN_GRID", "BOUNDARY_MASK",
            "BOUNDARY_MASK_L1", "NORM2",
            "SSTGV", "LBV", "UNWRAP_LAPLACIAN", "SHARP", "VSHARP", "RESHARP", "ISMV", "PDF"]


def test_gateway_count():
    assert len(GATEWAYS) == 29 + 8


@pytest.mark.parametrize("gw", GATEWAYS)
def test_shim_compiles(gw, tmp_path):
    src = os.path.join(ROOT, "qsm.m_gb300", "mex", "qsm_mex.c")
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-O2", "-c", f"-DQSM_MEX_{gw}",
           "-I", os.path.join(ROOT, "oracle", "ref", "mexshim"), "-I", os.path.join(ROOT, "include"), src,
           "-o", str(tmp_path / f"{gw}.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
