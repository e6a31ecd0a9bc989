"""The thin C-MEX shims over the C ABI (qsm.m_gb300/mex/qsm_mex.c) compile for
every gateway (syntax and types checked against the C ABI header; MATLAB is
not available to link them)."""
import os
import subprocess

import pytest

from conftest import ROOT

GATEWAYS = ["PD_TGV", "PD_TV", "GRADF", "GRADB", "GRADC", "GRADFM", "GRADBM", "GRADCM", "GRADF_ADJ", "GRADB_ADJ",
            "GRADFM_ADJ", "GRADBM_ADJ", "GRADFP", "GRADFP_ADJ", "LAP1", "LAPW", "MGPCG", "MG", "FMG"]


@pytest.mark.parametrize("gw", GATEWAYS)
def test_shim_compiles(gw):
    src = os.path.join(ROOT, "qsm.m_gb300", "mex", "qsm_mex.c")
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", f"-DQSM_MEX_{gw}",
           "-I", os.path.join(ROOT, "oracle", "ref", "mexshim"), "-I", os.path.join(ROOT, "include"), src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
