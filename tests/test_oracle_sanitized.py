"""The CPU oracle under AddressSanitizer and UndefinedBehaviorSanitizer: the
oracle's C (oracle/qsm_oracle.c) is built with -fsanitize=address,undefined
and no recovery, and the golden-vector tests (tests/test_oracle_golden.py:
every operator, both solvers, the multigrid pieces and solvers on their
fixtures, in FP32 and FP64) run against that build in a child process with
the ASan runtime preloaded.  Any out-of-bounds access, use of freed memory,
overflow or other undefined behaviour aborts the child and fails the test.
The CUDA kernels have no such tool on the GPU pool; the oracle they are
checked against does."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT


def _runtime(name):
    try:
        p = subprocess.run(["gcc", f"-print-file-name={name}"], capture_output=True, text=True, check=True).stdout
    except (OSError, subprocess.CalledProcessError):
        return None
    p = p.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


def test_oracle_golden_under_sanitizers(tmp_path):
    asan = _runtime("libasan.so")
    if asan is None or _runtime("libubsan.so") is None:
        pytest.skip("the gcc sanitizer runtimes are not installed")
    lib = tmp_path / "liborc_san.so"
    src = os.path.join(ROOT, "oracle", "qsm_oracle.c")
    subprocess.run(["gcc", "-std=c11", "-O1", "-g", "-fno-omit-frame-pointer", "-ffp-contract=off", "-fopenmp", "-fPIC",
                    "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-shared", "-o", str(lib), src, "-lm"],
                   check=True, capture_output=True)
    env = dict(os.environ, QSM_ORACLE_LIB=str(lib), LD_PRELOAD=asan, OMP_NUM_THREADS="4",
               ASAN_OPTIONS="detect_leaks=0:abort_on_error=1", UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    r = subprocess.run([sys.executable, "-m", "pytest", os.path.join(ROOT, "tests", "test_oracle_golden.py"), "-q",
                        "-x", "-p", "no:cacheprovider"], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    assert "passed" in r.stdout
    # the child really loaded the sanitized build
    chk = subprocess.run([sys.executable, "-c", "import sys; sys.path.insert(0, 'oracle'); import port; "
                          "port.lib(); print(port.LIB_PATH)"], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=120)
    assert chk.returncode == 0 and chk.stdout.strip() == str(lib), (chk.stdout, chk.stderr)


def test_sanitizer_build_catches_a_planted_overflow(tmp_path):
    """The same build and loading recipe on a C function that reads one
    element past a heap buffer (a mistake planted here, on the CPU): the child
    must abort with a sanitizer report, so a clean oracle run above means
    something."""
    asan = _runtime("libasan.so")
    if asan is None:
        pytest.skip("the gcc sanitizer runtimes are not installed")
    src = tmp_path / "planted.c"
    src.write_text("#include <stdlib.h>\n"
                   "double planted(int n) { double *a = malloc(n * sizeof(double)); double s = 0;\n"
                   "  for (int i = 0; i <= n; ++i) s += a[i];\n"
                   "  free(a); return s; }\n")
    lib = tmp_path / "libplanted.so"
    subprocess.run(["gcc", "-O1", "-g", "-fPIC", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
                    "-shared", "-o", str(lib), str(src)], check=True, capture_output=True)
    env = dict(os.environ, LD_PRELOAD=asan, ASAN_OPTIONS="detect_leaks=0:abort_on_error=1")
    code = ("import ctypes; L = ctypes.CDLL(%r); L.planted.restype = ctypes.c_double; "
            "L.planted.argtypes = [ctypes.c_int]; L.planted(8)" % str(lib))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=120)
    # whichever sanitizer sees it first (the object-size check of UBSan, or ASan) reports and aborts
    assert r.returncode != 0 and ("AddressSanitizer" in r.stderr or "runtime error" in r.stderr), \
        (r.returncode, r.stderr[-2000:])
