"""qsm_norm2_noalloc through the C ABI: the allocation-free masked 2-norm
for callers that must not let the library allocate device memory (a MATLAB
session lending its own gpuArray memory, pipelines that allocate only at
start-up).  Its result must equal the allocating entry point qsm_norm2 bit
for bit on two calls in a row -- the second call reuses the library's fixed
scratch array that the first one left behind -- and the reference MEX's
golden norm2 values; the largest documented size must work, sizes beyond it
must be rejected, and a device reset (a new CUDA context, as MATLAB's
reset(gpuDevice) makes) must not leave the entry point writing through the
old context's scratch address.  This file is collected last on purpose."""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
QSM_OK, QSM_ERR_DIMS = 0, 2
MAX_N = 1 << 25


@pytest.fixture(scope="module")
def capi():
    torch = pytest.importorskip("torch")
    import qsm_gb300.build as b

    L = ctypes.CDLL(b.build())
    L.qsm_norm2_noalloc.argtypes = [ctypes.c_int32, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p]
    L.qsm_norm2_noalloc.restype = ctypes.c_int
    L.qsm_ctx_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    L.qsm_ctx_create.restype = ctypes.c_int
    L.qsm_ctx_destroy.argtypes = [ctypes.c_void_p]
    L.qsm_norm2.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                            ctypes.POINTER(ctypes.c_double)]
    L.qsm_norm2.restype = ctypes.c_int
    ctx = ctypes.c_void_p()
    assert L.qsm_ctx_create(0, ctypes.byref(ctx)) == QSM_OK
    yield L, ctx, torch
    L.qsm_ctx_destroy(ctx)


def _existing(L, ctx, dt, x, g):
    # qsm_norm2 runs on the context's own stream: torch's writes of x and g
    # must be complete first
    import torch

    torch.cuda.current_stream().synchronize()
    out = ctypes.c_double()
    st = L.qsm_norm2(ctx, dt, x.numel(), ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(g.data_ptr()),
                     ctypes.byref(out))
    assert st == QSM_OK
    return out.value


def _noalloc(L, torch, dt, x, g):
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    st = L.qsm_norm2_noalloc(dt, x.numel(), ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(g.data_ptr()),
                             ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert st == QSM_OK
    stream.synchronize()
    return float(out.item())


@pytest.mark.parametrize("dt", [0, 1])
def test_noalloc_matches_existing_twice(capi, dt):
    L, ctx, torch = capi
    tdt = torch.float64 if dt == 0 else torch.float32
    gen = torch.Generator(device="cuda").manual_seed(1234 + dt)
    # two different sizes in a row: the second call must not depend on what
    # the first left in the shared scratch array
    for n in (3_000_017, 777_777):
        x = torch.randn(n, generator=gen, device="cuda", dtype=tdt)
        g = (torch.rand(n, generator=gen, device="cuda") > 0.3).to(torch.uint8)
        want = _existing(L, ctx, dt, x, g)
        got = _noalloc(L, torch, dt, x, g)
        assert got == want  # the same pairwise tree: bit for bit


def test_noalloc_reference_golden(capi):
    """The reference norm2_mex's own outputs (tests/golden/mg_ops.npz)."""
    L, ctx, torch = capi
    gold = np.load(os.path.join(ROOT, "tests", "golden", "mg_ops.npz"))
    for si in range(3):
        xn = gold[f"s{si}_xn"]
        gb = gold[f"s{si}_Gb"]
        x = torch.from_numpy(np.ascontiguousarray(xn.ravel(order="F"))).cuda()
        g = torch.from_numpy(np.ascontiguousarray(gb.ravel(order="F"))).cuda()
        assert _noalloc(L, torch, 0, x, g) == float(gold[f"s{si}_norm2"])


@pytest.mark.parametrize("dt", [0, 1])
def test_noalloc_at_size_limit(capi, dt):
    """n = QSM_NORM2_NOALLOC_MAX_N fills the scratch array's deepest tree."""
    L, ctx, torch = capi
    tdt = torch.float64 if dt == 0 else torch.float32
    gen = torch.Generator(device="cuda").manual_seed(77 + dt)
    x = torch.randn(MAX_N, generator=gen, device="cuda", dtype=tdt)
    g = (torch.rand(MAX_N, generator=gen, device="cuda") > 0.5).to(torch.uint8)
    want = _existing(L, ctx, dt, x, g)
    assert _noalloc(L, torch, dt, x, g) == want
    assert _noalloc(L, torch, dt, x, g) == want
    del x, g
    torch.cuda.empty_cache()


def test_noalloc_small_and_limits(capi):
    L, ctx, torch = capi
    for n in (1, 128, 129, 4097):
        x = torch.arange(1, n + 1, dtype=torch.float64, device="cuda")
        g = torch.ones(n, dtype=torch.uint8, device="cuda")
        got = _noalloc(L, torch, 0, x, g)
        assert got == pytest.approx(float(np.sqrt(np.sum(np.arange(1, n + 1, dtype=np.float64) ** 2))), rel=1e-12)
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    g = torch.ones(8, dtype=torch.uint8, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = [ctypes.c_void_p(t.data_ptr()) for t in (x, g, out)]
    assert L.qsm_norm2_noalloc(0, MAX_N + 1, p[0], p[1], p[2], None) == QSM_ERR_DIMS
    assert L.qsm_norm2_noalloc(0, 0, p[0], p[1], p[2], None) == QSM_ERR_DIMS


# A child process (no torch) allocates with the CUDA runtime itself, calls
# the entry point, resets the device -- which destroys the context and the
# library's scratch array with it -- and calls it again on fresh buffers.
_RESET_CHILD = r"""
import ctypes, json, sys
import numpy as np
L = ctypes.CDLL(sys.argv[1])
rt = ctypes.CDLL("libcudart.so.13")
P = ctypes.c_void_p
L.qsm_norm2_noalloc.argtypes = [ctypes.c_int32, ctypes.c_size_t, P, P, P, P]
rt.cudaMalloc.argtypes = [ctypes.POINTER(P), ctypes.c_size_t]
rt.cudaMemcpy.argtypes = [P, P, ctypes.c_size_t, ctypes.c_int]
rt.cudaFree.argtypes = [P]
rng = np.random.default_rng(5)
n = 1_000_003
x = rng.standard_normal(n)
g = (rng.random(n) > 0.4).astype(np.uint8)
res = []
for call in range(2):
    bufs = [P(), P(), P()]
    for b, nb in zip(bufs, (x.nbytes, g.nbytes, 8)):
        assert rt.cudaMalloc(ctypes.byref(b), nb) == 0
    assert rt.cudaMemcpy(bufs[0], x.ctypes.data, x.nbytes, 1) == 0
    assert rt.cudaMemcpy(bufs[1], g.ctypes.data, g.nbytes, 1) == 0
    st = L.qsm_norm2_noalloc(0, n, bufs[0], bufs[1], bufs[2], None)
    out = np.zeros(1)
    cp = rt.cudaMemcpy(out.ctypes.data, bufs[2], 8, 2)
    res.append({"status": st, "copy": cp, "value": float(out[0])})
    for b in bufs:
        rt.cudaFree(b)
    if call == 0:
        res.append({"reset": rt.cudaDeviceReset()})
print(json.dumps(res))
"""


def test_noalloc_after_device_reset(capi):
    L, ctx, torch = capi
    import qsm_gb300.build as b

    r = subprocess.run([sys.executable, "-c", _RESET_CHILD, b.build()], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    first, reset, second = json.loads(r.stdout.strip().splitlines()[-1])
    assert reset["reset"] == 0
    assert first["status"] == QSM_OK and second["status"] == QSM_OK
    assert first["copy"] == 0 and second["copy"] == 0
    rng = np.random.default_rng(5)
    n = 1_000_003
    x = torch.from_numpy(rng.standard_normal(n)).cuda()
    g = torch.from_numpy((rng.random(n) > 0.4).astype(np.uint8)).cuda()
    want = _existing(L, ctx, 0, x, g)
    assert first["value"] == want
    assert second["value"] == want
