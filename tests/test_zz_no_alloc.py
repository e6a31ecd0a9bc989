"""qsm_norm2_noalloc through the C ABI: the allocation-free masked 2-norm
for callers that must not let the library allocate device memory (a MATLAB
session lending its own gpuArray memory, pipelines that allocate only at
start-up).  Its result must match the allocating entry point qsm_norm2 on
two calls in a row -- the second call reuses the library's fixed scratch
array that the first one left behind -- and sizes beyond the documented
maximum must be rejected.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

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
        assert got == pytest.approx(want, rel=1e-12, abs=0.0)


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
