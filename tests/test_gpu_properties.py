"""The reference's own multigrid and operator properties, as assertions on
the GPU path.

QSM.m's Poisson-solver test scripts print residual and error histories
without asserting anything (src/utils/poisson_solver/test/
testMultigridPoisson.m, testPoissonSolvers.m).  Their properties are
restated here and checked through the library's gateways:

  * relaxation leaves the exact discrete solution fixed
    (testMultigridPoisson.m:241-296): forward and reverse red-black sweeps,
    n = 15, 16, 127, 128;
  * a V-cycle built from the level operators leaves it fixed too
    (:162-238): n = 31, 32, 126, 127;
  * the V-cycle's residual reduction per cycle on the sin*sin*sin model
    problem stays below the red-black smoothing factor 0.567 quoted in the
    script (:26-79);
  * MG, FMG and MG-PCG solve the model problem to their tolerance with
    second-order discretisation error, n = 63, 127, 255, 64, 128, 256
    (testPoissonSolvers.m:6-102);
  * the periodic gradient and its adjoint (gradfp_mex.c, gradfp_adj_mex.c)
    satisfy <grad u, p> = <u, grad^T p> to rounding.

Where the oracle finishes in seconds the GPU result is also compared with it
bit for bit."""
import numpy as np
import pytest

from conftest import bits_equal, first_diff

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def L2(u):
    return float(np.linalg.norm(np.ravel(u)) / np.sqrt(np.size(u)))


def model_problem(n, p=2 * np.pi):
    """u = sin(pX) sin(pY) sin(pZ) on the (n+1)^3 grid of [0, 1]^3, G its
    interior, f = -Delta u = 3 p^2 u (testPoissonSolvers.m:105-122)."""
    x = np.linspace(0.0, 1.0, n + 1)
    s = np.sin(p * x)
    u = np.asfortranarray(s[:, None, None] * s[None, :, None] * s[None, None, :])
    G = np.zeros(u.shape, np.uint8, order="F")
    G[1:-1, 1:-1, 1:-1] = 1
    f = np.asfortranarray(3 * p * p * u)
    return u, G, f


def residual(qsm, f, v, G, h):
    r = np.zeros_like(f, order="F")
    qsm.residual_mex(r, f, v, G, h)
    return r


def neg_lap(qsm, V, G, h):
    d = np.zeros_like(V, order="F")
    qsm.lapmg_mex(d, V, G, h)
    return np.asfortranarray(-d)


@pytest.mark.parametrize("rev", [0, 1])
@pytest.mark.parametrize("n", [15, 16, 127, 128])
def test_relaxation_fixed_point(gpu_ctx, qsm, port, n, rev):
    rng = np.random.default_rng(n + 7 * rev)
    h = [1.0 / n] * 3
    G = np.ones((n + 1,) * 3, np.uint8, order="F")
    V = np.asfortranarray(rng.standard_normal((n + 1,) * 3))
    f = neg_lap(qsm, V, G, h)
    v = V.copy(order="F")
    assert L2(residual(qsm, f, v, G, h)) <= 1e-12 * L2(f)
    qsm.gauss_seidel_mex(v, f, G, h, 100, rev)
    assert L2(v - V) <= 1e-11 * L2(V)
    assert L2(residual(qsm, f, v, G, h)) <= 1e-11 * L2(f)
    if n <= 16:
        w = V.copy(order="F")
        port.gauss_seidel_mex(w, f, G, h, 100, rev)
        assert bits_equal(v, w), first_diff(v, w)


def _coarsen(qsm, G):
    G2 = np.zeros(tuple((s - 2 + 1) // 2 + 2 for s in G.shape), np.uint8, order="F")
    qsm.coarsen_grid_mex(G2, G)
    return G2


@pytest.mark.parametrize("n", [31, 32, 126, 127])
def test_vcycle_fixed_point(gpu_ctx, qsm, n):
    rng = np.random.default_rng(100 + n)
    sz = n + 1
    G0 = np.zeros((sz + 2,) * 3, np.uint8, order="F")
    G0[1:-1, 1:-1, 1:-1] = 1
    V = np.asfortranarray(G0 * rng.standard_normal(G0.shape))
    h = np.array([1.0 / n] * 3)
    f = [neg_lap(qsm, V, G0, h)]
    v = [V.copy(order="F")]
    G = [G0]
    nlevels = int(np.floor(np.log2(n))) - 2
    for lv in range(nlevels):
        hl = 2.0 ** lv * h
        qsm.gauss_seidel_mex(v[lv], f[lv], G[lv], hl, 3, 0)
        r = residual(qsm, f[lv], v[lv], G[lv], hl)
        G.append(_coarsen(qsm, G[lv]))
        f2 = np.zeros(G[-1].shape, np.float64, order="F")
        qsm.restrict_mex(f2, r, G[-1])
        f.append(f2)
        v.append(np.zeros(G[-1].shape, np.float64, order="F"))
    hc = 2.0 ** nlevels * h
    qsm.gauss_seidel_mex(v[-1], f[-1], G[-1], hc, 2500, 0)
    qsm.gauss_seidel_mex(v[-1], f[-1], G[-1], hc, 2500, 1)
    for lv in range(nlevels - 1, -1, -1):
        qsm.correct_mex(v[lv], v[lv + 1], G[lv])
        qsm.gauss_seidel_mex(v[lv], f[lv], G[lv], 2.0 ** lv * h, 3, 1)
    assert L2(v[0] - V) <= 1e-10 * L2(V)


def _levels(n):
    return max(1, int(np.floor(np.log2(n + 1))) - 3)


@pytest.mark.parametrize("n", [64, 128, 256])
def test_vcycle_reduction_factor(gpu_ctx, qsm, n):
    """One V-cycle at a time (mu 1, one pre- and one post-sweep, two boundary
    sweeps): the residual falls by at least the smoothing factor 0.567 per
    cycle (about 0.24 per cycle at these sizes)."""
    u, G, f = model_problem(n)
    h = [1.0 / n] * 3
    v = np.zeros_like(f, order="F")
    res = [L2(residual(qsm, f, v, G, h))]
    for _ in range(6):
        v = qsm.mg_mex(v, f, G, h, 0.0, 1, 1, 1, 1, 2, _levels(n))
        res.append(L2(residual(qsm, f, v, G, h)))
    ratios = [res[k + 1] / res[k] for k in range(len(res) - 1)]
    assert max(ratios) <= 0.567, ratios


@pytest.mark.parametrize("n", [63, 127, 255, 64, 128, 256])
def test_poisson_solvers_model_problem(gpu_ctx, qsm, port, n):
    u, G, f = model_problem(n)
    h = [1.0 / n] * 3
    nl = _levels(n)
    tol = float(np.sqrt(EPS))
    z = np.zeros_like(f, order="F")
    v_mg = qsm.mg_mex(z, f, G, h, tol, max(f.shape), 1, 1, 1, 2, nl)
    v_fmg = qsm.fmg_mex(f, G, h, tol, 1, 1, 1, 1, 2, nl)
    info = {}
    v_pcg = qsm.mgpcg_mex(z, f, G, h, tol, f.size, -1.0, 1, 1, 1, 1, 2, nl, info=info)
    nf = L2(f)
    for v in (v_mg, v_pcg):
        assert L2(residual(qsm, f, v, G, h)) <= 10 * tol * nf
    e_pcg = L2(v_pcg - u) / L2(u)
    e_mg = L2(v_mg - u) / L2(u)
    e_fmg = L2(v_fmg - u) / L2(u)
    # MG and MG-PCG converge to the same discrete solution; one FMG pass
    # reaches the discretisation error
    assert abs(e_mg - e_pcg) <= 1e-3 * e_pcg
    assert e_fmg <= 2.0 * e_pcg
    # second order: the 7-point stencil's symbol on sin(p x) is off by
    # about (p h)^2 / 12, so the discrete solution's relative error is too
    assert 0.07 < e_pcg * n * n / (2 * np.pi) ** 2 < 0.1, e_pcg
    if n <= 64:
        assert bits_equal(v_mg, port.mg_mex(z, f, G, h, tol, max(f.shape), 1, 1, 1, 2, nl))
        assert bits_equal(v_fmg, port.fmg_mex(f, G, h, tol, 1, 1, 1, 1, 2, nl))
        oi = {}
        ref = port.mgpcg_mex(z, f, G, h, tol, f.size, -1.0, 1, 1, 1, 1, 2, nl, info=oi)
        assert info["iters"] == oi["iters"]
        assert bits_equal(v_pcg, ref), first_diff(v_pcg, ref)


@pytest.mark.parametrize("shape,h", [((13, 10, 7), [1, 0.9, 1.3]), ((64, 48, 40), [1, 1, 1]),
                                     ((97, 33, 65), [0.5, 1, 2])])
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_periodic_gradient_adjoint_identity(gpu_ctx, qsm, shape, h, dt):
    rng = np.random.default_rng(sum(shape))
    u = np.asfortranarray(rng.standard_normal(shape).astype(dt))
    p = [np.asfortranarray(rng.standard_normal(shape).astype(dt)) for _ in range(3)]
    g = [np.zeros(shape, dt, order="F") for _ in range(3)]
    qsm.gradfp_mex(*g, u, h)
    du = np.zeros(shape, dt, order="F")
    qsm.gradfp_adj_mex(du, *p, h)
    a = sum(np.vdot(g[i].astype(np.float64), p[i].astype(np.float64)) for i in range(3))
    b = np.vdot(u.astype(np.float64), du.astype(np.float64))
    scale = sum(np.vdot(np.abs(g[i]).astype(np.float64), np.abs(p[i]).astype(np.float64)) for i in range(3))
    tol = 64 * np.finfo(dt).eps
    assert abs(a - b) <= tol * scale, (a, b)
