"""The CPU restatement of tv.m (oracle/tv_admm.py): its k-space pieces
against independent formulas, and its u-subproblem against the normal
equations it solves.  (The loop itself is unpinned: no MATLAB here.)"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def tvo(port):
    import tv_admm
    return tv_admm


def test_laplace_symbol_matches_closed_form(tvo):
    sz, h = (12, 9, 7), (1.0, 0.8, 1.3)
    L = tvo.laplace_symbol(sz, h)
    i = np.indices(sz).astype(float)
    ref = sum((2.0 / h[a] ** 2) * (1 - np.cos(2 * np.pi * i[a] / sz[a])) for a in range(3))
    assert np.allclose(L, ref, rtol=0, atol=1e-13)


def test_dipole_kernel_matches_synthetic(tvo):
    from qsm_gb300 import synthetic
    sz, h = (16, 11, 10), (1.0, 1.0, 2.0)
    b = (0.2, 0.3, 0.9)
    D = tvo.dipole_kernel(sz, h, b)
    assert D[0, 0, 0] == 0.0
    assert np.allclose(D, synthetic.dipole_kernel(sz, h, b), rtol=0, atol=1e-15)


def test_u_subproblem_solves_normal_equations(tvo):
    """One u-update: (mu D^2 + rho L) u_hat = mu D f_hat + fft(r) wherever
    the operator is invertible (tv.m:172-175)."""
    rng = np.random.default_rng(0)
    sz = (10, 9, 8)
    f = np.asfortranarray(rng.standard_normal(sz))
    r = np.asfortranarray(rng.standard_normal(sz))
    mu, rho = 7.5e3, 9.0
    D = tvo.dipole_kernel(sz, (1, 1, 1))
    L = tvo.laplace_symbol(sz, (1, 1, 1))
    iA = tvo._inv(mu * D * D, L, rho)
    u = np.real(np.fft.ifftn(iA * (mu * D * np.fft.fftn(f) + np.fft.fftn(r))))
    lhs = (mu * D * D + rho * L) * np.fft.fftn(u)
    rhs = mu * D * np.fft.fftn(f) + np.fft.fftn(r)
    ok = (mu * D * D + rho * L) != 0
    assert np.allclose(lhs[ok], rhs[ok], rtol=1e-10, atol=1e-8)


def test_tv_reduces_residual_and_is_masked(tvo):
    from qsm_gb300 import synthetic
    sz = (24, 20, 16)
    m = synthetic.ellipsoid_mask(sz, (9, 8, 6))
    chi = np.zeros(sz)
    chi[8:14, 7:12, 5:10] = 0.1
    f = np.real(np.fft.ifftn(synthetic.dipole_kernel(sz) * np.fft.fftn(chi)))
    trace = []
    x = tvo.tv(f, m, [1, 1, 1], opts=dict(maxit=15), trace=trace)
    assert np.all(x[m == 0] == 0)
    assert trace[-1]["nr"] < trace[0]["nr"]
    err = np.linalg.norm((x - chi)[m != 0]) / np.linalg.norm(chi[m != 0])
    assert err < 0.9
