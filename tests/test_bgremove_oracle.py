"""The CPU restatement of the FFT background removal (oracle/bgremove.py):
padfastfft / nextfastfft sizes, the SMV kernel, and the defining property of
SHARP-type filtering: a harmonic background inside the mask is removed."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def bg(port):
    import bgremove
    return bgremove


def test_next_fast_and_padding(bg):
    assert [bg.next_fast(n) for n in (1, 11, 13, 17, 97, 121, 1000)] == [1, 12, 14, 18, 98, 125, 1000]
    # 11 + 2*3 -> 18: an odd total of 7, the extra zero before an odd size;
    # 12 + 6 = 18 is 7-smooth: 3 + 3; 20 + 6 -> 27: 7, the extra zero after an even size
    assert bg.pad_offsets((11, 12, 20), 3) == [(4, 3), (3, 3), (3, 4)]
    u = np.random.default_rng(0).standard_normal((11, 12, 7))
    p = bg.padfast(u, 3)
    assert all(bg.next_fast(n) == n for n in p.shape)
    assert np.array_equal(bg.unpadfast(p, u.shape, 3), u)


def test_smv_kernel_is_a_normalised_sphere(bg):
    k = bg.smv_kernel((20, 21, 22), 3.0, (1.0, 1.0, 1.0))
    assert abs(k.sum() - 1.0) < 1e-15 and k[10, 10, 11] > 0 and k[10, 10, 15] == 0
    H = np.fft.fftn(np.fft.ifftshift(k))
    assert np.max(np.abs(H.imag)) < 1e-12  # real and even


def test_sharp_removes_a_harmonic_background(bg):
    from qsm_gb300 import synthetic
    shape = (40, 38, 36)
    m = synthetic.ellipsoid_mask(shape, (15, 14, 13))
    g = np.indices(shape).astype(float)
    f = np.asfortranarray(0.3 * g[0] - 0.2 * g[1] + 0.1 * g[2])  # harmonic (linear)
    for fl, mo in (bg.sharp(f, m, [1, 1, 1], r=4), bg.vsharp(f, m, [1, 1, 1], rs=[5, 4, 3])):
        inside = mo != 0
        assert inside.sum() > 1000 and np.all(m[inside])
        assert np.linalg.norm(fl[inside]) < 1e-3 * np.linalg.norm(f[inside])
    fl, mo = bg.ismv(f, m, [1, 1, 1], r=3, maxit=300)
    inside = mo != 0
    assert np.linalg.norm(fl[inside]) < 0.05 * np.linalg.norm(f[inside])


def test_lsmr_solves_damped_least_squares(bg):
    """The LSMR restatement reaches the damped least-squares solution of a small
    dense system (normal equations solved directly)."""
    rng = np.random.default_rng(3)
    A = rng.normal(size=(60, 40))
    b = rng.normal(size=60)
    for lam in (0.0, 0.5):
        x, it = bg.lsmr(lambda v: A @ v, lambda v: A.T @ v, b, lam, 1e-12, 1e-12, 1e8, 200)
        ref = np.linalg.solve(A.T @ A + lam * lam * np.eye(40), A.T @ b)
        assert np.linalg.norm(x - ref) <= 1e-8 * np.linalg.norm(ref) and 0 < it <= 200


def test_lsmr_zero_rhs(bg):
    x, it = bg.lsmr(lambda v: v, lambda v: v, np.zeros(5))
    assert it == 0 and not x.any()


def test_dipole_kernel_image_space(bg):
    """dipoleKernel 'i': zero at the centre, even in r, and its transform is real
    (within roundoff, so psf2otf drops the imaginary part) when B is along an axis."""
    D = bg.dipole_kernel_i((9, 8, 7), (1.0, 1.0, 1.0))
    assert D[4, 4, 3] == 0.0
    assert D[4, 4, 4] == pytest.approx(2.0 / (4 * np.pi))
    assert D[5, 4, 3] == pytest.approx(-1.0 / (4 * np.pi))
    K = bg.psf2otf(D)
    assert not K.imag.any()
    Ko = bg.psf2otf(bg.dipole_kernel_i((9, 8, 7), (1.0, 1.0, 1.0), (0.0, 0.3, 1.0)))
    assert np.abs(Ko.imag).max() > 1e-6
