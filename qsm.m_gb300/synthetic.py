"""Seeded synthetic QSM inputs (numpy, FP64).

The reference measures on no public data set; these generators stand in for
scanner data with the shapes, sizes and value ranges of the benchmark
configurations:

* ``tgv_case(...)``: ellipsoid susceptibility phantom chi, a local field
  phi = real(ifftn(D * fftn(chi))) + noise with the k-space unit dipole
  D(k) = 1/3 - (k.b)^2 / |k|^2, D(0) = 0 (src/utils/kernels/dipoleKernel.m:56-65,
  B0 along z), and the TGV/TV right-hand side d2f = -lapw(phi)
  (src/inversion/sstgv.m:79-83);
* ``poisson_case(...)``: a smooth field (sum of Gaussians) inside a random
  ellipsoidal mask and f = -Delta_h u on the mask (the LBV / Laplacian
  unwrapping form of src/bgremove/lbv.m:108-113).

Volumes are MATLAB-ordered: shape (nx, ny, nz), Fortran order.
"""
from __future__ import annotations

import numpy as np


def dipole_kernel(shape, vsz=(1.0, 1.0, 1.0), bdir=(0.0, 0.0, 1.0)) -> np.ndarray:
    """k-space unit dipole response in FFT (ifftshifted) order."""
    k = [np.fft.fftfreq(n, d=h) for n, h in zip(shape, vsz)]
    kx, ky, kz = np.meshgrid(*k, indexing="ij")
    b = np.asarray(bdir, dtype=np.float64)
    b = b / np.linalg.norm(b)
    kb = b[0] * kx + b[1] * ky + b[2] * kz
    k2 = kx * kx + ky * ky + kz * kz
    with np.errstate(divide="ignore", invalid="ignore"):
        D = 1.0 / 3.0 - (kb * kb) / k2
    D[0, 0, 0] = 0.0
    return D


def sphere_mask(shape, radius, centre=None) -> np.ndarray:
    c = [(n - 1) / 2 for n in shape] if centre is None else centre
    g = np.ogrid[0:shape[0], 0:shape[1], 0:shape[2]]
    r2 = sum((g[i] - c[i]) ** 2 for i in range(3))
    return np.asfortranarray(r2 <= radius * radius).astype(np.uint8, order="F")


def ellipsoid_mask(shape, semi, centre=None) -> np.ndarray:
    c = [(n - 1) / 2 for n in shape] if centre is None else centre
    g = np.ogrid[0:shape[0], 0:shape[1], 0:shape[2]]
    q = sum(((g[i] - c[i]) / semi[i]) ** 2 for i in range(3))
    return np.asfortranarray(q <= 1.0).astype(np.uint8, order="F")


def ellipsoid_phantom(shape, count, rng, mask, semi=(4.0, 16.0), chi=(-0.1, 0.1)) -> np.ndarray:
    """Axis-aligned ellipsoids, centres uniform over the mask's voxels,
    semi-axes U[semi], values U[chi]; later ellipsoids overwrite earlier."""
    vol = np.zeros(shape, dtype=np.float64, order="F")
    idx = np.argwhere(mask != 0)
    for _ in range(count):
        c = idx[rng.integers(len(idx))].astype(np.float64) + rng.uniform(-0.5, 0.5, 3)
        a = rng.uniform(semi[0], semi[1], 3)
        val = rng.uniform(chi[0], chi[1])
        lo = [max(0, int(np.floor(c[i] - a[i]))) for i in range(3)]
        hi = [min(shape[i], int(np.ceil(c[i] + a[i])) + 1) for i in range(3)]
        g = np.ogrid[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
        q = sum(((g[i] - c[i]) / a[i]) ** 2 for i in range(3))
        sub = vol[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
        sub[q <= 1.0] = val
    return vol


def _wrap(x):
    out = x.copy()
    w = (x < -np.pi) | (x > np.pi)
    y = x[w] + np.pi
    out[w] = np.where(y < 0, np.fmod(y, 2 * np.pi) + np.pi, np.fmod(y, 2 * np.pi) - np.pi)
    return out


def lapw(u, vsz=(1.0, 1.0, 1.0)) -> np.ndarray:
    """Laplacian of a wrapped phase on the interior (faces stay 0)."""
    d = np.zeros_like(u)
    c = (slice(1, -1),) * 3
    for ax in range(3):
        hp = [slice(1, -1)] * 3
        hm = [slice(1, -1)] * 3
        hp[ax] = slice(2, None)
        hm[ax] = slice(0, -2)
        uf = _wrap(u[tuple(hp)] - u[c])
        ub = _wrap(u[c] - u[tuple(hm)])
        d[c] += (1.0 / (vsz[ax] * vsz[ax])) * (uf - ub)
    return d


def lap7(u, mask, vsz=(1.0, 1.0, 1.0)) -> np.ndarray:
    """7-point Laplacian on the interior voxels of the mask (0 elsewhere)."""
    d = np.zeros_like(u)
    c = (slice(1, -1),) * 3
    acc = np.zeros_like(u[c])
    for ax in range(3):
        hp = [slice(1, -1)] * 3
        hm = [slice(1, -1)] * 3
        hp[ax] = slice(2, None)
        hm[ax] = slice(0, -2)
        acc += (1.0 / (vsz[ax] * vsz[ax])) * (u[tuple(hp)] - 2.0 * u[c] + u[tuple(hm)])
    d[c] = np.where(mask[c] != 0, acc, 0.0)
    return d


def tgv_case(shape, seed, *, n_ell=12, chi=(-0.1, 0.1), noise=0.01, mask=None, semi=(4.0, 16.0),
             vsz=(1.0, 1.0, 1.0)):
    """Returns (d2f, mask, chi_true) for a TGV/TV inversion."""
    rng = np.random.default_rng(seed)
    if mask is None:
        mask = sphere_mask(shape, min(shape) / 2 - 4)
    chi_true = ellipsoid_phantom(shape, n_ell, rng, mask, semi=semi, chi=chi)
    D = dipole_kernel(shape, vsz)
    phi = np.real(np.fft.ifftn(D * np.fft.fftn(chi_true)))
    phi = phi + rng.normal(0.0, noise, shape)
    d2f = np.asfortranarray(-lapw(np.asfortranarray(phi), vsz))
    return d2f, mask, chi_true


def config0(seed=0):
    """64^3, 12 ellipsoids (semi-axes U[4,16], chi U[-0.1,0.1] ppm) in a
    sphere of radius 28 centred at (32,32,32), noise 0.01 ppm."""
    shape = (64, 64, 64)
    mask = sphere_mask(shape, 28.0, centre=(32.0, 32.0, 32.0))
    return tgv_case(shape, seed, n_ell=12, chi=(-0.1, 0.1), noise=0.01, mask=mask)


def config2(seed=2):
    """224x224x128, 60 ellipsoids (chi U[-0.15,0.15] ppm) inside an
    ellipsoidal brain mask with semi-axes (94, 94, 54), noise 0.02 ppm."""
    shape = (224, 224, 128)
    mask = ellipsoid_mask(shape, (94.0, 94.0, 54.0))
    return tgv_case(shape, seed, n_ell=60, chi=(-0.15, 0.15), noise=0.02, mask=mask)


def config3_sizes(seed=3, count=32):
    """Volume sizes of the batched TV configuration: each axis uniform over
    {96..256}, {96..256}, {64..176} in steps of 16."""
    rng = np.random.default_rng(seed)
    sx = rng.choice(np.arange(96, 257, 16), count)
    sy = rng.choice(np.arange(96, 257, 16), count)
    sz = rng.choice(np.arange(64, 177, 16), count)
    return [(int(a), int(b), int(c)) for a, b, c in zip(sx, sy, sz)]


def poisson_case(shape, seed, *, n_gauss=40, sigma=(5.0, 30.0), semi=(80.0, 120.0), jitter=8.0,
                 vsz=(1.0, 1.0, 1.0)):
    """Returns (f, mask, u_true): u = sum of n_gauss Gaussians, mask a random
    ellipsoid (semi-axes U[semi] clipped to the grid, centre jittered), and
    f = -Delta_h u on the mask."""
    rng = np.random.default_rng(seed)
    g = [np.arange(n, dtype=np.float64) for n in shape]
    ex = [np.empty((n_gauss, n)) for n in shape]
    for t in range(n_gauss):
        c = [rng.uniform(0, n - 1) for n in shape]
        s = rng.uniform(sigma[0], sigma[1])
        a = rng.uniform(-1.0, 1.0)
        for i in range(3):
            ex[i][t] = np.exp(-((g[i] - c[i]) ** 2) / (2 * s * s))
        ex[0][t] *= a
    # u[i,j,k] = sum_t ex0[t,i] ex1[t,j] ex2[t,k], as one contraction
    xy = np.einsum("ti,tj->tji", ex[0], ex[1]).reshape(n_gauss, -1)   # (t, j*nx + i)
    u = np.asfortranarray((ex[2].T @ xy).reshape(shape[2], shape[1], shape[0]).transpose(2, 1, 0))
    ctr = [(n - 1) / 2 + rng.uniform(-jitter, jitter) for n in shape]
    sa = [min(rng.uniform(semi[0], semi[1]), (n - 1) / 2 - 2) for n in shape]
    mask = ellipsoid_mask(shape, sa, centre=ctr)
    f = np.asfortranarray(-lap7(u, mask, vsz))
    return f, mask, u


def config1(seed=1):
    """256^3 Poisson problem of the LBV / Laplacian-unwrapping form."""
    return poisson_case((256, 256, 256), seed)


def field_case(shape, seed, *, echoes=1, n_ell=60, chi=(-0.15, 0.15), noise=0.01, mask=None,
               vsz=(1.0, 1.0, 1.0)):
    """Returns (f, local, mask): a total field f = (local + background) inside the
    mask for background-field removal and the MATLAB wrappers.  local is the
    dipole field of an ellipsoid phantom (as in tgv_case); the background is the
    harmonic field of four point sources outside the grid (1/r, scaled to ~10x
    the local field), growing by echo (echo t multiplies everything by t + 1).
    f is (nx, ny, nz) for one echo, else (nx, ny, nz, echoes); Fortran order."""
    rng = np.random.default_rng(seed)
    if mask is None:
        mask = ellipsoid_mask(shape, [0.42 * n for n in shape])
    chi_true = ellipsoid_phantom(shape, n_ell, rng, mask, chi=chi)
    local = np.real(np.fft.ifftn(dipole_kernel(shape, vsz) * np.fft.fftn(chi_true)))
    g = np.meshgrid(*[np.arange(n, dtype=np.float64) * h for n, h in zip(shape, vsz)], indexing="ij")
    ext = [n * h for n, h in zip(shape, vsz)]
    bg = np.zeros(shape)
    for _ in range(4):
        ax = int(rng.integers(0, 3))
        c = [float(rng.uniform(0.2, 0.8)) * e for e in ext]
        c[ax] = -0.25 * ext[ax] if rng.random() < 0.5 else 1.25 * ext[ax]
        r = np.sqrt((g[0] - c[0]) ** 2 + (g[1] - c[1]) ** 2 + (g[2] - c[2]) ** 2)
        bg += float(rng.uniform(0.5, 1.5)) / r
    bg *= 10.0 * np.abs(local).max() / np.abs(bg).max()
    m = mask != 0
    out = [np.where(m, (t + 1) * (local + bg) + rng.normal(0.0, noise, shape), 0.0) for t in range(echoes)]
    f = out[0] if echoes == 1 else np.stack(out, axis=3)
    return np.asfortranarray(f), np.asfortranarray(np.where(m, local, 0.0)), mask
