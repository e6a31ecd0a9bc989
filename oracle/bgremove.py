"""CPU restatement of QSM.m's FFT background-field removal.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the GPU
path; the product never imports it.

Follows src/bgremove/sharp.m:1-84, vsharp.m:1-153 and ismv.m:1-112 with
src/utils/cropIndices.m, padfastfft.m, unpadfastfft.m,
src/utils/kernels/smvKernel.m:25-37 and third_party/nextfastfft.m (the smallest
7-smooth integer >= n).  fft3 / ifft3 are numpy's pocketfft: complex128 for
the field (MATLAB double), complex64 for fft3(single(mask)) (MATLAB single).
The reference is MATLAB code that cannot run here and ships no fixture for
these functions, so parity of the restatement itself is unpinned.
"""
from __future__ import annotations

import math

import numpy as np


def next_fast(n: int) -> int:
    m = max(int(n), 1)
    while True:
        k = m
        for p in (2, 3, 5, 7):
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m += 1


def crop_slices(mask):
    m = np.asarray(mask) != 0
    idx = [np.flatnonzero(m.any(axis=tuple(b for b in range(3) if b != a))) for a in range(3)]
    if idx[0].size == 0:
        raise ValueError("empty mask")
    return tuple(slice(int(i[0]), int(i[-1]) + 1) for i in idx)


def pad_offsets(sz, pad):
    """padfastfft 'both' with pad per axis: (pre, post) zeros."""
    out = []
    for s in sz:
        tot = next_fast(s + 2 * pad) - s if pad else 0
        half, odd = tot // 2, tot & 1
        pre = half + (odd & (s & 1))
        out.append((pre, tot - pre))
    return out


def padfast(u, pad):
    return np.pad(u, [*pad_offsets(u.shape[:3], pad)] + [(0, 0)] * (u.ndim - 3))


def unpadfast(u, sz, pad):
    off = pad_offsets(sz, pad)
    return u[tuple(slice(p, p + s) for (p, _), s in zip(off, sz))]


def smv_kernel(sz, r, vsz):
    """smvKernel(sz, r, vsz): centred sphere of radius r (mm), normalised."""
    g = []
    for n, h in zip(sz, vsz):
        low = n // 2
        high = low - (1 - n % 2)
        g.append(np.arange(-low, high + 1) * float(h))
    X, Y, Z = np.meshgrid(*g, indexing="ij")
    k = ((Y * Y + X * X + Z * Z) <= r * r).astype(np.float64)
    return k / k.sum()


def smv_spectrum(sz, r, vsz):
    """real(fft3(ifftshift(h)))"""
    return np.real(np.fft.fftn(np.fft.ifftshift(smv_kernel(sz, r, vsz))))


def erode(H, mask_pad):
    """real(ifft3(h .* fft3(single(mask)))) > 0.999 in single precision."""
    M = np.fft.fftn(mask_pad.astype(np.float32))
    v = np.real(np.fft.ifftn(H.astype(np.float32) * M)).astype(np.float32)
    return v.astype(np.float64) > 0.999


def _echoes(f):
    f = np.asarray(f, dtype=np.float64)
    return f, ([f] if f.ndim == 3 else [f[..., t] for t in range(f.shape[3])])


def sharp(f, mask, vsz, r=9.0, thr=0.05):
    f, echoes = _echoes(f)
    b = crop_slices(mask)
    sz = tuple(s.stop - s.start for s in b)
    pad = int(math.ceil(r / min(vsz)))
    m1 = padfast(np.asarray(mask)[b] != 0, pad)
    H = smv_spectrum(m1.shape, r, vsz)
    mk = erode(H, m1)
    h = 1.0 - H
    fl = np.zeros(f.shape, order="F")
    for t, ft in enumerate(echoes):
        u = padfast(ft[b], pad)
        u = mk * np.real(np.fft.ifftn(h * np.fft.fftn(u)))
        U = np.fft.fftn(u) / h
        U[np.abs(h) < thr] = 0
        u = mk * np.real(np.fft.ifftn(U))
        out = unpadfast(u, sz, pad)
        if f.ndim == 3:
            fl[b] = out
        else:
            fl[b + (t,)] = out
    mo = np.zeros(np.shape(mask), np.uint8, order="F")
    mo[b] = unpadfast(mk, sz, pad)
    return fl, mo


def vsharp(f, mask, vsz, rs=None, thr=0.05):
    f, echoes = _echoes(f)
    if rs is None:
        hm = max(vsz)
        rs = list(np.arange(9.0, 2 * hm - 1e-12, -2 * hm))
        rs = [r for r in rs if r >= 2 * hm]
    rs = sorted([float(r) for r in rs], reverse=True)
    b = crop_slices(mask)
    sz = tuple(s.stop - s.start for s in b)
    pad = int(math.ceil(max(rs) / min(vsz)))
    m0 = padfast(np.asarray(mask)[b] != 0, pad)
    fl = np.zeros(f.shape, order="F")
    M = np.fft.fftn(m0.astype(np.float32))
    ret = None
    for t, ft in enumerate(echoes):
        F = np.fft.fftn(padfast(ft[b], pad))
        acc = np.zeros(m0.shape)
        mprev = np.zeros(m0.shape, bool)
        ih = None
        ii = 0
        while ii < len(rs):
            if ii + 1 < len(rs):
                # a pair of radii as one complex kernel (vsharp.m:89-125)
                h = smv_kernel(m0.shape, rs[ii], vsz) + 1j * smv_kernel(m0.shape, rs[ii + 1], vsz)
                h = np.fft.fftn(np.fft.ifftshift(h))
                m = np.fft.ifftn(h.astype(np.complex64) * M)
                mask1 = np.real(m).astype(np.float64) > 0.999
                mask2 = np.imag(m).astype(np.float64) > 0.999
                h = (1 + 1j) - h
                if ii == 0:
                    with np.errstate(divide="ignore"):
                        ih = 1.0 / np.real(h)
                    ih[np.abs(np.real(h)) < thr] = 0
                hf = np.fft.ifftn(h * F)
                acc = acc + (mask1.astype(float) - mprev) * np.real(hf) + (mask2.astype(float) - mask1) * np.imag(hf)
                mprev = mask2
                maskn = mask2
                ret = mask1
            else:
                H = smv_spectrum(m0.shape, rs[ii], vsz)
                mask1 = np.real(np.fft.ifftn(H.astype(np.float32) * M)).astype(np.float32).astype(np.float64) > 0.999
                hh = 1.0 - H
                acc = acc + (mask1.astype(float) - mprev) * np.real(np.fft.ifftn(hh * F))
                maskn = mask1
                ret = mask1
            ii += 2
        u = maskn * np.real(np.fft.ifftn(ih * np.fft.fftn(acc)))
        out = unpadfast(u, sz, pad)
        if f.ndim == 3:
            fl[b] = out
        else:
            fl[b + (t,)] = out
    mo = np.zeros(np.shape(mask), np.uint8, order="F")
    mo[b] = unpadfast(ret, sz, pad)
    return fl, mo


def ismv(f, mask, vsz, r=3.0, tol=None, maxit=500, info=None):
    f, echoes = _echoes(f)
    tol = math.sqrt(np.finfo(np.float64).eps) if tol is None else tol
    b = crop_slices(mask)
    sz = tuple(s.stop - s.start for s in b)
    pad = int(math.ceil(r / min(vsz)))
    m1 = padfast(np.asarray(mask)[b] != 0, pad).astype(np.float64)
    H = smv_spectrum(m1.shape, r, vsz)
    m = erode(H, m1).astype(np.float64)
    fl = np.zeros(f.shape, order="F")
    iters = []
    for t, ft in enumerate(echoes):
        u = padfast(ft[b], pad)
        bc = (m1 - m) * u
        x = u.copy()
        res = np.linalg.norm((m * x).ravel())
        reltol = res * tol
        it = 0
        for ii in range(1, maxit + 1):
            if res <= reltol:
                break
            x0 = x
            x = bc + m * np.real(np.fft.ifftn(H * np.fft.fftn(x)))
            res = np.linalg.norm((x0 - x).ravel())
            it = ii
        iters.append(it)
        out = unpadfast(m * (u - x), sz, pad)
        if f.ndim == 3:
            fl[b] = out
        else:
            fl[b + (t,)] = out
    if info is not None:
        info["iters"] = iters
    mo = np.zeros(np.shape(mask), np.uint8, order="F")
    mo[b] = unpadfast(m, sz, pad).astype(np.uint8)
    return fl, mo
