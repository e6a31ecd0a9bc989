"""CPU restatement of QSM.m's FFT background-field removal.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the oracle of the GPU
path; the product never imports it.

Follows src/bgremove/sharp.m:1-84, vsharp.m:1-153, ismv.m:1-112,
resharp.m:1-88 (MATLAB's cgs restated as the published CGS iteration) and
pdf.m:1-86 (third_party/lsmr/lsmr.m restated from Fong & Saunders 2011;
src/utils/kernels/dipoleKernel.m 'i'; psf2otf as ifftshift + fftn, real part
kept when the imaginary part is roundoff) with
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
        with np.errstate(divide="ignore", invalid="ignore"):
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


def cgs(A, b, tol, maxit):
    """Conjugate gradients squared (Sonneveld 1989; the unpreconditioned form of
    Barrett et al., Templates, 1994), x0 = 0, stopping when the recursively
    updated residual is <= tol * ||b||.  Returns (x, iterations)."""
    x = np.zeros_like(b)
    r = b.copy()
    rt = b.copy()
    nb = np.linalg.norm(b)
    it = 0
    if nb == 0:
        return x, 0
    rho1 = 1.0
    u = p = q = None
    for ii in range(1, maxit + 1):
        rho = float(np.dot(rt, r))
        if rho == 0.0:
            break
        if ii == 1:
            u = r.copy()
            p = r.copy()
        else:
            beta = rho / rho1
            u = r + beta * q
            p = u + beta * (q + beta * p)
        vh = A(p)
        sv = float(np.dot(rt, vh))
        if sv == 0.0:
            break
        alpha = rho / sv
        q = u - alpha * vh
        uh = u + q
        x = x + alpha * uh
        r = r - alpha * A(uh)
        rho1 = rho
        it = ii
        if np.linalg.norm(r) <= tol * nb:
            break
    return x, it


def resharp(f, mask, vsz, r=3.0, lam=1e-2, tol=None, maxit=None, info=None):
    """resharp.m:1-88 with MATLAB's cgs replaced by `cgs` above."""
    f, echoes = _echoes(f)
    tol = math.sqrt(np.finfo(np.float64).eps) if tol is None else tol
    maxit = maxit or int(math.ceil(math.sqrt(np.asarray(mask).size)))
    b = crop_slices(mask)
    sz = tuple(s.stop - s.start for s in b)
    pad = int(math.ceil(r / min(vsz)))
    m1 = padfast(np.asarray(mask)[b] != 0, pad)
    H = smv_spectrum(m1.shape, r, vsz)
    mk = erode(H, m1).astype(np.float64)
    h = 1.0 - H
    shape = m1.shape

    def A(v):
        v = v.reshape(shape)
        return (mk * np.real(np.fft.ifftn(h * np.fft.fftn(v))) + lam * v).ravel()

    fl = np.zeros(f.shape, order="F")
    iters = []
    for t, ft in enumerate(echoes):
        rhs = (mk * np.real(np.fft.ifftn(h * np.fft.fftn(padfast(ft[b], pad))))).ravel()
        x, it = cgs(A, rhs, tol, maxit)
        iters.append(it)
        out = unpadfast(mk * x.reshape(shape), sz, pad)
        if f.ndim == 3:
            fl[b] = out
        else:
            fl[b + (t,)] = out
    if info is not None:
        info["iters"] = iters
    mo = np.zeros(np.shape(mask), np.uint8, order="F")
    mo[b] = unpadfast(mk, sz, pad).astype(np.uint8)
    return fl, mo


def psf2otf(k):
    """fft3 of a centred kernel moved to index 0 (ifftshift); the real part when
    the imaginary part is roundoff: max|Im| / max|K| <= N log2(N) eps."""
    K = np.fft.fftn(np.fft.ifftshift(k))
    n = k.size
    eps = np.finfo(np.float32 if k.dtype == np.float32 else np.float64).eps
    if np.abs(K.imag).max() / np.abs(K).max() <= n * math.log2(n) * eps:
        K = K.real.astype(K.dtype)
    return K


def dipole_kernel_i(sz, vsz, bdir=(0.0, 0.0, 1.0)):
    """dipoleKernel(sz, vsz, bdir, 'i') (src/utils/kernels/dipoleKernel.m:44-51):
    (3 (b.r)^2 - |r|^2) / (4 pi |r|^5) on the centred grid, 0 at the centre."""
    b = np.asarray(bdir, np.float64)
    nb = math.sqrt(float(b @ b))
    if nb != 1.0:
        b = b / nb
    g = []
    for n, h in zip(sz, vsz):
        low = n // 2
        high = low - (1 - n % 2)
        g.append(np.arange(-low, high + 1) * float(h))
    X, Y, Z = np.meshgrid(*g, indexing="ij")
    rz = b[0] * X + b[1] * Y + b[2] * Z
    r2 = X * X + Y * Y + Z * Z
    den = 4 * math.pi * np.sqrt(r2 * r2 * r2 * r2 * r2)
    with np.errstate(divide="ignore", invalid="ignore"):
        D = (3 * (rz * rz) - r2) / den
    D[den == 0] = 0
    return D


def lsmr(A, AT, b, lam=0.0, atol=1e-6, btol=1e-6, conlim=1e8, itnlim=None):
    """LSMR (Fong & Saunders, SIAM J. Sci. Comput. 33(5), 2011) without local
    reorthogonalisation, with the stopping rules of the published algorithm
    (third_party/lsmr/lsmr.m).  Returns (x, itn)."""
    u = b.copy()
    beta = float(np.linalg.norm(u))
    if beta > 0:
        u = u / beta
    v = AT(u)
    alpha = float(np.linalg.norm(v))
    if alpha > 0:
        v = v / alpha
    x = np.zeros_like(v)
    itnlim = itnlim if itnlim is not None else min(b.size, v.size)
    if alpha * beta == 0:
        return x, 0
    zetabar, alphabar, rho, rhobar, cbar, sbar = alpha * beta, alpha, 1.0, 1.0, 1.0, 0.0
    h, hbar = v.copy(), np.zeros_like(v)
    betadd, betad, rhodold, tautildeold, thetatilde, zeta, d = beta, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0
    normA2, maxrbar, minrbar, normb = alpha * alpha, 0.0, 1e100, beta
    ctol = 1.0 / conlim if conlim > 0 else 0.0
    itn = 0
    while itn < itnlim:
        itn += 1
        u = A(v) - alpha * u
        beta = float(np.linalg.norm(u))
        if beta > 0:
            u = u / beta
            v = AT(u) - beta * v
            alpha = float(np.linalg.norm(v))
            if alpha > 0:
                v = v / alpha
        alphahat = math.hypot(alphabar, lam)
        chat, shat = alphabar / alphahat, lam / alphahat
        rhoold = rho
        rho = math.hypot(alphahat, beta)
        c, s = alphahat / rho, beta / rho
        thetanew = s * alpha
        alphabar = c * alpha
        rhobarold, zetaold, thetabar, rhotemp = rhobar, zeta, sbar * rho, cbar * rho
        rhobar = math.hypot(cbar * rho, thetanew)
        cbar = cbar * rho / rhobar
        sbar = thetanew / rhobar
        zeta = cbar * zetabar
        zetabar = -sbar * zetabar
        hbar = h - (thetabar * rho / (rhoold * rhobarold)) * hbar
        x = x + (zeta / (rho * rhobar)) * hbar
        h = v - (thetanew / rho) * h
        betaacute, betacheck = chat * betadd, -shat * betadd
        betahat = c * betaacute
        betadd = -s * betaacute
        thetatildeold = thetatilde
        rhotildeold = math.hypot(rhodold, thetabar)
        ctildeold, stildeold = rhodold / rhotildeold, thetabar / rhotildeold
        thetatilde = stildeold * rhobar
        rhodold = ctildeold * rhobar
        betad = -stildeold * betad + ctildeold * betahat
        tautildeold = (zetaold - thetatildeold * tautildeold) / rhotildeold
        taud = (zeta - thetatilde * tautildeold) / rhodold
        d = d + betacheck * betacheck
        normr = math.sqrt(d + (betad - taud) ** 2 + betadd * betadd)
        normA2 = normA2 + beta * beta
        normA = math.sqrt(normA2)
        normA2 = normA2 + alpha * alpha
        maxrbar = max(maxrbar, rhobarold)
        if itn > 1:
            minrbar = min(minrbar, rhobarold)
        condA = max(maxrbar, rhotemp) / min(minrbar, rhotemp)
        normAr = abs(zetabar)
        normx = float(np.linalg.norm(x))
        test1, test2, test3 = normr / normb, normAr / (normA * normr), 1.0 / condA
        t1 = test1 / (1 + normA * normx / normb)
        rtol = btol + atol * normA * normx / normb
        if (itn >= itnlim or 1 + test3 <= 1 or 1 + test2 <= 1 or 1 + t1 <= 1 or test3 <= ctol
                or test2 <= atol or test1 <= rtol):
            break
    return x, itn


def pdf(f, mask, vsz, w=None, bdir=(0.0, 0.0, 1.0), lam=0.0, tol=1e-5, maxit=None, info=None):
    """pdf.m:1-86 on the full grid with `lsmr` above."""
    f, echoes = _echoes(f)
    mask = np.asarray(mask) != 0
    maxit = maxit or int(math.ceil(math.sqrt(mask.size)))
    if w is None or not np.any(w):
        w = mask
    D = psf2otf(dipole_kernel_i(mask.shape, vsz, bdir))
    m = mask * np.asarray(w, np.float64)
    nm = (m == 0).astype(np.float64)
    shape = mask.shape

    def A(v):
        return (m * np.real(np.fft.ifftn(D * np.fft.fftn(nm * v.reshape(shape))))).ravel()

    def AT(v):
        return (nm * np.real(np.fft.ifftn(np.conj(D) * np.fft.fftn(m * v.reshape(shape))))).ravel()

    fl = np.zeros(f.shape, order="F")
    iters = []
    for t, ft in enumerate(echoes):
        xb, it = lsmr(A, AT, (m * ft).ravel(), lam, tol, tol, 1e8, maxit)
        iters.append(it)
        out = (m != 0) * (ft - np.real(np.fft.ifftn(D * np.fft.fftn(nm * xb.reshape(shape)))))
        if f.ndim == 3:
            fl[...] = out
        else:
            fl[..., t] = out
    if info is not None:
        info["iters"] = iters
    return fl
