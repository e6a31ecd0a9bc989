"""CPU restatement of QSM.m's FFT total-variation inversion (ADMM).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the oracle of the GPU
path; the product never imports it.

Follows src/inversion/tv.m (tv :1-98 defaults and echo loop, tv_ :101-277),
src/utils/kernels/dipoleKernel.m:56-65 (k-space dipole, ifftshifted, D(1)=0)
and src/utils/kernels/laplaceKernel.m (7-point stencil, whose negated,
zero-padded, centred FFT gives the Laplacian's symbol L, tv.m:140-142).  The
periodic gradient and its adjoint are the reference MEX gateways
gradfp_mex / gradfp_adj_mex, taken from the oracle library (bit-identical
with the reference C, pinned by the golden tests).  fft3/ifft3 are numpy's
pocketfft in FP64 (MATLAB's FFTW is not available here); norm2(x) =
||x(:)||_2 (src/utils/norm2.m).

Parity of this loop itself is unpinned: the reference is MATLAB code and no
MATLAB or Octave is available to run it; the reference ships no fixture for
tv.m.  The pieces it calls (gradfp, gradfp_adj) are pinned.
"""
from __future__ import annotations

import numpy as np

import port

DEFAULTS = dict(mu=7.5e3, tv=1, rtol=1e-1, atol=1e-4, maxit=20, verbose=0, rho=9.0, alpha=1.5, rtau=0.7,
                stau=1e2, gamma=3.0)  # tv.m:38-82


def dipole_kernel(sz, vsz, bdir=(0.0, 0.0, 1.0)):
    """dipoleKernel(sz, vsz, bdir, 'k'): D = 1/3 - (k.b)^2/|k|^2 on the grid
    k_a = i / (n_a h_a), ifftshifted (DC first), D(1) = 0."""
    b = np.asarray(bdir, dtype=np.float64)
    if np.linalg.norm(b) != 1.0:
        b = b / np.linalg.norm(b)
    k = [np.fft.fftfreq(int(n), d=float(h)) for n, h in zip(sz, vsz)]
    kx, ky, kz = np.meshgrid(*k, indexing="ij")
    kb = b[0] * kx + b[1] * ky + b[2] * kz
    k2 = kx * kx + ky * ky + kz * kz
    with np.errstate(divide="ignore", invalid="ignore"):
        D = 1.0 / 3.0 - (kb * kb) / k2
    D[0, 0, 0] = 0.0
    return np.asfortranarray(D)


def laplace_symbol(sz, vsz):
    """real(fft3(circshift(padarray(-laplaceKernel(vsz), sz-3, 'post'), -1)))
    (tv.m:140-142): the negated 7-point stencil centred at index (1,1,1).

    Its DC entry is the stencil's coefficient sum, zero in exact arithmetic;
    an FFT can leave +-1e-15 there when 1/h^2 is not exact (h = 0.9 ...),
    which turns tv.m's intended iA(DC) = 0 (1/0 -> inf -> 0, :144-145) into
    ~1e14 and amplifies round-off at DC.  The restatement keeps the exact
    zero, as the GPU path does."""
    ih = [1.0 / (h * h) for h in vsz]
    L = np.zeros(tuple(int(n) for n in sz))
    L[0, 0, 0] = 2.0 * (ih[0] + ih[1] + ih[2])
    for a in range(3):
        for s in (1, -1):
            idx = [0, 0, 0]
            idx[a] = s
            L[tuple(idx)] += -ih[a]
    out = np.asfortranarray(np.real(np.fft.fftn(L)))
    out[0, 0, 0] = 0.0
    return out


def _grad(u, h):
    dx, dy, dz = (np.zeros_like(u, order="F") for _ in range(3))
    port.gradfp_mex(dx, dy, dz, u, h)
    return dx, dy, dz


def _grad_adj(x, y, z, h):
    du = np.zeros_like(x, order="F")
    port.gradfp_adj_mex(du, np.asfortranarray(x), np.asfortranarray(y), np.asfortranarray(z), h)
    return du


def _inv(K, L, rho):
    with np.errstate(divide="ignore", invalid="ignore"):
        iA = 1.0 / (K + rho * L)
    iA[~np.isfinite(iA)] = 0.0
    return iA


def tv_(f, mask, D, vsz, opts, trace=None):
    """tv.m:101-277 for one 3-D volume (FP64)."""
    f = np.asfortranarray(f, dtype=np.float64)
    h = np.asarray(vsz, dtype=np.float64)
    n = f.size
    rtol, atol = opts["rtol"], opts["atol"]
    atolp = np.sqrt(3 * n) * atol
    atold = np.sqrt(n) * atol
    mu, rho, alpha = opts["mu"], opts["rho"], opts["alpha"]
    rtau, stau, gamma = opts["rtau"], opts["stau"], opts["gamma"]
    irho = 1.0 / rho
    F = mu * np.conj(D) * np.fft.fftn(f)
    K = mu * np.abs(D) ** 2
    L = laplace_symbol(f.shape, h)
    iA = _inv(K, L, rho)
    u = f.copy(order="F")
    l1, l2, l3 = (np.zeros_like(f, order="F") for _ in range(3))
    v1, v2, v3 = _grad(u, h)
    nr = np.sum(np.sqrt(v1 * v1 + v2 * v2 + v3 * v3))
    flag = 0
    it = 0
    for ii in range(1, opts["maxit"] + 1):
        it = ii
        # u-subproblem
        r1 = _grad_adj(rho * v1 - l1, rho * v2 - l2, rho * v3 - l3, h)
        b = F + np.fft.fftn(r1)
        u = np.asfortranarray(np.real(np.fft.ifftn(iA * b)))
        # v-subproblem
        v1_, v2_, v3_ = v1, v2, v3
        dx, dy, dz = _grad(u, h)
        dx1 = alpha * dx + (1 - alpha) * v1
        dy1 = alpha * dy + (1 - alpha) * v2
        dz1 = alpha * dz + (1 - alpha) * v3
        r1 = dx1 + irho * l1
        r2 = dy1 + irho * l2
        r3 = dz1 + irho * l3
        if opts["tv"] == 1:
            v1 = np.maximum(np.abs(r1) - irho, 0) * np.sign(r1)
            v2 = np.maximum(np.abs(r2) - irho, 0) * np.sign(r2)
            v3 = np.maximum(np.abs(r3) - irho, 0) * np.sign(r3)
        else:
            s = np.sqrt(r1 * r1 + r2 * r2 + r3 * r3)
            with np.errstate(divide="ignore", invalid="ignore"):
                s = (s - irho) * (s > irho) / s
            s[~np.isfinite(s)] = 0
            v1, v2, v3 = r1 * s, r2 * s, r3 * s
        # multiplier update
        l1 = l1 + rho * (dx1 - v1)
        l2 = l2 + rho * (dy1 - v2)
        l3 = l3 + rho * (dz1 - v3)
        # convergence check
        nr_ = nr
        r1, r2, r3 = dx - v1, dy - v2, dz - v3
        s = rho * _grad_adj(v1 - v1_, v2 - v2_, v3 - v3_, h)
        nr = np.sum(np.sqrt(r1 * r1 + r2 * r2 + r3 * r3))
        ns = np.linalg.norm(s.ravel())
        na = np.sum(np.sqrt(dx * dx + dy * dy + dz * dz))
        nb = np.sum(np.sqrt(v1 * v1 + v2 * v2 + v3 * v3))
        ep = atolp + rtol * max(na, nb)
        ed = atold + rtol * np.linalg.norm((rho * _grad_adj(l1, l2, l3, h)).ravel())
        if trace is not None:
            trace.append(dict(iter=ii, nr=nr, ep=ep, ns=ns, ed=ed, rho=rho))
        if nr < ep and ns < ed:
            break
        # parameter update
        if nr > stau * ns or (nr > rtau * nr_ and flag < 3):
            rho = gamma * rho
            irho = 1.0 / rho
            iA = _inv(K, L, rho)
            if flag > 5:
                flag = 0
        elif nr < ns / stau:
            rho = rho / gamma ** 2
            irho = 1.0 / rho
            iA = _inv(K, L, rho)
            flag = flag + 1
    return np.asfortranarray(mask * u), it


def tv(f, mask, vsz, bdir=(0.0, 0.0, 1.0), opts=None, trace=None):
    """x = tv(f, mask, vsz, bdir, opts) (tv.m:1-98): 3-D or 4-D (echoes) f."""
    o = dict(DEFAULTS)
    if opts:
        o.update({k: v for k, v in opts.items() if v is not None})
    vsz = np.broadcast_to(np.asarray(vsz, dtype=np.float64), (3,))
    f = np.asarray(f, dtype=np.float64)
    D = dipole_kernel(mask.shape, vsz, bdir)
    m = np.asarray(mask, dtype=np.float64)
    if f.ndim == 3:
        return tv_(f, m, D, vsz, o, trace)[0]
    x = np.zeros(f.shape, order="F")
    for t in range(f.shape[3]):
        x[..., t] = tv_(f[..., t], m, D, vsz, o, trace)[0]
    return x
