"""CPU ORACLE of the spectral right preconditioner (test infrastructure only; never imported by
the product).

The reference has no preconditioner: its GMRES (ForwardMap/ForwardMap.tpp:658-697,
ForwardMap/opGMRES.hpp:68-269) is unpreconditioned.  The product adds a right preconditioner
for the combined-field operator A = 1/2 I + K - i eta S on closed curves, built from the
operator's flat-boundary symbol (the leading term of its pseudo-differential symbol; the
complexified wavenumber that smooths the glancing singularity is the on-surface radiation
condition device of Antoine and Darbas, M2AN 2005):

    sigma(xi) = 1/2 + eta / (2 sqrt(k_eps^2 - xi^2)),   k_eps = k + i eps,  Im sqrt >= 0,

xi the arc-length frequency.  The preconditioner is

    M r = 2 r + B F^{-1} [ (1/sigma - 2) F (W r) ],

with W the resampling of the quadrature-node values of each closed curve onto a uniform
arc-length grid of nu = 2^m >= n points (per point of the grid, the Lagrange interpolant of its
patch's Np nodes), F the discrete Fourier transform along the curve and B the resampling back
to the nodes (per node, the degree-(T-1) Lagrange interpolant of the T uniform grid points
around it).  This module restates that algorithm in numpy, independently of the product's C++
tables, so that the device preconditioner can be checked against it.
"""
from __future__ import annotations

import numpy as np

CURVE_CIRCLE, CURVE_KITE, CURVE_LINE, CURVE_STAR = 0, 1, 2, 3


def curve_speed(ctype, p):
    """|x'(t)| of the curve types of include/ifgf2d.h (circle, kite, star)."""
    p = np.asarray(p, dtype=np.float64)
    if ctype == CURVE_CIRCLE:
        return lambda t: np.abs(p[2]) * np.ones_like(np.asarray(t, dtype=np.float64))
    if ctype == CURVE_KITE:
        return lambda t: np.hypot(-p[0] * np.sin(t) - 2.0 * p[1] * np.sin(2.0 * t), p[3] * np.cos(t))
    if ctype == CURVE_STAR:
        M = int(p[2])
        a, b = p[3:3 + M], p[3 + M:3 + 2 * M]

        def speed(t):
            t = np.asarray(t, dtype=np.float64)
            m = np.arange(1, M + 1)
            ang = np.multiply.outer(t, m)
            r = 1.0 + np.cos(ang) @ a + np.sin(ang) @ b
            dr = -np.sin(ang) @ (m * a) + np.cos(ang) @ (m * b)
            return np.hypot(dr, r)
        return speed
    raise ValueError("the spectral preconditioner needs a closed curve")


class CurveTables:
    """Resampling tables of one closed curve whose points (in the given order) lie on patches
    [t1[p], t2[p]] with Np nodes each, node parameters tp."""

    def __init__(self, speed, t1, t2, tp, Np, taps_back=8, nu=None):
        t1 = np.asarray(t1, float); t2 = np.asarray(t2, float); tp = np.asarray(tp, float)
        P = t1.size
        n = P * Np
        assert tp.size == n
        self.n = n
        self.nu = nu if nu is not None else 1 << int(np.ceil(np.log2(max(n, 64))))
        gx, gw = np.polynomial.legendre.leggauss(32)

        def seg(a, b):
            a = np.asarray(a, float); b = np.asarray(b, float)
            tm = 0.5 * (a + b)[..., None] + 0.5 * (b - a)[..., None] * gx
            return 0.5 * (b - a) * (speed(tm) @ gw)

        Lp = seg(t1, t2)
        S = np.concatenate([[0.0], np.cumsum(Lp)])
        self.L = L = S[-1]
        patch = np.repeat(np.arange(P), Np)
        self.s_nodes = S[patch] + seg(t1[patch], tp)
        # uniform grid: parameter by Newton on the patch's arc length (the device interpolates it
        # through the nodes' arc lengths instead; both agree to rounding)
        h = L / self.nu
        su = h * np.arange(self.nu)
        # a grid point on a patch boundary (up to rounding) belongs to the patch that starts there
        pu = np.clip(np.searchsorted(S, su + 1e-10 * L, side="right") - 1, 0, P - 1)
        a, b = t1[pu], t2[pu]
        t = a + (su - S[pu]) / Lp[pu] * (b - a)
        for _ in range(12):
            t = np.clip(t - (S[pu] + seg(a, t) - su) / speed(t), a, b)
        u = (2.0 * t - a - b) / (b - a)
        un = (2.0 * tp - t1[patch] - t2[patch]) / (t2[patch] - t1[patch])
        un = un.reshape(P, Np)
        # barycentric weights of each patch's nodes
        diff = un[:, :, None] - un[:, None, :]
        diff[:, np.arange(Np), np.arange(Np)] = 1.0
        lam = 1.0 / np.prod(diff, axis=2)
        du = u[:, None] - un[pu]
        exact = np.abs(du) == 0.0
        du[exact] = 1.0
        q = lam[pu] / du
        W = q / q.sum(axis=1, keepdims=True)
        rows = np.nonzero(exact.any(axis=1))[0]
        W[rows] = exact[rows].astype(float)
        self.fw_base = pu * Np
        self.fw_w = W
        # back: T-tap Lagrange on the uniform grid
        T = taps_back
        x = self.s_nodes / h
        q0 = np.floor(x).astype(np.int64) - (T // 2 - 1)
        xr = x - q0                                   # position relative to the first tap
        idx = np.arange(T)
        num = xr[:, None] - idx[None, :]
        Wb = np.empty((n, T))
        for i in range(T):
            o = np.delete(idx, i)
            Wb[:, i] = np.prod(num[:, o], axis=1) / np.prod(i - o)
        self.bk_base = q0 % self.nu
        self.bk_w = Wb
        self.T = T

    def forward(self, r):
        Np = self.fw_w.shape[1]
        g = r[self.fw_base[:, None] + np.arange(Np)[None, :]]
        return np.sum(g * self.fw_w, axis=1)

    def back(self, u):
        idx = (self.bk_base[:, None] + np.arange(self.T)[None, :]) % self.nu
        return np.sum(u[idx] * self.bk_w, axis=1)

    def multiplier(self, k, eta, eps, which=0):
        """the multiplier m of z = b v + B F^-1 [m F W v]: 0 the preconditioner (1/sigma - 2, b = 2),
        1 the flat symbol's magnitude (|sigma| - 1/2, b = 1/2), 2 its inverse (1/|sigma| - 2, b = 2)"""
        xi = 2.0 * np.pi * np.fft.fftfreq(self.nu, self.L / self.nu)
        ke = k + 1j * eps
        sig = 0.5 + eta / (2.0 * np.sqrt(ke * ke - xi * xi + 0j))
        if which == 1:
            return np.abs(sig) - 0.5
        if which == 2:
            return 1.0 / np.abs(sig) - 2.0
        return 1.0 / sig - 2.0


def eps_default(k, scale=0.25):
    """The glancing damping eps = scale k^(1/3), the device's default scale."""
    return scale * k ** (1.0 / 3.0)


class SpectralPreconditioner:
    """M for all closed curves of a discretisation: curves = list of (ctype, params, t1, t2, tp)
    with each curve's points contiguous, in order."""

    def __init__(self, curves, Np, k, eta=None, eps=None, taps_back=8):
        self.k = k
        self.eta = k if eta is None else eta
        self.eps = eps_default(k) if eps is None else eps
        self.tables = []
        self.off = [0]
        for ctype, params, t1, t2, tp in curves:
            tb = CurveTables(curve_speed(ctype, params), t1, t2, tp, Np, taps_back)
            self.tables.append(tb)
            self.off.append(self.off[-1] + tb.n)
        self.mult = [tb.multiplier(k, self.eta, self.eps) for tb in self.tables]

    def __call__(self, r, which=0):
        """z = M r (which 0), or Op(|sigma|) r (1), Op(1/|sigma|) r (2)"""
        r = np.asarray(r, dtype=np.complex128)
        z = (0.5 if which == 1 else 2.0) * r
        for c, tb in enumerate(self.tables):
            a, b = self.off[c], self.off[c + 1]
            m = self.mult[c] if which == 0 else tb.multiplier(self.k, self.eta, self.eps, which)
            u = np.fft.ifft(m * np.fft.fft(tb.forward(r[a:b])))
            z[a:b] += tb.back(u)
        return z
