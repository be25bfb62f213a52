"""Independent FP64 Ewald direct sums -- TEST INFRASTRUCTURE ONLY.

A vectorised numpy restatement of the reference's MATLAB direct sums in
PE/tests/matlab_sums/*.m, used by PE/tests/direct_sums_test.m to check the
MEX output.  No grid, no FFT, no cell list: the real-space part sums every
source over the 3x3 periodic images with the exact exponential integral
(scipy.special.exp1), and the k-space part sums the Fourier modes directly
through structure factors.

* ``slp_real_ds``  -- stokes_slp_real_ds.m:26-69 (self term at r < 1e-13:
  -(gamma/2 + log xi + 1) f, :42-46)
* ``dlp_real_ds``  -- stokes_dlp_real_ds.m:28-76 (r < 1e-13 skipped, :44-46)
* ``slp_kspace_ds`` -- stokes_slp_kspace_ds.m:21-75 (modes jk in [-kinf+1, kinf]^2,
  k = 0 excluded, real part / (Lx Ly))
* ``dlp_kspace_ds`` -- stokes_dlp_kspace_ds.m:23-85 (plus the zero-mode term
  -sum((f.n) x_src)/(Lx Ly), :67-69)

The Ewald-split direct sums define the periodic sums (the raw 2D Stokeslet
lattice sum is only conditionally convergent).  Inputs are 1-D arrays as in
the MATLAB scripts; outputs are (2, Ntar).
"""
from __future__ import annotations

import numpy as np
from scipy.special import exp1

EULER_GAMMA = 0.57721566490153286061


def _images(Lx, Ly):
    return [(jx * Lx, jy * Ly) for jx in (-1, 0, 1) for jy in (-1, 0, 1)]


def slp_real_ds(xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, xi, chunk=2048):
    xsrc, ysrc, f1, f2 = map(np.asarray, (xsrc, ysrc, f1, f2))
    xtar, ytar = np.asarray(xtar), np.asarray(ytar)
    u = np.zeros((2, xtar.size))
    self_c = -(EULER_GAMMA / 2 + np.log(xi) + 1)
    for t0 in range(0, xtar.size, chunk):
        tx = xtar[t0:t0 + chunk, None]
        ty = ytar[t0:t0 + chunk, None]
        a1 = np.zeros(tx.shape[0])
        a2 = np.zeros(tx.shape[0])
        for ox, oy in _images(Lx, Ly):
            r1 = xsrc[None, :] + ox - tx
            r2 = ysrc[None, :] + oy - ty
            rr = r1 * r1 + r2 * r2
            near = np.sqrt(rr) < 1e-13
            rs = np.where(near, 1.0, rr)
            e = np.exp(-xi * xi * rs)
            E = exp1(xi * xi * rs)
            rf = r1 * f1[None, :] + r2 * f2[None, :]
            v1 = e * (r1 * rf / rs - f1[None, :]) + f1[None, :] * E / 2
            v2 = e * (r2 * rf / rs - f2[None, :]) + f2[None, :] * E / 2
            v1 = np.where(near, self_c * f1[None, :], v1)
            v2 = np.where(near, self_c * f2[None, :], v2)
            a1 += v1.sum(axis=1)
            a2 += v2.sum(axis=1)
        u[0, t0:t0 + chunk] = a1
        u[1, t0:t0 + chunk] = a2
    return u / (4 * np.pi)


def dlp_real_ds(xsrc, ysrc, xtar, ytar, n1, n2, f1, f2, Lx, Ly, xi, chunk=2048):
    xsrc, ysrc, n1, n2, f1, f2 = map(np.asarray, (xsrc, ysrc, n1, n2, f1, f2))
    xtar, ytar = np.asarray(xtar), np.asarray(ytar)
    u = np.zeros((2, xtar.size))
    for t0 in range(0, xtar.size, chunk):
        tx = xtar[t0:t0 + chunk, None]
        ty = ytar[t0:t0 + chunk, None]
        a1 = np.zeros(tx.shape[0])
        a2 = np.zeros(tx.shape[0])
        for ox, oy in _images(Lx, Ly):
            r1 = xsrc[None, :] + ox - tx
            r2 = ysrc[None, :] + oy - ty
            rr = r1 * r1 + r2 * r2
            near = np.sqrt(rr) < 1e-13
            rs = np.where(near, 1.0, rr)
            rf = r1 * f1 + r2 * f2
            rn = r1 * n1 + r2 * n2
            nf = n1 * f1 + n2 * f2
            e = np.exp(-xi * xi * rs)
            c = -4 * rn * rf / rs ** 2 * (1 + xi * xi * rs)
            v1 = e * (c * r1 + 2 * xi * xi * (f1 * rn + n1 * rf + nf * r1))
            v2 = e * (c * r2 + 2 * xi * xi * (f2 * rn + n2 * rf + nf * r2))
            a1 += np.where(near, 0.0, v1).sum(axis=1)
            a2 += np.where(near, 0.0, v2).sum(axis=1)
        u[0, t0:t0 + chunk] = a1
        u[1, t0:t0 + chunk] = a2
    return u / (4 * np.pi)


def default_kinf(xi, Lx, Ly, decay=41.0):
    """Smallest kinf with exp(-k^2/(4 xi^2)) < e^-decay at |k| = 2 pi kinf / max(L)."""
    return int(np.ceil(2 * xi * np.sqrt(decay) * max(Lx, Ly) / (2 * np.pi))) + 1


def _modes(Lx, Ly, kinf):
    j = np.arange(-kinf + 1, kinf + 1)
    J1, J2 = np.meshgrid(j, j, indexing="ij")
    k1 = (2 * np.pi / Lx * J1).ravel()
    k2 = (2 * np.pi / Ly * J2).ravel()
    keep = ~((k1 == 0) & (k2 == 0))
    return k1[keep], k2[keep]


def _structure(k1, k2, xs, ys, weights, chunk=512):
    """S_w(k) = sum_s w_s exp(+i k.x_s) for each weight vector w (list)."""
    out = [np.zeros(k1.size, complex) for _ in weights]
    for s0 in range(0, xs.size, chunk):
        ph = np.exp(1j * (np.outer(k1, xs[s0:s0 + chunk]) + np.outer(k2, ys[s0:s0 + chunk])))
        for o, w in zip(out, weights):
            o += ph @ w[s0:s0 + chunk]
    return out


def _structure_grid(Lx, Ly, kinf, xs, ys, weights, chunk=4096):
    """_structure on the full mode grid, in _modes' order (k = 0 removed),
    as sums over source chunks of (X w) Y^T with X[a, s] = exp(i k1_a x_s) and
    Y[b, s] = exp(i k2_b y_s): the phases factor per axis, so the cost is two
    small exponential tables and one matrix product per chunk instead of one
    exponential per mode and source."""
    j = np.arange(-kinf + 1, kinf + 1)
    out = [np.zeros((j.size, j.size), complex) for _ in weights]
    for s0 in range(0, xs.size, chunk):
        X = np.exp(1j * (2 * np.pi / Lx) * np.outer(j, xs[s0:s0 + chunk]))
        Y = np.exp(1j * (2 * np.pi / Ly) * np.outer(j, ys[s0:s0 + chunk]))
        for o, w in zip(out, weights):
            o += (X * w[s0:s0 + chunk]) @ Y.T
    keep = np.ones(j.size * j.size, bool)
    keep[(kinf - 1) * j.size + (kinf - 1)] = False          # j1 = j2 = 0
    return [o.ravel()[keep] for o in out]


def _evaluate_grid(Lx, Ly, kinf, coefs, xt, yt, chunk=4096):
    """_evaluate for coefficients in _modes' order (k = 0 removed), through
    per-axis phase tables: u(t) = Re sum_a X_t[a] (C Y_t)[a]."""
    j = np.arange(-kinf + 1, kinf + 1)
    n = j.size
    u = np.zeros((len(coefs), xt.size))
    grids = []
    for co in coefs:
        g = np.zeros(n * n, complex)
        keep = np.ones(n * n, bool)
        keep[(kinf - 1) * n + (kinf - 1)] = False
        g[keep] = co
        grids.append(g.reshape(n, n))
    for t0 in range(0, xt.size, chunk):
        X = np.exp(-1j * (2 * np.pi / Lx) * np.outer(j, xt[t0:t0 + chunk]))
        Y = np.exp(-1j * (2 * np.pi / Ly) * np.outer(j, yt[t0:t0 + chunk]))
        for c, g in enumerate(grids):
            u[c, t0:t0 + chunk] = np.einsum("at,at->t", X, g @ Y).real
    return u


def _evaluate(k1, k2, coefs, xt, yt, chunk=512):
    """u_c(t) = Re sum_k coefs_c(k) exp(-i k.x_t)."""
    u = np.zeros((len(coefs), xt.size))
    for t0 in range(0, xt.size, chunk):
        ph = np.exp(-1j * (np.outer(xt[t0:t0 + chunk], k1) + np.outer(yt[t0:t0 + chunk], k2)))
        for c, co in enumerate(coefs):
            u[c, t0:t0 + chunk] = (ph @ co).real
    return u


def _sums(Lx, Ly, kinf, k1, k2, xs, ys, weights, grid):
    if grid:
        return _structure_grid(Lx, Ly, kinf, xs, ys, weights)
    return _structure(k1, k2, xs, ys, weights)


def _values(Lx, Ly, kinf, k1, k2, coefs, xt, yt, grid):
    if grid:
        return _evaluate_grid(Lx, Ly, kinf, coefs, xt, yt)
    return _evaluate(k1, k2, coefs, xt, yt)


def slp_kspace_ds(xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, xi, kinf=None, grid=False):
    """grid=True sums the same modes through per-axis phase tables (for
    thousands of sources and modes)."""
    if kinf is None:
        kinf = default_kinf(xi, Lx, Ly)
    k1, k2 = _modes(Lx, Ly, kinf)
    K2 = k1 * k1 + k2 * k2
    A = (1 + K2 / (4 * xi * xi)) * np.exp(-K2 / (4 * xi * xi)) / K2
    F1, F2 = _sums(Lx, Ly, kinf, k1, k2, np.asarray(xsrc, float), np.asarray(ysrc, float),
                   [np.asarray(f1, float), np.asarray(f2, float)], grid)
    # (f - k (k.f)/k^2) A: stokeslet_k_sum, stokes_slp_kspace_ds.m:67-74
    c1 = A * ((1 - k1 * k1 / K2) * F1 - k1 * k2 / K2 * F2)
    c2 = A * (-k1 * k2 / K2 * F1 + (1 - k2 * k2 / K2) * F2)
    return _values(Lx, Ly, kinf, k1, k2, [c1, c2], np.asarray(xtar, float),
                   np.asarray(ytar, float), grid) / (Lx * Ly)


def dlp_kspace_ds(xsrc, ysrc, xtar, ytar, n1, n2, f1, f2, Lx, Ly, xi, kinf=None, grid=False):
    """grid=True as for slp_kspace_ds."""
    if kinf is None:
        kinf = default_kinf(xi, Lx, Ly)
    xsrc, ysrc, n1, n2, f1, f2 = map(lambda a: np.asarray(a, float),
                                      (xsrc, ysrc, n1, n2, f1, f2))
    k1, k2 = _modes(Lx, Ly, kinf)
    K2 = k1 * k1 + k2 * k2
    B = (1 + K2 / (4 * xi * xi)) * np.exp(-K2 / (4 * xi * xi)) / K2
    # S_ab = f_a n_b per source, summed into structure factors.
    S11, S12, S21, S22 = _sums(Lx, Ly, kinf, k1, k2, xsrc, ysrc,
                               [f1 * n1, f1 * n2, f2 * n1, f2 * n2], grid)
    # stokes_dlp_k_sum (stokes_dlp_kspace_ds.m:73-85), linear in S_ab:
    #   f1 (k.n) = k1 S11 + k2 S12 ; n1 (k.f) = k1 S11 + k2 S21 ; k1 (f.n) = k1 (S11 + S22)
    #   (k.n)(k.f) = k1^2 S11 + k1 k2 (S12 + S21) + k2^2 S22
    kk = k1 * k1 * S11 + k1 * k2 * (S12 + S21) + k2 * k2 * S22
    fn = S11 + S22
    g1 = (k1 * S11 + k2 * S12) + (k1 * S11 + k2 * S21) + k1 * fn - 2 * k1 * kk / K2
    g2 = (k1 * S21 + k2 * S22) + (k1 * S12 + k2 * S22) + k2 * fn - 2 * k2 * kk / K2
    u = _values(Lx, Ly, kinf, k1, k2, [1j * B * g1, 1j * B * g2], np.asarray(xtar, float),
                np.asarray(ytar, float), grid)
    u /= (Lx * Ly)
    fdotn = f1 * n1 + f2 * n2
    u[0] -= np.sum(fdotn * xsrc) / (Lx * Ly)
    u[1] -= np.sum(fdotn * ysrc) / (Lx * Ly)
    return u
