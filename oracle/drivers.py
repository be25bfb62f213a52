"""Restatement of the MATLAB driver logic -- TEST INFRASTRUCTURE ONLY.

The parameter selection of PE/src/matlab/StokesSLP_ewald_2p.m:27-104,
:147-202 and PE/src/matlab/StokesDLP_ewald_2p.m:30-125, :171-224, written as
plain loops so the golden fixtures can record which (nside, xi, M, w, eta)
the MATLAB drivers would pick.  The product's own host-side estimators are
checked against these values.
"""
from __future__ import annotations

import math

import numpy as np


def matlab_round(x: float) -> float:
    """MATLAB round: half away from zero."""
    return math.copysign(math.floor(abs(x) + 0.5), x)


def rat(x: float, tol: float | None = None):
    """MATLAB rat(X) for a positive scalar: continued-fraction N/D with
    |X - N/D| < tol, tol = 1e-6*|X| by default."""
    if tol is None:
        tol = 1e-6 * abs(x)
    y = x
    n_prev, d_prev = 1.0, 0.0
    n, d = matlab_round(y), 1.0
    frac = y - n
    while abs(x - n / d) >= tol:
        flip = 1.0 / frac
        step = matlab_round(flip)
        frac = flip - step
        n, n_prev = n * step + n_prev, n
        d, d_prev = d * step + d_prev, d
    return int(n * np.sign(d)), int(abs(d))


def _newton(f, fp, x0, tol, maxit=100):
    x, it = x0, 0
    while abs(f(x)) > tol:
        if it > maxit:
            break
        x = x - min(f(x) / fp(x), 0.9 * x)
        it += 1
    return x


def slp_find_xi(Q, Lx, Ly, rc, tol):
    """StokesSLP_ewald_2p.m:178-202."""
    c = math.sqrt(Q * math.pi / (4 * Lx * Ly))
    f = lambda x: math.sqrt(Q * math.pi / (4 * Lx * Ly * x)) * math.exp(-x * x * rc * rc) - tol
    fp = lambda x: -c * math.exp(-x * x * rc * rc) * (0.5 * x ** -1.5 + 2 * rc * rc * x * math.sqrt(1 / x))
    return _newton(f, fp, 4 / rc, tol)


def slp_find_kinfb(Q, Lx, Ly, xi, tol):
    """StokesSLP_ewald_2p.m:147-173 (called with Ly := Lx, :96)."""
    mx = max(Lx, Ly)
    f = lambda k: math.sqrt(4 * Q * math.pi * mx / (Lx ** 3 * Ly ** 3 * k)) * math.exp(-k * k / (4 * xi * xi)) - tol
    fp = lambda k: -math.sqrt(4 * Q * math.pi * mx / (Lx ** 3 * Ly ** 3)) * math.exp(-k * k / (4 * xi * xi)) * \
        (0.5 * k ** -1.5 + math.sqrt(1 / k) * 2 * k / (4 * xi * xi))
    k = _newton(f, fp, matlab_round(5 * xi), tol)
    return int(matlab_round(Lx * k / (2 * math.pi)))


def dlp_find_xi(Q, Lx, Ly, rc, tol):
    """StokesDLP_ewald_2p.m:204-224."""
    c = math.sqrt(2 * math.pi * Q / (Lx * Ly))
    f = lambda a: math.exp(-a * a * rc * rc) * a * rc * c - tol
    fp = lambda a: (1 - 2 * a * a * rc * rc) * math.exp(-a * a * rc * rc) * c * rc
    return _newton(f, fp, 1 / rc, tol)


def dlp_find_kinfb(Q, Lx, Ly, xi, tol):
    """StokesDLP_ewald_2p.m:171-199, keeping its precedence: k*8*pi*Q*max/Lx^3*Ly^3."""
    mx = max(Lx, Ly)
    f = lambda k: math.sqrt(k * 8 * math.pi * Q * mx / Lx ** 3 * Ly ** 3) * math.exp(-k * k / (4 * xi * xi)) - tol
    fp = lambda k: math.sqrt(8 * math.pi * Q * mx / Lx ** 3 * Ly ** 3) * math.exp(-k * k / (4 * xi * xi)) * \
        (0.5 * k ** -0.5 - 2 * k ** 1.5 / (4 * xi * xi))
    k = _newton(f, fp, matlab_round(5 * xi), tol)
    return int(matlab_round(Lx * k / (2 * math.pi)))


def params(kind, nsrc, ntar, fsq_sum, Lx, Ly, P=24, Nb=None, tol=1e-16):
    """(nside_x, nside_y, xi, Mx, My, w, eta) as the MATLAB driver picks them.

    fsq_sum = sum(f.^2) over both components (the Q estimate uses Q = fsq_sum + 1).
    """
    npts = nsrc + ntar
    if Nb is None:
        Nb = min(P * matlab_round(math.log2(npts)), npts / 4)
    A, B = rat(Lx / Ly)
    Q = fsq_sum + 1
    a = math.ceil(math.sqrt(npts / (Nb * A * B)))
    m = 0.95 * math.sqrt(math.pi * P)
    nside_x, nside_y = a * A, a * B
    rc = Lx / nside_x
    if kind == "slp":
        xi = slp_find_xi(Q, Lx, Ly, rc, tol)
        kinf = slp_find_kinfb(Q, Lx, Lx, xi, tol)
    else:
        xi = dlp_find_xi(Q, Lx, Ly, rc, tol)
        kinf = dlp_find_kinfb(Q, Lx, Lx, xi, tol)
    M = min(2 * kinf, 10000)
    My, Mx = B * M, A * M
    w = P * Lx / Mx / 2
    eta = (2 * xi * w / m) ** 2
    return dict(nside_x=int(nside_x), nside_y=int(nside_y), xi=xi, Mx=int(Mx), My=int(My),
                w=w, eta=eta, P=int(P), Nb=Nb, tol=tol)
