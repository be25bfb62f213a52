"""Driver layer: the MATLAB functions StokesSLP_ewald_2p / StokesDLP_ewald_2p of
FastTools2D (PeriodicEwald/src/matlab/*.m) on top of libse2p.

``StokesSLP_ewald_2p(xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, P=24, Nb=None,
tol=1e-16, verbose=False)`` returns ``(u1, u2, ur, uk, xi)`` like the MATLAB
function; ``StokesDLP_ewald_2p(xsrc, ysrc, xtar, ytar, n1, n2, f1, f2, Lx, Ly,
...)`` likewise.  Parameter selection (rc from Nb, xi and kinf from the
Palsson-Tornberg error estimates by Newton iteration, M, w, eta) follows
StokesSLP_ewald_2p.m:27-104 and :147-202, StokesDLP_ewald_2p.m:30-125 and
:171-224, including their differences (the SLP passes Lx twice to its kinf
estimate; the DLP kinf estimate keeps the expression k*8*pi*Q*max/Lx^3*Ly^3
as MATLAB parses it).

The lower-level ``slp_ewald``, ``dlp_ewald`` and ``stokes_ewald`` take the
Ewald parameters directly (an :class:`EwaldParams`) and call the C ABI
composites se2p_slp_ewald / se2p_dlp_ewald / se2p_stokes_ewald.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import _lib
from .mex import _Arg, _Out, _bind_stream, _plan, _same_n


@dataclass
class EwaldParams:
    xi: float
    nside_x: int
    nside_y: int
    Mx: int
    My: int
    P: int
    Lx: float
    Ly: float
    w: float
    eta: float

    @staticmethod
    def derived(xi, nside_x, nside_y, Mx, My, P, Lx, Ly):
        """w = P Lx/Mx/2, eta = (2 xi w/m)^2 with m = 0.95 sqrt(pi P)
        (StokesSLP_ewald_2p.m:90, :103-104)."""
        w = P * Lx / Mx / 2
        m = 0.95 * math.sqrt(math.pi * P)
        return EwaldParams(float(xi), int(nside_x), int(nside_y), int(Mx), int(My), int(P),
                           float(Lx), float(Ly), w, (2 * xi * w / m) ** 2)

    def as_c(self) -> _lib.Params:
        return _lib.Params(self.xi, self.nside_x, self.nside_y, self.Mx, self.My, self.P,
                           self.Lx, self.Ly, self.w, self.eta)


# ----------------------------------------------------------------------------
# Parameter selection
# ----------------------------------------------------------------------------
def _round_half_away(x: float) -> float:
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


def rational(x: float):
    """(A, B) with A/B ~ x to 1e-6 relative by continued fractions (MATLAB rat)."""
    tol = 1e-6 * abs(x)
    num, den = _round_half_away(x), 1.0
    pnum, pden = 1.0, 0.0
    rest = x - num
    while abs(x - num / den) >= tol:
        inv = 1.0 / rest
        a = _round_half_away(inv)
        rest = inv - a
        num, pnum = a * num + pnum, num
        den, pden = a * den + pden, den
    sign = -1 if den < 0 else 1
    return int(sign * num), int(abs(den))


def _newton_limited(g, dg, x, tol, maxit=100):
    """x <- x - min(g/g', 0.9 x) until |g| <= tol (at most maxit+2 steps)."""
    for _ in range(maxit + 2):
        gx = g(x)
        if abs(gx) <= tol:
            break
        x -= min(gx / dg(x), 0.9 * x)
    return x


def _xi_slp(Q, Lx, Ly, rc, tol):
    c = math.sqrt(Q * math.pi / (4 * Lx * Ly))
    g = lambda x: c / math.sqrt(x) * math.exp(-(x * rc) ** 2) - tol
    dg = lambda x: -c * math.exp(-(x * rc) ** 2) * (0.5 * x ** -1.5 + 2 * rc * rc * math.sqrt(x))
    return _newton_limited(g, dg, 4 / rc, tol)


def _kinf_slp(Q, L1, L2, xi, tol):
    c = math.sqrt(4 * Q * math.pi * max(L1, L2) / (L1 ** 3 * L2 ** 3))
    s = 4 * xi * xi
    g = lambda k: c / math.sqrt(k) * math.exp(-k * k / s) - tol
    dg = lambda k: -c * math.exp(-k * k / s) * (0.5 * k ** -1.5 + 2 * math.sqrt(k) / s)
    k = _newton_limited(g, dg, _round_half_away(5 * xi), tol)
    return int(_round_half_away(L1 * k / (2 * math.pi)))


def _xi_dlp(Q, Lx, Ly, rc, tol):
    c = math.sqrt(2 * math.pi * Q / (Lx * Ly))
    g = lambda a: math.exp(-(a * rc) ** 2) * a * rc * c - tol
    dg = lambda a: (1 - 2 * (a * rc) ** 2) * math.exp(-(a * rc) ** 2) * c * rc
    return _newton_limited(g, dg, 1 / rc, tol)


def _kinf_dlp(Q, L1, L2, xi, tol, compat=True):
    # MATLAB parses sqrt(k*8*pi*Q*max(Lx,Ly)/Lx^3*Ly^3) as ((...)/Lx^3)*Ly^3;
    # compat=False uses the estimate's intended 1/(Lx^3 Ly^3).
    if compat:
        c = math.sqrt(8 * math.pi * Q * max(L1, L2) / L1 ** 3 * L2 ** 3)
    else:
        c = math.sqrt(8 * math.pi * Q * max(L1, L2) / (L1 ** 3 * L2 ** 3))
    s = 4 * xi * xi
    g = lambda k: c * math.sqrt(k) * math.exp(-k * k / s) - tol
    dg = lambda k: c * math.exp(-k * k / s) * (0.5 / math.sqrt(k) - 2 * k ** 1.5 / s)
    k = _newton_limited(g, dg, _round_half_away(5 * xi), tol)
    return int(_round_half_away(L1 * k / (2 * math.pi)))


def select_params(kind: str, nsrc: int, ntar: int, fsq_sum: float, Lx: float, Ly: float,
                  P: int = 24, Nb=None, tol: float = 1e-16, compat: bool = True) -> EwaldParams:
    """Ewald parameters as the MATLAB drivers choose them; fsq_sum = sum(f.^2).

    compat=True (the default) reproduces the drivers' own arithmetic, so the
    same inputs give the reference's xi, nside and M: the SLP k_inf estimate
    receives (Lx, Lx) (StokesSLP_ewald_2p.m:96) and the DLP one keeps MATLAB's
    parse of /Lx^3*Ly^3 (StokesDLP_ewald_2p.m:177).  compat=False passes
    (Lx, Ly) and divides by Lx^3 Ly^3, as the estimates are written."""
    npts = nsrc + ntar
    if Nb is None:
        Nb = min(P * _round_half_away(math.log2(npts)), npts / 4)
    A, B = rational(Lx / Ly)
    Q = fsq_sum + 1
    a = math.ceil(math.sqrt(npts / (Nb * A * B)))
    nside_x, nside_y = a * A, a * B
    rc = Lx / nside_x
    L2 = Lx if compat else Ly
    if kind == "slp":
        xi = _xi_slp(Q, Lx, Ly, rc, tol)
        kinf = _kinf_slp(Q, Lx, L2, xi, tol)
    elif kind == "dlp":
        xi = _xi_dlp(Q, Lx, Ly, rc, tol)
        kinf = _kinf_dlp(Q, Lx, L2, xi, tol, compat)
    else:
        raise ValueError("kind must be 'slp' or 'dlp'")
    M = min(2 * kinf, 10000)
    return EwaldParams.derived(xi, nside_x, nside_y, A * M, B * M, P, Lx, Ly)


# ----------------------------------------------------------------------------
# Composites with given parameters
# ----------------------------------------------------------------------------
def slp_ewald(psrc, ptar, f, prm: EwaldParams, parts=False, plan=None):
    """u = ur + uk after wrapping (StokesSLP_ewald_2p.m:74-82, :119-133).

    MATLAB-shaped (2, N) numpy arrays or (N, 2) CUDA tensors.  Returns u, or
    (u, ur, uk) with parts=True."""
    pl = _plan(plan)
    s, t, ff = _Arg(psrc, "psrc"), _Arg(ptar, "ptar"), _Arg(f, "f")
    _same_n(s, ff, "psrc and f must be the same size.")
    _bind_stream(pl, t.torch)
    outs = [_Out(t.n, t.torch, pl.device) for _ in range(3 if parts else 1)]
    c = prm.as_c()
    pl.check(pl.lib.se2p_slp_ewald(pl.handle, ctypes.byref(c), s.ptr, s.n, t.ptr, t.n, ff.ptr,
                                   outs[0].ptr, outs[1].ptr if parts else None,
                                   outs[2].ptr if parts else None))
    r = [o.result() for o in outs]
    return tuple(r) if parts else r[0]


def dlp_ewald(psrc, ptar, f, n, prm: EwaldParams, parts=False, plan=None):
    """u = -(ur + uk - sum((f.n) x_src)/(Lx Ly)) (StokesDLP_ewald_2p.m:295-360).
    The zero-mode term uses the caller's unwrapped source positions."""
    pl = _plan(plan)
    s, t, ff, nn = _Arg(psrc, "psrc"), _Arg(ptar, "ptar"), _Arg(f, "f"), _Arg(n, "n")
    _same_n(s, ff, "psrc and f must be the same size.")
    _same_n(s, nn, "psrc and n must be the same size.")
    _bind_stream(pl, t.torch)
    outs = [_Out(t.n, t.torch, pl.device) for _ in range(3 if parts else 1)]
    c = prm.as_c()
    pl.check(pl.lib.se2p_dlp_ewald(pl.handle, ctypes.byref(c), s.ptr, s.n, t.ptr, t.n, ff.ptr,
                                   nn.ptr, outs[0].ptr, outs[1].ptr if parts else None,
                                   outs[2].ptr if parts else None))
    r = [o.result() for o in outs]
    return tuple(r) if parts else r[0]


def stokes_ewald(psrc, ptar, f_slp, f_dlp, n, prm: EwaldParams, plan=None):
    """(u_slp, u_dlp) on one point set in one pass (se2p_stokes_ewald)."""
    pl = _plan(plan)
    s, t = _Arg(psrc, "psrc"), _Arg(ptar, "ptar")
    fs, fd, nn = _Arg(f_slp, "f_slp"), _Arg(f_dlp, "f_dlp"), _Arg(n, "n")
    for a, nm in ((fs, "f_slp"), (fd, "f_dlp"), (nn, "n")):
        _same_n(s, a, f"psrc and {nm} must be the same size.")
    _bind_stream(pl, t.torch)
    o1, o2 = _Out(t.n, t.torch, pl.device), _Out(t.n, t.torch, pl.device)
    c = prm.as_c()
    pl.check(pl.lib.se2p_stokes_ewald(pl.handle, ctypes.byref(c), s.ptr, s.n, t.ptr, t.n,
                                      fs.ptr, fd.ptr, nn.ptr, o1.ptr, o2.ptr))
    return o1.result(), o2.result()


def stokes_ewald_adjoint(psrc, ptar, f_slp, f_dlp, n, w_slp, w_dlp, prm: EwaldParams,
                         plan=None):
    """Gradients of J = sum_t w_slp(t).u_slp(t) + w_dlp(t).u_dlp(t) (u as returned
    by :func:`stokes_ewald`) with respect to source positions, SLP forces, DLP
    densities and normals: returns (g_psrc, g_fslp, g_fdlp, g_n).  Pass None
    for (f_slp, w_slp) or (f_dlp, n, w_dlp) to drop that term; its gradients
    come back as None."""
    pl = _plan(plan)
    s, t = _Arg(psrc, "psrc"), _Arg(ptar, "ptar")
    fs, fd, nn = _Arg(f_slp, "f_slp"), _Arg(f_dlp, "f_dlp"), _Arg(n, "n")
    ws, wd = _Arg(w_slp, "w_slp"), _Arg(w_dlp, "w_dlp")
    slp = fs.ptr is not None and ws.ptr is not None
    dlp = fd.ptr is not None and nn.ptr is not None and wd.ptr is not None
    for a, nm in ((fs, "f_slp"), (fd, "f_dlp"), (nn, "n")):
        if a.ptr is not None:
            _same_n(s, a, f"psrc and {nm} must be the same size.")
    for a, nm in ((ws, "w_slp"), (wd, "w_dlp")):
        if a.ptr is not None:
            _same_n(t, a, f"ptar and {nm} must be the same size.")
    _bind_stream(pl, s.torch)
    outs = [_Out(s.n, s.torch, pl.device) for _ in range(4)]
    c = prm.as_c()
    pl.check(pl.lib.se2p_stokes_ewald_adjoint(
        pl.handle, ctypes.byref(c), s.ptr, s.n, t.ptr, t.n, fs.ptr if slp else None,
        fd.ptr if dlp else None, nn.ptr if dlp else None, ws.ptr if slp else None,
        wd.ptr if dlp else None, outs[0].ptr, outs[1].ptr if slp else None,
        outs[2].ptr if dlp else None, outs[3].ptr if dlp else None))
    r = [o.result() for o in outs]
    return r[0], (r[1] if slp else None), (r[2] if dlp else None), (r[3] if dlp else None)


# ----------------------------------------------------------------------------
# The MATLAB drivers
# ----------------------------------------------------------------------------
def _col(a):
    return np.asarray(a, dtype=np.float64).reshape(-1)


def _verbose_print(kind, prm, ns, nt, tol, Nb):
    name = "SINGLE" if kind == "slp" else "DOUBLE"
    print(f"SPECTRAL EWALD FOR THE STOKES {name}-LAYER POTENTIAL")
    print(f"NUMBER OF SOURCES: {ns}\nNUMBER OF TARGETS: {nt}\nTOLERANCE: {tol:3.3e}")
    print(f"P: {prm.P}\nPoints per box: {Nb}")
    print(f"\txi: {prm.xi:3.3f}\n\trc: {prm.Lx / prm.nside_x:3.3f}\n\tMx: {prm.Mx}\n"
          f"\tMy: {prm.My}\n\tw: {prm.w:3.3f}\n\teta: {prm.eta:3.3f}")


def StokesSLP_ewald_2p(xsrc, ysrc, xtar, ytar, f1, f2, Lx, Ly, P=24, Nb=None, tol=1e-16,
                       verbose=False, plan=None):
    """Doubly-periodic Stokeslet by spectral Ewald (StokesSLP_ewald_2p.m:1-138).

    Returns (u1, u2, ur, uk, xi); ur and uk are 2 x Ntar like the MATLAB
    outputs."""
    xs, ys, xt, yt = map(_col, (xsrc, ysrc, xtar, ytar))
    f = np.vstack([_col(f1), _col(f2)])
    npts = xs.size + xt.size
    if Nb is None:
        Nb = min(P * _round_half_away(math.log2(npts)), npts / 4)
    prm = select_params("slp", xs.size, xt.size, float(np.sum(f ** 2)), Lx, Ly, P, Nb, tol)
    if verbose:
        _verbose_print("slp", prm, xs.size, xt.size, tol, Nb)
    u, ur, uk = slp_ewald(np.vstack([xs, ys]), np.vstack([xt, yt]), f, prm, parts=True,
                          plan=plan)
    return u[0], u[1], ur, uk, prm.xi


def StokesDLP_ewald_2p(xsrc, ysrc, xtar, ytar, n1, n2, f1, f2, Lx, Ly, P=24, Nb=None,
                       tol=1e-16, verbose=False, unit_normal_fix=True, plan=None):
    """Doubly-periodic stresslet by spectral Ewald (StokesDLP_ewald_2p.m:1-365).

    unit_normal_fix mirrors the driver's guard for MATLAB releases after
    R2017a (StokesDLP_ewald_2p.m:69-80): n1 -= 1e-60, n2 = sqrt(1-n1^2) sign(n2),
    f += 1e-60, i.e. normals are re-normalised from n1 and the sign of n2.
    Returns (u1, u2, ur, uk, xi)."""
    xs, ys, xt, yt = map(_col, (xsrc, ysrc, xtar, ytar))
    n1, n2, f1, f2 = map(_col, (n1, n2, f1, f2))
    if unit_normal_fix:
        off = 1e-60
        n1 = n1 - off
        if np.all(n1 < -1):
            n1 = n1 + 2 * off
        n2 = np.sqrt(1 - n1 ** 2) * np.sign(n2)
        f1 = f1 + off
        f2 = f2 + off
    f = np.vstack([f1, f2])
    npts = xs.size + xt.size
    if Nb is None:
        Nb = min(P * _round_half_away(math.log2(npts)), npts / 4)
    # the DLP driver recomputes npts as length(psrc)+length(ptar) (:309)
    ns_len = max(xs.size, 2) if xs.size else 0
    nt_len = max(xt.size, 2) if xt.size else 0
    prm = select_params("dlp", ns_len, nt_len, float(np.sum(f ** 2)), Lx, Ly, P, Nb, tol)
    if verbose:
        _verbose_print("dlp", prm, xs.size, xt.size, tol, Nb)
    u, ur, uk = dlp_ewald(np.vstack([xs, ys]), np.vstack([xt, yt]), f, np.vstack([n1, n2]), prm,
                          parts=True, plan=plan)
    return u[0], u[1], ur, uk, prm.xi


class Geometry:
    """One point set for many right-hand sides (se2p_geom_*).

    Sorts the points, builds the cell lists and stores the real-space
    operator once; :meth:`apply` then evaluates any number of densities, each
    exactly as :func:`stokes_ewald` (or :func:`slp_ewald` / :func:`dlp_ewald`
    for one kind) would.  ``kinds`` is "slp", "dlp" or "both"; normals ``n``
    belong to the geometry (DLP).  Arrays are MATLAB-shaped 2xN numpy arrays
    or (N, 2) CUDA tensors, as elsewhere in this package.
    """

    _KINDS = {"slp": 1, "dlp": 2, "both": 3}

    def __init__(self, psrc, ptar, prm: EwaldParams, n=None, kinds: str = "both", plan=None):
        self.plan = _plan(plan)
        self.kinds = self._KINDS[kinds]
        self.prm = prm
        s, t, nn = _Arg(psrc, "psrc"), _Arg(ptar, "ptar"), _Arg(n, "n")
        if self.kinds & 2:
            _same_n(s, nn, "psrc and n must be the same size.")
        self.ns, self.nt, self.torch = s.n, t.n, t.torch
        self.handle = ctypes.c_void_p()
        c = prm.as_c()
        self.plan.check(self.plan.lib.se2p_geom_create(self.plan.handle, ctypes.byref(c), s.ptr,
                                                       s.n, t.ptr, t.n, nn.ptr, self.kinds,
                                                       ctypes.byref(self.handle)))

    @property
    def bytes(self) -> int:
        return self.plan.lib.se2p_geom_bytes(self.handle)

    @property
    def pairs(self) -> int:
        return self.plan.lib.se2p_geom_pairs(self.handle)

    def _rhs(self, f, name):
        """nrhs x 2 x N numpy (or nrhs x N x 2 CUDA tensor) -> (pointer, nrhs, keep)."""
        if f is None:
            return None, None, None
        if _is_torch(f):
            import torch
            t = f.to(torch.float64).contiguous()
            if t.dim() != 3 or t.shape[1] != self.ns or t.shape[2] != 2:
                raise ValueError(f"{name} must be an (nrhs, nsrc, 2) CUDA tensor")
            return t.data_ptr(), t.shape[0], t
        x = np.asarray(f, dtype=np.float64)
        if x.ndim == 2:
            x = x[None]
        if x.ndim != 3 or x.shape[1] != 2 or x.shape[2] != self.ns:
            raise ValueError(f"{name} must be nrhs x 2 x nsrc")
        buf = np.ascontiguousarray(np.transpose(x, (0, 2, 1)))
        return buf.ctypes.data, x.shape[0], buf

    def apply(self, f_slp=None, f_dlp=None):
        """u for each right-hand side: (u_slp, u_dlp), each nrhs x 2 x ntar (or
        nrhs x ntar x 2 tensors); the kind not in the geometry is None."""
        ps, ns_, ks = self._rhs(f_slp if self.kinds & 1 else None, "f_slp")
        pd, nd_, kd = self._rhs(f_dlp if self.kinds & 2 else None, "f_dlp")
        nrhs = ns_ if ns_ is not None else nd_
        if nrhs is None:
            raise ValueError("no right-hand side given")
        if ns_ is not None and nd_ is not None and ns_ != nd_:
            raise ValueError("f_slp and f_dlp must hold the same number of right-hand sides")
        use_torch = any(k is not None and not isinstance(k, np.ndarray) for k in (ks, kd))
        outs = []
        for on in (self.kinds & 1, self.kinds & 2):
            if not on:
                outs.append(None)
            elif use_torch:
                import torch
                outs.append(torch.empty((nrhs, self.nt, 2), dtype=torch.float64,
                                        device=f"cuda:{self.plan.device}"))
            else:
                outs.append(np.zeros((nrhs, self.nt, 2)))
        ptr = lambda o: None if o is None else (o.data_ptr() if not isinstance(o, np.ndarray)
                                                 else o.ctypes.data)
        self.plan.check(self.plan.lib.se2p_geom_apply(self.handle, nrhs, ps, pd, ptr(outs[0]),
                                                      ptr(outs[1])))
        res = []
        for o in outs:
            if o is None or not isinstance(o, np.ndarray):
                res.append(o)
            else:
                res.append(np.transpose(o, (0, 2, 1)).copy())
        return tuple(res)

    def close(self):
        if self.handle:
            self.plan.lib.se2p_geom_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _is_torch(a):
    return type(a).__module__.startswith("torch")
