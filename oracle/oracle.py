"""CPU oracle for the spectral-Ewald SLP/DLP path -- TEST INFRASTRUCTURE ONLY.

Python side of the oracle: ctypes glue over ``libse2p_oracle.so`` (the C
restatement in ``se2p_oracle.c``) plus the FFT step, which the reference
delegates to MATLAB's ``fft2``/``ifft2`` via ``mexCallMATLAB``
(PE/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:148-149, :236-241;
PE/src/mex/StokesDLP/mex_stokes_dlp_kspace.cpp:167-170, :300-305) and which
is done here with scipy's FP64 FFT on full complex spectra.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, always as the checker or the timed CPU
baseline, never as the product path.

All array arguments follow MATLAB's MEX layout: ``(2, N)`` arrays (row 0 = x
components, row 1 = y components), i.e. interleaved (x, y) per point in
column-major memory.  Results are ``(2, N)`` numpy arrays.

Parity of this oracle is pinned against the reference's own sources compiled
under ``oracle/_ref`` (see ``ref_mex.py``) and against the committed
fixtures in ``tests/golden`` generated from them.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libse2p_oracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)


def build(force: bool = False) -> str:
    """Compile the C restatement (``make -C oracle``); returns the .so path."""
    src = os.path.join(_HERE, "se2p_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-C", _HERE, "libse2p_oracle.so"], check=True,
                       stdout=subprocess.DEVNULL)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        i64, i32, d = ctypes.c_int64, ctypes.c_int, ctypes.c_double
        L.or_assign.argtypes = [_dp, i64, d, d, i32, i32, _ip, _ip]
        L.or_find_closest_node.argtypes = [d, d, d, d, d, i32, ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_int), _dp, _dp]
        L.or_e1.argtypes = [d, _dp]
        L.or_e1.restype = d
        L.or_slp_real.argtypes = [_dp, i64, _dp, i64, _dp, d, i32, i32, d, d, _dp]
        L.or_dlp_real.argtypes = [_dp, i64, _dp, i64, _dp, _dp, d, i32, i32, d, d, _dp]
        L.or_spread.argtypes = [_dp, i64, _dp, _dp, d, d, i32, i32, d, d, d, i32, _dp]
        L.or_slp_filter.argtypes = [_dp, _dp, i32, i32, d, d, d, d]
        L.or_dlp_filter.argtypes = [_dp, _dp, i32, i32, d, d, d, d]
        L.or_gather.argtypes = [_dp, i64, _dp, d, d, i32, i32, d, d, d, i32, _dp]
        L.or_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def num_threads() -> int:
    return lib().or_num_threads()


def _il(a):
    """MATLAB (2, N) -> contiguous interleaved (N, 2) float64 buffer."""
    a = np.asarray(a, dtype=np.float64)
    if a.ndim != 2 or a.shape[0] != 2:
        raise ValueError("expected a 2xN array")
    return np.ascontiguousarray(a.T)


def _p(a):
    return a.ctypes.data_as(_dp)


# --------------------------------------------------------------------------
# Building blocks (exposed for fine-grained tests)
# --------------------------------------------------------------------------
def assign(p, Lx, Ly, nside_x, nside_y):
    """Cell binning (PE/src/mex/common/ewald_tools.cpp:7-80): (perm, start)."""
    q = _il(p)
    n = q.shape[0]
    perm = np.zeros(max(n, 1), np.int32)
    start = np.zeros(nside_x * nside_y + 1, np.int32)
    lib().or_assign(_p(q), n, Lx, Ly, nside_x, nside_y, perm.ctypes.data_as(_ip),
                    start.ctypes.data_as(_ip))
    return perm[:n], start


def find_closest_node(x, y, Lx, Ly, h, P):
    """PE/src/mex/common/ewald_tools.cpp:86-114 -> (mx, my, px, py)."""
    mx, my = ctypes.c_int(), ctypes.c_int()
    px, py = ctypes.c_double(), ctypes.c_double()
    lib().or_find_closest_node(x, y, Lx, Ly, h, P, ctypes.byref(mx), ctypes.byref(my),
                               ctypes.byref(px), ctypes.byref(py))
    return mx.value, my.value, px.value, py.value


def e1(x):
    """The reference's Pade E1 (PE/src/mex/StokesSLP/mex_stokes_slp_real.cpp:166-205)."""
    e = ctypes.c_double()
    return lib().or_e1(float(x), ctypes.byref(e)), e.value


def spread(psrc, f, n, xi, eta, Mx, My, Lx, Ly, w, P):
    """Gaussian spread; returns (ncomp, Mx, My) (each an My x Mx col-major grid)."""
    s = _il(psrc)
    ff = _il(f)
    nn = _il(n) if n is not None else None
    nc = 4 if nn is not None else 2
    H = np.zeros((nc, Mx, My))
    lib().or_spread(_p(s), s.shape[0], _p(ff), _p(nn) if nn is not None else None,
                    xi, eta, Mx, My, Lx, Ly, w, P, _p(H))
    return H


def gather(ptar, Ht, xi, eta, Mx, My, Lx, Ly, w, P):
    t = _il(ptar)
    Ht = np.ascontiguousarray(Ht, dtype=np.float64)
    u = np.zeros((t.shape[0], 2))
    lib().or_gather(_p(t), t.shape[0], _p(Ht), xi, eta, Mx, My, Lx, Ly, w, P, _p(u))
    return u.T.copy()


def _fft2(a, inverse=False, workers=-1):
    import scipy.fft as sfft
    return (sfft.ifft2 if inverse else sfft.fft2)(a, axes=(-2, -1), workers=workers)


def filtered_grids(kind, psrc, f, n, xi, eta, Mx, My, Lx, Ly, w, P, workers=-1):
    """Spread -> fft2 -> filter -> ifft2; returns the 2 real grids the gather reads."""
    H = spread(psrc, f, n, xi, eta, Mx, My, Lx, Ly, w, P)
    Hh = _fft2(H, workers=workers)
    re = np.ascontiguousarray(Hh.real)
    im = np.ascontiguousarray(Hh.imag)
    del Hh
    filt = lib().or_slp_filter if kind == "slp" else lib().or_dlp_filter
    filt(_p(re), _p(im), Mx, My, Lx, Ly, xi, eta)
    Ht = _fft2(re[:2] + 1j * im[:2], inverse=True, workers=workers)
    # SLP keeps the real part (mex_stokes_slp_kspace.cpp:239-241), DLP the
    # imaginary part (mex_stokes_dlp_kspace.cpp:303-305).
    return np.ascontiguousarray(Ht.real if kind == "slp" else Ht.imag)


# --------------------------------------------------------------------------
# The four MEX entry points (same argument order as the gateways)
# --------------------------------------------------------------------------
def mex_stokes_slp_real(psrc, ptar, f, xi, nside_x, nside_y, Lx, Ly):
    s, t, ff = _il(psrc), _il(ptar), _il(f)
    u = np.zeros((t.shape[0], 2))
    lib().or_slp_real(_p(s), s.shape[0], _p(t), t.shape[0], _p(ff), xi, int(nside_x),
                      int(nside_y), Lx, Ly, _p(u))
    return u.T.copy()


def mex_stokes_dlp_real(psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly):
    s, t, ff, nn = _il(psrc), _il(ptar), _il(f), _il(n)
    u = np.zeros((t.shape[0], 2))
    lib().or_dlp_real(_p(s), s.shape[0], _p(t), t.shape[0], _p(ff), _p(nn), xi, int(nside_x),
                      int(nside_y), Lx, Ly, _p(u))
    return u.T.copy()


def mex_stokes_slp_kspace(psrc, ptar, xi, eta, f, Mx, My, Lx, Ly, w, P, workers=-1):
    Mx, My, P = int(Mx), int(My), int(P)
    Ht = filtered_grids("slp", psrc, f, None, xi, eta, Mx, My, Lx, Ly, w, P, workers)
    return gather(ptar, Ht, xi, eta, Mx, My, Lx, Ly, w, P)


def mex_stokes_dlp_kspace(psrc, ptar, xi, eta, f, n, Mx, My, Lx, Ly, w, P, workers=-1):
    Mx, My, P = int(Mx), int(My), int(P)
    Ht = filtered_grids("dlp", psrc, f, n, xi, eta, Mx, My, Lx, Ly, w, P, workers)
    return gather(ptar, Ht, xi, eta, Mx, My, Lx, Ly, w, P)


# --------------------------------------------------------------------------
# Driver-level composites (PE/src/matlab/Stokes{SLP,DLP}_ewald_2p.m with the
# parameters given instead of estimated)
# --------------------------------------------------------------------------
def wrap(x, L):
    """MATLAB mod(x + L/2, L) - L/2 (StokesSLP_ewald_2p.m:75-78)."""
    x = np.asarray(x, dtype=np.float64)
    return np.mod(x + L / 2, L) - L / 2


def slp_ewald(psrc, ptar, f, xi, nside_x, nside_y, Mx, My, Lx, Ly, P, w=None, eta=None,
              workers=-1):
    """u = ur + uk (StokesSLP_ewald_2p.m:119-133); returns (u, ur, uk)."""
    w, eta = derived_w_eta(xi, Mx, Lx, P, w, eta)
    ps = np.vstack([wrap(psrc[0], Lx), wrap(psrc[1], Ly)])
    pt = np.vstack([wrap(ptar[0], Lx), wrap(ptar[1], Ly)])
    ur = mex_stokes_slp_real(ps, pt, f, xi, nside_x, nside_y, Lx, Ly)
    uk = mex_stokes_slp_kspace(ps, pt, xi, eta, f, Mx, My, Lx, Ly, w, P, workers)
    return ur + uk, ur, uk


def dlp_zero_mode(psrc, f, n, Lx, Ly):
    """k=0 term sum((f.n) x_src)/(Lx Ly) on UNWRAPPED sources (StokesDLP_ewald_2p.m:150-151)."""
    fn = f[0] * n[0] + f[1] * n[1]
    return np.array([np.sum(fn * psrc[0]), np.sum(fn * psrc[1])]) / (Lx * Ly)


def dlp_ewald(psrc, ptar, f, n, xi, nside_x, nside_y, Mx, My, Lx, Ly, P, w=None, eta=None,
              workers=-1):
    """u = -(ur + uk - zero mode) (StokesDLP_ewald_2p.m:140-158); returns (u, ur, uk)."""
    w, eta = derived_w_eta(xi, Mx, Lx, P, w, eta)
    ps = np.vstack([wrap(psrc[0], Lx), wrap(psrc[1], Ly)])
    pt = np.vstack([wrap(ptar[0], Lx), wrap(ptar[1], Ly)])
    ur = mex_stokes_dlp_real(ps, pt, f, n, xi, nside_x, nside_y, Lx, Ly)
    uk = mex_stokes_dlp_kspace(ps, pt, xi, eta, f, n, Mx, My, Lx, Ly, w, P, workers)
    uk = uk - dlp_zero_mode(psrc, f, n, Lx, Ly)[:, None]
    return -(ur + uk), ur, uk


def derived_w_eta(xi, Mx, Lx, P, w=None, eta=None):
    """w = P Lx / Mx / 2 and eta = (2 xi w / m)^2, m = 0.95 sqrt(pi P)
    (StokesSLP_ewald_2p.m:90, :103-104)."""
    if w is None:
        w = P * Lx / Mx / 2
    if eta is None:
        m = 0.95 * np.sqrt(np.pi * P)
        eta = (2 * xi * w / m) ** 2
    return w, eta
