"""The four spectral-Ewald MEX gateways of FastTools2D, on the GB300.

Same names, argument order and meaning as
    mex_stokes_slp_real(psrc, ptar, f, xi, nside_x, nside_y, Lx, Ly)
        (PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_real.cpp:58-83)
    mex_stokes_slp_kspace(psrc, ptar, xi, eta, f, Mx, My, Lx, Ly, w, P)
        (PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:8-42)
    mex_stokes_dlp_real(psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly)
        (PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:15-52)
    mex_stokes_dlp_kspace(psrc, ptar, xi, eta, f, n, Mx, My, Lx, Ly, w, P)
        (PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_kspace.cpp:10-53)

Arrays are MATLAB-shaped ``(2, N)``: row 0 holds x components, row 1 y
components.  numpy inputs run through host staging and return numpy
``(2, N)`` results.  torch CUDA tensors of shape ``(N, 2)`` (interleaved,
contiguous float64) are passed to the library by device pointer and the
result is a torch CUDA tensor ``(N, 2)`` on the plan's stream.

Shape errors raise ValueError with the gateway's message
(mex_stokes_slp_kspace.cpp:10-17, mex_stokes_dlp_real.cpp:20-34); library
failures raise Se2pError.
"""
from __future__ import annotations

import numpy as np

from . import _lib


def _is_torch_cuda(a):
    return type(a).__module__.startswith("torch") and getattr(a, "is_cuda", False)


class _Arg:
    """A 2xN argument as a C pointer; keeps the backing buffer alive."""

    def __init__(self, a, name):
        if a is None:
            self.ptr, self.n, self.keep, self.torch = None, 0, None, False
            return
        if _is_torch_cuda(a):
            import torch
            if a.dim() != 2 or a.shape[1] != 2:
                raise ValueError(f"{name} must be an (N, 2) CUDA tensor")
            t = a.to(torch.float64).contiguous()
            self.ptr, self.n, self.keep, self.torch = t.data_ptr(), t.shape[0], t, True
            return
        x = np.asarray(a, dtype=np.float64)
        if x.ndim != 2 or x.shape[0] != 2:
            raise ValueError(f"{name} must be a 2xn matrix.")
        buf = np.ascontiguousarray(x.T)
        self.ptr, self.n, self.keep, self.torch = buf.ctypes.data, buf.shape[0], buf, False


class _Out:
    def __init__(self, n, like_torch, device):
        if like_torch:
            import torch
            self.t = torch.empty((n, 2), dtype=torch.float64, device=f"cuda:{device}")
            self.ptr = self.t.data_ptr()
            self.np = None
        else:
            self.np = np.zeros((max(n, 0), 2))
            self.ptr = self.np.ctypes.data
            self.t = None

    def result(self):
        return self.t if self.t is not None else self.np.T.copy()


def _plan(plan):
    return plan if plan is not None else _lib.default_plan()


def _bind_stream(pl, use_torch):
    if use_torch:
        import torch
        pl.set_stream(torch.cuda.current_stream(pl.device).cuda_stream)


def _same_n(a, b, msg):
    if a.n != b.n:
        raise ValueError(msg)


def mex_stokes_slp_real(psrc, ptar, f, xi, nside_x, nside_y, Lx, Ly, plan=None):
    pl = _plan(plan)
    s, t, ff = _Arg(psrc, "psrc"), _Arg(ptar, "ptar"), _Arg(f, "f")
    _same_n(s, ff, "psrc and f must be the same size.")
    _bind_stream(pl, t.torch)
    out = _Out(t.n, t.torch, pl.device)
    pl.check(pl.lib.se2p_slp_real(pl.handle, s.ptr, s.n, t.ptr, t.n, ff.ptr, float(xi),
                                  int(nside_x), int(nside_y), float(Lx), float(Ly), out.ptr))
    return out.result()


def mex_stokes_slp_kspace(psrc, ptar, xi, eta, f, Mx, My, Lx, Ly, w, P, plan=None):
    pl = _plan(plan)
    s, t, ff = _Arg(psrc, "psrc"), _Arg(ptar, "ptar"), _Arg(f, "f")
    _same_n(s, ff, "psrc and f must be the same size.")
    _bind_stream(pl, t.torch)
    out = _Out(t.n, t.torch, pl.device)
    pl.check(pl.lib.se2p_slp_kspace(pl.handle, s.ptr, s.n, t.ptr, t.n, float(xi), float(eta),
                                    ff.ptr, int(Mx), int(My), float(Lx), float(Ly), float(w),
                                    int(P), out.ptr))
    return out.result()


def mex_stokes_dlp_real(psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly, plan=None):
    pl = _plan(plan)
    s, t, ff, nn = _Arg(psrc, "psrc"), _Arg(ptar, "ptar"), _Arg(f, "f"), _Arg(n, "n")
    _same_n(s, ff, "psrc and f must be the same size.")
    _same_n(s, nn, "psrc and n must be the same size.")
    _bind_stream(pl, t.torch)
    out = _Out(t.n, t.torch, pl.device)
    pl.check(pl.lib.se2p_dlp_real(pl.handle, s.ptr, s.n, t.ptr, t.n, ff.ptr, nn.ptr, float(xi),
                                  int(nside_x), int(nside_y), float(Lx), float(Ly), out.ptr))
    return out.result()


def mex_stokes_dlp_kspace(psrc, ptar, xi, eta, f, n, Mx, My, Lx, Ly, w, P, plan=None):
    pl = _plan(plan)
    s, t, ff, nn = _Arg(psrc, "psrc"), _Arg(ptar, "ptar"), _Arg(f, "f"), _Arg(n, "n")
    _same_n(s, ff, "psrc and f must be the same size.")
    _same_n(s, nn, "psrc and n must be the same size.")
    _bind_stream(pl, t.torch)
    out = _Out(t.n, t.torch, pl.device)
    pl.check(pl.lib.se2p_dlp_kspace(pl.handle, s.ptr, s.n, t.ptr, t.n, float(xi), float(eta),
                                    ff.ptr, nn.ptr, int(Mx), int(My), float(Lx), float(Ly),
                                    float(w), int(P), out.ptr))
    return out.result()
