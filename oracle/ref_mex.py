"""Loader for the reference MEX gateways compiled under ``oracle/_ref``.

ORACLE / TEST INFRASTRUCTURE ONLY.  ``make -C oracle ref`` compiles
FastTools2D's own spectral-Ewald sources (PE/src/mex/StokesSLP/*.cpp,
PE/src/mex/StokesDLP/*.cpp, PE/src/mex/common/ewald_tools.cpp) unchanged
against the MATLAB stand-in in ``oracle/mexshim``.  This module builds
``mxArray`` arguments, serves the ``fft2``/``ifft2`` calls the sources make
through ``mexCallMATLAB`` with scipy's FP64 FFT (MATLAB uses FFTW; both are
FP64-accurate transforms with 1/(M*N) on the inverse), and returns the
gateway's ``plhs[0]`` as a numpy ``(2, N)`` array, i.e. MATLAB's 2xN layout.

The compiled reference needs x86-64 (SSE3 intrinsics) and the reference
tree, so it exists only where the fixtures are generated; the committed
fixtures under ``tests/golden`` carry its outputs elsewhere.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(_HERE, "_ref")
NAMES = ("mex_stokes_slp_real", "mex_stokes_slp_kspace",
         "mex_stokes_dlp_real", "mex_stokes_dlp_kspace")

_FFT_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t,
                           ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                           ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double))


def available() -> bool:
    return all(os.path.exists(os.path.join(REF_DIR, n + ".so")) for n in NAMES) and \
        os.path.exists(os.path.join(REF_DIR, "libmexshim.so"))


def _fft2_callback(inverse, m, n, re, im, out_re, out_im):
    """MATLAB fft2/ifft2 of an m x n column-major array (numpy view n x m)."""
    try:
        import scipy.fft as sfft
        x = np.ctypeslib.as_array(re, shape=(n, m)).astype(np.complex128)
        if im:
            x = x + 1j * np.ctypeslib.as_array(im, shape=(n, m))
        y = sfft.ifft2(x, workers=-1) if inverse else sfft.fft2(x, workers=-1)
        np.ctypeslib.as_array(out_re, shape=(n, m))[...] = y.real
        np.ctypeslib.as_array(out_im, shape=(n, m))[...] = y.imag
        return 0
    except Exception:  # pragma: no cover - reported as a MEX error
        return 1


class MexSet:
    """Four MEX gateways loaded from ``lib_dir``, called with MATLAB-shaped numpy args.

    ``shim`` is the MATLAB stand-in they were linked against.  Used for the
    reference's own gateways (``RefMex``) and for the GPU gateways in
    ``fasttools2d_gb300/mexgw`` built against the same stand-in.
    """

    def __init__(self, lib_dir, shim, ext=".so"):
        self.shim = ctypes.CDLL(shim, mode=ctypes.RTLD_GLOBAL)
        s = self.shim
        s.mxCreateDoubleMatrix.restype = ctypes.c_void_p
        s.mxCreateDoubleMatrix.argtypes = [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int]
        s.mxGetPr.restype = ctypes.POINTER(ctypes.c_double)
        s.mxGetPr.argtypes = [ctypes.c_void_p]
        s.mxGetM.restype = ctypes.c_size_t
        s.mxGetM.argtypes = [ctypes.c_void_p]
        s.mxGetN.restype = ctypes.c_size_t
        s.mxGetN.argtypes = [ctypes.c_void_p]
        s.mxDestroyArray.argtypes = [ctypes.c_void_p]
        s.shim_call.restype = ctypes.c_int
        s.shim_call.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                ctypes.c_char_p, ctypes.c_size_t]
        self._cb = _FFT_CB(_fft2_callback)
        s.shim_set_fft.argtypes = [_FFT_CB]
        s.shim_set_fft(self._cb)
        self.fn = {}
        for n in NAMES:
            lib = ctypes.CDLL(os.path.join(lib_dir, n + ext), mode=ctypes.RTLD_LOCAL)
            self.fn[n] = ctypes.cast(lib.mexFunction, ctypes.c_void_p).value
            setattr(self, "_lib_" + n, lib)

    def clear(self):
        """MATLAB's ``clear mex``: run the functions the gateways gave mexAtExit."""
        self.shim.shim_run_atexit()

    def _mx(self, a):
        a = np.asarray(a, dtype=np.float64)
        if a.ndim == 0:
            a = a.reshape(1, 1)
        m, n = a.shape
        p = self.shim.mxCreateDoubleMatrix(m, n, 0)
        if m * n:
            dst = np.ctypeslib.as_array(self.shim.mxGetPr(p), shape=(n, m))
            dst[...] = a.T
        return p

    def call(self, name, *args):
        prhs = (ctypes.c_void_p * len(args))(*[self._mx(a) for a in args])
        plhs = (ctypes.c_void_p * 1)()
        err = ctypes.create_string_buffer(512)
        try:
            rc = self.shim.shim_call(self.fn[name], 1, plhs, len(args), prhs, err, 512)
            if rc:
                raise RuntimeError(f"{name}: {err.value.decode()}")
            out = plhs[0]
            m, n = self.shim.mxGetM(out), self.shim.mxGetN(out)
            res = np.ctypeslib.as_array(self.shim.mxGetPr(out), shape=(n, m)).T.copy() \
                if m * n else np.zeros((m, n))
            self.shim.mxDestroyArray(out)
            return res
        finally:
            for p in prhs:
                self.shim.mxDestroyArray(p)

    # MEX argument orders: PE/src/mex/StokesSLP/mex_stokes_slp_real.cpp:65-83,
    # mex_stokes_slp_kspace.cpp:20-42, PE/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:37-52,
    # mex_stokes_dlp_kspace.cpp:29-53.
    def slp_real(self, psrc, ptar, f, xi, nside_x, nside_y, Lx, Ly):
        return self.call("mex_stokes_slp_real", psrc, ptar, f, xi, nside_x, nside_y, Lx, Ly)

    def slp_kspace(self, psrc, ptar, xi, eta, f, Mx, My, Lx, Ly, w, P):
        return self.call("mex_stokes_slp_kspace", psrc, ptar, xi, eta, f, Mx, My, Lx, Ly, w, P)

    def dlp_real(self, psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly):
        return self.call("mex_stokes_dlp_real", psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly)

    def dlp_kspace(self, psrc, ptar, xi, eta, f, n, Mx, My, Lx, Ly, w, P):
        return self.call("mex_stokes_dlp_kspace", psrc, ptar, xi, eta, f, n, Mx, My, Lx, Ly, w, P)


class RefMex(MexSet):
    """The reference's own four MEX gateways compiled under ``oracle/_ref``."""

    def __init__(self):
        if not available():
            raise RuntimeError("oracle/_ref not built (run `make -C oracle ref` on x86-64)")
        super().__init__(REF_DIR, os.path.join(REF_DIR, "libmexshim.so"))
