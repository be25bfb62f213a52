"""ctypes binding of libse2p.so (the C ABI declared in include/se2p.h).

The CUDA library is the only compute path: if libse2p.so is missing or no
GPU is present, loading fails with an error instead of falling back to any
CPU implementation.
"""
from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libse2p.so")

SE2P_OK, SE2P_ERR_ARG, SE2P_ERR_CUDA, SE2P_ERR_CUFFT, SE2P_ERR_ALLOC, SE2P_ERR_UNSUPPORTED = range(6)
NOALLOC_SCRATCH_BYTES = 32 << 20   # SE2P_NOALLOC_SCRATCH_BYTES
STATUS_NAMES = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_CUFFT", 4: "ERR_ALLOC",
                5: "ERR_UNSUPPORTED"}

# Every symbol include/se2p.h declares, for load checks.
EXPORTS = (
    "se2p_version", "se2p_plan_create", "se2p_plan_destroy", "se2p_plan_set_stream",
    "se2p_plan_last_error", "se2p_plan_workspace_bytes", "se2p_plan_kernel_launches",
    "se2p_slp_real", "se2p_slp_kspace", "se2p_dlp_real", "se2p_dlp_kspace",
    "se2p_slp_ewald", "se2p_dlp_ewald", "se2p_stokes_ewald",
    "se2p_plan_enable_timing", "se2p_num_stages", "se2p_stage_name", "se2p_plan_stage_times",
    "se2p_plan_probe_atomics",
    "se2p_plan_count_pairs", "se2p_slp_real_noalloc", "se2p_plan_set_precision",
    "se2p_plan_set_overlap", "se2p_stokes_ewald_adjoint",
    "se2p_geom_create", "se2p_geom_apply", "se2p_geom_bytes", "se2p_geom_pairs",
    "se2p_geom_destroy",
)
PRECISION_FP64, PRECISION_FP32_GRID, PRECISION_FP64_NATIVE = 0, 1, 2
_PRECISIONS = {"fp64": PRECISION_FP64, "fp32_grid": PRECISION_FP32_GRID,
               "fp64_native": PRECISION_FP64_NATIVE}


class Se2pError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"se2p {STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    """se2p_params (include/se2p.h)."""
    _fields_ = [("xi", ctypes.c_double), ("nside_x", ctypes.c_int), ("nside_y", ctypes.c_int),
                ("Mx", ctypes.c_int), ("My", ctypes.c_int), ("P", ctypes.c_int),
                ("Lx", ctypes.c_double), ("Ly", ctypes.c_double), ("w", ctypes.c_double),
                ("eta", ctypes.c_double)]


_lib = None
_lock = threading.Lock()
_dp = ctypes.c_void_p   # double* (host or device address)


def load(path: str = LIB_PATH):
    """Load libse2p.so and declare its signatures (no CUDA call is made)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(f"libse2p.so not built ({path}); run "
                               "`python -m fasttools2d_gb300.build` (needs nvcc)")
        L = ctypes.CDLL(path)
        i64, i32, d, P = ctypes.c_int64, ctypes.c_int, ctypes.c_double, ctypes.c_void_p
        L.se2p_version.restype = ctypes.c_char_p
        L.se2p_plan_create.argtypes = [ctypes.POINTER(P), i32]
        L.se2p_plan_destroy.argtypes = [P]
        L.se2p_plan_set_stream.argtypes = [P, P]
        L.se2p_plan_last_error.argtypes = [P]
        L.se2p_plan_last_error.restype = ctypes.c_char_p
        L.se2p_plan_workspace_bytes.argtypes = [P]
        L.se2p_plan_workspace_bytes.restype = i64
        L.se2p_plan_kernel_launches.argtypes = [P]
        L.se2p_plan_kernel_launches.restype = i64
        L.se2p_slp_real.argtypes = [P, _dp, i64, _dp, i64, _dp, d, i32, i32, d, d, _dp]
        L.se2p_slp_kspace.argtypes = [P, _dp, i64, _dp, i64, d, d, _dp, i32, i32, d, d, d, i32, _dp]
        L.se2p_dlp_real.argtypes = [P, _dp, i64, _dp, i64, _dp, _dp, d, i32, i32, d, d, _dp]
        L.se2p_dlp_kspace.argtypes = [P, _dp, i64, _dp, i64, d, d, _dp, _dp, i32, i32, d, d, d,
                                      i32, _dp]
        L.se2p_plan_enable_timing.argtypes = [P, i32]
        L.se2p_stage_name.argtypes = [i32]
        L.se2p_stage_name.restype = ctypes.c_char_p
        L.se2p_plan_probe_atomics.argtypes = [P, ctypes.POINTER(ctypes.c_double)]
        L.se2p_plan_stage_times.argtypes = [P, ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_int64), i32]
        L.se2p_plan_count_pairs.argtypes = [P, i32, ctypes.POINTER(ctypes.c_int64), i32]
        L.se2p_plan_set_precision.argtypes = [P, i32]
        L.se2p_plan_set_overlap.argtypes = [P, i32]
        L.se2p_slp_real_noalloc.argtypes = [_dp, i64, _dp, i64, _dp, d, i32, i32, d, d, _dp, P]
        PP = ctypes.POINTER(Params)
        L.se2p_slp_ewald.argtypes = [P, PP, _dp, i64, _dp, i64, _dp, _dp, _dp, _dp]
        L.se2p_dlp_ewald.argtypes = [P, PP, _dp, i64, _dp, i64, _dp, _dp, _dp, _dp, _dp]
        L.se2p_stokes_ewald.argtypes = [P, PP, _dp, i64, _dp, i64, _dp, _dp, _dp, _dp, _dp]
        L.se2p_stokes_ewald_adjoint.argtypes = [P, PP, _dp, i64, _dp, i64, _dp, _dp, _dp, _dp, _dp,
                                                _dp, _dp, _dp, _dp]
        L.se2p_geom_create.argtypes = [P, PP, _dp, i64, _dp, i64, _dp, i32, ctypes.POINTER(P)]
        L.se2p_geom_apply.argtypes = [P, i32, _dp, _dp, _dp, _dp]
        L.se2p_geom_bytes.argtypes = [P]
        L.se2p_geom_bytes.restype = i64
        L.se2p_geom_pairs.argtypes = [P]
        L.se2p_geom_pairs.restype = i64
        L.se2p_geom_destroy.argtypes = [P]
        for name in EXPORTS:
            if name not in ("se2p_version",):
                getattr(L, name).restype = getattr(L, name).restype or ctypes.c_int
        _lib = L
        return L


class Plan:
    """Owns an se2p_plan (stream, workspace, cuFFT plans) on one device."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.handle = ctypes.c_void_p()
        rc = self.lib.se2p_plan_create(ctypes.byref(self.handle), device)
        if rc != SE2P_OK:
            raise Se2pError(rc, f"cannot create a plan on CUDA device {device}")
        self.device = device
        self.precision = "fp64"

    def check(self, rc):
        if rc != SE2P_OK:
            raise Se2pError(rc, self.lib.se2p_plan_last_error(self.handle).decode())

    def set_stream(self, stream_ptr):
        self.check(self.lib.se2p_plan_set_stream(self.handle, ctypes.c_void_p(stream_ptr or 0)))

    @property
    def workspace_bytes(self) -> int:
        return self.lib.se2p_plan_workspace_bytes(self.handle)

    @property
    def kernel_launches(self) -> int:
        return self.lib.se2p_plan_kernel_launches(self.handle)

    def set_precision(self, precision):
        """'fp64' (default: FP64 results, float-float hot loops), 'fp64_native'
        (every operation in FP64) or 'fp32_grid' (mixed precision, tolerances >= 1e-6)."""
        code = _PRECISIONS.get(precision, precision)
        self.check(self.lib.se2p_plan_set_precision(self.handle, int(code)))
        self.precision = {v: k for k, v in _PRECISIONS.items()}[int(code)]

    def set_overlap(self, on: bool = True):
        self.check(self.lib.se2p_plan_set_overlap(self.handle, 1 if on else 0))

    def enable_timing(self, on: bool = True):
        self.check(self.lib.se2p_plan_enable_timing(self.handle, 1 if on else 0))

    def stage_times(self, reset: bool = True):
        """{stage: (total_ms, calls)} accumulated since the last reset."""
        n = self.lib.se2p_num_stages()
        ms = (ctypes.c_double * n)()
        calls = (ctypes.c_int64 * n)()
        self.check(self.lib.se2p_plan_stage_times(self.handle, ms, calls, 1 if reset else 0))
        return {self.lib.se2p_stage_name(i).decode(): (ms[i], calls[i]) for i in range(n)}

    def probe_atomics(self) -> float:
        """Coalesced 64-bit integer L2 atomics per second on this device, in G/s."""
        g = ctypes.c_double()
        self.check(self.lib.se2p_plan_probe_atomics(self.handle, ctypes.byref(g)))
        return g.value

    def count_pairs(self, on: bool = True, reset: bool = True):
        """Turn the real-space counters on/off; returns (candidates, slp_pairs, dlp_pairs)."""
        c = (ctypes.c_int64 * 3)()
        self.check(self.lib.se2p_plan_count_pairs(self.handle, 1 if on else 0, c,
                                                  1 if reset else 0))
        return tuple(c)

    def close(self):
        if self.handle:
            self.lib.se2p_plan_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass


_default_plans = {}


def default_plan(device: int = 0) -> Plan:
    p = _default_plans.get(device)
    if p is None:
        p = _default_plans[device] = Plan(device)
    return p
