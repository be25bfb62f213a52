"""se2p_slp_real_noalloc: the SLP real-space sum for callers that cannot
allocate device memory (MEX code inside MATLAB, whose gpuArray allocator owns
the GPU memory; solver loops that must not allocate).  It keeps its working
arrays in a fixed 32 MiB device array instead of cudaMalloc'd workspace.

Checked through the C ABI against the regular entry point se2p_slp_real on
two calls in a row with different sizes and box grids, so a result that
leaned on the previous call's leftovers in the shared array would show up;
and timed against the regular entry point and the all-FP64 form, to show
that it runs the default float-float real-space form.
This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu
PARITY = 1e-12


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    import fasttools2d_gb300 as ft
    lib = ft.load()
    plan = ft.Plan(0)
    stream = torch.cuda.current_stream().cuda_stream
    cases = [(101, 40000, 30000, 24, 80.0), (202, 7000, 9000, 9, 35.0)]
    for seed, ns, nt, nside, xi in cases:
        rng = np.random.default_rng(seed)
        ps = _dev(torch, rng.random((ns, 2)) - 0.5)
        pt = _dev(torch, rng.random((nt, 2)) - 0.5)
        f = _dev(torch, rng.standard_normal((ns, 2)))
        ref = ft.mex_stokes_slp_real(ps, pt, f, xi, nside, nside, 1.0, 1.0, plan=plan)
        u = torch.full((nt, 2), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.se2p_slp_real_noalloc(ps.data_ptr(), ns, pt.data_ptr(), nt, f.data_ptr(),
                                       ctypes.c_double(xi), nside, nside, ctypes.c_double(1.0),
                                       ctypes.c_double(1.0), u.data_ptr(),
                                       ctypes.c_void_p(stream))
        assert rc == 0
        torch.cuda.synchronize()
        assert relerr(u.cpu().numpy(), ref.cpu().numpy()) < PARITY
    plan.close()


def test_noalloc_rejects_oversize_and_host_pointers():
    torch = pytest.importorskip("torch")
    import fasttools2d_gb300 as ft
    lib = ft.load()
    big = 400000                      # 52*big + 56*big bytes > 32 MiB
    ps = torch.zeros((8, 2), dtype=torch.float64, device="cuda")
    rc = lib.se2p_slp_real_noalloc(ps.data_ptr(), big, ps.data_ptr(), big, ps.data_ptr(),
                                   ctypes.c_double(10.0), 4, 4, ctypes.c_double(1.0),
                                   ctypes.c_double(1.0), ps.data_ptr(), None)
    assert rc == ft._lib.SE2P_ERR_UNSUPPORTED
    host = np.zeros((8, 2))
    rc = lib.se2p_slp_real_noalloc(host.ctypes.data, 8, host.ctypes.data, 8, host.ctypes.data,
                                   ctypes.c_double(10.0), 4, 4, ctypes.c_double(1.0),
                                   ctypes.c_double(1.0), host.ctypes.data, None)
    assert rc == ft._lib.SE2P_ERR_ARG


def _time_ms(torch, fn, reps=3):
    best = 1e30
    for _ in range(reps):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        s.record()
        fn()
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e))
    return best


def test_noalloc_runs_the_default_float_float_form():
    """At 250,000 + 250,000 points the all-FP64 real space is about three
    times slower than the float-float form that se2p_slp_real runs by
    default; the allocation-free entry point must run at the latter's speed."""
    torch = pytest.importorskip("torch")
    import fasttools2d_gb300 as ft
    lib = ft.load()
    n, nside, xi = 250000, 86, 415.0
    rng = np.random.default_rng(303)
    ps = _dev(torch, rng.random((n, 2)) - 0.5)
    pt = _dev(torch, rng.random((n, 2)) - 0.5)
    f = _dev(torch, rng.standard_normal((n, 2)))
    stream = torch.cuda.current_stream().cuda_stream
    u = torch.empty((n, 2), dtype=torch.float64, device="cuda")

    def noalloc():
        assert lib.se2p_slp_real_noalloc(ps.data_ptr(), n, pt.data_ptr(), n, f.data_ptr(),
                                         ctypes.c_double(xi), nside, nside, ctypes.c_double(1.0),
                                         ctypes.c_double(1.0), u.data_ptr(),
                                         ctypes.c_void_p(stream)) == 0
    times = {}
    outs = {}
    for prec in ("fp64", "fp64_native"):
        plan = ft.Plan(0)
        plan.set_stream(stream)
        plan.set_precision(prec)
        out = {}

        def regular():
            out["u"] = ft.mex_stokes_slp_real(ps, pt, f, xi, nside, nside, 1.0, 1.0, plan=plan)
        regular()
        times[prec] = _time_ms(torch, regular)
        outs[prec] = out["u"].cpu().numpy()
        plan.close()
    noalloc()
    times["noalloc"] = _time_ms(torch, noalloc)
    got = u.cpu().numpy()
    assert relerr(got, outs["fp64"]) < PARITY
    assert relerr(got, outs["fp64_native"]) < PARITY
    assert times["noalloc"] < 1.5 * times["fp64"], times
    assert times["noalloc"] < 0.6 * times["fp64_native"], times
