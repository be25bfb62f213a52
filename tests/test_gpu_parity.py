"""GPU parity tests: libse2p (CUDA, sm_103a) against the reference outputs in
tests/golden and against the CPU oracle, called through the C ABI.

Tolerance: the FP64 path must match the reference to <= 1e-12 relative
(normwise, max|a-b|/max|b|).  Differences come only from FP64 summation
order (atomics, cuFFT vs FFTW) and are ~1e-15.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden, relerr

pytestmark = pytest.mark.gpu
PARITY = 1e-12


@pytest.fixture(scope="module")
def ft():
    import fasttools2d_gb300 as ft
    return ft


@pytest.fixture(scope="module")
def plan(ft):
    p = ft.Plan(0)
    yield p
    p.close()


@pytest.mark.parametrize("name", golden_names())
def test_mex_gateways_match_reference(ft, plan, name):
    g = load_golden(name)
    ps, pt, f, n = g["psrc"], g["ptar"], g["f"], g["n"]
    xi, nx, ny, Lx, Ly = g["xi"], g["nside_x"], g["nside_y"], g["Lx"], g["Ly"]
    Mx, My, w, eta, P = g["Mx"], g["My"], g["w"], g["eta"], g["P"]
    got = {
        "slp_real": ft.mex_stokes_slp_real(ps, pt, f, xi, nx, ny, Lx, Ly, plan=plan),
        "slp_kspace": ft.mex_stokes_slp_kspace(ps, pt, xi, eta, f, Mx, My, Lx, Ly, w, P, plan=plan),
        "dlp_real": ft.mex_stokes_dlp_real(ps, pt, f, n, xi, nx, ny, Lx, Ly, plan=plan),
        "dlp_kspace": ft.mex_stokes_dlp_kspace(ps, pt, xi, eta, f, n, Mx, My, Lx, Ly, w, P,
                                               plan=plan),
    }
    for k, v in got.items():
        err = relerr(v, g["out_" + k])
        assert err < PARITY, (name, k, err)


def _uniform(seed, N, L=1.0):
    rng = np.random.default_rng(seed)
    p = rng.random((2, N)) * L
    f = rng.standard_normal((2, N))
    g = rng.standard_normal((2, N))
    th = rng.random(N) * 2 * np.pi
    return p, f, g, np.vstack([np.cos(th), np.sin(th)])


def test_driver_composites_match_oracle(ft, plan):
    from oracle import oracle as O
    p, f, g, n = _uniform(11, 1000)
    q = np.random.default_rng(12).random((2, 700)) * 1.3 - 0.2      # some targets outside the cell
    prm = ft.EwaldParams.derived(19.2, 4, 4, 64, 64, 24, 1.0, 1.0)
    u, ur, uk = ft.slp_ewald(p, q, f, prm, parts=True, plan=plan)
    ru, rr, rk = O.slp_ewald(p, q, f, prm.xi, 4, 4, 64, 64, 1.0, 1.0, 24)
    assert relerr(u, ru) < PARITY and relerr(ur, rr) < PARITY and relerr(uk, rk) < PARITY
    u, ur, uk = ft.dlp_ewald(p, q, g, n, prm, parts=True, plan=plan)
    ru, rr, rk = O.dlp_ewald(p, q, g, n, prm.xi, 4, 4, 64, 64, 1.0, 1.0, 24)
    assert relerr(u, ru) < PARITY and relerr(ur, rr) < PARITY and relerr(uk, rk) < PARITY
    us, ud = ft.stokes_ewald(p, q, f, g, n, prm, plan=plan)
    assert relerr(us, O.slp_ewald(p, q, f, prm.xi, 4, 4, 64, 64, 1.0, 1.0, 24)[0]) < PARITY
    assert relerr(ud, O.dlp_ewald(p, q, g, n, prm.xi, 4, 4, 64, 64, 1.0, 1.0, 24)[0]) < PARITY


def test_rectangular_driver(ft, plan):
    from oracle import oracle as O
    rng = np.random.default_rng(5)
    p = np.vstack([rng.random(800), 2 * rng.random(800)])
    f = rng.standard_normal((2, 800))
    th = rng.random(800) * 2 * np.pi
    n = np.vstack([np.cos(th), np.sin(th)])
    prm = ft.EwaldParams.derived(14.0, 3, 6, 40, 80, 24, 1.0, 2.0)
    us, ud = ft.stokes_ewald(p, p, f, f, n, prm, plan=plan)
    assert relerr(us, O.slp_ewald(p, p, f, 14.0, 3, 6, 40, 80, 1.0, 2.0, 24)[0]) < PARITY
    assert relerr(ud, O.dlp_ewald(p, p, f, n, 14.0, 3, 6, 40, 80, 1.0, 2.0, 24)[0]) < PARITY


def test_slp1000_meets_ewald_tolerance(ft, plan):
    """SLP, 1000 points (xi=19.2, rc=0.25, M=64, P=24) against the FP64 direct lattice sum."""
    g = load_golden("slp1000_xi19")
    ps, f = g["psrc"], g["f"]
    u = ft.mex_stokes_slp_real(ps, ps, f, g["xi"], 4, 4, 1.0, 1.0, plan=plan) + \
        ft.mex_stokes_slp_kspace(ps, ps, g["xi"], g["eta"], f, 64, 64, 1.0, 1.0, g["w"], 24,
                                 plan=plan)
    ds = g["out_slp_real_ds"] + g["out_slp_kspace_ds"]
    assert relerr(u, ds) < 1e-10


def test_circles_full_size(ft, plan):
    """8 circles x 8192 points (65,536 DLP sources), 65,536 targets
    outside the circles, xi=60, rc=0.08 (nside 12), M=192, P=24."""
    from oracle import oracle as O
    from tests.golden.make_golden import circles, targets_outside
    rng = np.random.default_rng(20261203 + 2)
    ps, f, n, cs = circles(rng, 8, 8192)
    pt = targets_outside(rng, 65536, cs)
    prm = ft.EwaldParams.derived(60.0, 12, 12, 192, 192, 24, 1.0, 1.0)
    ur = ft.mex_stokes_dlp_real(ps, pt, f, n, 60.0, 12, 12, 1.0, 1.0, plan=plan)
    uk = ft.mex_stokes_dlp_kspace(ps, pt, 60.0, prm.eta, f, n, 192, 192, 1.0, 1.0, prm.w, 24,
                                  plan=plan)
    assert relerr(ur, O.mex_stokes_dlp_real(ps, pt, f, n, 60.0, 12, 12, 1.0, 1.0)) < PARITY
    assert relerr(uk, O.mex_stokes_dlp_kspace(ps, pt, 60.0, prm.eta, f, n, 192, 192, 1.0, 1.0,
                                              prm.w, 24)) < PARITY


def test_host_and_device_pointers_agree(ft, plan):
    torch = pytest.importorskip("torch")
    p, f, g, n = _uniform(21, 3000)
    prm = ft.EwaldParams.derived(30.0, 6, 6, 96, 96, 24, 1.0, 1.0)
    us, ud = ft.stokes_ewald(p, p, f, g, n, prm, plan=plan)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    ts, td = ft.stokes_ewald(dev(p), dev(p), dev(f), dev(g), dev(n), prm, plan=plan)
    torch.cuda.synchronize()
    assert relerr(ts.cpu().numpy().T, us) < 1e-14
    assert relerr(td.cpu().numpy().T, ud) < 1e-14


def test_repeatable(ft, plan):
    p, f, g, n = _uniform(31, 5000)
    prm = ft.EwaldParams.derived(40.0, 8, 8, 128, 128, 24, 1.0, 1.0)
    a = ft.stokes_ewald(p, p, f, g, n, prm, plan=plan)
    b = ft.stokes_ewald(p, p, f, g, n, prm, plan=plan)
    assert relerr(a[0], b[0]) < 1e-13 and relerr(a[1], b[1]) < 1e-13


def test_linearity_in_forces(ft, plan):
    p, f, g, n = _uniform(41, 4000)
    prm = ft.EwaldParams.derived(40.0, 8, 8, 128, 128, 24, 1.0, 1.0)
    a = ft.slp_ewald(p, p, f, prm, plan=plan)
    b = ft.slp_ewald(p, p, g, prm, plan=plan)
    c = ft.slp_ewald(p, p, 2.0 * f - 3.0 * g, prm, plan=plan)
    assert relerr(c, 2.0 * a - 3.0 * b) < 1e-12


def test_empty_inputs(ft, plan):
    prm = ft.EwaldParams.derived(19.2, 4, 4, 64, 64, 24, 1.0, 1.0)
    t = np.random.default_rng(1).random((2, 10)) - 0.5
    z = np.zeros((2, 0))
    assert np.all(ft.slp_ewald(z, t, z, prm, plan=plan) == 0)
    assert ft.slp_ewald(t, z, t, prm, plan=plan).shape == (2, 0)


def test_argument_errors(ft, plan):
    p = np.zeros((2, 4))
    with pytest.raises(ft.Se2pError):        # odd grid size
        ft.mex_stokes_slp_kspace(p, p, 10.0, 0.8, p, 63, 64, 1.0, 1.0, 0.1, 24, plan=plan)
    with pytest.raises(ft.Se2pError):        # odd P
        ft.mex_stokes_slp_kspace(p, p, 10.0, 0.8, p, 64, 64, 1.0, 1.0, 0.1, 23, plan=plan)
    with pytest.raises(ft.Se2pError):        # nside < 1
        ft.mex_stokes_slp_real(p, p, p, 10.0, 0, 4, 1.0, 1.0, plan=plan)
    with pytest.raises(ValueError):          # MEX shape check
        ft.mex_stokes_dlp_real(p, p, np.zeros((2, 3)), p, 10.0, 4, 4, 1.0, 1.0, plan=plan)
    # the plan stays usable after errors
    g = load_golden("slp1000_xi19")
    u = ft.mex_stokes_slp_real(g["psrc"], g["ptar"], g["f"], g["xi"], 4, 4, 1.0, 1.0, plan=plan)
    assert relerr(u, g["out_slp_real"]) < PARITY


def test_pending_runtime_error_of_other_code_is_not_reported(ft, plan):
    """An error that other code left pending in the CUDA runtime (here an
    invalid device ordinal from cudaSetDevice, which touches no GPU state) is
    not this library's: the next call clears it on entry and succeeds.  Its
    launch checks read cudaGetLastError, so without that the call reported the
    other code's error as its own."""
    import ctypes
    import ctypes.util
    names = ["libcudart.so.13", "libcudart.so.12", ctypes.util.find_library("cudart")]
    rt = None
    for name in filter(None, names):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            continue
    if rt is None:
        pytest.skip("libcudart not loadable")
    g = load_golden(golden_names()[0])
    ps, pt, f = g["psrc"], g["ptar"], g["f"]
    ref = ft.mex_stokes_slp_real(ps, pt, f, g["xi"], g["nside_x"], g["nside_y"], g["Lx"], g["Ly"],
                                 plan=plan)
    assert rt.cudaSetDevice(ctypes.c_int(1 << 20)) != 0        # left pending
    got = ft.mex_stokes_slp_real(ps, pt, f, g["xi"], g["nside_x"], g["nside_y"], g["Lx"], g["Ly"],
                                 plan=plan)                       # does not raise
    # (not bitwise: the within-box order of the sort comes from atomics)
    assert relerr(got, ref) < 1e-13


def test_matlab_driver_stresslet_identity(ft, plan):
    """stresslet_identity_test.m through StokesDLP_ewald_2p (parameters chosen by the driver)."""
    r, L, ns, nt = 1.0, 4.0, 256, 16
    hs = 2 * np.pi / ns
    th = hs * np.arange(1, ns + 1)
    tt = 2 * np.pi / nt * np.arange(1, nt + 1)
    xt = np.concatenate([0.5 * np.cos(tt), 1.5 * np.cos(tt)])
    yt = np.concatenate([0.5 * np.sin(tt), 1.5 * np.sin(tt)])
    for comp in (0, 1):
        f = [np.zeros(ns), np.zeros(ns)]
        f[comp][:] = hs
        u1, u2, _, _, _ = ft.StokesDLP_ewald_2p(r * np.cos(th), r * np.sin(th), xt, yt,
                                               np.cos(th), np.sin(th), f[0], f[1], L, L,
                                               plan=plan)
        inside = u1[:nt] + 1j * u2[:nt]
        assert np.abs(inside - (1 if comp == 0 else 1j)).max() < 1e-9
        assert np.abs(u1[nt:] + 1j * u2[nt:]).max() < 1e-9


def test_matlab_driver_direct_sums(ft, plan):
    """direct_sums_test.m: the driver's ur/uk against the direct sums (tol=1e-16)."""
    for kind in ("slp", "dlp"):
        g = load_golden("direct_" + kind)
        xs, xt, f, n = g["raw_src"], g["raw_tar"], g["f"], g["n"]
        if kind == "slp":
            _, _, ur, uk, xi = ft.StokesSLP_ewald_2p(xs[0], xs[1], xt[0], xt[1], f[0], f[1],
                                                     1.0, 2.0, tol=1e-16, plan=plan)
        else:
            _, _, ur, uk, xi = ft.StokesDLP_ewald_2p(xs[0], xs[1], xt[0], xt[1], n[0], n[1],
                                                     f[0], f[1], 1.0, 2.0, tol=1e-16,
                                                     unit_normal_fix=False, plan=plan)
        assert xi == pytest.approx(g["xi"], rel=1e-13)
        assert relerr(ur, g[f"out_{kind}_real_ds"]) < 1e-11
        assert relerr(uk, g[f"out_{kind}_kspace_ds"]) < 1e-11
