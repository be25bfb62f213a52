"""GPU tests of the FP32-grid (mixed-precision) form against the FP64 oracle.

The FP32-grid form targets Ewald tolerances >= 1e-6: spread, FFT, filter,
gather and the far real-space pairs run in FP32; near pairs (E1 at small
argument), the self term and the DLP k=0 term stay FP64.  Its arithmetic
error must stay below the tolerance: here <= 2e-6 max and <= 1e-6 RMS,
relative to the FP64 result, per potential.
"""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu


def _inputs(N, seed):
    rng = np.random.default_rng(seed)
    p = rng.random((2, N))
    q = rng.random((2, N))
    f = rng.standard_normal((2, N))
    g = rng.standard_normal((2, N))
    th = rng.random(N) * 2 * np.pi
    return p, q, f, g, np.vstack([np.cos(th), np.sin(th)])


def _rms(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


@pytest.fixture(scope="module")
def ft():
    import fasttools2d_gb300 as ft
    return ft


def test_fp32grid_vs_fp64_oracle(ft):
    """xi rc = 3.61, P = 12 (the 1M-point mixed-precision workload's ratios) at N = 2^15 against the oracle."""
    from oracle import oracle as O
    N = 2 ** 15
    p, q, f, g, n = _inputs(N, 17)
    nside = 42
    xi, M, P = 3.614 * nside, 384, 12
    prm = ft.EwaldParams.derived(xi, nside, nside, M, M, P, 1.0, 1.0)
    plan = ft.Plan(0)
    plan.set_precision("fp32_grid")
    us, ud = ft.stokes_ewald(p, q, f, g, n, prm, plan=plan)
    rs = O.slp_ewald(p, q, f, xi, nside, nside, M, M, 1.0, 1.0, P)[0]
    rd = O.dlp_ewald(p, q, g, n, xi, nside, nside, M, M, 1.0, 1.0, P)[0]
    for got, ref in ((us, rs), (ud, rd)):
        assert relerr(got, ref) < 2e-6
        assert _rms(got, ref) < 1e-6
    plan.close()


@pytest.mark.parametrize("kind", ["slp_real", "dlp_real", "slp_kspace", "dlp_kspace"])
def test_fp32grid_mex_gateways(ft, kind):
    """Each gateway in FP32-grid mode stays within the FP32 error budget."""
    from conftest import load_golden
    g = load_golden("slp1000_xi19")
    ps, f, n = g["psrc"], g["f"], g["n"]
    plan = ft.Plan(0)
    plan.set_precision("fp32_grid")
    args = {"slp_real": (ft.mex_stokes_slp_real, (ps, ps, f, g["xi"], 4, 4, 1.0, 1.0)),
            "dlp_real": (ft.mex_stokes_dlp_real, (ps, ps, f, n, g["xi"], 4, 4, 1.0, 1.0)),
            "slp_kspace": (ft.mex_stokes_slp_kspace,
                           (ps, ps, g["xi"], g["eta"], f, 64, 64, 1.0, 1.0, g["w"], 24)),
            "dlp_kspace": (ft.mex_stokes_dlp_kspace,
                           (ps, ps, g["xi"], g["eta"], f, n, 64, 64, 1.0, 1.0, g["w"], 24))}
    fn, a = args[kind]
    got = fn(*a, plan=plan)
    assert relerr(got, g["out_" + kind]) < 2e-6
    plan.close()


def test_overlap_switch_gives_same_result(ft):
    p, q, f, g, n = _inputs(20000, 5)
    prm = ft.EwaldParams.derived(120.0, 30, 30, 192, 192, 24, 1.0, 1.0)
    plan = ft.Plan(0)
    a = ft.stokes_ewald(p, q, f, g, n, prm, plan=plan)
    plan.set_overlap(False)
    b = ft.stokes_ewald(p, q, f, g, n, prm, plan=plan)
    assert relerr(a[0], b[0]) < 1e-13 and relerr(a[1], b[1]) < 1e-13
    plan.close()


def test_fp32grid_real_space_close_pairs(ft):
    """Clusters and near-coincident pairs (r = 1e-6, 1e-7, 1e-9) with targets
    on the sources (self terms): real space against the oracle."""
    from oracle import oracle as O
    rng = np.random.default_rng(23)
    c = rng.random((2, 30))
    p = (c[:, rng.integers(0, 30, 3000)] + 0.003 * rng.standard_normal((2, 3000))) % 1.0
    p = np.hstack([p, p[:, :40] + 1e-6, p[:, 40:80] + 1e-7, p[:, 80:120] + 1e-9])
    N = p.shape[1]
    f = rng.standard_normal((2, N))
    th = rng.random(N) * 2 * np.pi
    n = np.vstack([np.cos(th), np.sin(th)])
    plan = ft.Plan(0)
    plan.set_precision("fp32_grid")
    xi, ns = 40.0, 8
    a = ft.mex_stokes_slp_real(p, p, f, xi, ns, ns, 1.0, 1.0, plan=plan)
    b = ft.mex_stokes_dlp_real(p, p, f, n, xi, ns, ns, 1.0, 1.0, plan=plan)
    ra = O.mex_stokes_slp_real(p, p, f, xi, ns, ns, 1.0, 1.0)
    rb = O.mex_stokes_dlp_real(p, p, f, n, xi, ns, ns, 1.0, 1.0)
    assert relerr(a, ra) < 2e-6 and _rms(a, ra) < 1e-6, (relerr(a, ra), _rms(a, ra))
    assert relerr(b, rb) < 2e-6 and _rms(b, rb) < 1e-6, (relerr(b, rb), _rms(b, rb))
    plan.close()
