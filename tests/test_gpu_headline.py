"""Parity at the headline sizes: 2^20 sources and 2^20 targets.

The 1M-point SLP+DLP workload (xi = 860, rc = 0.0056 -> nside = 178,
M = 2688, P = 24, tolerance 1e-10) in the default FP64 form and the all-FP64
form against the CPU oracle on the same inputs, per potential, normwise and
RMS-relative (<= 1e-12); and the FP32-grid form on the mixed-precision
parameters of the same points (xi = 860, rc = 0.0042 -> nside = 238,
M = 2048, P = 12, tolerance 1e-6) against the oracle run with those
parameters, its error stated and bounded.

The reference paths being matched: mex_stokes_slp_real.cpp:58-357,
mex_stokes_slp_kspace.cpp:64-329, mex_stokes_dlp_real.cpp:15-211,
mex_stokes_dlp_kspace.cpp:10-406 and the driver corrections of
StokesDLP_ewald_2p.m:140-158 (PeriodicEwald).
"""
import math

import numpy as np
import pytest

from conftest import normwise_err, relerr, rms_err

pytestmark = pytest.mark.gpu

N = 2 ** 20
PARITY = 1e-12


def _workload():
    """Seeded uniform points, N(0,1) forces and densities, random unit normals
    (MATLAB 2xN layout)."""
    rng = np.random.default_rng(20261203 + 3)
    psrc = rng.random((N, 2))
    ptar = rng.random((N, 2))
    f = rng.standard_normal((N, 2))
    g = rng.standard_normal((N, 2))
    th = rng.random(N) * 2 * np.pi
    n = np.stack([np.cos(th), np.sin(th)], axis=1)
    return psrc.T.copy(), ptar.T.copy(), f.T.copy(), g.T.copy(), n.T.copy()


@pytest.fixture(scope="module")
def data():
    return _workload()


@pytest.fixture(scope="module")
def oracle_headline(data):
    from oracle import oracle as O
    p, q, f, g, n = data
    nside = int(math.floor(1.0 / 0.0056))
    us = O.slp_ewald(p, q, f, 860.0, nside, nside, 2688, 2688, 1.0, 1.0, 24)[0]
    ud = O.dlp_ewald(p, q, g, n, 860.0, nside, nside, 2688, 2688, 1.0, 1.0, 24)[0]
    return us, ud


@pytest.mark.parametrize("precision", ["fp64", "fp64_native"])
def test_headline_1m_points_against_oracle(data, oracle_headline, precision):
    import fasttools2d_gb300 as ft
    p, q, f, g, n = data
    nside = int(math.floor(1.0 / 0.0056))
    prm = ft.EwaldParams.derived(860.0, nside, nside, 2688, 2688, 24, 1.0, 1.0)
    plan = ft.Plan(0)
    plan.set_precision(precision)
    us, ud = ft.stokes_ewald(p, q, f, g, n, prm, plan=plan)
    plan.close()
    for got, ref in zip((us, ud), oracle_headline):
        assert np.isfinite(got).all()
        err = (normwise_err(got, ref), rms_err(got, ref))
        assert relerr(got, ref) < PARITY, err


def test_fp32grid_1m_points_against_oracle(data):
    """The FP32-grid form's error against the FP64 oracle on the
    mixed-precision parameters: <= 2e-6 normwise and <= 1e-6 RMS-relative per
    potential (measured: about 7e-7 and 3e-7)."""
    import fasttools2d_gb300 as ft
    from oracle import oracle as O
    p, q, f, g, n = data
    nside = int(math.floor(1.0 / 0.0042))
    prm = ft.EwaldParams.derived(860.0, nside, nside, 2048, 2048, 12, 1.0, 1.0)
    plan = ft.Plan(0)
    plan.set_precision("fp32_grid")
    us, ud = ft.stokes_ewald(p, q, f, g, n, prm, plan=plan)
    plan.close()
    rs = O.slp_ewald(p, q, f, 860.0, nside, nside, 2048, 2048, 1.0, 1.0, 12)[0]
    rd = O.dlp_ewald(p, q, g, n, 860.0, nside, nside, 2048, 2048, 1.0, 1.0, 12)[0]
    for got, ref in ((us, rs), (ud, rd)):
        assert normwise_err(got, ref) < 2e-6
        assert rms_err(got, ref) < 1e-6, rms_err(got, ref)
