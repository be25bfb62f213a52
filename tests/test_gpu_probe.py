"""The atomic-rate probe behind the integer spread's roofline
(se2p_plan_probe_atomics).

It times coalesced 64-bit integer atomic adds into an L2-resident array on
the plan's stream.  The tests check that it returns a finite rate of a
plausible size and that a plan stays usable after it (it borrows 32 MB of the
plan's workspace).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ft():
    import fasttools2d_gb300 as ft
    return ft


def test_probe_returns_a_plausible_rate(ft):
    plan = ft.Plan(0)
    g = plan.probe_atomics()
    assert math.isfinite(g)
    # well above one atomic per SM clock, well below one per lane per clock
    assert 50.0 < g < 20000.0, g
    assert plan.workspace_bytes >= 32 << 20


def test_plan_evaluates_after_probe(ft):
    plan = ft.Plan(0)
    plan.probe_atomics()
    rng = np.random.default_rng(3)
    n = 4000
    p, q = rng.random((2, n)), rng.random((2, n))
    f, g = rng.standard_normal((2, n)), rng.standard_normal((2, n))
    th = rng.random(n) * 2 * np.pi
    nrm = np.stack([np.cos(th), np.sin(th)])
    prm = ft.EwaldParams.derived(40.0, 8, 8, 96, 96, 24, 1.0, 1.0)
    u = ft.stokes_ewald(p, q, f, g, nrm, prm, plan=plan)
    v = ft.stokes_ewald(p, q, f, g, nrm, prm, plan=ft.Plan(0))
    # (the box sort's within-box order comes from atomics, so the real-space
    # summation order, and the last bits, may differ between calls)
    for a, b in zip(u, v):
        a, b = np.asarray(a), np.asarray(b)
        assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()
