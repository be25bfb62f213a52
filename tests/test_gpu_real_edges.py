"""Real space on box edges and half-lines, against the CPU oracle.

The pair set is the reference's (mex_stokes_slp_real.cpp:131-333,
mex_stokes_dlp_real.cpp:103-187): every pair of the target's own box, and
pairs of the 8 neighbour boxes with r2 < Lx*Ly/nside_x/nside_y.  Box
indices (ewald_tools.cpp:28-33) and the cutoff test decide discrete outcomes
at the boundaries, so these cases put points on box edges and half-lines and
a few ulps either side, outside the unit cell (clamped into the edge boxes
by the reference's Assign), and on a lattice 4x finer than the boxes, in
square and non-square boxes.  Exact coincidences with a periodic image give
NaN in the reference, and must give NaN at the same targets here.
"""
import zlib

import numpy as np
import pytest

from conftest import relerr

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


def _edge_coords(L, n, rng, m):
    """Box edges and half-lines (in the reference's [-L/2, L/2) frame), moved
    by -3..3 ulps, with 5 % of the values anywhere in 1.2 cells."""
    b = rng.integers(0, n + 1, m)
    edge = L * (b / n - 0.5)
    half = L * ((b + 0.5) / n - 0.5)
    v = np.where(rng.random(m) < 0.5, edge, half)
    v = v + rng.integers(-3, 4, m) * np.spacing(np.abs(v) + 1e-300)
    out = rng.random(m) < 0.05
    return np.where(out, (rng.random(m) - 0.5) * 2.4 * L, v)


def _points(kind, Lx, Ly, nx, ny, rng, m):
    if kind == "uniform":
        return np.vstack([(rng.random(m) - 0.5) * Lx, (rng.random(m) - 0.5) * Ly])
    if kind == "edges":
        # one coordinate on an edge or half-line, the other uniform; both on
        # them for a fifth of the points (exact coincidences with periodic
        # images give NaN, as in the reference, and must coincide)
        ux, uy = (rng.random(m) - 0.5) * Lx, (rng.random(m) - 0.5) * Ly
        ex, ey = _edge_coords(Lx, nx, rng, m), _edge_coords(Ly, ny, rng, m)
        c = rng.random(m)
        return np.vstack([np.where(c < 0.6, ex, ux), np.where((c >= 0.4) | (c < 0.2), ey, uy)])
    g = 4 * max(nx, ny)                       # points on a lattice 4x finer than the boxes
    return np.vstack([Lx * (rng.integers(0, g, m) / g - 0.5), Ly * (rng.integers(0, g, m) / g - 0.5)])


@pytest.mark.parametrize("box", [(1.0, 1.0, 5, 5), (1.0, 1.0, 2, 2), (1.0, 1.0, 1, 1),
                                 (1.0, 2.0, 3, 6), (1.0, 2.0, 4, 4), (2.0, 1.0, 4, 4),
                                 (1.0, 1.3, 5, 4)])
@pytest.mark.parametrize("kind", ["uniform", "edges", "lattice"])
def test_real_space_on_box_edges_and_half_lines(ft, plan, box, kind):
    from oracle import oracle as O
    Lx, Ly, nx, ny = box
    rng = np.random.default_rng(zlib.crc32(repr((box, kind)).encode()))
    m = 1200
    ps = _points(kind, Lx, Ly, nx, ny, rng, m)
    pt = np.hstack([ps[:, rng.permutation(m)[:400]], _points(kind, Lx, Ly, nx, ny, rng, 400)])
    f = rng.standard_normal((2, m))
    th = rng.random(m) * 2 * np.pi
    n = np.vstack([np.cos(th), np.sin(th)])
    xi = 3.0 * max(nx / Lx, ny / Ly)
    got = ft.mex_stokes_slp_real(ps, pt, f, xi, nx, ny, Lx, Ly, plan=plan)
    ref = O.mex_stokes_slp_real(ps, pt, f, xi, nx, ny, Lx, Ly)
    assert relerr(got, ref) < PARITY, ("slp", box, kind, relerr(got, ref))
    got = ft.mex_stokes_dlp_real(ps, pt, f, n, xi, nx, ny, Lx, Ly, plan=plan)
    ref = O.mex_stokes_dlp_real(ps, pt, f, n, xi, nx, ny, Lx, Ly)
    assert relerr(got, ref) < PARITY, ("dlp", box, kind, relerr(got, ref))


@pytest.mark.parametrize("box", [(1.0, 1.0, 5, 5, 64, 64), (1.0, 2.0, 3, 6, 40, 80)])
def test_drivers_on_box_edges_and_half_lines(ft, plan, box):
    """The composite SLP+DLP evaluation (wrap, sort, real and k space) on
    the same kind of boundary points, against the oracle's drivers."""
    from oracle import oracle as O
    Lx, Ly, nx, ny, Mx, My = box
    rng = np.random.default_rng(zlib.crc32(repr(box).encode()))
    m = 1500
    p = _points("edges", Lx, Ly, nx, ny, rng, m)
    q = np.hstack([p[:, :500], _points("edges", Lx, Ly, nx, ny, rng, 500)])
    f = rng.standard_normal((2, m))
    g = rng.standard_normal((2, m))
    th = rng.random(m) * 2 * np.pi
    n = np.vstack([np.cos(th), np.sin(th)])
    xi = 3.0 * max(nx / Lx, ny / Ly)
    prm = ft.EwaldParams.derived(xi, nx, ny, Mx, My, 24, Lx, Ly)
    us, ud = ft.stokes_ewald(p, q, f, g, n, prm, plan=plan)
    rs = O.slp_ewald(p, q, f, prm.xi, nx, ny, Mx, My, Lx, Ly, 24)[0]
    rd = O.dlp_ewald(p, q, g, n, prm.xi, nx, ny, Mx, My, Lx, Ly, 24)[0]
    assert relerr(us, rs) < PARITY, ("slp", box, relerr(us, rs))
    assert relerr(ud, rd) < PARITY, ("dlp", box, relerr(ud, rd))
