"""Generate the golden fixtures in tests/golden/*.npz from the REFERENCE itself.

Run on an x86-64 host that has the FastTools2D tree:

    make -C oracle ref            # compiles the reference MEX sources (oracle/_ref)
    python tests/golden/make_golden.py

Each fixture stores seeded inputs, the MEX-level parameters and the outputs
of the four reference gateways (mex_stokes_{slp,dlp}_{real,kspace}) run
through oracle/ref_mex.py, plus (where cheap) the FP64 Ewald direct sums of
oracle/direct.py.  The fixtures travel with the repository, so the tests can
pin the oracle and the CUDA library where the reference cannot run.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import direct, drivers, ref_mex  # noqa: E402
from oracle.oracle import derived_w_eta, wrap  # noqa: E402

SEED0 = 20261203


def _unit_normals(rng, n):
    th = rng.random(n) * 2 * np.pi
    return np.vstack([np.cos(th), np.sin(th)])


def _run_ref(R, ps, pt, f, n, prm, with_direct=False, raw_src=None):
    """All four gateways on wrapped points; returns a dict of outputs."""
    Lx, Ly = prm["Lx"], prm["Ly"]
    out = {}
    out["slp_real"] = R.slp_real(ps, pt, f, prm["xi"], prm["nside_x"], prm["nside_y"], Lx, Ly)
    out["slp_kspace"] = R.slp_kspace(ps, pt, prm["xi"], prm["eta"], f, prm["Mx"], prm["My"],
                                     Lx, Ly, prm["w"], prm["P"])
    out["dlp_real"] = R.dlp_real(ps, pt, f, n, prm["xi"], prm["nside_x"], prm["nside_y"], Lx, Ly)
    out["dlp_kspace"] = R.dlp_kspace(ps, pt, prm["xi"], prm["eta"], f, n, prm["Mx"], prm["My"],
                                     Lx, Ly, prm["w"], prm["P"])
    if with_direct:
        xi = prm["xi"]
        out["slp_real_ds"] = direct.slp_real_ds(ps[0], ps[1], pt[0], pt[1], f[0], f[1], Lx, Ly, xi)
        out["slp_kspace_ds"] = direct.slp_kspace_ds(ps[0], ps[1], pt[0], pt[1], f[0], f[1], Lx, Ly, xi)
        out["dlp_real_ds"] = direct.dlp_real_ds(ps[0], ps[1], pt[0], pt[1], n[0], n[1], f[0], f[1],
                                                Lx, Ly, xi)
        src = ps if raw_src is None else raw_src
        out["dlp_kspace_ds"] = direct.dlp_kspace_ds(src[0], src[1], pt[0], pt[1], n[0], n[1],
                                                    f[0], f[1], Lx, Ly, xi)
    return out


def _save(name, ps, pt, f, n, prm, out, **extra):
    scal = {k: np.float64(v) for k, v in prm.items()}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), psrc=ps, ptar=pt, f=f, n=n,
                        **scal, **{"out_" + k: v for k, v in out.items()}, **extra)
    print(f"wrote {name}.npz  Ns={ps.shape[1]} Nt={pt.shape[1]}")


def mex_params(xi, nside_x, nside_y, Mx, My, Lx, Ly, P):
    w, eta = derived_w_eta(xi, Mx, Lx, P)
    return dict(xi=xi, nside_x=nside_x, nside_y=nside_y, Mx=Mx, My=My, Lx=Lx, Ly=Ly, P=P,
                w=w, eta=eta)


def uniform_case(R, name, seed, N, xi, nside, M, P, L=1.0, targets_are_sources=False,
                 with_direct=False):
    rng = np.random.default_rng(seed)
    p = rng.random((2, N)) * L
    ps = np.vstack([wrap(p[0], L), wrap(p[1], L)])
    f = rng.standard_normal((2, N))
    n = _unit_normals(rng, N)
    if targets_are_sources:
        pt = ps.copy()
    else:
        q = rng.random((2, N)) * L
        pt = np.vstack([wrap(q[0], L), wrap(q[1], L)])
    prm = mex_params(xi, nside, nside, M, M, L, L, P)
    out = _run_ref(R, ps, pt, f, n, prm, with_direct=with_direct)
    _save(name, ps, pt, f, n, prm, out)


def circles(rng, ncirc, per, L=1.0, rmin=0.05, rmax=0.1, modes=8):
    """Non-overlapping circles, equispaced points, outward normals, trapezoid
    weights 2 pi r / per, density = random Fourier series (modes <= 8)."""
    cs = []
    while len(cs) < ncirc:
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(-L / 2 + r, L / 2 - r, size=2)
        if all(np.hypot(*(c - c2)) > r + r2 + 0.01 for c2, r2 in cs):
            cs.append((c, r))
    th = 2 * np.pi * np.arange(per) / per
    P_, F_, N_ = [], [], []
    for c, r in cs:
        x = np.vstack([c[0] + r * np.cos(th), c[1] + r * np.sin(th)])
        nrm = np.vstack([np.cos(th), np.sin(th)])
        dens = np.zeros((2, per))
        for comp in range(2):
            for m in range(modes + 1):
                a, b = rng.standard_normal(2)
                dens[comp] += a * np.cos(m * th) + b * np.sin(m * th)
        P_.append(x)
        N_.append(nrm)
        F_.append(dens * 2 * np.pi * r / per)
    return np.hstack(P_), np.hstack(F_), np.hstack(N_), cs


def targets_outside(rng, nt, cs, L=1.0):
    pts = []
    while sum(p.shape[1] for p in pts) < nt:
        q = rng.random((2, 4 * nt)) * L - L / 2
        ok = np.ones(q.shape[1], bool)
        for c, r in cs:
            ok &= np.hypot(q[0] - c[0], q[1] - c[1]) > r
        pts.append(q[:, ok])
    return np.hstack(pts)[:, :nt]


def main():
    R = ref_mex.RefMex()
    # SLP FP64, N=1000, targets = sources (the self term enters at r2 == 0).
    uniform_case(R, "slp1000_xi19", SEED0 + 1, 1000, 19.2, 4, 64, 24, targets_are_sources=True,
                 with_direct=True)

    # Circle geometry at reduced size: 8 circles x 256 points, 2048 targets outside.
    rng = np.random.default_rng(SEED0 + 2)
    ps, f, n, cs = circles(rng, 8, 256)
    pt = targets_outside(rng, 2048, cs)
    prm = mex_params(60.0, 12, 12, 192, 192, 1.0, 1.0, 24)
    _save("circles2048_xi60", ps, pt, f, n, prm, _run_ref(R, ps, pt, f, n, prm))

    # direct_sums_test.m layout: N=10, Lx=1, Ly=2, driver parameters at tol=1e-16
    # (PE/tests/direct_sums_test.m:13-38), separate SLP and DLP parameter sets.
    rng = np.random.default_rng(SEED0 + 10)
    Lx, Ly, N = 1.0, 2.0, 10
    f = 10 * rng.random((2, N))
    n1 = rng.random(N)
    n = np.vstack([n1, np.sqrt(1 - n1 ** 2)])
    xs = np.vstack([Lx * rng.random(N), Ly * rng.random(N)])
    xt = np.vstack([Lx * rng.random(N), Ly * rng.random(N)])
    ps = np.vstack([wrap(xs[0], Lx), wrap(xs[1], Ly)])
    pt = np.vstack([wrap(xt[0], Lx), wrap(xt[1], Ly)])
    for kind in ("slp", "dlp"):
        d = drivers.params(kind, N, N, float(np.sum(f ** 2)), Lx, Ly, tol=1e-16)
        prm = mex_params(d["xi"], d["nside_x"], d["nside_y"], d["Mx"], d["My"], Lx, Ly, d["P"])
        out = _run_ref(R, ps, pt, f, n, prm, with_direct=True, raw_src=xs)
        _save(f"direct_{kind}", ps, pt, f, n, prm, out, raw_src=xs, raw_tar=xt,
              Nb=np.float64(d["Nb"]), tol=np.float64(1e-16))

    # Edge cases.
    rng = np.random.default_rng(SEED0 + 20)
    L, M, P = 1.0, 64, 24
    h = L / M
    k = rng.integers(0, M, size=(2, 40))
    on_nodes = -L / 2 + k * h                      # exactly on grid nodes
    near_nodes = on_nodes + rng.choice([-1, 1], size=on_nodes.shape) * 3e-14  # inside the snap
    edge = np.array([[-0.5, -0.5, 0.5 - 1e-16, -0.5 + 1e-17, 0.0, 0.25, -0.25, 0.49999999999999994],
                     [-0.5, 0.49999999999999994, -0.5, 0.0, 0.0, -0.5, 0.5 - 1e-16, -0.5]])
    rand = rng.random((2, 120)) - 0.5
    ps = np.hstack([on_nodes, near_nodes, edge, rand])
    pt = np.hstack([ps[:, ::2], rng.random((2, 60)) - 0.5, edge])   # shares points -> self terms
    ps = np.hstack([ps, ps[:, :5]])                                 # duplicate sources
    f = rng.standard_normal((2, ps.shape[1]))
    n = _unit_normals(rng, ps.shape[1])
    prm = mex_params(12.0, 4, 4, M, M, L, L, P)
    _save("edge_nodes", ps, pt, f, n, prm, _run_ref(R, ps, pt, f, n, prm))

    # Rectangular box with distinct nside and M per axis (Lx/Mx == Ly/My).
    rng = np.random.default_rng(SEED0 + 21)
    ps = np.vstack([rng.random(300) - 0.5, 2 * rng.random(300) - 1.0])
    pt = np.vstack([rng.random(200) - 0.5, 2 * rng.random(200) - 1.0])
    f = rng.standard_normal((2, 300))
    n = _unit_normals(rng, 300)
    prm = mex_params(15.0, 3, 6, 48, 96, 1.0, 2.0, 16)
    _save("rect", ps, pt, f, n, prm, _run_ref(R, ps, pt, f, n, prm))

    # Few boxes (nside 1 and 2) and a grid barely larger than the stencil.
    for nside, M_, P_, name in ((1, 26, 24, "nside1_M26"), (2, 32, 24, "nside2_M32"),
                                (3, 40, 8, "nside3_P8"), (5, 48, 12, "nside5_P12")):
        rng = np.random.default_rng(SEED0 + 30 + nside)
        ps = rng.random((2, 150)) - 0.5
        pt = rng.random((2, 90)) - 0.5
        f = rng.standard_normal((2, 150))
        n = _unit_normals(rng, 150)
        prm = mex_params(6.0, nside, nside, M_, M_, 1.0, 1.0, P_)
        _save(name, ps, pt, f, n, prm, _run_ref(R, ps, pt, f, n, prm))

    # All points clustered in one box (one heavy box, the rest empty).
    rng = np.random.default_rng(SEED0 + 40)
    ps = 0.02 * rng.random((2, 400)) + 0.11
    pt = 0.03 * rng.random((2, 300)) + 0.1
    f = rng.standard_normal((2, 400))
    n = _unit_normals(rng, 400)
    prm = mex_params(20.0, 6, 6, 64, 64, 1.0, 1.0, 24)
    _save("cluster", ps, pt, f, n, prm, _run_ref(R, ps, pt, f, n, prm))


if __name__ == "__main__":
    main()
