"""CPU-only tests of the C-ABI library and the host-side driver logic.

No CUDA call is made: the library is loaded and its exports inspected, and
the parameter selection of the MATLAB drivers is compared with the oracle's
restatement (oracle/drivers.py).
"""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "se2p.h")


def _declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(se2p_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from fasttools2d_gb300 import build
    build.build()
    return ctypes.CDLL(build.LIB)


def test_library_exports_every_declared_symbol(lib):
    names = _declared_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), f"libse2p.so does not export {n}"
    from fasttools2d_gb300 import _lib
    assert set(_lib.EXPORTS) == set(names)


def test_version_string(lib):
    lib.se2p_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.se2p_version()


def test_null_plan_is_rejected_without_gpu(lib):
    # argument checks run before any CUDA call
    assert lib.se2p_slp_real(None, None, 0, None, 0, None, ctypes.c_double(1.0), 1, 1,
                             ctypes.c_double(1.0), ctypes.c_double(1.0), None) == 1


def test_rational_matches_matlab_rat():
    from fasttools2d_gb300.ewald import rational
    from oracle import drivers
    for x in (1.0, 0.5, 2.0, 1.5, 2 / 3, 0.75, 4 / 3, 3.14159, 0.1, 7.0, 1 / 7, np.sqrt(2)):
        assert rational(x) == drivers.rat(x), x


@pytest.mark.parametrize("kind", ["slp", "dlp"])
@pytest.mark.parametrize("N,L,tol,Nb,P", [
    (10, (1.0, 2.0), 1e-16, None, 24), (1000, (1.0, 1.0), 1e-10, None, 24),
    (10000, (1.0, 2.0), 1e-12, 9, 24), (65536, (1.0, 1.0), 1e-10, 27, 24),
    (2 ** 20, (1.0, 1.0), 1e-6, None, 12), (300, (4.0, 4.0), 1e-16, None, 24),
    (5000, (2.0, 1.0), 1e-8, 3, 16)])
def test_select_params_matches_driver(kind, N, L, tol, Nb, P):
    from fasttools2d_gb300.ewald import select_params
    from oracle import drivers
    rng = np.random.default_rng(N)
    fsq = float(np.sum(rng.standard_normal((2, N)) ** 2))
    got = select_params(kind, N, N, fsq, L[0], L[1], P=P, Nb=Nb, tol=tol)
    ref = drivers.params(kind, N, N, fsq, L[0], L[1], P=P, Nb=Nb, tol=tol)
    for k in ("nside_x", "nside_y", "Mx", "My", "P"):
        assert getattr(got, k) == ref[k], k
    for k in ("xi", "w", "eta"):
        assert getattr(got, k) == pytest.approx(ref[k], rel=1e-13), k


def test_params_meet_estimated_tolerance():
    """The chosen xi puts the SLP real-space estimate within the driver's stopping
    rule |estimate - tol| <= tol (StokesSLP_ewald_2p.m:190)."""
    from fasttools2d_gb300.ewald import select_params
    prm = select_params("slp", 5000, 5000, 2e4, 1.0, 1.0, tol=1e-10)
    rc = prm.Lx / prm.nside_x
    Q = 2e4 + 1
    est = np.sqrt(Q * np.pi / (4 * prm.xi)) * np.exp(-(prm.xi * rc) ** 2)
    assert 0 < est <= 2e-10


def test_select_params_compat_switch():
    """compat=True keeps the drivers' arithmetic; compat=False the estimates as
    written.  They coincide for a unit square and differ for Lx != Ly."""
    from fasttools2d_gb300.ewald import select_params
    a = select_params("dlp", 4000, 4000, 3e3, 1.0, 1.0, tol=1e-10, compat=True)
    b = select_params("dlp", 4000, 4000, 3e3, 1.0, 1.0, tol=1e-10, compat=False)
    assert (a.xi, a.Mx, a.My) == (b.xi, b.Mx, b.My)
    for kind, Ly in (("slp", 2.0), ("dlp", 8.0)):
        c = select_params(kind, 4000, 4000, 3e3, 1.0, Ly, tol=1e-10, compat=True)
        d = select_params(kind, 4000, 4000, 3e3, 1.0, Ly, tol=1e-10, compat=False)
        assert c.xi == d.xi and c.Mx > d.Mx


def test_autograd_rejects_target_position_gradients():
    """ptar requiring a gradient (e.g. psrc passed again as the targets) raises
    before any GPU work, instead of returning a gradient without its
    target-position part."""
    torch = pytest.importorskip("torch")
    from fasttools2d_gb300.autograd import stokes_ewald_torch
    p = torch.zeros((4, 2), dtype=torch.float64, requires_grad=True)
    with pytest.raises(NotImplementedError):
        stokes_ewald_torch(p, p, p, p, p, None)
