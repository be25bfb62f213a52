"""The GPU MEX gateways (fasttools2d_gb300/mexgw) called the way MATLAB calls them.

The four gateways are compiled against the MATLAB stand-in in oracle/mexshim
and linked to libse2p.  They are then driven with mxArray arguments exactly
as the drivers pass them (PE/src/matlab/StokesSLP_ewald_2p.m:119,126 and
StokesDLP_ewald_2p.m:140,147).  The CPU tests cover the argument checks and
messages of the reference gateways (PE/src/mex/StokesSLP/mex_stokes_slp_real.cpp:65-83
and the other three); the GPU tests compare plhs[0] with the reference's
outputs held in tests/golden.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_names, load_golden, relerr

MEXGW = os.path.join(ROOT, "fasttools2d_gb300", "mexgw")
OUT = os.path.join(MEXGW, "_build")
SHIM = os.path.join(ROOT, "oracle", "libmexshim.so")


@pytest.fixture(scope="module")
def gw():
    from oracle.ref_mex import MexSet
    if not os.path.exists(os.path.join(ROOT, "fasttools2d_gb300", "libse2p.so")):
        pytest.fail("libse2p.so not built (python -c 'import __graft_entry__ as g; g.build()')")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "libmexshim.so"], check=True)
    os.makedirs(OUT, exist_ok=True)
    subprocess.run(["make", "-s", "-j4", "-C", MEXGW, f"MEX_INC={os.path.join(ROOT, 'oracle', 'mexshim')}",
                    f"MEX_LIBS=-L{os.path.dirname(SHIM)} -lmexshim -Wl,-rpath,{os.path.dirname(SHIM)}",
                    f"OUT={OUT}"], check=True)
    g = MexSet(OUT, SHIM)
    yield g
    g.clear()


def _z(*shape):
    return np.zeros(shape)


def test_argument_errors(gw):
    p = np.random.default_rng(0).random((2, 5))
    cases = [
        ("mex_stokes_slp_real", (p, p, p, 1.0, 2, 2, 1.0), "Incorrect number of input parameters"),
        ("mex_stokes_slp_real", (_z(3, 5), p, p, 1.0, 2, 2, 1.0, 1.0), "psrc must be a 2xn matrix."),
        ("mex_stokes_slp_real", (p, _z(1, 5), p, 1.0, 2, 2, 1.0, 1.0), "ptar must be a 2xn matrix."),
        ("mex_stokes_slp_real", (p, p, _z(2, 4), 1.0, 2, 2, 1.0, 1.0), "psrc and f must be the same size."),
        ("mex_stokes_slp_kspace", (p, p, 1.0, 1.0, p, 8, 8, 1.0, 1.0, 0.1), "Incorrect number of input parameters"),
        ("mex_stokes_slp_kspace", (p, p, 1.0, 1.0, _z(5, 2), 8, 8, 1.0, 1.0, 0.1, 4), "f must be a 2xn matrix."),
        ("mex_stokes_dlp_real", (p, p, p, _z(2, 3), 1.0, 2, 2, 1.0, 1.0), "psrc and n must be the same size."),
        ("mex_stokes_dlp_real", (p, p, p, _z(3, 5), 1.0, 2, 2, 1.0, 1.0), "n must be a 2xn matrix."),
        ("mex_stokes_dlp_kspace", (p, p, 1.0, 1.0, p, p, 8, 8, 1.0, 1.0, 0.1), "Incorrect number of input parameters"),
        ("mex_stokes_dlp_kspace", (p, p, 1.0, 1.0, p, _z(2, 4), 8, 8, 1.0, 1.0, 0.1, 4), "psrc and n must be the same size."),
    ]
    for name, args, msg in cases:
        with pytest.raises(RuntimeError, match=msg):
            gw.call(name, *args)


def _args(d, kind):
    if kind == "slp_real":
        return (d["psrc"], d["ptar"], d["f"], d["xi"], d["nside_x"], d["nside_y"], d["Lx"], d["Ly"])
    if kind == "slp_kspace":
        return (d["psrc"], d["ptar"], d["xi"], d["eta"], d["f"], d["Mx"], d["My"], d["Lx"], d["Ly"],
                d["w"], d["P"])
    if kind == "dlp_real":
        return (d["psrc"], d["ptar"], d["f"], d["n"], d["xi"], d["nside_x"], d["nside_y"], d["Lx"], d["Ly"])
    return (d["psrc"], d["ptar"], d["xi"], d["eta"], d["f"], d["n"], d["Mx"], d["My"], d["Lx"], d["Ly"],
            d["w"], d["P"])


KINDS = ("slp_real", "slp_kspace", "dlp_real", "dlp_kspace")


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_names())
def test_gateways_match_reference(gw, name):
    d = load_golden(name)
    if "out_slp_real" not in d:
        pytest.skip("fixture holds no gateway outputs")
    for kind in KINDS:
        u = gw.call("mex_stokes_" + kind, *_args(d, kind))
        assert u.shape == d["out_" + kind].shape
        e = relerr(u, d["out_" + kind])
        assert e <= 1e-12, (name, kind, e)


@pytest.mark.gpu
def test_gateways_plan_reuse_and_clear(gw):
    d = load_golden("slp1000_xi19")
    a = gw.call("mex_stokes_slp_real", *_args(d, "slp_real"))
    b = gw.call("mex_stokes_slp_real", *_args(d, "slp_real"))
    assert relerr(a, b) <= 1e-13
    gw.clear()   # destroys the session plan; the next call makes a new one
    c = gw.call("mex_stokes_dlp_kspace", *_args(d, "dlp_kspace"))
    assert relerr(c, d["out_dlp_kspace"]) <= 1e-12


@pytest.mark.gpu
def test_gateways_empty_targets(gw):
    d = load_golden("slp1000_xi19")
    for kind in KINDS:
        a = list(_args(d, kind))
        a[1] = np.zeros((2, 0))
        u = gw.call("mex_stokes_" + kind, *a)
        assert u.shape == (2, 0)
