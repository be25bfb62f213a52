"""Times the oracle port against the compiled reference on the same inputs.

ORACLE / TEST INFRASTRUCTURE ONLY.  Runs where ``make -C oracle ref`` built
the reference's own MEX sources into ``oracle/_ref`` (x86-64 hosts holding
the FastTools2D tree: the real-space sources use SSE3 intrinsics).  The GPU
host is aarch64, so there the CPU baseline and the reference arm of bench.py
time the port; this script records, on a host where both exist, how the port
compares with the reference in time and in results.

    python oracle/compare_ref_port.py [--n 262144] [--reps 3]

For each gateway (SLP/DLP real and k space) and for the full SLP+DLP
evaluation it prints the median wall time of the reference and of the port
(after one warm-up each), their ratio, and the normwise difference of their
outputs.  Inputs: N uniform sources and N uniform targets in the unit box,
N(0,1) forces and densities, random unit normals; xi, nside and M scaled from
the 1M-point workload (xi = 860, nside = 178, M = 2688, P = 24) so that the
points per box and per grid node stay the same.
"""
from __future__ import annotations

import argparse
import math
import os
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# run as a script, the oracle directory itself heads sys.path; the package
# import below needs the repository root instead
sys.path[:] = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402
from oracle import ref_mex  # noqa: E402


def _median_time(fn, reps):
    fn()
    ts = []
    out = None
    for _ in range(reps):
        t0 = time.perf_counter()
        out = fn()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts), out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=2 ** 18)
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    if not ref_mex.available():
        sys.exit("the compiled reference is absent: run `make -C oracle ref` on an x86-64 host")
    N = args.n
    r = math.sqrt(2 ** 20 / N)
    xi, nside, M, P = 860.0 / r, int(math.floor(1.0 / (0.0056 * r))), int(round(2688 / r)) // 2 * 2, 24
    w, eta = O.derived_w_eta(xi, M, 1.0, P)
    rng = np.random.default_rng(20261203 + 3)
    ps = O.wrap(rng.random((2, N)), 1.0)
    pt = O.wrap(rng.random((2, N)), 1.0)
    f = rng.standard_normal((2, N))
    g = rng.standard_normal((2, N))
    th = rng.random(N) * 2 * np.pi
    n = np.vstack([np.cos(th), np.sin(th)])
    R = ref_mex.RefMex()
    cases = {
        "slp_real": (lambda: R.slp_real(ps, pt, f, xi, nside, nside, 1.0, 1.0),
                     lambda: O.mex_stokes_slp_real(ps, pt, f, xi, nside, nside, 1.0, 1.0)),
        "slp_kspace": (lambda: R.slp_kspace(ps, pt, xi, eta, f, M, M, 1.0, 1.0, w, P),
                       lambda: O.mex_stokes_slp_kspace(ps, pt, xi, eta, f, M, M, 1.0, 1.0, w, P)),
        "dlp_real": (lambda: R.dlp_real(ps, pt, g, n, xi, nside, nside, 1.0, 1.0),
                     lambda: O.mex_stokes_dlp_real(ps, pt, g, n, xi, nside, nside, 1.0, 1.0)),
        "dlp_kspace": (lambda: R.dlp_kspace(ps, pt, xi, eta, g, n, M, M, 1.0, 1.0, w, P),
                       lambda: O.mex_stokes_dlp_kspace(ps, pt, xi, eta, g, n, M, M, 1.0, 1.0, w, P)),
    }
    print(f"N = {N} sources + {N} targets, xi = {xi:.1f}, nside = {nside}, M = {M}, P = {P}, "
          f"{O.num_threads()} threads, {os.cpu_count()} cores")
    print(f"{'gateway':12s} {'reference s':>12s} {'port s':>10s} {'port/ref':>9s} {'max|d|/max|ref|':>16s}")
    tot_r = tot_p = 0.0
    for name, (fr, fp) in cases.items():
        tr, a = _median_time(fr, args.reps)
        tp, b = _median_time(fp, args.reps)
        tot_r += tr
        tot_p += tp
        d = np.abs(a - b).max() / np.abs(a).max()
        print(f"{name:12s} {tr:12.3f} {tp:10.3f} {tp / tr:9.2f} {d:16.2e}")
    print(f"{'total':12s} {tot_r:12.3f} {tot_p:10.3f} {tot_p / tot_r:9.2f}")


if __name__ == "__main__":
    main()
