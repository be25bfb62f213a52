#!/usr/bin/env python
"""Benchmark: doubly-periodic spectral Ewald, 2D Stokeslet (SLP) + stresslet
(DLP), FP64, N = 2^20 sources and targets, on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = one SE evaluation of both potentials on the workload (sort, real
space, spread, FFTs, filter, gather, DLP k=0 term) through se2p_stokes_ewald.

Workload (xi=860, rc=0.0056 -> nside=178, M=2688, P=24, tolerance 1e-10):
1,048,576 sources and 1,048,576 separate targets uniform in the unit box,
SLP forces and DLP densities N(0,1), uniformly random unit normals, seed
20261203+3.  Synthetic data: the reference names no dataset.

Printed JSON line:
  value         evals/s with inputs resident in HBM (whole job, all ranks)
  e2e           evals/s through the C ABI with pinned HOST buffers, the
                host->device copies of the inputs and device->host copies of
                both outputs inside the timed region
  roofline      dominant kernel: its arithmetic work per launch over its
                CUDA-event time against the peak of the pipe that bounds it
                (real space: FP32 thread instructions of the float-float pair
                evaluations against 128 lanes x SMs x SM clock), plus its
                HBM side against the measured copy bandwidth
  cpu_baseline  the CPU oracle (a restatement of the reference's OpenMP path)
                on this host's cores, median of full evaluations
  parity_vs_oracle  the end-to-end outputs against the oracle's on the same
                inputs, per potential: normwise, RMS-relative and the
                99.9-percentile of the pointwise relative error
  fp64_native   the all-FP64 form on the same workload (rate and parity)
  gpu_launches  this library's kernel launches in the timed region
  clocks        nvidia-smi samples taken during the timed region

L2 (126 MB) is flushed between timed steps by writing a 256 MB buffer
(outside the timed intervals); the evaluation's own working set is ~0.9 GB.

With --impl reference the CPU reference path is timed instead (the
reference's own sources built under oracle/_ref where they compile, else the
oracle port), on all host threads, on the same workload; one step = one full
evaluation.  Under torchrun only rank 0 runs it.

Multi-GPU (torchrun, N > 1): independent replicas, one per GPU, no
collective on the data path (weak scaling); the timed region is bracketed by
barriers and the maximum time over ranks is reported.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 2 ** 20
XI, RC, M, P, L = 860.0, 0.0056, 2688, 24, 1.0
SEED = 20261203 + 3
METRIC = "SE Stokes evals/s @1M pts: FP64 tol 1e-10 vs FP32-grid tol 1e-6; fwd+adjoint time"
UNIT = "evals/s"
# Roofline inputs of the library's own kernels on this workload (FP64 form).
# * real space (k_real, far pairs in float-float on the FP32 pipe): bound by
#   the FP32 pipe; work = the FP32 thread instructions (FADD + FFMA + FMUL,
#   ncu) of one SLP+DLP pair evaluation, times the accepted pairs counted in
#   this run; peak = 128 FP32 lanes x SMs x the SM clock sampled in this run.
#   Issue utilisation (warp instructions per evaluation, ncu) is reported
#   beside it.
# * spread (k_spread_fix, exact int64 sums): bound by L2 atomics; work = one
#   64-bit reduction per stencil node and grid, (P+1)^2 C_in per source with
#   C_in = 5 grids (SLP f1, f2; DLP S11, S12+S21, S22); peak = coalesced int64
#   atomics measured in this run (se2p_plan_probe_atomics).
# * gather (k_gather_fix, int64 sums of exact products): bound by issue and
#   load latency; work = warp instructions per target (ncu).
# * filter: FP64 FLOP against cuBLAS DGEMM.
# DRAM bytes per launch are ncu's dram__bytes_read + _write of one launch
# (profiles/).
C_IN, C_OUT = 5, 4
SPREAD_RED_PER_SOURCE = (P + 1) ** 2 * C_IN
FILTER_FLOP_PER_MODE = 60
DRAM_BYTES = {"spread": 1.925e9, "gather": 0.281e9, "real": 0.213e9}
REAL_WARP_INST_PER_PAIR = 39.7     # ncu smsp__inst_executed / SLP+DLP pair evaluations
REAL_FP32_INST_PER_EVAL = 556.0    # ncu FADD 374 + FFMA 130 + FMUL 52 thread instructions per evaluation
GATHER_WARP_INST_PER_TARGET = 1508.0   # ncu smsp__inst_executed / targets (k_gather_fix<4,24>)
# Algorithmic HBM bytes of one launch, each array read or written once:
# real space reads per sorted source its position (16 B), FP32 copy (8 B), 5
# FP64 coefficients and 7 float-float ones (96 B), and per target its
# position, FP32 copy and box (28 B), and writes 2 x 16 B of sums.
REAL_ALG_BYTES_PER_POINT = (16 + 8 + 96, 16 + 8 + 4 + 32)   # (per source, per target)
FALLBACK_HBM_GBS = 6800.0


def workload(N):
    rng = np.random.default_rng(SEED)
    psrc = rng.random((N, 2))
    ptar = rng.random((N, 2))
    f = rng.standard_normal((N, 2))
    g = rng.standard_normal((N, 2))
    th = rng.random(N) * 2 * np.pi
    n = np.stack([np.cos(th), np.sin(th)], axis=1)
    return psrc, ptar, f, g, n


def params(N):
    import fasttools2d_gb300 as ft
    nside = int(math.floor(L / RC))
    return ft.EwaldParams.derived(XI, nside, nside, M, M, P, L, L)


def config(N, extra=None):
    c = {"workload": f"SE SLP+DLP FP64, N={N} sources + {N} targets uniform in L=1, "
                     f"xi={XI}, rc={RC} (nside={int(L / RC)}), M={M}, P={P}, tol 1e-10",
         "N_sources": N, "N_targets": N, "xi": XI, "rc": RC, "nside": int(L / RC), "M": M,
         "P": P, "L": L, "l2": "flushed between timed steps (256 MB write)"}
    if extra:
        c.update(extra)
    return c


def err_stats(a, b):
    """Error of a against b, both (N, 2): normwise max|a-b| / max|b|, RMS-relative
    ||a-b|| / ||b||, and the 99.9-percentile over targets of the pointwise
    relative error |a_t - b_t| / |b_t| (2-norms per target)."""
    a = np.asarray(a, dtype=np.float64).reshape(-1, 2)
    b = np.asarray(b, dtype=np.float64).reshape(-1, 2)
    ok = np.isfinite(b).all(axis=1) & np.isfinite(a).all(axis=1)
    a, b = a[ok], b[ok]
    d = a - b
    nb = np.hypot(b[:, 0], b[:, 1])
    pw = np.hypot(d[:, 0], d[:, 1]) / np.where(nb > 0, nb, np.inf)
    return {"max_rel": float(np.abs(d).max() / np.abs(b).max()),
            "rms_rel": float(np.sqrt(np.mean(d * d) / np.mean(b * b))),
            "p999_rel": float(np.quantile(pw, 0.999)),
            "nonfinite_mismatch": int((~ok).sum())}


def measured_hbm_gbs():
    """(GB/s, source): the copy bandwidth in MEASURED_PEAKS.json, else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, ValueError, KeyError):
        return FALLBACK_HBM_GBS, "fallback (one earlier GB300 measurement)"


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples (every 100 ms, time-stamped) while the context is
    open; summary() keeps those inside the windows marked with window(), the
    timed regions, with one sampling interval of slack."""
    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    PERIOD_S = 0.1

    def __init__(self, gpu_id):
        self.gpu_id = gpu_id
        self.proc = None
        self.windows = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu_id), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(int(self.PERIOD_S * 1000))],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def window(self, t0, t1):
        self.windows.append((t0, t1))

    def __exit__(self, *exc):
        self.rows = []
        if self.proc is None:
            return False
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for line in out.splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 8:
                try:
                    t = time.mktime(time.strptime(parts[0].split(".")[0], "%Y/%m/%d %H:%M:%S"))
                    t += float("0." + parts[0].split(".")[1]) if "." in parts[0] else 0.0
                except (ValueError, IndexError):
                    t = None
                self.rows.append((t, parts[1:]))
        return False

    def summary(self):
        if not getattr(self, "rows", None):
            return None
        sl = self.PERIOD_S
        inside = [r for t, r in self.rows if t is not None and
                  any(t0 - sl <= t <= t1 + sl for t0, t1 in self.windows)]
        rows = inside or [r for _, r in self.rows]
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows), "in_timed_regions": bool(inside)}


# ---------------------------------------------------------------------------
# CPU paths (oracle port / compiled reference), used for cpu_baseline and
# the reference arm
# ---------------------------------------------------------------------------
def cpu_eval_fn(N, prefer_reference):
    from oracle import oracle as O
    psrc, ptar, f, g, n = workload(N)
    prm = params(N)
    S, T = psrc.T.copy(), ptar.T.copy()
    F, G, Nn = f.T.copy(), g.T.copy(), n.T.copy()
    kind = "port"
    if prefer_reference:
        from oracle import ref_mex
        if ref_mex.available():
            kind = "reference"
            R = ref_mex.RefMex()

            def run():
                ps = np.vstack([O.wrap(S[0], L), O.wrap(S[1], L)])
                pt = np.vstack([O.wrap(T[0], L), O.wrap(T[1], L)])
                R.slp_real(ps, pt, F, prm.xi, prm.nside_x, prm.nside_y, L, L)
                R.slp_kspace(ps, pt, prm.xi, prm.eta, F, M, M, L, L, prm.w, P)
                R.dlp_real(ps, pt, G, Nn, prm.xi, prm.nside_x, prm.nside_y, L, L)
                R.dlp_kspace(ps, pt, prm.xi, prm.eta, G, Nn, M, M, L, L, prm.w, P)
                O.dlp_zero_mode(S, G, Nn, L, L)
            return run, kind

    def run():
        """(u_slp, u_dlp) as (N, 2) arrays."""
        us = O.slp_ewald(S, T, F, prm.xi, prm.nside_x, prm.nside_y, M, M, L, L, P)[0]
        ud = O.dlp_ewald(S, T, G, Nn, prm.xi, prm.nside_x, prm.nside_y, M, M, L, L, P)[0]
        return us.T, ud.T
    return run, kind


def cpu_threads():
    from oracle import oracle as O
    return O.num_threads()


def cpu_baseline(N, reps=5):
    """The oracle port on the host cores: the median of `reps` full
    evaluations after one warm-up (about 10 s at N = 2^20).  Returns the
    baseline record and the oracle's outputs (u_slp, u_dlp), which the GPU
    results are checked against."""
    run, kind = cpu_eval_fn(N, prefer_reference=False)
    out = run()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        run()
        ts.append(time.perf_counter() - t0)
    dt = statistics.median(ts)
    return {"value": 1.0 / dt, "unit": UNIT, "cores": cpu_threads(), "kind": kind,
            "sample": f"median of {reps} full SLP+DLP evaluations at N={N} after one warm-up "
                      f"(oracle C restatement, OpenMP, scipy FFT), {dt:.2f} s each"}, out


def reference_arm(args, rank, world):
    if rank != 0:
        return
    N = args.n
    run, kind = cpu_eval_fn(N, prefer_reference=True)
    for _ in range(args.warmup):
        run()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        run()
        ts.append(time.perf_counter() - t0)
    total = sum(ts)
    value = args.steps / total
    cores = cpu_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config(N, {"parallelism": "cpu-openmp"}),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"full SLP+DLP evaluation at N={N} per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def fp64_peak_tflops(torch, dev):
    """FP64 peak of this GPU measured as cuBLAS DGEMM throughput (best of 5)."""
    n = 2048
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize(dev)
    best = 1e30
    for _ in range(5):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e))
    return 2 * n ** 3 / (best * 1e-3) / 1e12


# The mixed-precision workload (same points), tolerance 1e-6.
XI4, RC4, M4, P4 = 860.0, 0.0042, 2048, 12


# ncu dram__bytes_read + _write of one launch of the FP32-grid k-space kernels
# at the mixed-precision workload (profiles/).
F32_DRAM_BYTES = {"spread": 0.172e9, "gather": 0.0955e9}


def mixed_precision_leg(plan, tens, u_dev, N, steps, timed, dev, with_oracle):
    """FP32-grid vs FP64 on the mixed-precision workload: evals/s of each, speed-up, the
    FP32-grid error against the FP64 result and (with_oracle) against the CPU oracle run
    on the same points and parameters, per potential; and the HBM roofline of the
    FP32-grid spread and gather from a serialised pass with stage timing."""
    import torch
    import fasttools2d_gb300 as ft
    nside = int(math.floor(L / RC4))
    prm4p = ft.EwaldParams.derived(XI4, nside, nside, M4, M4, P4, L, L)
    prm4 = prm4p.as_c()
    L_ = plan.lib
    out = {}
    res = {}
    stages = None
    for prec in ("fp64", "fp32_grid"):
        plan.set_precision(prec)
        u = [torch.empty_like(u_dev[0]), torch.empty_like(u_dev[1])]

        def step():
            plan.check(L_.se2p_stokes_ewald(plan.handle, ctypes.byref(prm4), tens[0].data_ptr(), N,
                                            tens[1].data_ptr(), N, tens[2].data_ptr(),
                                            tens[3].data_ptr(), tens[4].data_ptr(),
                                            u[0].data_ptr(), u[1].data_ptr()))
        for _ in range(3):
            step()
        ms = timed(step, steps) / steps
        res[prec] = [x.double().cpu().numpy() for x in u]
        out[prec] = {"evals_per_s": 1e3 / ms, "ms_per_step": ms}
        if prec == "fp32_grid":
            plan.set_overlap(False)
            plan.enable_timing(True)
            plan.stage_times(reset=True)
            for _ in range(2):
                step()
            torch.cuda.synchronize(dev)
            stages = plan.stage_times(reset=True)
            plan.enable_timing(False)
            plan.set_overlap(True)
    plan.set_precision("fp64")
    err = {name: err_stats(res["fp32_grid"][i], res["fp64"][i])
           for i, name in enumerate(("slp", "dlp"))}
    line = {"workload": f"SE SLP+DLP, same 1M points, xi={XI4}, rc={RC4} (nside={nside}), M={M4}, "
                        f"P={P4}, tol 1e-6",
            "value": out["fp32_grid"]["evals_per_s"], "unit": UNIT,
            "ms_per_step": out["fp32_grid"]["ms_per_step"],
            "fp64_same_workload": out["fp64"],
            "speedup_vs_fp64_same_workload": out["fp32_grid"]["evals_per_s"] / out["fp64"]["evals_per_s"],
            "error_vs_fp64": err}
    if with_oracle:
        from oracle import oracle as O
        psrc, ptar, f, g, n = workload(N)
        S, T = psrc.T.copy(), ptar.T.copy()
        ros = O.slp_ewald(S, T, f.T.copy(), XI4, nside, nside, M4, M4, L, L, P4)[0].T
        rod = O.dlp_ewald(S, T, g.T.copy(), n.T.copy(), XI4, nside, nside, M4, M4, L, L, P4)[0].T
        line["error_vs_oracle"] = {"fp32_grid": {"slp": err_stats(res["fp32_grid"][0], ros),
                                                 "dlp": err_stats(res["fp32_grid"][1], rod)},
                                   "fp64": {"slp": err_stats(res["fp64"][0], ros),
                                            "dlp": err_stats(res["fp64"][1], rod)},
                                   "oracle": "CPU oracle (FP64) on the same points and parameters"}
    # HBM roofline of the FP32-grid k-space kernels (serialised stage times):
    # the spread reads per source its position and 5 FP64 coefficients (56 B)
    # and writes the 5 FP32 grids once; the gather reads per target its
    # position (16 B), the 4 FP32 grids once, and writes 2 x 16 B.
    hbm, hbm_src = measured_hbm_gbs()
    G4 = M4 * M4
    alg = {"spread": N * 56 + G4 * 5 * 4, "gather": N * (16 + 32) + G4 * 4 * 4}
    roof = {}
    for k in ("spread", "gather"):
        if stages and k in stages and stages[k][1] > 0:
            ms = stages[k][0] / stages[k][1]
            gbs = alg[k] / (ms * 1e-3) / 1e9
            roof[k] = {"kernel": f"k_{k}_f32", "bound": "hbm", "ms_per_launch": ms,
                       "alg_bytes": alg[k], "achieved": gbs, "peak": hbm, "unit": "GB/s",
                       "frac": gbs / hbm, "peak_source": hbm_src,
                       "traffic": F32_DRAM_BYTES[k], "traffic_unit": "bytes/launch (ncu)"}
    line["roofline"] = roof
    line["stage_ms"] = {k: round(v[0] / 2, 4) for k, v in (stages or {}).items()
                        if v[1] > 0}
    return line


def native_leg(plan, tens, u_dev, N, steps, timed, oracle_out):
    """The all-FP64 form (every floating-point step an FP64 instruction, as the
    reference computes it) on the headline workload: its rate, and its parity
    with the oracle when the oracle's outputs are at hand."""
    import torch
    L_ = plan.lib
    cprm = params(N).as_c()
    u = [torch.empty_like(u_dev[0]), torch.empty_like(u_dev[1])]
    plan.set_precision("fp64_native")

    def step():
        plan.check(L_.se2p_stokes_ewald(plan.handle, ctypes.byref(cprm), tens[0].data_ptr(), N,
                                        tens[1].data_ptr(), N, tens[2].data_ptr(),
                                        tens[3].data_ptr(), tens[4].data_ptr(),
                                        u[0].data_ptr(), u[1].data_ptr()))
    try:
        for _ in range(2):
            step()
        k = max(2, steps // 2)
        ms = timed(step, k) / k
    finally:
        plan.set_precision("fp64")
    line = {"workload": "the headline workload, precision SE2P_PRECISION_FP64_NATIVE",
            "evals_per_s": 1e3 / ms, "ms_per_step": ms, "steps": k}
    if oracle_out is not None:
        got = [x.cpu().numpy() for x in u]
        line["parity_vs_oracle"] = {"slp": err_stats(got[0], oracle_out[0]),
                                    "dlp": err_stats(got[1], oracle_out[1])}
    return line


# The adjoint workload: forward + adjoint, N = 2^18.
N5, XI5, RC5, M5, P5 = 2 ** 18, 430.0, 0.011, 1344, 24
FD_COORDS = 64


def multi_rhs_leg(plan, tens, N, ms_single, dev, nrhs=4):
    """Many right-hand sides on the 1M-point geometry (se2p_geom_*): time to
    build the geometry (sort, cell lists, real-space operator), and time per
    right-hand side of one apply over nrhs densities, against the single-RHS
    evaluation.  Every apply is checked against se2p_stokes_ewald on its
    first right-hand side."""
    import time
    import torch
    import fasttools2d_gb300 as ft
    prm = ft.EwaldParams.derived(XI, int(math.floor(L / RC)), int(math.floor(L / RC)), M, M, P, L, L)
    rng = torch.Generator(device=dev).manual_seed(SEED + 100)
    F = torch.randn((nrhs, N, 2), dtype=torch.float64, device=dev, generator=rng)
    G = torch.randn((nrhs, N, 2), dtype=torch.float64, device=dev, generator=rng)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    geo = ft.Geometry(tens[0], tens[1], prm, n=tens[4], plan=plan)
    torch.cuda.synchronize(dev)
    build_ms = (time.perf_counter() - t0) * 1e3
    us, ud = geo.apply(F, G)                       # warm-up (cuFFT plans, workspace)
    best = 1e30
    for _ in range(3):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        us, ud = geo.apply(F, G)
        torch.cuda.synchronize(dev)
        best = min(best, (time.perf_counter() - t0) * 1e3)
    vs, vd = ft.stokes_ewald(tens[0], tens[1], F[0], G[0], tens[4], prm, plan=plan)
    err = max(float((us[0] - vs).abs().max() / vs.abs().max()),
              float((ud[0] - vd).abs().max() / vd.abs().max()))
    out = {"workload": f"SE SLP+DLP, same 1M points and parameters, {nrhs} right-hand sides "
                       "per apply (densities ~ N(0,1))",
           "nrhs": nrhs, "geometry_build_ms": build_ms, "apply_ms_per_rhs": best / nrhs,
           "single_rhs_ms": ms_single, "speedup_per_rhs": ms_single / (best / nrhs),
           "geometry_bytes": geo.bytes, "pairs": geo.pairs,
           "max_rel_diff_vs_single_rhs": err}
    geo.close()
    return out


def adjoint_leg(plan, steps, timed, dev):
    """Adjoint workload: time of the forward and of forward + adjoint (gradients of
    J = sum_t w_slp.u_slp + w_dlp.u_dlp w.r.t. source positions, forces,
    densities, normals), and a central-difference check of the gradients on
    64 random coordinates (h = 1e-6, J from the GPU forward)."""
    import torch
    import fasttools2d_gb300 as ft
    rng = np.random.default_rng(20261203 + 5)
    N = N5
    arrs = [rng.random((N, 2)), rng.random((N, 2)), rng.standard_normal((N, 2)),
            rng.standard_normal((N, 2))]
    th = rng.random(N) * 2 * np.pi
    arrs.append(np.stack([np.cos(th), np.sin(th)], axis=1))
    w = [rng.standard_normal((N, 2)), rng.standard_normal((N, 2))]
    T = [torch.from_numpy(a).to(dev) for a in arrs]
    Wt = [torch.from_numpy(a).to(dev) for a in w]
    nside = int(math.floor(L / RC5))
    prm = ft.EwaldParams.derived(XI5, nside, nside, M5, M5, P5, L, L)
    c = prm.as_c()
    Lb = plan.lib
    u = [torch.empty((N, 2), dtype=torch.float64, device=dev) for _ in range(2)]
    g = [torch.empty((N, 2), dtype=torch.float64, device=dev) for _ in range(4)]

    def fwd():
        plan.check(Lb.se2p_stokes_ewald(plan.handle, ctypes.byref(c), T[0].data_ptr(), N,
                                        T[1].data_ptr(), N, T[2].data_ptr(), T[3].data_ptr(),
                                        T[4].data_ptr(), u[0].data_ptr(), u[1].data_ptr()))

    def adj():
        plan.check(Lb.se2p_stokes_ewald_adjoint(
            plan.handle, ctypes.byref(c), T[0].data_ptr(), N, T[1].data_ptr(), N,
            T[2].data_ptr(), T[3].data_ptr(), T[4].data_ptr(), Wt[0].data_ptr(),
            Wt[1].data_ptr(), g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(),
            g[3].data_ptr()))

    def both():
        fwd()
        adj()
    for _ in range(3):
        both()
    t_f = timed(fwd, steps) / steps
    t_fa = timed(both, steps) / steps
    # finite differences on 64 coordinates: positions, forces, densities, normals
    both()
    torch.cuda.synchronize(dev)
    G = [x.cpu().numpy() for x in g]
    pick = np.random.default_rng(1)
    worst = 0.0
    h = 1e-6
    which = {0: 0, 2: 1, 3: 2, 4: 3}          # input array -> gradient array

    def J():
        fwd()
        return float((Wt[0] * u[0]).sum() + (Wt[1] * u[1]).sum())
    for _ in range(FD_COORDS):
        a = int(pick.choice([0, 2, 3, 4]))
        i, k = int(pick.integers(0, N)), int(pick.integers(0, 2))
        x0 = float(T[a][i, k])
        T[a][i, k] = x0 + h
        jp = J()
        T[a][i, k] = x0 - h
        jm = J()
        T[a][i, k] = x0
        gi = G[which[a]]
        worst = max(worst, abs((jp - jm) / (2 * h) - gi[i, k]) / np.abs(gi).max())
    return {"workload": f"SE SLP+DLP forward+adjoint, N={N} sources + {N} targets uniform, xi={XI5}, rc={RC5} "
                        f"(nside={nside}), M={M5}, P={P5}, FP64; J = sum_t w.u with w ~ N(0,1)",
            "fwd_ms": t_f, "fwd_adjoint_ms": t_fa, "ratio_fwd_adjoint_over_fwd": t_fa / t_f,
            "fd_check": {"coords": FD_COORDS, "h": h, "max_err_rel_to_max_grad": worst}}


def aggregate_replicas(local_ms, steps, world, device=None):
    """(max over ranks of a timed region in ms, whole-job evals/s).

    Replicas: every rank evaluates its own copy of the workload, so the job
    rate is world * steps over the slowest rank's time.  With world > 1 this
    is an all-reduce (MAX) in the process group (NCCL on GPUs, gloo in the
    CPU tests)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        local_ms = float(t.item())
    return local_ms, world * steps / (local_ms * 1e-3)


def gpu_arm(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    import fasttools2d_gb300 as ft

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    N = args.n
    prm = params(N)
    psrc, ptar, f, g, n = workload(N)
    tens = [torch.from_numpy(a).to(dev) for a in (psrc, ptar, f, g, n)]
    plan = ft.Plan(local_rank)
    stream = torch.cuda.current_stream(dev)
    plan.set_stream(stream.cuda_stream)
    flush = torch.empty(64 * 2 ** 20, dtype=torch.float32, device=dev)   # 256 MB
    cprm = prm.as_c()
    L_ = plan.lib

    u_dev = [torch.empty((N, 2), dtype=torch.float64, device=dev) for _ in range(2)]

    def step_device():
        plan.check(L_.se2p_stokes_ewald(plan.handle, ctypes.byref(cprm), tens[0].data_ptr(), N,
                                        tens[1].data_ptr(), N, tens[2].data_ptr(),
                                        tens[3].data_ptr(), tens[4].data_ptr(),
                                        u_dev[0].data_ptr(), u_dev[1].data_ptr()))

    pin = [torch.from_numpy(a).pin_memory() for a in (psrc, ptar, f, g, n)]
    u_host = [torch.empty((N, 2), dtype=torch.float64).pin_memory() for _ in range(2)]

    def step_host():
        plan.check(L_.se2p_stokes_ewald(plan.handle, ctypes.byref(cprm), pin[0].data_ptr(), N,
                                        pin[1].data_ptr(), N, pin[2].data_ptr(),
                                        pin[3].data_ptr(), pin[4].data_ptr(),
                                        u_host[0].data_ptr(), u_host[1].data_ptr()))

    def timed(step, steps):
        ms = []
        for _ in range(steps):
            flush.zero_()
            s = torch.cuda.Event(enable_timing=True)
            e = torch.cuda.Event(enable_timing=True)
            s.record(stream)
            step()
            e.record(stream)
            ms.append((s, e))
        torch.cuda.synchronize(dev)
        return sum(s.elapsed_time(e) for s, e in ms)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    def max_over_ranks(x):
        return aggregate_replicas(x, 1, world, dev)[0]

    gpu_id = local_rank
    try:
        gpu_id = str(torch.cuda.get_device_properties(dev).uuid)
        gpu_id = gpu_id if gpu_id.startswith("GPU-") else "GPU-" + gpu_id
    except Exception:
        pass
    # the clock sampler starts before the warm-up, so that it is sampling
    # when the timed regions begin; it keeps the samples taken inside them
    with ClockSampler(gpu_id) as clk:
        for _ in range(args.warmup):
            step_device()
        torch.cuda.synchronize(dev)

        # ---- device-resident timed region (no stage events, no pair counters)
        launches0 = plan.kernel_launches
        barrier()
        t0 = time.time()
        total_ms = timed(step_device, args.steps)
        barrier()
        clk.window(t0, time.time())
        launches = plan.kernel_launches - launches0
        total_ms, value = aggregate_replicas(total_ms, args.steps, world, dev)
        ms_per_step = total_ms / args.steps

        # ---- end to end through the C ABI with pinned host buffers --------
        for _ in range(max(1, args.warmup // 2)):
            step_host()
        barrier()
        t0 = time.time()
        e2e_ms = max_over_ranks(timed(step_host, args.steps))
        barrier()
        clk.window(t0, time.time())
    e2e = {"value": world * args.steps / (e2e_ms * 1e-3), "unit": UNIT,
           "h2d_bytes_per_step": 5 * N * 16, "d2h_bytes_per_step": 2 * N * 16,
           "ms_per_step": e2e_ms / args.steps}

    # ---- per-kernel times without overlap (for the roofline) -------------
    # Real space normally runs concurrently with the k-space chain; for the
    # per-kernel roofline the stages are timed once more, in order.
    # The real-space pair counters run here too (they add ballots to the
    # candidate loop, so the timed region above runs without them).
    plan.set_overlap(False)
    plan.enable_timing(True)
    plan.stage_times(reset=True)
    plan.count_pairs(True, reset=True)
    n_serial = 2
    for _ in range(n_serial):
        step_device()
    torch.cuda.synchronize(dev)
    counts = plan.count_pairs(False, reset=True)
    stages = plan.stage_times(reset=True)
    plan.enable_timing(False)
    plan.set_overlap(True)

    # ---- the oracle on the same inputs: CPU baseline and parity ----------
    legs = set(args.legs.split(","))
    cpu = oracle_out = parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, oracle_out = cpu_baseline(N)
        got = [x.numpy() for x in u_host]               # the end-to-end (host) outputs
        dev_out = [x.cpu().numpy() for x in u_dev]       # the device-resident outputs
        parity = {"slp": err_stats(got[0], oracle_out[0]), "dlp": err_stats(got[1], oracle_out[1]),
                  "device_vs_host_outputs": max(err_stats(dev_out[i], got[i])["max_rel"]
                                                for i in range(2)),
                  "oracle": "CPU oracle (FP64 restatement of the reference) on the same inputs",
                  "bar": "normwise and RMS-relative <= 1e-12 per potential"}

    # ---- the all-FP64 form on the same workload ---------------------------
    native = native_leg(plan, tens, u_dev, N, args.steps, timed, oracle_out) \
        if "fp64_native" in legs else None

    # ---- FP32-grid form (mixed-precision workload) next to the FP64 form on the same workload
    mixed = mixed_precision_leg(plan, tens, u_dev, N, args.steps, timed, dev,
                                with_oracle=oracle_out is not None) \
        if "fp32_grid" in legs else None
    if mixed is not None:
        # the metric's own pairing: FP32-grid at tolerance 1e-6 against the
        # FP64 form at tolerance 1e-10 (the headline workload above)
        mixed["speedup_vs_fp64_tol1e-10"] = mixed["value"] / (1e3 / ms_per_step)
    adjoint = adjoint_leg(plan, args.steps, timed, dev) if "adjoint" in legs else None
    multi = multi_rhs_leg(plan, tens, N, ms_per_step, dev) if "multi_rhs" in legs else None

    # ---- roofline of the dominant kernel ---------------------------------
    # Stage times come from CUDA events on each kernel's own stream, taken in
    # the serialised pass above; the top one among this library's kernels
    # (cuFFT excluded) gets the roofline.
    kstages = {k: v for k, v in stages.items() if k not in ("h2d", "d2h") and v[1] > 0}
    per = {k: v[0] / v[1] for k, v in kstages.items()}
    own = {k: per[k] for k in ("real", "spread", "gather", "filter") if k in per}
    top = max(own, key=own.get)
    top_ms = own[top]
    pairs_per_launch = (counts[1] + counts[2]) / n_serial       # counted in the serialised pass
    evals_per_launch = pairs_per_launch / 2                     # SLP and DLP share each evaluation
    clock_ghz = (clk.summary().get("sm_mhz") or 2070.0) / 1e3
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    issue_peak = 4 * sms * clock_ghz * 1e9 / 1e12
    issue_src = "4 warp instructions per clock per SM x SMs x measured SM clock"
    fp32_peak = 128 * sms * clock_ghz * 1e9 / 1e12
    hbm, hbm_src = measured_hbm_gbs()
    # the integer spread against the L2 atomic rate, whichever kernel is on top
    spread_atomics = None
    if "spread" in per:
        red_peak = plan.probe_atomics()
        red_done = N * SPREAD_RED_PER_SOURCE / (per["spread"] * 1e-3) / 1e9
        spread_atomics = {"kernel": "k_spread_fix<5>", "achieved": red_done, "peak": red_peak,
                          "unit": "G int64 atomics/s", "frac": red_done / red_peak,
                          "ms_per_launch": per["spread"],
                          "hbm_side": {"traffic": DRAM_BYTES["spread"],
                                       "alg_bytes": N * (16 + 8 * C_IN) + M * M * C_IN * 8}}
    real_side = None
    if "real" in per:
        rms_ = per["real"]
        alg = N * (REAL_ALG_BYTES_PER_POINT[0] + REAL_ALG_BYTES_PER_POINT[1])
        real_side = {
            "kernel": "k_real<SLP,DLP,float-float>", "ms_per_launch": rms_,
            "accepted_pairs_per_launch": pairs_per_launch,
            "evaluations_per_launch": evals_per_launch,
            "candidates_per_launch": counts[0] / n_serial,
            "candidates_per_evaluation": counts[0] / n_serial / max(1.0, evals_per_launch),
            "pairs_per_s": pairs_per_launch / (rms_ * 1e-3),
            "fp32_pipe": {"achieved": evals_per_launch * REAL_FP32_INST_PER_EVAL / (rms_ * 1e-3) / 1e12,
                          "peak": fp32_peak, "unit": "T FP32 thread-inst/s",
                          "work_per_evaluation": REAL_FP32_INST_PER_EVAL,
                          "peak_source": "128 FP32 lanes per SM x SMs x measured SM clock"},
            "issue": {"achieved": evals_per_launch * REAL_WARP_INST_PER_PAIR / (rms_ * 1e-3) / 1e12,
                      "peak": issue_peak, "unit": "T warp-inst/s",
                      "work_per_evaluation": REAL_WARP_INST_PER_PAIR, "peak_source": issue_src},
            "hbm_side": {"alg_bytes": alg, "achieved": alg / (rms_ * 1e-3) / 1e9, "peak": hbm,
                         "unit": "GB/s", "traffic": DRAM_BYTES["real"]}}
        for k in ("fp32_pipe", "issue", "hbm_side"):
            real_side[k]["frac"] = real_side[k]["achieved"] / real_side[k]["peak"]
    if top == "real":
        roof = {"kernel": "k_real<SLP,DLP,float-float> (fused real-space pair sum)",
                "bound": "fp32", "achieved": real_side["fp32_pipe"]["achieved"],
                "peak": fp32_peak, "unit": "T FP32 thread-inst/s",
                "peak_source": real_side["fp32_pipe"]["peak_source"],
                "work": f"{REAL_FP32_INST_PER_EVAL:.0f} FP32 thread instructions (FADD+FFMA+FMUL, ncu) "
                        "per SLP+DLP pair evaluation x evaluations counted in this run"}
    elif top == "gather":
        roof = {"kernel": "k_gather_fix<4,24> (integer gather, 4 grids)", "bound": "issue",
                "achieved": N * GATHER_WARP_INST_PER_TARGET / (top_ms * 1e-3) / 1e12,
                "peak": issue_peak, "unit": "T warp-inst/s", "peak_source": issue_src}
    elif top == "spread":
        roof = {"kernel": "k_spread_fix<5> (integer spread, 5 grids)", "bound": "l2_atomics",
                "achieved": N * SPREAD_RED_PER_SOURCE / (top_ms * 1e-3) / 1e9,
                "peak": spread_atomics["peak"], "unit": "G int64 atomics/s",
                "peak_source": "coalesced 64-bit integer atomics into an L2-resident array, "
                               "se2p_plan_probe_atomics in this run "
                               "(MEASURED_PEAKS.json holds no atomic figure)"}
    else:
        flops = M * (M // 2 + 1) * FILTER_FLOP_PER_MODE
        roof = {"kernel": "k_filter", "bound": "fp64", "achieved": flops / (top_ms * 1e-3) / 1e12,
                "peak": fp64_peak_tflops(torch, dev), "unit": "TFLOP/s",
                "peak_source": "cuBLAS DGEMM 2048^3 measured in this run "
                               "(MEASURED_PEAKS.json holds no FP64 figure)"}
    roof.update({"frac": roof["achieved"] / roof["peak"],
                 "traffic": DRAM_BYTES.get(top), "traffic_unit": "bytes/launch (ncu)",
                 "ms_per_launch": top_ms, "top_stage": top,
                 "spread_atomics": spread_atomics, "real_space": real_side})
    # per evaluation (a stage may be timed in parts: the sources' and the
    # targets' sort, the two coefficient kernels)
    stage_ms = {k: round(v[0] / n_serial, 4) for k, v in stages.items() if v[1] > 0}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config(N, {"parallelism": f"replicas x{world}" if world > 1 else "single GPU"}),
        "e2e": e2e, "roofline": roof, "gpu_launches": launches, "stage_ms": stage_ms,
        "clocks": clk.summary(), "parity_vs_oracle": parity, "fp64_native": native,
        "fp32_grid": mixed, "adjoint": adjoint, "multi_rhs": multi,
        # the metric's secondary unit: targets evaluated per second (N_t / t)
        "target_evals_per_s": value * N,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)
    plan.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT, help="points (sources = targets count)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--legs", default="fp64_native,fp32_grid,adjoint,multi_rhs",
                    help="extra legs after the headline workload: fp64_native, fp32_grid, adjoint, "
                         "multi_rhs, or none "
                         "(a profiling run of the headline workload alone uses none)")
    ap.add_argument("--shrink", type=int, default=1, choices=[1, 4, 16],
                    help="profiling cases: N / shrink points with xi, 1/rc and M divided by "
                         "sqrt(shrink), so the points per box and per grid node stay the same "
                         "(4: 2^18 points, xi=430, nside=89, M=1344)")
    args = ap.parse_args()
    if args.shrink > 1:
        global XI, RC, M
        r = int(round(math.sqrt(args.shrink)))
        XI, RC, M = XI / r, RC * r, M // r
        args.n //= args.shrink
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if args.gpus == 1 else 1)))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    gpu_arm(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
