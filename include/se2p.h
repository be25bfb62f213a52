/*
 * se2p.h -- C ABI of libse2p: doubly-periodic spectral Ewald (SE) summation of
 * the 2D Stokeslet (single layer, SLP) and stresslet (double layer, DLP) on a
 * GB300 GPU (sm_103a).
 *
 * Drop-in for the spectral-Ewald path of FastTools2D (PeriodicEwald):
 *   - the four MEX gateways keep their argument order and meaning,
 *   - the two driver composites reproduce the MATLAB drivers' post-processing
 *     (wrap into [-L/2, L/2), real + k-space parts, DLP k=0 term, DLP sign)
 *     for given Ewald parameters.
 *
 * Data layout is MATLAB's: a "2xN" array is N interleaved (x, y) doubles.
 * Every array argument may be host memory (pageable or pinned) or device
 * memory of the plan's device; the library stages host data itself.  With
 * any host argument the call returns after the results are in host memory;
 * with device-only arguments the work is queued on the plan's stream and the
 * call returns without synchronising.
 *
 * Calls on one plan must not overlap; distinct plans are independent.
 * Every function returns an se2p_status; se2p_plan_last_error() gives the
 * message of the last failure on that plan.
 */
#ifndef SE2P_H
#define SE2P_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SE2P_OK = 0,
    SE2P_ERR_ARG = 1,          /* bad shape or parameter (the MEX gateways' mexErrMsgTxt cases) */
    SE2P_ERR_CUDA = 2,         /* CUDA runtime failure */
    SE2P_ERR_CUFFT = 3,        /* cuFFT failure */
    SE2P_ERR_ALLOC = 4,        /* device allocation failure */
    SE2P_ERR_UNSUPPORTED = 5   /* valid for the reference, outside this library's limits */
} se2p_status;

typedef struct se2p_plan_st *se2p_plan;

/* Ewald parameters of one evaluation (the MEX-level arguments). */
typedef struct {
    double xi;            /* Ewald splitting parameter */
    int nside_x, nside_y; /* real-space boxes per axis; cutoff^2 = Lx*Ly/nside_x/nside_y */
    int Mx, My;           /* k-space grid, even, with Lx/Mx == Ly/My */
    int P;                /* Gaussian support: P+1 nodes per axis, P even, P <= 30 */
    double Lx, Ly;        /* periodic box */
    double w;             /* Gaussian width P*h/2 (as passed by the drivers) */
    double eta;           /* spectral splitting parameter */
} se2p_params;

/* ---- plans ---------------------------------------------------------------
 * A plan owns a CUDA stream, reusable device workspace and cached cuFFT
 * plans.  No reference counterpart (the MEX gateways allocate per call). */
int se2p_plan_create(se2p_plan *plan, int device);
int se2p_plan_destroy(se2p_plan plan);
/* Queue the plan's work on an existing cudaStream_t; NULL selects CUDA's
 * legacy default stream (as cublasSetStream / cufftSetStream do).  A new plan
 * uses a private non-blocking stream. */
int se2p_plan_set_stream(se2p_plan plan, void *cuda_stream);
const char *se2p_plan_last_error(se2p_plan plan);
/* Real space runs on a plan-owned side stream, concurrently with the k-space
 * chain, unless overlap is switched off (on = 0): then every stage runs in
 * order on the plan's stream, e.g. to time kernels in isolation. */
int se2p_plan_set_overlap(se2p_plan plan, int on);
/* Bytes of device workspace the plan currently holds. */
int64_t se2p_plan_workspace_bytes(se2p_plan plan);
/* Number of kernels this plan has launched so far (its own, not cuFFT's). */
int64_t se2p_plan_kernel_launches(se2p_plan plan);
const char *se2p_version(void);

/* ---- precision ----------------------------------------------------------------
 * SE2P_PRECISION_FP64 (default): FP64 inputs and outputs, results within
 * 1e-12 of the reference (normwise and RMS-relative, per potential).  Each
 * stage runs in the narrowest arithmetic that keeps that bound, because GB300
 * issues FP32 some 70 times faster than FP64:
 *   - real space: the far pairs (1 < xi^2 r^2 < 64) in float-float arithmetic
 *     (pairs of FP32 values carrying about 48 bits); near pairs, the SLP self
 *     term and the exact cutoff decisions in FP64;
 *   - spread and gather: exact integer arithmetic -- every Gaussian factor
 *     rounded once to 62 bits, products as the high words of 64 x 64-bit
 *     integer products rounded to nearest, sums as exact int64 additions (the
 *     spread grid is bitwise reproducible); crowded grids or non-finite
 *     values fall back to the FP64 spread and gather;
 *   - FFT: float-float mixed-radix row transforms (cuFFT Z2Z for lengths with
 *     prime factors above 7);
 *   - filter, DLP k=0 term and the final sums: FP64.
 * SE2P_PRECISION_FP64_NATIVE: every floating-point step an FP64 instruction,
 * as the reference computes it (FP64 atomics, cuFFT Z2Z).
 * SE2P_PRECISION_FP32_GRID: the mixed form for tolerances >= 1e-6 --
 * spreading, FFT, filter and gather in FP32 and the far real-space pairs
 * (xi^2 r^2 > 1) in FP32, while the near real-space pairs (E1 at small
 * argument), the SLP self term and the DLP k=0 term stay FP64; the pair set,
 * box assignment and stencil origins stay exactly the reference's.
 * No reference counterpart (the reference is FP64 only).  Applies to all
 * later calls on the plan. */
typedef enum {
    SE2P_PRECISION_FP64 = 0,
    SE2P_PRECISION_FP32_GRID = 1,
    SE2P_PRECISION_FP64_NATIVE = 2
} se2p_precision;
int se2p_plan_set_precision(se2p_plan plan, int precision);

/* ---- stage timing ------------------------------------------------------------
 * Replaces the drivers' `verbose` tic/toc prints (StokesSLP_ewald_2p.m:106-131):
 * with timing on, every stage of every call (h2d, wrap, sort, coef, real,
 * spread, fft_fwd, filter, fft_inv, gather, zero_mode, assemble, d2h) is
 * bracketed by CUDA events on the plan's stream.  se2p_plan_stage_times
 * waits for the pending events and returns, per stage, the accumulated
 * milliseconds and call counts (arrays of se2p_num_stages() entries). */
int se2p_plan_enable_timing(se2p_plan plan, int on);
int se2p_num_stages(void);
const char *se2p_stage_name(int stage);
int se2p_plan_stage_times(se2p_plan plan, double *ms, int64_t *calls, int reset);

/* Measurement helper, no reference counterpart: the rate of coalesced 64-bit
 * integer atomic adds into an L2-resident array on the plan's device, in G/s
 * (best of 5 CUDA-event timings on the plan's stream; 32 MB of workspace).
 * It is the denominator of the integer spread's roofline, which issues one
 * such atomic per stencil node and grid. */
int se2p_plan_probe_atomics(se2p_plan plan, double *gops);

/* Real-space work counters: with counting on, the real-space kernel adds up
 * per call the candidate sources it examined and the SLP and DLP pairs it
 * accepted.  Sets counting on/off and returns the totals so far in
 * counts[3] = {candidates, slp_pairs, dlp_pairs} (optionally resetting them). */
int se2p_plan_count_pairs(se2p_plan plan, int on, int64_t *counts, int reset);

/* ---- MEX gateways ----------------------------------------------------------
 * Replaces mex_stokes_slp_real(psrc, ptar, f, xi, nside_x, nside_y, Lx, Ly)
 * (PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_real.cpp:58-83). */
int se2p_slp_real(se2p_plan plan, const double *psrc, int64_t nsrc, const double *ptar,
                  int64_t ntar, const double *f, double xi, int nside_x, int nside_y,
                  double Lx, double Ly, double *u);

/* Replaces mex_stokes_slp_kspace(psrc, ptar, xi, eta, f, Mx, My, Lx, Ly, w, P)
 * (PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:8-42). */
int se2p_slp_kspace(se2p_plan plan, const double *psrc, int64_t nsrc, const double *ptar,
                    int64_t ntar, double xi, double eta, const double *f, int Mx, int My,
                    double Lx, double Ly, double w, int P, double *u);

/* Replaces mex_stokes_dlp_real(psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly)
 * (PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:15-52). */
int se2p_dlp_real(se2p_plan plan, const double *psrc, int64_t nsrc, const double *ptar,
                  int64_t ntar, const double *f, const double *n, double xi, int nside_x,
                  int nside_y, double Lx, double Ly, double *u);

/* Replaces mex_stokes_dlp_kspace(psrc, ptar, xi, eta, f, n, Mx, My, Lx, Ly, w, P)
 * (PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_kspace.cpp:10-53). */
int se2p_dlp_kspace(se2p_plan plan, const double *psrc, int64_t nsrc, const double *ptar,
                    int64_t ntar, double xi, double eta, const double *f, const double *n,
                    int Mx, int My, double Lx, double Ly, double w, int P, double *u);

/* ---- driver composites -----------------------------------------------------
 * The part of StokesSLP_ewald_2p.m after parameter selection
 * (PeriodicEwald/src/matlab/StokesSLP_ewald_2p.m:74-82, :119-133):
 * wrap points into [-L/2, L/2), u = ur + uk.  ur / uk may be NULL. */
int se2p_slp_ewald(se2p_plan plan, const se2p_params *prm, const double *psrc, int64_t nsrc,
                   const double *ptar, int64_t ntar, const double *f, double *u, double *ur,
                   double *uk);

/* StokesDLP_ewald_2p.m:295-360 after parameter selection: wrap, ur, uk,
 * uk -= sum((f.n) x_src)/(Lx Ly) over the UNWRAPPED sources, u = -(ur + uk).
 * ur / uk (may be NULL) receive the parts as the driver returns them. */
int se2p_dlp_ewald(se2p_plan plan, const se2p_params *prm, const double *psrc, int64_t nsrc,
                   const double *ptar, int64_t ntar, const double *f, const double *n,
                   double *u, double *ur, double *uk);

/* Both drivers on one point set in one pass: u_slp as se2p_slp_ewald with
 * forces f_slp, u_dlp as se2p_dlp_ewald with density f_dlp and normals n.
 * Sorting, Gaussian weights, cuFFT batches and the real-space walk are
 * shared.  No single reference counterpart: it equals calling
 * StokesSLP_ewald_2p.m and StokesDLP_ewald_2p.m with the same parameters. */
int se2p_stokes_ewald(se2p_plan plan, const se2p_params *prm, const double *psrc,
                      int64_t nsrc, const double *ptar, int64_t ntar, const double *f_slp,
                      const double *f_dlp, const double *n, double *u_slp, double *u_dlp);

/* ---- adjoint ---------------------------------------------------------------------
 * Gradients of J = sum_t w_slp(t).u_slp(t) + w_dlp(t).u_dlp(t), where u_slp and
 * u_dlp are exactly what se2p_stokes_ewald returns for the same arguments,
 * with respect to the source positions psrc (as given, before wrapping), the
 * SLP forces f_slp, the DLP densities f_dlp and the normals n.  The SLP term
 * is present when f_slp and w_slp are given, the DLP term when f_dlp, n and
 * w_dlp are; any gradient pointer may be NULL.  Real space is differentiated
 * over exactly the forward's pair set (E1'(x) = -exp(-x)/x), k space by the
 * transposed spread/filter/gather chain with the Gaussian weights and their
 * derivatives recomputed, and the DLP k=0 term analytically.  No reference
 * counterpart (the reference has no derivatives). */
int se2p_stokes_ewald_adjoint(se2p_plan plan, const se2p_params *prm, const double *psrc,
                              int64_t nsrc, const double *ptar, int64_t ntar,
                              const double *f_slp, const double *f_dlp, const double *n,
                              const double *w_slp, const double *w_dlp, double *g_psrc,
                              double *g_fslp, double *g_fdlp, double *g_n);

/* ---- reusable geometry: many right-hand sides on one point set ---------------
 * No reference counterpart.  Boundary-integral solvers apply the same SE
 * operator to a new density every GMRES iteration.  se2p_geom_create sorts
 * the sources and targets once, builds the cell lists and precomputes the
 * real-space operator for prm: per target, every accepted (source, pair) with
 * its SLP 2x2 block (h - g x2^2, g x1 x2, h - g x1^2) and DLP 2x3 block --
 * float-float for far pairs, FP64 for near pairs and the self term (60 bytes
 * per pair; se2p_geom_bytes reports the total, about 6.6 GB at 2^20 + 2^20
 * uniform points with nside = 178).  kinds
 * = 1 (SLP), 2 (DLP, normals n fixed with the geometry) or 3 (both).
 * se2p_geom_apply evaluates nrhs right-hand sides -- f_slp and f_dlp are nrhs
 * consecutive 2 x nsrc arrays, u_slp and u_dlp nrhs consecutive 2 x ntar
 * arrays, host or device -- each as se2p_stokes_ewald (or se2p_slp_ewald /
 * se2p_dlp_ewald for one kind) would: the real space by the stored operator
 * (several RHS per pass over it), the k space and the DLP k=0 term per RHS at
 * the plan's precision.  Results agree with the single-RHS entry points to
 * ~1e-13.  The geometry uses its plan's stream and workspace: destroy it
 * before the plan, and do not run it concurrently with other calls on the plan. */
typedef struct se2p_geom_st *se2p_geom;
int se2p_geom_create(se2p_plan plan, const se2p_params *prm, const double *psrc, int64_t nsrc,
                     const double *ptar, int64_t ntar, const double *n, int kinds,
                     se2p_geom *geom);
int se2p_geom_apply(se2p_geom geom, int nrhs, const double *f_slp, const double *f_dlp,
                    double *u_slp, double *u_dlp);
int64_t se2p_geom_bytes(se2p_geom geom);
int64_t se2p_geom_pairs(se2p_geom geom);
int se2p_geom_destroy(se2p_geom geom);

/* ---- allocation-free SLP real space ------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory: a MEX function running inside MATLAB, where gpuArray's caching
 * allocator owns the GPU's memory, or a solver's time-step loop that must not
 * stall or fail on cudaMalloc.  Computes what se2p_slp_real computes on a
 * plan of the default precision (SE2P_PRECISION_FP64: far pairs in
 * float-float, near pairs and the self term in FP64), but all working arrays
 * live in one fixed file-scope device array of SE2P_NOALLOC_SCRATCH_BYTES
 * (32 MiB), beside an 18 KB table of the E1 fit, which every GPU that loads
 * this library holds until the process exits; nothing is allocated or freed
 * per call.
 *
 *  - psrc, ptar, f and u must be device memory of the current device,
 *    16-byte aligned; the work is queued on `cuda_stream` (NULL = legacy
 *    default stream) and the call returns without synchronising.
 *  - Size limit: 256-byte-rounded arrays totalling about
 *    68*nsrc + 56*ntar + 12*nside_x*nside_y bytes must fit in 32 MiB
 *    (e.g. 265,000 sources plus 265,000 targets with nside 178); larger
 *    calls return SE2P_ERR_UNSUPPORTED before touching the GPU.
 *  - Every call looks the arrays' device addresses up (cudaGetSymbolAddress,
 *    a host-side lookup) with the current device's context, and copies the
 *    E1 table in from host memory on `cuda_stream`.  A context created anew
 *    (after cudaDeviceReset, or MATLAB's reset(gpuDevice)) thus gets its own
 *    arrays; the first call in a context also loads the module, so make it
 *    before any stream capture.
 *  - Every call reuses the same array, which keeps the previous call's
 *    contents (the per-box counters are cleared on each call); calls whose
 *    GPU work overlaps, on any stream or thread, race on it. */
#define SE2P_NOALLOC_SCRATCH_BYTES (32u << 20)
int se2p_slp_real_noalloc(const double *psrc, int64_t nsrc, const double *ptar, int64_t ntar,
                          const double *f, double xi, int nside_x, int nside_y, double Lx,
                          double Ly, double *u, void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* SE2P_H */
