// se2p_api.cu -- C ABI of libse2p (include/se2p.h): argument checks, device
// workspace, staging of host arrays, cuFFT plans and the order of kernel
// launches for each entry point.
//
// One evaluation runs as
//   [wrap] -> sort sources/targets into boxes -> per-source coefficients
//   -> real space (k_real)                     \  both read the sorted data
//   -> spread -> 2D FFT -> filter -> inverse FFT -> gather /
//   -> [DLP zero mode] -> assemble in the caller's target order.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <algorithm>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/se2p.h"
#include "se2p_internal.cuh"

using namespace se2p;

namespace {

#ifndef SE2P_PATCH_NODES
#define SE2P_PATCH_NODES 48
#endif
constexpr double kPatchNodes = SE2P_PATCH_NODES;   // side of a gather patch, in grid nodes

enum Slot {
    S_IN_PS, S_IN_PT, S_IN_F, S_IN_FD, S_IN_N,   // staged inputs
    S_WPS, S_WPT,                               // wrapped positions
    S_SBOX, S_SRANK, S_TBOX, S_TRANK, S_COUNT,  // binning scratch
    S_SSTART, S_TSTART, S_SPERM, S_TPERM, S_TBOXS,
    S_SP, S_TP, S_SPF, S_TPF, S_COEF,           // sorted data
    S_UR_SLP, S_UR_DLP, S_UK,                   // partial results (sorted order)
    S_GRID, S_SPEC, S_E1, S_ZPART, S_ZM, S_COUNTERS,
    S_OUT0, S_OUT1, S_OUT2, S_OUT3,             // staged outputs
    S_IN_W1, S_IN_W2, S_WCOEF, S_GR, S_GK, S_SBOXS, S_ZEROS,   // adjoint
    S_GTAB, S_COEF_FF,                          // float-float real space
    S_ZGRID,                                    // complex pairs of grids (1D-pass FFT)
    S_GCOUNT, S_GTGT, S_GMETA,                  // geometry build scratch
    S_GCOEF, S_GCOEFF, S_GUR0, S_GUR1,          // geometry apply scratch
    S_SBINS, S_GMAX,                            // fixed-point spread bound, gather scale
    S_TWY, S_TWX,                               // float-float FFT twiddles (y, x lengths)
    S_SPL, S_TPL,                               // low halves of sorted positions (FP32 grid)
    S_MTAB,                                     // cached per-mode filter multipliers
    S_PROBE,                                    // the atomic-rate probe's array
    S_MGRID, S_MGMAX, S_MUK, S_MZM,             // k space of several right-hand sides
    S_GORDER, S_GPCNT, S_GPSTART,               // patch-major target order of the gather
    S_COUNT_SLOTS
};

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

}  // namespace

// Stages timed with CUDA events when timing is on (se2p_plan_enable_timing).
enum Stage {
    T_STAGE_IN, T_WRAP, T_SORT, T_COEF, T_REAL, T_SPREAD, T_FFT_FWD, T_FILTER, T_FFT_INV,
    T_GATHER, T_ZERO_MODE, T_ASSEMBLE, T_STAGE_OUT, T_NUM_STAGES
};
static const char *kStageNames[T_NUM_STAGES] = {
    "h2d", "wrap", "sort", "coef", "real", "spread", "fft_fwd", "filter", "fft_inv",
    "gather", "zero_mode", "assemble", "d2h"};

struct se2p_plan_st {
    int device = 0;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;     // real space runs here, concurrently with k space
    cudaStream_t kst = nullptr;      // k space beside real space (highest priority)
    cudaEvent_t fork = nullptr, join = nullptr, kjoin = nullptr;
    cudaEvent_t cin0 = nullptr, cin1 = nullptr;   // densities' host copies on the side stream
    std::string err;
    int64_t launches = 0;
    DevBuf buf[S_COUNT_SLOTS];
    std::map<std::tuple<int, int, int, int>, cufftHandle> ffts;  // (Mx, My, batch, dir)
    int precision = SE2P_PRECISION_FP64;
    bool overlap = true;             // real space concurrent with the k-space chain
    bool timing = false;
    bool count_pairs = false;
    double mtab_key[7] = {0, 0, 0, 0, 0, 0, -1};   // (Mx, My, Lx, Ly, xi, eta, layout) of S_MTAB
    bool gtab_ready = false;                   // S_GTAB holds the E1 fit
    // float-float FFT twiddles: the length and device copy each slot holds,
    // and the host tables the (asynchronous) uploads read from
    int tw_len[2] = {0, 0};
    const void *tw_dev[2] = {nullptr, nullptr};
    std::vector<float4> tw_host[2];
    // pending (start, end) event pairs per stage, resolved by se2p_plan_stage_times
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending[T_NUM_STAGES];
    double stage_ms[T_NUM_STAGES] = {0};
    int64_t stage_calls[T_NUM_STAGES] = {0};
};

namespace {

int fail(se2p_plan pl, int code, const char *fmt, ...)
{
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    if (pl) pl->err = msg;
    return code;
}

#define CK(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return fail(pl, SE2P_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));     \
    } while (0)

#define CKF(call)                                                                       \
    do {                                                                                \
        cufftResult r_ = (call);                                                        \
        if (r_ != CUFFT_SUCCESS) return fail(pl, SE2P_ERR_CUFFT, "%s: cufft error %d", #call, (int)r_); \
    } while (0)

#define CKS(call)                       \
    do {                                \
        int s_ = (call);                \
        if (s_ != SE2P_OK) return s_;   \
    } while (0)

// Brackets one stage of one call with events on the plan's stream.
struct StageTimer {
    se2p_plan pl;
    int stage;
    cudaStream_t st;
    cudaEvent_t a = nullptr, b = nullptr;
    StageTimer(se2p_plan p, int stg, cudaStream_t s = nullptr) : pl(p), stage(stg)
    {
        st = s ? s : pl->stream;
        if (!pl->timing) return;
        if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
            cudaGetLastError();
            a = b = nullptr;
            return;
        }
        cudaEventRecord(a, st);
    }
    ~StageTimer()
    {
        if (!a) return;
        cudaEventRecord(b, st);
        pl->pending[stage].emplace_back(a, b);
    }
};

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        // an error left pending by earlier calls of other code is not this
        // call's: the launch checks below read cudaGetLastError (a sticky
        // error persists and is still reported)
        (void)cudaGetLastError();
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

int ensure(se2p_plan pl, int slot, size_t bytes, void **out)
{
    DevBuf &b = pl->buf[slot];
    if (bytes == 0) bytes = 16;
    if (b.bytes < bytes) {
        if (b.p) {
            CK(cudaStreamSynchronize(pl->stream));
            if (pl->side) CK(cudaStreamSynchronize(pl->side));
            if (pl->kst) CK(cudaStreamSynchronize(pl->kst));
            CK(cudaFree(b.p));
            b.p = nullptr;
            b.bytes = 0;
        }
        size_t want = bytes + bytes / 8;  // headroom for slightly larger calls
        cudaError_t e = cudaMalloc(&b.p, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(pl, SE2P_ERR_ALLOC, "cudaMalloc(%zu bytes): %s", want, cudaGetErrorString(e));
        }
        b.bytes = want;
    }
    *out = b.p;
    return SE2P_OK;
}

template <class T>
int ensure_t(se2p_plan pl, int slot, size_t count, T **out)
{
    void *p = nullptr;
    int s = ensure(pl, slot, count * sizeof(T), &p);
    *out = static_cast<T *>(p);
    return s;
}

// Device memory of this plan's device, aligned for 16-byte loads?
bool device_ready(const se2p_plan pl, const void *p)
{
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const bool dev = at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
    return dev && at.device == pl->device && (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

// Input array of `count` double2: use in place when it is usable device
// memory, otherwise copy it into workspace slot `slot`.
int stage_in(se2p_plan pl, int slot, const double *p, int64_t count, const double2 **out,
             bool *host_io, cudaStream_t cs = nullptr)
{
    *out = nullptr;
    if (count <= 0 || !p) return SE2P_OK;
    if (device_ready(pl, p)) {
        *out = reinterpret_cast<const double2 *>(p);
        return SE2P_OK;
    }
    double2 *d = nullptr;
    CKS(ensure_t(pl, slot, (size_t)count, &d));
    CK(cudaMemcpyAsync(d, p, sizeof(double2) * (size_t)count, cudaMemcpyDefault,
                       cs ? cs : pl->stream));
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) == cudaSuccess && at.type != cudaMemoryTypeDevice &&
        at.type != cudaMemoryTypeManaged)
        *host_io = true;
    cudaGetLastError();
    *out = d;
    return SE2P_OK;
}

// Output array: write directly into usable device memory, else into a slot
// that is copied back by finish_out().
struct OutBuf {
    double *user = nullptr;
    double2 *dev = nullptr;
    int64_t count = 0;
    bool staged = false;
};

int stage_out(se2p_plan pl, int slot, double *user, int64_t count, OutBuf *o, bool *host_io)
{
    o->user = user;
    o->count = count;
    o->dev = nullptr;
    o->staged = false;
    if (!user || count <= 0) return SE2P_OK;
    if (device_ready(pl, user)) {
        o->dev = reinterpret_cast<double2 *>(user);
        return SE2P_OK;
    }
    CKS(ensure_t(pl, slot, (size_t)count, &o->dev));
    o->staged = true;
    *host_io = true;
    return SE2P_OK;
}

int finish_out(se2p_plan pl, const OutBuf &o)
{
    if (o.staged && o.count > 0)
        CK(cudaMemcpyAsync(o.user, o.dev, sizeof(double2) * (size_t)o.count, cudaMemcpyDefault,
                           pl->stream));
    return SE2P_OK;
}

// dir: 0 = D2Z, 1 = Z2D, 2 = R2C (FP32), 3 = C2R (FP32) -- 2D, batch grids;
// 4 = Z2Z along y (batch contiguous rows of My); 5 = Z2Z along x of one
// Mx x (My/2+1) half spectrum (stride My/2+1, My/2+1 transforms); 6 = Z2Z
// along x of transposed half spectra (batch contiguous rows of Mx);
// 10 + W = R2C of batch grids interleaved per node with stride W (FP32);
// 20 + W = C2R into grids interleaved with stride W (FP32).
int get_fft(se2p_plan pl, cudaStream_t st, int Mx, int My, int batch, int dir, cufftHandle *h)
{
    auto key = std::make_tuple(Mx, My, batch, dir);
    auto it = pl->ffts.find(key);
    if (it != pl->ffts.end()) {
        *h = it->second;
        CKF(cufftSetStream(*h, st));
        return SE2P_OK;
    }
    int n[2] = {Mx, My};
    const int real_dist = Mx * My, cplx_dist = Mx * (My / 2 + 1);
    cufftHandle p;
    if (dir == 4) {
        int ny = My;
        CKF(cufftPlanMany(&p, 1, &ny, nullptr, 1, My, nullptr, 1, My, CUFFT_Z2Z, batch));
        CKF(cufftSetStream(p, st));
        pl->ffts[key] = p;
        *h = p;
        return SE2P_OK;
    }
    if (dir == 6) {
        int nx = Mx;
        CKF(cufftPlanMany(&p, 1, &nx, nullptr, 1, Mx, nullptr, 1, Mx, CUFFT_Z2Z, batch));
        CKF(cufftSetStream(p, st));
        pl->ffts[key] = p;
        *h = p;
        return SE2P_OK;
    }
    if (dir == 5) {
        int nx = Mx, emb = Mx;
        const int H1 = My / 2 + 1;
        CKF(cufftPlanMany(&p, 1, &nx, &emb, H1, 1, &emb, H1, 1, CUFFT_Z2Z, H1));
        CKF(cufftSetStream(p, st));
        pl->ffts[key] = p;
        *h = p;
        return SE2P_OK;
    }
    if (dir > 10) {
        const int W = dir % 10, H1 = My / 2 + 1;
        int re[2] = {Mx, My}, ce[2] = {Mx, H1};
        if (dir < 20)
            CKF(cufftPlanMany(&p, 2, n, re, W, 1, ce, 1, cplx_dist, CUFFT_R2C, batch));
        else
            CKF(cufftPlanMany(&p, 2, n, ce, 1, cplx_dist, re, W, 1, CUFFT_C2R, batch));
        CKF(cufftSetStream(p, st));
        pl->ffts[key] = p;
        *h = p;
        return SE2P_OK;
    }
    const bool fwd = dir == 0 || dir == 2;
    const cufftType type = dir == 0 ? CUFFT_D2Z : dir == 1 ? CUFFT_Z2D : dir == 2 ? CUFFT_R2C : CUFFT_C2R;
    if (fwd)
        CKF(cufftPlanMany(&p, 2, n, nullptr, 1, real_dist, nullptr, 1, cplx_dist, type, batch));
    else
        CKF(cufftPlanMany(&p, 2, n, nullptr, 1, cplx_dist, nullptr, 1, real_dist, type, batch));
    CKF(cufftSetStream(p, st));
    pl->ffts[key] = p;
    *h = p;
    return SE2P_OK;
}

// The filters' effective per-mode multipliers (k_filter_matrix_table) depend
// only on (Mx, My, Lx, Ly, xi, eta) and the layout; the plan keeps them
// between calls, like cuFFT keeps its twiddles.  k_filter and k_filter_adj
// then do two small complex mat-vecs per mode (about 20 FP64 operations
// instead of 60).
int filter_matrix(se2p_plan pl, FilterArgs &fa, cudaStream_t st)
{
    const double key[7] = {(double)fa.Mx, (double)fa.My, fa.Lx, fa.Ly, fa.xi, fa.eta,
                           (double)fa.transposed};
    const size_t H = (size_t)fa.Mx * (fa.My / 2 + 1);
    const bool have = pl->buf[S_MTAB].p &&
                      pl->buf[S_MTAB].bytes >= H * kFilterMat * sizeof(double) &&
                      memcmp(key, pl->mtab_key, sizeof key) == 0;
    double *tab = nullptr;
    CKS(ensure_t(pl, S_MTAB, H * kFilterMat, &tab));
    if (!have) {
        CK(launch_filter_matrix_table(fa, tab, st, pl->launches));
        memcpy(pl->mtab_key, key, sizeof key);
    }
    fa.mtab = tab;
    return SE2P_OK;
}

// --------------------------------------------------------------------------
// Piecewise fit of g(x) = exp(x) E1(x) in the reference's Pade form
// (PE/src/mex/StokesSLP/mex_stokes_slp_real.cpp:19-47: z + p(z)/(q(z) + x),
// z = 1/x, mid set for 1 < x < 16, far set from 16) for the float-float real
// space.  Each of the 64 pieces per octave on [1, 64) is interpolated at 7
// Chebyshev nodes in long double and stored as a degree-6 polynomial in
// d = x - centre: c0..c3 as float-float, c4..c6 as floats (|c_k d^k| falls
// by ~2^-7 per degree, so FP32 suffices from c4 on).  Built once per process
// and checked against the Pade form at 33 points per piece.
// --------------------------------------------------------------------------
static const double kE1Host[3][22] = SE2P_E1_PADE;

static long double pade_g(long double x)
{
    const double *c = x >= 16 ? kE1Host[0] : kE1Host[1];
    const long double z = 1.0L / x;
    long double pa = c[0], pb = c[1];
    for (int i = 2; i < 22; i += 2) {
        pa = z * pa + c[i];
        pb = z * pb + c[i + 1];
    }
    return z + pa / (pb + x);
}

struct GFit {
    std::vector<float> tab;   // kGPieces x 12 floats
    double worst = 0;         // largest relative deviation of the stored fit
};

static const GFit &gfit()
{
    static GFit F;
    static std::once_flag once;
    std::call_once(once, [] {
        constexpr int n = 7;
        const long double pi = 3.141592653589793238462643383279502884L;
        F.tab.assign((size_t)kGPieces * 12, 0.f);
        for (int oct = 0; oct < kGOctaves; ++oct)
            for (int m = 0; m < kGPiecesPerOctave; ++m) {
                const long double lo = ldexpl(1.0L + m / 64.0L, oct);
                const long double hi = ldexpl(1.0L + (m + 1) / 64.0L, oct);
                const long double c = (lo + hi) / 2, hw = (hi - lo) / 2;
                long double A[n][n + 1];
                for (int i = 0; i < n; ++i) {
                    const long double u = cosl(pi * (i + 0.5L) / n);
                    long double pw = 1;
                    for (int k = 0; k < n; ++k) {
                        A[i][k] = pw;
                        pw *= u;
                    }
                    A[i][n] = pade_g(c + hw * u);
                }
                for (int col = 0; col < n; ++col) {           // elimination, partial pivoting
                    int piv = col;
                    for (int r = col + 1; r < n; ++r)
                        if (fabsl(A[r][col]) > fabsl(A[piv][col])) piv = r;
                    for (int k = 0; k <= n; ++k) std::swap(A[col][k], A[piv][k]);
                    for (int r = 0; r < n; ++r) {
                        if (r == col) continue;
                        const long double f = A[r][col] / A[col][col];
                        for (int k = col; k <= n; ++k) A[r][k] -= f * A[col][k];
                    }
                }
                long double ck[n];
                long double sc = 1;
                for (int k = 0; k < n; ++k) {
                    ck[k] = A[k][n] / A[k][k] / sc;           // coefficient of d^k
                    sc *= hw;
                }
                float *o = F.tab.data() + (size_t)12 * (oct * kGPiecesPerOctave + m);
                long double stored[n];
                for (int k = 0; k < 4; ++k) {
                    const float h = (float)ck[k];
                    const float l = (float)(ck[k] - h);
                    o[2 * k] = h;
                    o[2 * k + 1] = l;
                    stored[k] = (long double)h + l;
                }
                for (int k = 4; k < n; ++k) {
                    o[4 + k] = (float)ck[k];
                    stored[k] = o[4 + k];
                }
                for (int i = 0; i <= 32; ++i) {
                    const long double x = lo + (hi - lo) * i / 32.0L * (i == 32 ? 0.999999L : 1);
                    const long double d = x - c;
                    long double v = stored[n - 1];
                    for (int k = n - 2; k >= 0; --k) v = v * d + stored[k];
                    const long double g = pade_g(x);
                    F.worst = std::max(F.worst, (double)fabsl((v - g) / g));
                }
            }
    });
    return F;
}

// Uploads the fit once per plan; fails if it is not accurate to 1e-14.
int gtab_device(se2p_plan pl, cudaStream_t st, const float4 **out)
{
    const GFit &F = gfit();
    if (!(F.worst < 1e-14))
        return fail(pl, SE2P_ERR_UNSUPPORTED, "E1 fit deviates by %.3g", F.worst);
    float4 *d = nullptr;
    CKS(ensure_t(pl, S_GTAB, (size_t)kGPieces * 3, &d));
    if (!pl->gtab_ready) {
        CK(cudaMemcpyAsync(d, F.tab.data(), F.tab.size() * sizeof(float), cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));   // the host vector is static, but keep the copy ordered
        pl->gtab_ready = true;
    }
    *out = d;
    return SE2P_OK;
}

// --------------------------------------------------------------------------
// Argument checks (the MEX gateways' checks plus this library's limits)
// --------------------------------------------------------------------------
bool finite_pos(double v) { return std::isfinite(v) && v > 0; }

int check_common(se2p_plan pl, const double *psrc, int64_t ns, const double *ptar, int64_t nt,
                 double xi, double Lx, double Ly, const double *u)
{
    if (!pl) return SE2P_ERR_ARG;
    if (ns < 0 || nt < 0) return fail(pl, SE2P_ERR_ARG, "negative point count");
    if (ns > 0x7fffffff || nt > 0x7fffffff)
        return fail(pl, SE2P_ERR_UNSUPPORTED, "more than 2^31-1 points");
    if ((ns > 0 && !psrc) || (nt > 0 && !ptar)) return fail(pl, SE2P_ERR_ARG, "null point array");
    if (nt > 0 && !u) return fail(pl, SE2P_ERR_ARG, "null output array");
    if (!finite_pos(xi)) return fail(pl, SE2P_ERR_ARG, "xi must be positive and finite");
    if (!finite_pos(Lx) || !finite_pos(Ly)) return fail(pl, SE2P_ERR_ARG, "Lx, Ly must be positive");
    return SE2P_OK;
}

int check_real(se2p_plan pl, int nx, int ny)
{
    if (nx < 1 || ny < 1) return fail(pl, SE2P_ERR_ARG, "nside_x, nside_y must be >= 1");
    if ((int64_t)nx * ny > (1 << 26)) return fail(pl, SE2P_ERR_UNSUPPORTED, "more than 2^26 boxes");
    return SE2P_OK;
}

int check_kspace(se2p_plan pl, double eta, int Mx, int My, double w, int P)
{
    if (Mx < 2 || My < 2) return fail(pl, SE2P_ERR_ARG, "Mx, My must be >= 2");
    if ((Mx & 1) || (My & 1))
        return fail(pl, SE2P_ERR_UNSUPPORTED, "odd grid sizes are not supported (Mx=%d My=%d)", Mx, My);
    if ((int64_t)Mx * My > ((int64_t)1 << 30)) return fail(pl, SE2P_ERR_UNSUPPORTED, "grid larger than 2^30 nodes");
    if (P < 0 || (P & 1)) return fail(pl, SE2P_ERR_ARG, "P must be even and >= 0");
    if (P > kMaxP) return fail(pl, SE2P_ERR_UNSUPPORTED, "P > %d is not supported", kMaxP);
    if (!std::isfinite(eta) || eta <= 0) return fail(pl, SE2P_ERR_ARG, "eta must be positive");
    if (!std::isfinite(w)) return fail(pl, SE2P_ERR_ARG, "w must be finite");
    return SE2P_OK;
}

// --------------------------------------------------------------------------
// The evaluation pipeline
// --------------------------------------------------------------------------
struct Job {
    bool slp = false, dlp = false;     // which kernels
    bool real = false, kspace = false; // which parts
    bool wrap = false;                 // wrap points first (driver composites)
    bool zero_mode = false;            // DLP k=0 term
    // the plan's wrapped and sorted copies already hold these points (the
    // k-space runs of one geometry apply after its first): skip wrap and sort
    bool reuse_sort = false;
    double xi = 0, eta = 0, w = 0, Lx = 0, Ly = 0;
    int nx = 1, ny = 1, Mx = 0, My = 0, P = 0;
};

struct Io {
    const double *psrc = nullptr, *ptar = nullptr, *f_slp = nullptr, *f_dlp = nullptr,
                 *nrm = nullptr;
    int64_t ns = 0, nt = 0;
    // outputs: per kind, the total u and optionally the parts
    double *u_slp = nullptr, *ur_slp = nullptr, *uk_slp = nullptr;
    double *u_dlp = nullptr, *ur_dlp = nullptr, *uk_dlp = nullptr;
    int mode_slp = 0, mode_dlp = 1;   // k_assemble modes
};

// Spread with integer accumulation (k_spread_fix) when the source Gaussian's
// x and y factors stay below 2^3: sets kY (2^kY bounds each factor) and kfac
// (the factor of the bin bound).  The factors exceed 1 only when w differs
// from h P/2, by at most exp(2 |a| h (h P/2 - w)); the bound grows by 2^(2 kY),
// so the integer unit coarsens with it (kY = 3, w = 0.7 h P/2: 8e-14 from
// the FP64 spread), and beyond that the FP64 spread runs.
static bool spread_fixed_ok(const SpreadArgs &sa, int &kY, double &kfac, int &mult)
{
    const double wf = std::exp(-2.0 * sa.a * sa.h * std::max(0.0, sa.h * sa.P / 2 - sa.w));
    if (!(wf <= 8.0)) return false;
    kY = 0;
    if (wf > 1.5) {
        int e = 0;
        std::frexp(wf, &e);                             // wf < 2^e
        kY = e;
    }
    mult = ((sa.P + sa.Mx) / sa.Mx) * ((sa.P + sa.My) / sa.My);   // <= 16^2
    kfac = std::ldexp((double)mult, 2 * kY);
    return true;
}

// Bg of the fixed-point gather (k_gather_fix): 64 - log2(SX SY), SX = SY the
// largest sum over a stencil row of the Gaussian factors
// exp(a (p - h (i - P/2))^2), p in [0, h) (times wf >= 1 when w < h P/2).
static int gather_fixed_bits(const SpreadArgs &sa)
{
    double sx = 0.0;
    for (int i = 0; i <= sa.P; i++) {
        const double c = sa.h * (i - sa.P / 2);
        const double d = c < 0 ? -c : (c > sa.h ? c - sa.h : 0.0);
        sx += std::exp(sa.a * d * d);
    }
    sx *= std::exp(-2.0 * sa.a * sa.h * std::max(0.0, sa.h * sa.P / 2 - sa.w));
    int e = 0;
    std::frexp(sx * sx, &e);                         // SX SY < 2^e
    return std::min(62, 64 - e);
}

// Runs the spread of nc components of sa.coef into sa.grid.  With *fixb set
// on return, the grid holds k_spread_fix's integers or (when the bound slot
// *fixb is all ones: crowded sources) the FP64 spread's doubles, and the pack
// of fft_fwd_1d reads which; with *fixb null it holds doubles.
static int spread(se2p_plan pl, SpreadArgs &sa, int nc, bool allow_fixed, cudaStream_t ks,
                  const unsigned long long **fixb)
{
    int kY = 0, mult = 1;
    double kfac = 1.0;
    *fixb = nullptr;
    sa.bound = nullptr;
    if (allow_fixed && spread_fixed_ok(sa, kY, kfac, mult)) {
        double *ws = nullptr;
        CKS(ensure_t(pl, S_SBINS, (size_t)spread_bound_words(sa.Mx, sa.My, sa.P), &ws));
        sa.bound = reinterpret_cast<const unsigned long long *>(
            ws + spread_bound_slot(sa.Mx, sa.My, sa.P));
        CK(launch_spread_bound(sa, nc, kfac, mult, ws, ks, pl->launches));
        CK(launch_spread_fix(sa, nc, kY, ks, pl->launches));
        *fixb = sa.bound;
    }
    CK(launch_spread(sa, nc, ks, pl->launches));
    return SE2P_OK;
}

// Twiddle table of the float-float row FFT of length L in slot S_TWY
// (which = 0) or S_TWX (which = 1), built and uploaded once per length.
static int fft_ff_table(se2p_plan pl, cudaStream_t st, int L, int which, const float4 **tw)
{
    float4 *d = nullptr;
    CKS(ensure_t(pl, which ? S_TWX : S_TWY, (size_t)L, &d));
    if (pl->tw_len[which] != L || pl->tw_dev[which] != d) {
        std::vector<float4> &h = pl->tw_host[which];
        h.resize((size_t)L);
        fft_rows_ff_twiddles(L, h.data());
        CK(cudaMemcpyAsync(d, h.data(), sizeof(float4) * (size_t)L, cudaMemcpyHostToDevice, st));
        pl->tw_len[which] = L;
        pl->tw_dev[which] = d;
    }
    *tw = d;
    return SE2P_OK;
}

// The 1D passes in float-float (se2p_fft_ff.cu) when both lengths factor
// into the supported radices; otherwise, and in the FP64_NATIVE form, cuFFT.
static bool fft_ff_ok(int Mx, int My)
{
    FftRowsFF a, b;
    return fft_rows_ff_plan(Mx, a) && fft_rows_ff_plan(My, b);
}

// One batch of 1D row transforms: cuFFT plan `dir` or the float-float rows.
static int fft_rows(se2p_plan pl, cudaStream_t ks, bool ff, int Mx, int My, int L, int64_t rows,
                    int dir, double2 *data, int sign, const FftRowsFF *io = nullptr)
{
    if (ff) {
        FftRowsFF p;
        if (io) p = *io;                             // fused pack / unpack fields
        fft_rows_ff_plan(L, p);
        p.sign = sign;
        const float4 *tw = nullptr;
        CKS(fft_ff_table(pl, ks, L, L == My ? 0 : 1, &tw));
        CK(launch_fft_rows_ff(data, rows, p, tw, ks, pl->launches));
        return SE2P_OK;
    }
    cufftHandle h;
    CKS(get_fft(pl, ks, Mx, My, (int)rows, dir, &h));
    cufftDoubleComplex *z = reinterpret_cast<cufftDoubleComplex *>(data);
    CKF(cufftExecZ2Z(h, z, z, sign < 0 ? CUFFT_FORWARD : CUFFT_INVERSE));
    return SE2P_OK;
}

// D2Z of nc real grids into transposed half spectra, as 1D complex passes:
// pack pairs, C2C along y, Hermitian split (transposing), C2C along x.
// zg holds ceil(nc/2) complex grids.  With fixb the grids are the
// fixed-point integers of k_spread_fix at the scale that *fixb gives.
static int fft_fwd_1d(se2p_plan pl, cudaStream_t ks, int Mx, int My, const double *grid, int nc,
                      cufftDoubleComplex *zg, cufftDoubleComplex *spec,
                      const unsigned long long *fixb, bool ff)
{
    const int H1 = My / 2 + 1, ncg = (nc + 1) / 2;
    const size_t G = (size_t)Mx * My;
    double2 *zgd = reinterpret_cast<double2 *>(zg);
    // an odd plane count's last plane goes in as half as many rows, its rows x
    // and x + Mx/2 in one complex row (the pair's imaginary half is otherwise
    // zero): 2.5 instead of 3 grids of y transforms for SLP+DLP
    const bool fold = ff && (nc & 1) && Mx % 2 == 0;
    if (ff) {
        // the pack is fused into the float-float y pass
        FftRowsFF io;
        io.Mx = Mx;
        io.G = (int64_t)G;
        io.pack_in = grid;
        io.bound = fixb;
        io.npl_in = nc;
        io.fold = fold ? 1 : 0;
        const int64_t rows = fold ? (int64_t)(nc / 2) * Mx + Mx / 2 : (int64_t)ncg * Mx;
        CKS(fft_rows(pl, ks, ff, Mx, My, My, rows, 4, zgd, -1, &io));
    } else {
        if (fixb)
            CK(launch_pack_fixed_pairs(reinterpret_cast<const long long *>(grid), nc, (int64_t)G,
                                       fixb, zgd, ks, pl->launches));
        else
            CK(launch_pack_real_pairs(grid, nc, (int64_t)G, zgd, ks, pl->launches));
        CKS(fft_rows(pl, ks, ff, Mx, My, My, (int64_t)ncg * Mx, 4, zgd, -1));
    }
    CK(launch_split_half_spectra_t(zgd, nc, Mx, My, reinterpret_cast<double2 *>(spec), ks,
                                   pl->launches, fold));
    CKS(fft_rows(pl, ks, ff, Mx, My, Mx, (int64_t)nc * H1, 6, reinterpret_cast<double2 *>(spec), -1));
    return SE2P_OK;
}

// Z2D of nout transposed half spectra into real grids (the mirror of
// fft_fwd_1d); zg holds ceil(nout/2) complex grids.
static int fft_inv_1d(se2p_plan pl, cudaStream_t ks, int Mx, int My, cufftDoubleComplex *spec,
                      int nout, cufftDoubleComplex *zg, double *grid, bool ff,
                      unsigned long long *gmax = nullptr)
{
    const int H1 = My / 2 + 1, npo = (nout + 1) / 2;
    const size_t G = (size_t)Mx * My;
    double2 *zgd = reinterpret_cast<double2 *>(zg);
    CKS(fft_rows(pl, ks, ff, Mx, My, Mx, (int64_t)nout * H1, 6, reinterpret_cast<double2 *>(spec), 1));
    CK(launch_join_half_spectra_t(reinterpret_cast<double2 *>(spec), nout, Mx, My, zgd, ks,
                                  pl->launches));
    if (ff) {
        // the unpack (and the grid maximum) is fused into the float-float y pass
        FftRowsFF io;
        io.Mx = Mx;
        io.G = (int64_t)G;
        io.unpack_out = grid;
        io.npl_out = nout;
        io.gmax = gmax;
        CKS(fft_rows(pl, ks, ff, Mx, My, My, (int64_t)npo * Mx, 4, zgd, 1, &io));
    } else {
        CKS(fft_rows(pl, ks, ff, Mx, My, My, (int64_t)npo * Mx, 4, zgd, 1));
        CK(launch_unpack_real_pairs(zgd, nout, (int64_t)G, grid, ks, pl->launches, gmax));
    }
    return SE2P_OK;
}

int run(se2p_plan pl, const Job &J, const Io &io)
{
    DeviceGuard guard(pl->device);
    cudaStream_t st = pl->stream;
    bool host_io = false;
    const int64_t ns = io.ns, nt = io.nt;

    const double2 *ps = nullptr, *pt = nullptr, *fs = nullptr, *fd = nullptr, *nr = nullptr;
    StageTimer *t_in = new StageTimer(pl, T_STAGE_IN);
    CKS(stage_in(pl, S_IN_PS, io.psrc, ns, &ps, &host_io));
    CKS(stage_in(pl, S_IN_PT, io.ptar, nt, &pt, &host_io));
    // Host densities and normals are copied on the side stream, beside the
    // wrap and sort that need only the positions; the stream waits for
    // everything queued before (the staging slots' last readers), and the
    // coefficient kernel waits for the copies.
    CK(cudaEventRecord(pl->cin0, st));
    CK(cudaStreamWaitEvent(pl->side, pl->cin0, 0));
    if (J.slp) CKS(stage_in(pl, S_IN_F, io.f_slp, ns, &fs, &host_io, pl->side));
    if (J.dlp) {
        CKS(stage_in(pl, S_IN_FD, io.f_dlp, ns, &fd, &host_io, pl->side));
        CKS(stage_in(pl, S_IN_N, io.nrm, ns, &nr, &host_io, pl->side));
    }
    CK(cudaEventRecord(pl->cin1, pl->side));
    OutBuf o_us, o_urs, o_uks, o_ud, o_urd, o_ukd;
    CKS(stage_out(pl, S_OUT0, io.u_slp, nt, &o_us, &host_io));
    CKS(stage_out(pl, S_OUT1, io.u_dlp, nt, &o_ud, &host_io));
    // Parts are rarely requested; they share two extra slots per kind.
    CKS(stage_out(pl, S_OUT2, io.ur_slp ? io.ur_slp : io.ur_dlp, nt, io.ur_slp ? &o_urs : &o_urd, &host_io));
    CKS(stage_out(pl, S_OUT3, io.uk_slp ? io.uk_slp : io.uk_dlp, nt, io.uk_slp ? &o_uks : &o_ukd, &host_io));
    delete t_in;
    if (io.ur_slp && io.ur_dlp) return fail(pl, SE2P_ERR_ARG, "internal: both part outputs requested");

    if (nt == 0) {
        // The staging copies on the side stream read the caller's inputs:
        // the caller's stream waits for them, and host inputs are waited for.
        CK(cudaStreamWaitEvent(st, pl->cin1, 0));
        if (host_io) CK(cudaStreamSynchronize(pl->side));
        return SE2P_OK;
    }

    // Wrapped positions (driver composites); the raw sources stay for the zero mode.
    const double2 *ws = ps, *wt = pt;
    if (J.wrap && !J.reuse_sort) {
        StageTimer tm(pl, T_WRAP);
        double2 *a = nullptr, *b = nullptr;
        if (ns > 0) {
            CKS(ensure_t(pl, S_WPS, (size_t)ns, &a));
            CK(launch_wrap(ns, ps, J.Lx, J.Ly, a, st, pl->launches));
            ws = a;
        }
        CKS(ensure_t(pl, S_WPT, (size_t)nt, &b));
        CK(launch_wrap(nt, pt, J.Lx, J.Ly, b, st, pl->launches));
        wt = b;
    }

    // Boxes: the real-space cell list when the real part runs, otherwise
    // tiles of about 16 grid cells (locality only).
    int nx = J.nx, ny = J.ny;
    if (!J.real) {
        nx = J.Mx / 16 > 1 ? J.Mx / 16 : 1;
        ny = J.My / 16 > 1 ? J.My / 16 : 1;
    }
    const int nbox = nx * ny;
    int *sbox, *srank, *tbox, *trank, *count, *sstart, *tstart, *sperm, *tperm, *tboxs;
    double2 *sp, *tp;
    const size_t nsz = (size_t)(ns > 0 ? ns : 1), ntz = (size_t)nt;
    CKS(ensure_t(pl, S_SBOX, nsz, &sbox));
    CKS(ensure_t(pl, S_SRANK, nsz, &srank));
    CKS(ensure_t(pl, S_TBOX, ntz, &tbox));
    CKS(ensure_t(pl, S_TRANK, ntz, &trank));
    CKS(ensure_t(pl, S_COUNT, (size_t)nbox, &count));
    CKS(ensure_t(pl, S_SSTART, (size_t)nbox + 1, &sstart));
    CKS(ensure_t(pl, S_TSTART, (size_t)nbox + 1, &tstart));
    CKS(ensure_t(pl, S_SPERM, nsz, &sperm));
    CKS(ensure_t(pl, S_TPERM, ntz, &tperm));
    CKS(ensure_t(pl, S_TBOXS, ntz, &tboxs));
    CKS(ensure_t(pl, S_SP, nsz, &sp));
    CKS(ensure_t(pl, S_TP, ntz, &tp));

    float2 *spf = nullptr, *tpf = nullptr, *spl = nullptr, *tpl = nullptr;
    const bool f32 = pl->precision == SE2P_PRECISION_FP32_GRID;
    if (J.real) {
        CKS(ensure_t(pl, S_SPF, nsz, &spf));
        CKS(ensure_t(pl, S_TPF, ntz, &tpf));
        if (f32) {
            CKS(ensure_t(pl, S_SPL, nsz, &spl));
            CKS(ensure_t(pl, S_TPL, ntz, &tpl));
        }
    }
    if (!J.reuse_sort) {
    StageTimer tm(pl, T_SORT);
    BinArgs bs{ws, ns, J.Lx, J.Ly, nx, ny, sbox, srank, count};
    CK(launch_bin(bs, sstart, nbox, sperm, nullptr, sp, spf, st, pl->launches, spl));
    BinArgs bt{wt, nt, J.Lx, J.Ly, nx, ny, tbox, trank, count};
    CK(launch_bin(bt, tstart, nbox, tperm, tboxs, tp, tpf, st, pl->launches, tpl));
    }

    const int nc = (J.slp ? 2 : 0) + (J.dlp ? 3 : 0);
    const int doff = J.slp ? 2 : 0;
    double *coef = nullptr;
    CKS(ensure_t(pl, S_COEF, (size_t)nc * nsz, &coef));
    CK(cudaStreamWaitEvent(st, pl->cin1, 0));        // the densities are in
    {
        StageTimer tm(pl, T_COEF);
        CK(launch_src_coef(ns, sperm, J.slp ? fs : nullptr, J.dlp ? fd : nullptr, nr, coef, nc, st,
                           pl->launches));
    }

    double2 *ur_slp = nullptr, *ur_dlp = nullptr, *uk = nullptr;
    if (J.real) {
        if (J.slp) CKS(ensure_t(pl, S_UR_SLP, ntz, &ur_slp));
        if (J.dlp) CKS(ensure_t(pl, S_UR_DLP, ntz, &ur_dlp));
        RealArgs ra{};
        ra.sp = sp;
        ra.spf = spf;
        ra.tpf = tpf;
        ra.coef = coef;
        ra.nc = nc;
        ra.doff = doff;
        ra.sstart = sstart;
        ra.tp = tp;
        ra.tbox = tboxs;
        ra.ntar = nt;
        ra.nx = nx;
        ra.ny = ny;
        ra.Lx = J.Lx;
        ra.Ly = J.Ly;
        ra.xi = J.xi;
        ra.xi2 = J.xi * J.xi;
        ra.cut2 = J.Lx * J.Ly / nx / ny;                 // mex_stokes_slp_real.cpp:127
        ra.cut2f = (float)ra.cut2;
        ra.xi2f = (float)(J.xi * J.xi);
        ra.inv_xi2 = 1.0 / (J.xi * J.xi);
        ra.pf = 2.0 * J.xi * J.xi;
        // (len*(per_source - t))/nside with per_source - t = -+nside
        // (mex_stokes_slp_real.cpp:248-249)
        ra.zxm = (J.Lx * (double)(-nx)) / nx;
        ra.zxp = (J.Lx * (double)nx) / nx;
        ra.zym = (J.Ly * (double)(-ny)) / ny;
        ra.zyp = (J.Ly * (double)ny) / ny;
        ra.self_c = -1.288607832450766155 - std::log(J.xi);  // mex_stokes_slp_real.cpp:124
        ra.u_slp = ur_slp;
        ra.u_dlp = ur_dlp;
        ra.counters = nullptr;
        if (pl->count_pairs) {
            if (!pl->buf[S_COUNTERS].p) {
                unsigned long long *c = nullptr;
                CKS(ensure_t(pl, S_COUNTERS, 3, &c));
                CK(cudaMemsetAsync(c, 0, 3 * sizeof(unsigned long long), st));
            }
            ra.counters = static_cast<unsigned long long *>(pl->buf[S_COUNTERS].p);
        }
        const int form = pl->precision == SE2P_PRECISION_FP32_GRID    ? kFormF32
                         : pl->precision == SE2P_PRECISION_FP64_NATIVE ? kFormFP64
                                                                        : kFormFF;
        ra.coef_ff = nullptr;
        ra.ncf = 0;
        ra.doff_ff = 0;
        ra.gtab = nullptr;
        ra.spl = spl;
        ra.tpl = tpl;
        if (form == kFormFF || form == kFormF32) {
            // float-float coefficients (the FP32-grid form reads their high halves)
            const int ncf = (J.slp ? 2 : 0) + (J.dlp ? 5 : 0);
            float2 *cff = nullptr;
            CKS(ensure_t(pl, S_COEF_FF, (size_t)ncf * nsz, &cff));
            if (form == kFormFF) CKS(gtab_device(pl, st, &ra.gtab));
            StageTimer tm(pl, T_COEF);
            CK(launch_src_coef_ff(ns, coef, nc, J.slp, J.dlp, cff, ncf, st, pl->launches));
            ra.coef_ff = cff;
            ra.ncf = ncf;
            ra.doff_ff = J.slp ? 2 : 0;
        }
        // Real space on the side stream, overlapping the k-space chain.
        const bool side = J.kspace && pl->overlap;
        cudaStream_t rs = side ? pl->side : st;
        if (side) {
            CK(cudaEventRecord(pl->fork, st));
            CK(cudaStreamWaitEvent(rs, pl->fork, 0));
        }
        {
            StageTimer tm(pl, T_REAL, rs);
            CK(launch_real(ra, J.slp, J.dlp, rs, pl->launches, form));
        }
        if (side) CK(cudaEventRecord(pl->join, rs));
    }

    // The k-space chain runs on a high-priority plan stream when real space
    // runs beside it, so its (FP64-bound) kernels take SMs first and the real
    // space fills the remaining issue slots.
    cudaStream_t ks = st;
    if (J.real && J.kspace && pl->overlap) {
        ks = pl->kst;
        CK(cudaStreamWaitEvent(ks, pl->fork, 0));
    }
    if (J.kspace && pl->precision == SE2P_PRECISION_FP32_GRID) {
        // FP32-grid form: spread, FFT, filter and gather in FP32 (se2p_kernels_f32.cu)
        const int Mx = J.Mx, My = J.My, P = J.P;
        const size_t G = (size_t)Mx * My, H = (size_t)Mx * (My / 2 + 1);
        const int nout = (J.slp ? 2 : 0) + (J.dlp ? 2 : 0);
        const double h = J.Lx / Mx;
        // grids interleaved per node: the first min(nc, 4) components with
        // stride W (2 for SLP, 4 otherwise), a fifth one plain after them
        const int W = nc == 2 ? 2 : 4, nci = std::min(nc, 4), ncp = nc - nci;
        float *grid = nullptr;
        cufftComplex *spec = nullptr;
        CKS(ensure_t(pl, S_GRID, G * (size_t)std::max(W + ncp, nout), &grid));
        CKS(ensure_t(pl, S_SPEC, H * nc, &spec));
        CKS(ensure_t(pl, S_UK, ntz * (nout / 2), &uk));
        CK(cudaMemsetAsync(grid, 0, sizeof(float) * G * (W + ncp), ks));
        SpreadArgsF sa{sp, coef, ns, grid, Mx, My, P, J.Lx / 2.0, J.Ly / 2.0, h, J.w,
                       -2 * J.xi * J.xi / J.eta};
        {
            StageTimer tm(pl, T_SPREAD, ks);
            CK(launch_spread_f32(sa, nc, sm_count(), ks, pl->launches));
        }
        cufftHandle fwd, fwd1, inv;
        CKS(get_fft(pl, ks, Mx, My, nci, 10 + W, &fwd));
        {
            StageTimer tm(pl, T_FFT_FWD, ks);
            CKF(cufftExecR2C(fwd, grid, spec));
            if (ncp) {
                CKS(get_fft(pl, ks, Mx, My, ncp, 2, &fwd1));
                CKF(cufftExecR2C(fwd1, grid + (size_t)W * G, spec + (size_t)nci * H));
            }
        }
        FilterArgsF fa;
        fa.spec = reinterpret_cast<float2 *>(spec);
        fa.Mx = Mx;
        fa.My = My;
        fa.Lx = J.Lx;
        fa.Ly = J.Ly;
        fa.xi = J.xi;
        fa.eta = J.eta;
        fa.scale = (float)(1.0 / ((double)Mx * (double)My));
        fa.c1 = (float)(0.25 / (J.xi * J.xi));
        fa.c2 = (float)(0.25 * (1 - J.eta) / (J.xi * J.xi));
        fa.dkx = 2.0 * kPi / J.Lx;
        fa.dky = 2.0 * kPi / J.Ly;
        fa.slp_in = J.slp ? 0 : -1;
        fa.dlp_in = J.dlp ? doff : -1;
        fa.slp_out = 0;
        fa.dlp_out = J.slp ? 2 : 0;
        {
            StageTimer tm(pl, T_FILTER, ks);
            CK(launch_filter_f32(fa, ks, pl->launches));
        }
        CKS(get_fft(pl, ks, Mx, My, nout, 20 + nout, &inv));   // gather reads [node][nout]
        {
            StageTimer tm(pl, T_FFT_INV, ks);
            CKF(cufftExecC2R(inv, spec, grid));
        }
        double s = 4 * J.xi * J.xi / J.eta;               // mex_stokes_slp_kspace.cpp:325-328
        s = s * s * h * h / kPi;
        GatherArgsF ga{tp, nt, grid, Mx, My, P, J.Lx / 2.0, J.Ly / 2.0, h, J.w,
                       -2 * J.xi * J.xi / J.eta, s / (4 * kPi), uk};
        StageTimer tm(pl, T_GATHER, ks);
        CK(launch_gather_f32(ga, nout, ks, pl->launches));
    } else if (J.kspace) {
        const int Mx = J.Mx, My = J.My, P = J.P;
        const size_t G = (size_t)Mx * My, H = (size_t)Mx * (My / 2 + 1);
        const int nout = (J.slp ? 2 : 0) + (J.dlp ? 2 : 0);
        const double h = J.Lx / Mx;
        double *grid = nullptr, *e1 = nullptr;
        cufftDoubleComplex *spec = nullptr;
        CKS(ensure_t(pl, S_GRID, G * nc, &grid));
        CKS(ensure_t(pl, S_SPEC, H * nc, &spec));
        CKS(ensure_t(pl, S_E1, (size_t)P + 1, &e1));
        CKS(ensure_t(pl, S_UK, ntz * (nout / 2), &uk));
        // e1[j] = exp(-2 xi^2/eta h^2 j^2) (mex_stokes_slp_kspace.cpp:64-67)
        double e1h[kMaxP + 1];
        const double t = -2 * J.xi * J.xi / J.eta * h * h;
        for (int j = -P / 2; j <= P / 2; j++) e1h[j + P / 2] = std::exp(t * j * j);
        CK(cudaMemcpyAsync(e1, e1h, sizeof(double) * (P + 1), cudaMemcpyHostToDevice, ks));
        CK(cudaMemsetAsync(grid, 0, sizeof(double) * G * nc, ks));

        SpreadArgs sa;
        sa.sp = sp;
        sa.coef = coef;
        sa.ns = ns;
        sa.grid = grid;
        sa.Mx = Mx;
        sa.My = My;
        sa.P = P;
        sa.Lhx = J.Lx / 2.0;
        sa.Lhy = J.Ly / 2.0;
        sa.h = h;
        sa.w = J.w;
        sa.a = -2 * J.xi * J.xi / J.eta;
        sa.e1 = e1;
        const unsigned long long *fixb = nullptr;
        {
            StageTimer tm(pl, T_SPREAD, ks);
            CKS(spread(pl, sa, nc, pl->precision == SE2P_PRECISION_FP64, ks, &fixb));
        }
        const bool ffft = pl->precision == SE2P_PRECISION_FP64 && fft_ff_ok(Mx, My);

        // D2Z as 1D complex passes: pack pairs, C2C along y, split, C2C along x
        const int ncg = (nc + 1) / 2, npo = (nout + 1) / 2;
        cufftDoubleComplex *zg = nullptr;
        CKS(ensure_t(pl, S_ZGRID, G * (size_t)std::max(ncg, npo), &zg));
        // (the half spectra are kept transposed, [c][ky][x], so the x passes
        // are contiguous batched rows like the y passes)
        {
            StageTimer tm(pl, T_FFT_FWD, ks);
            CKS(fft_fwd_1d(pl, ks, Mx, My, grid, nc, zg, spec, fixb, ffft));
        }

        FilterArgs fa;
        fa.spec = spec;
        fa.Mx = Mx;
        fa.My = My;
        fa.Lx = J.Lx;
        fa.Ly = J.Ly;
        fa.xi = J.xi;
        fa.eta = J.eta;
        fa.scale = 1.0 / ((double)Mx * (double)My);
        fa.slp_in = J.slp ? 0 : -1;
        fa.dlp_in = J.dlp ? doff : -1;
        fa.slp_out = 0;
        fa.dlp_out = J.slp ? 2 : 0;
        fa.transposed = 1;
        {
            StageTimer tm(pl, T_FILTER, ks);
            CKS(filter_matrix(pl, fa, ks));
            CK(launch_filter(fa, ks, pl->launches));
        }

        // Z2D as 1D complex passes: C2C along x, Hermitian join, C2C along y, unpack
        // FP64 form: the fixed-point gather, whenever the spread could run
        // fixed-point (the same Gaussian-factor condition)
        unsigned long long *gmax = nullptr;
        int Bg = 0;
        {
            int kY = 0, mult = 1;
            double kfac = 1.0;
            if (pl->precision == SE2P_PRECISION_FP64 && spread_fixed_ok(sa, kY, kfac, mult) &&
                kY == 0) {
                CKS(ensure_t(pl, S_GMAX, kGmaxWords, &gmax));
                CK(cudaMemsetAsync(gmax, 0, sizeof(unsigned long long) * kGmaxWords, ks));
                Bg = gather_fixed_bits(sa);
            }
        }
        {
            StageTimer tm(pl, T_FFT_INV, ks);
            CKS(fft_inv_1d(pl, ks, Mx, My, spec, nout, zg, grid, ffft, gmax));
        }

        GatherArgs ga;
        ga.tp = tp;
        ga.nt = nt;
        ga.grid = grid;
        ga.Mx = Mx;
        ga.My = My;
        ga.P = P;
        ga.Lhx = J.Lx / 2.0;
        ga.Lhy = J.Ly / 2.0;
        ga.h = h;
        ga.w = J.w;
        ga.a = -2 * J.xi * J.xi / J.eta;
        double s = 4 * J.xi * J.xi / J.eta;               // mex_stokes_slp_kspace.cpp:325-328
        s = s * s * h * h / kPi;
        ga.scale = s / (4 * kPi);
        ga.e1 = e1;
        ga.out = uk;
        ga.gmax = gmax;
        ga.Bg = Bg;
        StageTimer tm(pl, T_GATHER, ks);
        if (gmax) {
            CK(launch_grid_to_fixed(grid, nout, (int64_t)G, gmax, Bg, ks, pl->launches));
            // the box-sorted targets visited patch by patch (about kPatchNodes
            // grid nodes a side), so that a block's targets in flight share
            // their grid lines in L1
            const int pw = std::max(1, (int)std::lround(kPatchNodes * nx / (double)Mx));
            const int ph = std::max(1, (int)std::lround(kPatchNodes * ny / (double)My));
            int *order = nullptr, *pcnt = nullptr, *pst = nullptr;
            CKS(ensure_t(pl, S_GORDER, ntz, &order));
            CKS(ensure_t(pl, S_GPCNT, (size_t)nbox, &pcnt));
            CKS(ensure_t(pl, S_GPSTART, (size_t)nbox + 1, &pst));
            CK(launch_patch_order(tstart, tboxs, nt, nx, ny, pw, ph, pcnt, pst, order, ks,
                                  pl->launches));
            ga.order = order;
        }
        CK(launch_gather(ga, nout, ks, pl->launches));
    }

    if (ks != st) {
        CK(cudaEventRecord(pl->kjoin, ks));
        CK(cudaStreamWaitEvent(st, pl->kjoin, 0));
    }

    double2 *zm = nullptr;
    if (J.zero_mode && J.dlp) {
        double2 *part = nullptr;
        CKS(ensure_t(pl, S_ZPART, (size_t)kZeroModeParts, &part));
        CKS(ensure_t(pl, S_ZM, 1, &zm));
        // sum over the caller's (unwrapped) sources
        StageTimer tm(pl, T_ZERO_MODE);
        CK(launch_zero_mode(ns, ps, fd, nr, 1.0 / (J.Lx * J.Ly), part, zm, st, pl->launches));
    }

    if (J.real && J.kspace && pl->overlap) CK(cudaStreamWaitEvent(st, pl->join, 0));
    StageTimer *t_asm = new StageTimer(pl, T_ASSEMBLE);
    const double2 *uk_slp = (J.kspace && J.slp) ? uk : nullptr;
    const double2 *uk_dlp = (J.kspace && J.dlp) ? uk + (J.slp ? nt : 0) : nullptr;
    if (J.slp && o_us.dev)
        CK(launch_assemble(nt, io.mode_slp, tperm, J.real ? ur_slp : nullptr, uk_slp, nullptr,
                           o_us.dev, o_urs.dev, o_uks.dev, st, pl->launches));
    if (J.dlp && o_ud.dev)
        CK(launch_assemble(nt, io.mode_dlp, tperm, J.real ? ur_dlp : nullptr, uk_dlp, zm,
                           o_ud.dev, o_urd.dev, o_ukd.dev, st, pl->launches));

    delete t_asm;
    StageTimer *t_out = new StageTimer(pl, T_STAGE_OUT);
    CKS(finish_out(pl, o_us));
    CKS(finish_out(pl, o_ud));
    CKS(finish_out(pl, o_urs));
    CKS(finish_out(pl, o_urd));
    CKS(finish_out(pl, o_uks));
    CKS(finish_out(pl, o_ukd));
    delete t_out;
    if (host_io) CK(cudaStreamSynchronize(st));
    else CK(cudaGetLastError());
    return SE2P_OK;
}

// --------------------------------------------------------------------------
// Adjoint: gradients of J = sum_t w_slp(t).u_slp(t) + w_dlp(t).u_dlp(t), with
// u_slp, u_dlp exactly as se2p_stokes_ewald returns them, with respect to the
// (unwrapped) source positions, SLP forces, DLP densities and normals.
// --------------------------------------------------------------------------
struct AdjIo {
    const double *psrc, *ptar, *f_slp, *f_dlp, *nrm, *w_slp, *w_dlp;
    int64_t ns, nt;
    double *g_pos, *g_fs, *g_fd, *g_n;
};

int run_adjoint(se2p_plan pl, const Job &J, const AdjIo &io)
{
    DeviceGuard guard(pl->device);
    cudaStream_t st = pl->stream;
    bool host_io = false;
    const int64_t ns = io.ns, nt = io.nt;
    const bool slp = J.slp, dlp = J.dlp;
    const double2 *ps, *pt, *fs = nullptr, *fd = nullptr, *nr = nullptr, *w1 = nullptr, *w2 = nullptr;
    CKS(stage_in(pl, S_IN_PS, io.psrc, ns, &ps, &host_io));
    CKS(stage_in(pl, S_IN_PT, io.ptar, nt, &pt, &host_io));
    if (slp) {
        CKS(stage_in(pl, S_IN_F, io.f_slp, ns, &fs, &host_io));
        CKS(stage_in(pl, S_IN_W1, io.w_slp, nt, &w1, &host_io));
    }
    if (dlp) {
        CKS(stage_in(pl, S_IN_FD, io.f_dlp, ns, &fd, &host_io));
        CKS(stage_in(pl, S_IN_N, io.nrm, ns, &nr, &host_io));
        CKS(stage_in(pl, S_IN_W2, io.w_dlp, nt, &w2, &host_io));
    }
    OutBuf o_p, o_fs, o_fd, o_n;
    CKS(stage_out(pl, S_OUT0, io.g_pos, ns, &o_p, &host_io));
    CKS(stage_out(pl, S_OUT1, slp ? io.g_fs : nullptr, ns, &o_fs, &host_io));
    CKS(stage_out(pl, S_OUT2, dlp ? io.g_fd : nullptr, ns, &o_fd, &host_io));
    CKS(stage_out(pl, S_OUT3, dlp ? io.g_n : nullptr, ns, &o_n, &host_io));
    if (ns == 0) return SE2P_OK;

    const size_t nsz = (size_t)ns, ntz = (size_t)(nt > 0 ? nt : 1);
    double2 *ws = nullptr, *wt = nullptr;
    CKS(ensure_t(pl, S_WPS, nsz, &ws));
    CKS(ensure_t(pl, S_WPT, ntz, &wt));
    CK(launch_wrap(ns, ps, J.Lx, J.Ly, ws, st, pl->launches));
    CK(launch_wrap(nt, pt, J.Lx, J.Ly, wt, st, pl->launches));

    const int nx = J.nx, ny = J.ny, nbox = nx * ny;
    int *sbox, *srank, *tbox, *trank, *count, *sstart, *tstart, *sperm, *tperm, *tboxs, *sboxs;
    double2 *sp, *tp;
    float2 *spf, *tpf;
    CKS(ensure_t(pl, S_SBOX, nsz, &sbox));
    CKS(ensure_t(pl, S_SRANK, nsz, &srank));
    CKS(ensure_t(pl, S_TBOX, ntz, &tbox));
    CKS(ensure_t(pl, S_TRANK, ntz, &trank));
    CKS(ensure_t(pl, S_COUNT, (size_t)nbox, &count));
    CKS(ensure_t(pl, S_SSTART, (size_t)nbox + 1, &sstart));
    CKS(ensure_t(pl, S_TSTART, (size_t)nbox + 1, &tstart));
    CKS(ensure_t(pl, S_SPERM, nsz, &sperm));
    CKS(ensure_t(pl, S_TPERM, ntz, &tperm));
    CKS(ensure_t(pl, S_TBOXS, ntz, &tboxs));
    CKS(ensure_t(pl, S_SBOXS, nsz, &sboxs));
    CKS(ensure_t(pl, S_SP, nsz, &sp));
    CKS(ensure_t(pl, S_TP, ntz, &tp));
    CKS(ensure_t(pl, S_SPF, nsz, &spf));
    CKS(ensure_t(pl, S_TPF, ntz, &tpf));
    {
        StageTimer tm(pl, T_SORT);
        BinArgs bs{ws, ns, J.Lx, J.Ly, nx, ny, sbox, srank, count};
        CK(launch_bin(bs, sstart, nbox, sperm, sboxs, sp, spf, st, pl->launches));
        BinArgs bt{wt, nt, J.Lx, J.Ly, nx, ny, tbox, trank, count};
        CK(launch_bin(bt, tstart, nbox, tperm, tboxs, tp, tpf, st, pl->launches));
    }
    // 5 coefficients per sorted source (absent kinds as zeros) and the
    // targets' weights (w_slp, w_dlp) in sorted order.
    double *coef = nullptr, *wcoef = nullptr;
    double2 *zeros = nullptr;
    CKS(ensure_t(pl, S_COEF, 5 * nsz, &coef));
    CKS(ensure_t(pl, S_WCOEF, 4 * ntz, &wcoef));
    CKS(ensure_t(pl, S_ZEROS, nsz, &zeros));
    CK(cudaMemsetAsync(zeros, 0, sizeof(double2) * nsz, st));
    {
        StageTimer tm(pl, T_COEF);
        CK(launch_src_coef(ns, sperm, slp ? fs : zeros, dlp ? fd : zeros, dlp ? nr : zeros, coef, 5,
                           st, pl->launches));
        CK(launch_sorted_pair(nt, tperm, w1, w2, wcoef, st, pl->launches));
    }
    double *gr = nullptr, *gk = nullptr;
    CKS(ensure_t(pl, S_GR, 7 * nsz, &gr));
    CKS(ensure_t(pl, S_GK, 7 * nsz, &gk));

    // real space (side stream) ...
    RealArgs ra{};
    ra.sp = sp;
    ra.spf = spf;
    ra.coef = coef;
    ra.nc = 5;
    ra.doff = 2;
    ra.sstart = tstart;            // candidate (inner) cell list: the targets
    ra.tp = tp;
    ra.tpf = tpf;
    ra.tbox = tboxs;
    ra.ntar = nt;
    ra.nx = nx;
    ra.ny = ny;
    ra.Lx = J.Lx;
    ra.Ly = J.Ly;
    ra.xi = J.xi;
    ra.xi2 = J.xi * J.xi;
    ra.cut2 = J.Lx * J.Ly / nx / ny;
    ra.cut2f = (float)ra.cut2;
    ra.xi2f = (float)(J.xi * J.xi);
    ra.inv_xi2 = 1.0 / (J.xi * J.xi);
    ra.pf = 2.0 * J.xi * J.xi;
    ra.zxm = (J.Lx * (double)(-nx)) / nx;
    ra.zxp = (J.Lx * (double)nx) / nx;
    ra.zym = (J.Ly * (double)(-ny)) / ny;
    ra.zyp = (J.Ly * (double)ny) / ny;
    ra.self_c = -1.288607832450766155 - std::log(J.xi);
    ra.nouter = ns;
    ra.obox = sboxs;
    ra.wcoef = wcoef;
    ra.gout = gr;
    const bool side = pl->overlap;
    cudaStream_t rs = side ? pl->side : st;
    if (side) {
        CK(cudaEventRecord(pl->fork, st));
        CK(cudaStreamWaitEvent(rs, pl->fork, 0));
    }
    const int form = pl->precision == SE2P_PRECISION_FP64_NATIVE ? kFormFP64 : kFormFF;
    ra.gtab = nullptr;
    if (form == kFormFF) CKS(gtab_device(pl, st, &ra.gtab));
    {
        StageTimer tm(pl, T_REAL, rs);
        CK(launch_real_adj(ra, slp, dlp, rs, pl->launches, form));
    }
    if (side) CK(cudaEventRecord(pl->join, rs));

    // k space on the high-priority plan stream beside the real space
    cudaStream_t ks = st;
    if (side) {
        ks = pl->kst;
        CK(cudaStreamWaitEvent(ks, pl->fork, 0));
    }
    // ... k space: spread w at the targets, D2Z, adjoint filter, Z2D, gather
    // with weight gradients at the sources.
    const int Mx = J.Mx, My = J.My, P = J.P;
    const size_t G = (size_t)Mx * My, H = (size_t)Mx * (My / 2 + 1);
    const double h = J.Lx / Mx;
    double *grid = nullptr, *e1 = nullptr;
    cufftDoubleComplex *spec = nullptr;
    CKS(ensure_t(pl, S_GRID, G * 5, &grid));
    CKS(ensure_t(pl, S_SPEC, H * 5, &spec));
    CKS(ensure_t(pl, S_E1, (size_t)P + 1, &e1));
    double e1h[kMaxP + 1];
    const double t = -2 * J.xi * J.xi / J.eta * h * h;
    for (int j = -P / 2; j <= P / 2; j++) e1h[j + P / 2] = std::exp(t * j * j);
    CK(cudaMemcpyAsync(e1, e1h, sizeof(double) * (P + 1), cudaMemcpyHostToDevice, ks));
    CK(cudaMemsetAsync(grid, 0, sizeof(double) * G * 4, ks));
    SpreadArgs sa;
    sa.sp = tp;
    sa.coef = wcoef;
    sa.ns = nt;
    sa.grid = grid;
    sa.Mx = Mx;
    sa.My = My;
    sa.P = P;
    sa.Lhx = J.Lx / 2.0;
    sa.Lhy = J.Ly / 2.0;
    sa.h = h;
    sa.w = J.w;
    sa.a = -2 * J.xi * J.xi / J.eta;
    sa.e1 = e1;
    const unsigned long long *fixb = nullptr;
    {
        StageTimer tm(pl, T_SPREAD, ks);
        CKS(spread(pl, sa, 4, form == kFormFF, ks, &fixb));
    }
    const bool ffft = form == kFormFF && fft_ff_ok(Mx, My);
    cufftDoubleComplex *zg = nullptr;
    CKS(ensure_t(pl, S_ZGRID, G * 3, &zg));
    {
        StageTimer tm(pl, T_FFT_FWD, ks);
        CKS(fft_fwd_1d(pl, ks, Mx, My, grid, 4, zg, spec, fixb, ffft));
    }
    FilterArgs fa;
    fa.spec = spec;
    fa.Mx = Mx;
    fa.My = My;
    fa.Lx = J.Lx;
    fa.Ly = J.Ly;
    fa.xi = J.xi;
    fa.eta = J.eta;
    fa.scale = 1.0 / ((double)Mx * (double)My);
    fa.slp_in = 0;
    fa.slp_out = 0;
    fa.dlp_in = 2;
    fa.dlp_out = 2;
    fa.transposed = 1;
    {
        StageTimer tm(pl, T_FILTER, ks);
        CKS(filter_matrix(pl, fa, ks));
        CK(launch_filter_adj(fa, ks, pl->launches));
    }
    // float-float gather (FP64 form) when float's range holds the weights;
    // it needs the grid maximum from the unpack and reuses zg for its planes
    unsigned long long *gmax = nullptr;
    const double a_gauss = -2 * J.xi * J.xi / J.eta;
    const bool ffg = form == kFormFF && adj_gather_ff_ok(a_gauss, h, J.w, P);
    if (ffg) {
        CKS(ensure_t(pl, S_GMAX, kGmaxWords, &gmax));
        CK(cudaMemsetAsync(gmax, 0, sizeof(unsigned long long) * kGmaxWords, ks));
    }
    {
        StageTimer tm(pl, T_FFT_INV, ks);
        CKS(fft_inv_1d(pl, ks, Mx, My, spec, 5, zg, grid, ffft, gmax));
    }
    GatherAdjArgs ga;
    ga.sp = sp;
    ga.ns = ns;
    ga.coef = coef;
    ga.grid = grid;
    ga.Mx = Mx;
    ga.My = My;
    ga.P = P;
    ga.Lhx = J.Lx / 2.0;
    ga.Lhy = J.Ly / 2.0;
    ga.h = h;
    ga.w = J.w;
    ga.a = -2 * J.xi * J.xi / J.eta;
    double sg = 4 * J.xi * J.xi / J.eta;
    sg = sg * sg * h * h / kPi;
    ga.scale = sg / (4 * kPi);
    ga.e1 = e1;
    ga.out = gk;
    if (ffg) {
        ga.gmax = gmax;
        ga.gff = reinterpret_cast<float2 *>(zg);     // 5 G float2 within its 3 G double2
    }
    {
        StageTimer tm(pl, T_GATHER, ks);
        CK(launch_gather_adj(ga, ks, pl->launches));
    }
    if (ks != st) {
        CK(cudaEventRecord(pl->kjoin, ks));
        CK(cudaStreamWaitEvent(st, pl->kjoin, 0));
    }
    if (side) CK(cudaStreamWaitEvent(st, pl->join, 0));

    double2 *part = nullptr;
    CKS(ensure_t(pl, S_ZPART, (size_t)kZeroModeParts + 1, &part));
    {
        StageTimer tm(pl, T_ASSEMBLE);
        CK(launch_adj_assemble(ns, sperm, gr, gk, wcoef, nt, part, ps, dlp ? fd : zeros,
                               dlp ? nr : zeros, 1.0 / (J.Lx * J.Ly), slp, dlp, o_p.dev,
                               o_fs.dev, o_fd.dev, o_n.dev, st, pl->launches));
    }
    CKS(finish_out(pl, o_p));
    CKS(finish_out(pl, o_fs));
    CKS(finish_out(pl, o_fd));
    CKS(finish_out(pl, o_n));
    if (host_io) CK(cudaStreamSynchronize(st));
    else CK(cudaGetLastError());
    return SE2P_OK;
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

const char *se2p_version(void) { return "se2p 0.1 (sm_103a)"; }

int se2p_plan_create(se2p_plan *plan, int device)
{
    if (!plan) return SE2P_ERR_ARG;
    *plan = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return SE2P_ERR_CUDA;
    }
    se2p_plan pl = new se2p_plan_st;
    pl->device = device;
    DeviceGuard guard(device);
    if (cudaStreamCreateWithFlags(&pl->own, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete pl;
        return SE2P_ERR_CUDA;
    }
    pl->stream = pl->own;
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (cudaStreamCreateWithFlags(&pl->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithPriority(&pl->kst, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaEventCreateWithFlags(&pl->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&pl->join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&pl->kjoin, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&pl->cin0, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&pl->cin1, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        se2p_plan_destroy(pl);
        return SE2P_ERR_CUDA;
    }
    *plan = pl;
    return SE2P_OK;
}

int se2p_plan_destroy(se2p_plan pl)
{
    if (!pl) return SE2P_OK;
    DeviceGuard guard(pl->device);
    cudaStreamSynchronize(pl->stream);
    if (pl->side) cudaStreamSynchronize(pl->side);
    if (pl->kst) cudaStreamSynchronize(pl->kst);
    for (auto &v : pl->pending)
        for (auto &ev : v) {
            cudaEventDestroy(ev.first);
            cudaEventDestroy(ev.second);
        }
    for (auto &kv : pl->ffts) cufftDestroy(kv.second);
    for (auto &b : pl->buf)
        if (b.p) cudaFree(b.p);
    if (pl->side) {
        cudaStreamSynchronize(pl->side);
        cudaStreamDestroy(pl->side);
    }
    if (pl->kst) {
        cudaStreamSynchronize(pl->kst);
        cudaStreamDestroy(pl->kst);
    }
    if (pl->fork) cudaEventDestroy(pl->fork);
    if (pl->join) cudaEventDestroy(pl->join);
    if (pl->kjoin) cudaEventDestroy(pl->kjoin);
    if (pl->cin0) cudaEventDestroy(pl->cin0);
    if (pl->cin1) cudaEventDestroy(pl->cin1);
    if (pl->own) cudaStreamDestroy(pl->own);
    delete pl;
    return SE2P_OK;
}

int se2p_plan_set_stream(se2p_plan pl, void *s)
{
    if (!pl) return SE2P_ERR_ARG;
    pl->stream = static_cast<cudaStream_t>(s);   // NULL = the legacy default stream
    return SE2P_OK;
}

const char *se2p_plan_last_error(se2p_plan pl) { return pl ? pl->err.c_str() : "null plan"; }

int64_t se2p_plan_workspace_bytes(se2p_plan pl)
{
    if (!pl) return 0;
    int64_t s = 0;
    for (auto &b : pl->buf) s += (int64_t)b.bytes;
    return s;
}

int64_t se2p_plan_kernel_launches(se2p_plan pl) { return pl ? pl->launches : 0; }

int se2p_plan_enable_timing(se2p_plan pl, int on)
{
    if (!pl) return SE2P_ERR_ARG;
    pl->timing = on != 0;
    return SE2P_OK;
}

int se2p_num_stages(void) { return T_NUM_STAGES; }

int se2p_plan_set_overlap(se2p_plan pl, int on)
{
    if (!pl) return SE2P_ERR_ARG;
    pl->overlap = on != 0;
    return SE2P_OK;
}

int se2p_plan_set_precision(se2p_plan pl, int precision)
{
    if (!pl) return SE2P_ERR_ARG;
    if (precision != SE2P_PRECISION_FP64 && precision != SE2P_PRECISION_FP32_GRID &&
        precision != SE2P_PRECISION_FP64_NATIVE)
        return fail(pl, SE2P_ERR_ARG, "unknown precision %d", precision);
    pl->precision = precision;
    return SE2P_OK;
}

int se2p_plan_count_pairs(se2p_plan pl, int on, int64_t *counts, int reset)
{
    if (!pl) return SE2P_ERR_ARG;
    DeviceGuard guard(pl->device);
    unsigned long long h[3] = {0, 0, 0};
    void *c = pl->buf[S_COUNTERS].p;
    if (c) {
        CK(cudaStreamSynchronize(pl->stream));
        CK(cudaMemcpy(h, c, sizeof h, cudaMemcpyDeviceToHost));
        if (reset) CK(cudaMemset(c, 0, sizeof h));
    }
    if (counts)
        for (int i = 0; i < 3; i++) counts[i] = (int64_t)h[i];
    pl->count_pairs = on != 0;
    return SE2P_OK;
}

const char *se2p_stage_name(int i) { return (i >= 0 && i < T_NUM_STAGES) ? kStageNames[i] : ""; }

int se2p_plan_probe_atomics(se2p_plan pl, double *gops)
{
    if (!pl || !gops) return SE2P_ERR_ARG;
    DeviceGuard guard(pl->device);
    cudaStream_t st = pl->stream;
    const int64_t n = (int64_t)1 << 22;              // 32 MB
    unsigned long long *a = nullptr;
    CKS(ensure_t(pl, S_PROBE, (size_t)n, &a));
    CK(cudaMemsetAsync(a, 0, sizeof(unsigned long long) * (size_t)n, st));
    int64_t count = 0;
    CK(launch_probe_red64(a, n, 64, &count, st));    // warm-up
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    cudaError_t err = cudaSuccess;
    for (int r = 0; r < 5 && err == cudaSuccess; r++) {
        err = cudaEventRecord(e0, st);
        if (err == cudaSuccess) err = launch_probe_red64(a, n, 1024, &count, st);
        if (err == cudaSuccess) err = cudaEventRecord(e1, st);
        if (err == cudaSuccess) err = cudaEventSynchronize(e1);
        float t = 0.f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
        if (err == cudaSuccess && t > 0.f) best = std::min(best, t);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CK(err);
    *gops = (double)count / (best * 1e-3) / 1e9;
    return SE2P_OK;
}

int se2p_plan_stage_times(se2p_plan pl, double *ms, int64_t *calls, int reset)
{
    if (!pl) return SE2P_ERR_ARG;
    DeviceGuard guard(pl->device);
    for (int i = 0; i < T_NUM_STAGES; i++) {
        for (auto &ev : pl->pending[i]) {
            float t = 0.f;
            if (cudaEventSynchronize(ev.second) == cudaSuccess &&
                cudaEventElapsedTime(&t, ev.first, ev.second) == cudaSuccess) {
                pl->stage_ms[i] += t;
                pl->stage_calls[i]++;
            } else {
                cudaGetLastError();
            }
            cudaEventDestroy(ev.first);
            cudaEventDestroy(ev.second);
        }
        pl->pending[i].clear();
        if (ms) ms[i] = pl->stage_ms[i];
        if (calls) calls[i] = pl->stage_calls[i];
        if (reset) {
            pl->stage_ms[i] = 0;
            pl->stage_calls[i] = 0;
        }
    }
    return SE2P_OK;
}

int se2p_slp_real(se2p_plan pl, const double *psrc, int64_t ns, const double *ptar, int64_t nt,
                  const double *f, double xi, int nside_x, int nside_y, double Lx, double Ly,
                  double *u)
{
    CKS(check_common(pl, psrc, ns, ptar, nt, xi, Lx, Ly, u));
    CKS(check_real(pl, nside_x, nside_y));
    if (ns > 0 && !f) return fail(pl, SE2P_ERR_ARG, "null f");
    Job J;
    J.slp = J.real = true;
    J.xi = xi; J.Lx = Lx; J.Ly = Ly; J.nx = nside_x; J.ny = nside_y;
    Io io;
    io.psrc = psrc; io.ptar = ptar; io.f_slp = f; io.ns = ns; io.nt = nt;
    io.u_slp = u; io.mode_slp = 0;
    return run(pl, J, io);
}

int se2p_dlp_real(se2p_plan pl, const double *psrc, int64_t ns, const double *ptar, int64_t nt,
                  const double *f, const double *n, double xi, int nside_x, int nside_y,
                  double Lx, double Ly, double *u)
{
    CKS(check_common(pl, psrc, ns, ptar, nt, xi, Lx, Ly, u));
    CKS(check_real(pl, nside_x, nside_y));
    if (ns > 0 && (!f || !n)) return fail(pl, SE2P_ERR_ARG, "null f or n");
    Job J;
    J.dlp = J.real = true;
    J.xi = xi; J.Lx = Lx; J.Ly = Ly; J.nx = nside_x; J.ny = nside_y;
    Io io;
    io.psrc = psrc; io.ptar = ptar; io.f_dlp = f; io.nrm = n; io.ns = ns; io.nt = nt;
    io.u_dlp = u; io.mode_dlp = 1;
    return run(pl, J, io);
}

int se2p_slp_kspace(se2p_plan pl, const double *psrc, int64_t ns, const double *ptar,
                    int64_t nt, double xi, double eta, const double *f, int Mx, int My,
                    double Lx, double Ly, double w, int P, double *u)
{
    CKS(check_common(pl, psrc, ns, ptar, nt, xi, Lx, Ly, u));
    CKS(check_kspace(pl, eta, Mx, My, w, P));
    if (ns > 0 && !f) return fail(pl, SE2P_ERR_ARG, "null f");
    Job J;
    J.slp = J.kspace = true;
    J.xi = xi; J.eta = eta; J.w = w; J.Lx = Lx; J.Ly = Ly; J.Mx = Mx; J.My = My; J.P = P;
    Io io;
    io.psrc = psrc; io.ptar = ptar; io.f_slp = f; io.ns = ns; io.nt = nt;
    io.u_slp = u; io.mode_slp = 2;
    return run(pl, J, io);
}

int se2p_dlp_kspace(se2p_plan pl, const double *psrc, int64_t ns, const double *ptar,
                    int64_t nt, double xi, double eta, const double *f, const double *n, int Mx,
                    int My, double Lx, double Ly, double w, int P, double *u)
{
    CKS(check_common(pl, psrc, ns, ptar, nt, xi, Lx, Ly, u));
    CKS(check_kspace(pl, eta, Mx, My, w, P));
    if (ns > 0 && (!f || !n)) return fail(pl, SE2P_ERR_ARG, "null f or n");
    Job J;
    J.dlp = J.kspace = true;
    J.xi = xi; J.eta = eta; J.w = w; J.Lx = Lx; J.Ly = Ly; J.Mx = Mx; J.My = My; J.P = P;
    Io io;
    io.psrc = psrc; io.ptar = ptar; io.f_dlp = f; io.nrm = n; io.ns = ns; io.nt = nt;
    io.u_dlp = u; io.mode_dlp = 2;
    return run(pl, J, io);
}

static int check_params(se2p_plan pl, const se2p_params *p)
{
    if (!p) return fail(pl, SE2P_ERR_ARG, "null params");
    CKS(check_real(pl, p->nside_x, p->nside_y));
    CKS(check_kspace(pl, p->eta, p->Mx, p->My, p->w, p->P));
    return SE2P_OK;
}

static void job_from_params(Job &J, const se2p_params *p)
{
    J.real = J.kspace = J.wrap = true;
    J.xi = p->xi; J.eta = p->eta; J.w = p->w; J.Lx = p->Lx; J.Ly = p->Ly;
    J.nx = p->nside_x; J.ny = p->nside_y; J.Mx = p->Mx; J.My = p->My; J.P = p->P;
}

int se2p_slp_ewald(se2p_plan pl, const se2p_params *prm, const double *psrc, int64_t ns,
                   const double *ptar, int64_t nt, const double *f, double *u, double *ur,
                   double *uk)
{
    if (!pl) return SE2P_ERR_ARG;
    CKS(check_params(pl, prm));
    CKS(check_common(pl, psrc, ns, ptar, nt, prm->xi, prm->Lx, prm->Ly, u));
    if (ns > 0 && !f) return fail(pl, SE2P_ERR_ARG, "null f");
    Job J;
    job_from_params(J, prm);
    J.slp = true;
    Io io;
    io.psrc = psrc; io.ptar = ptar; io.f_slp = f; io.ns = ns; io.nt = nt;
    io.u_slp = u; io.ur_slp = ur; io.uk_slp = uk; io.mode_slp = 3;
    return run(pl, J, io);
}

int se2p_dlp_ewald(se2p_plan pl, const se2p_params *prm, const double *psrc, int64_t ns,
                   const double *ptar, int64_t nt, const double *f, const double *n, double *u,
                   double *ur, double *uk)
{
    if (!pl) return SE2P_ERR_ARG;
    CKS(check_params(pl, prm));
    CKS(check_common(pl, psrc, ns, ptar, nt, prm->xi, prm->Lx, prm->Ly, u));
    if (ns > 0 && (!f || !n)) return fail(pl, SE2P_ERR_ARG, "null f or n");
    Job J;
    job_from_params(J, prm);
    J.dlp = true;
    J.zero_mode = true;
    Io io;
    io.psrc = psrc; io.ptar = ptar; io.f_dlp = f; io.nrm = n; io.ns = ns; io.nt = nt;
    io.u_dlp = u; io.ur_dlp = ur; io.uk_dlp = uk; io.mode_dlp = 4;
    return run(pl, J, io);
}

int se2p_stokes_ewald(se2p_plan pl, const se2p_params *prm, const double *psrc, int64_t ns,
                      const double *ptar, int64_t nt, const double *f_slp, const double *f_dlp,
                      const double *n, double *u_slp, double *u_dlp)
{
    if (!pl) return SE2P_ERR_ARG;
    CKS(check_params(pl, prm));
    CKS(check_common(pl, psrc, ns, ptar, nt, prm->xi, prm->Lx, prm->Ly, u_slp));
    if (nt > 0 && !u_dlp) return fail(pl, SE2P_ERR_ARG, "null u_dlp");
    if (ns > 0 && (!f_slp || !f_dlp || !n)) return fail(pl, SE2P_ERR_ARG, "null f or n");
    Job J;
    job_from_params(J, prm);
    J.slp = J.dlp = true;
    J.zero_mode = true;
    Io io;
    io.psrc = psrc; io.ptar = ptar; io.f_slp = f_slp; io.f_dlp = f_dlp; io.nrm = n;
    io.ns = ns; io.nt = nt;
    io.u_slp = u_slp; io.u_dlp = u_dlp; io.mode_slp = 3; io.mode_dlp = 4;
    return run(pl, J, io);
}

// --------------------------------------------------------------------------
// Reusable geometry: sorted points, cell lists and the real-space operator of
// one point set, applied to many right-hand sides (se2p_geom.cu).
// --------------------------------------------------------------------------
struct se2p_geom_st {
    se2p_plan pl = nullptr;
    se2p_params prm{};
    bool slp = false, dlp = false;
    int64_t ns = 0, nt = 0, nnz = 0;
    std::vector<void *> owned;
    size_t bytes = 0;
    double2 *ps = nullptr, *pt = nullptr, *nr = nullptr;   // caller's arrays, original order
    double2 *sp = nullptr, *tp = nullptr;                  // sorted, wrapped
    float2 *spf = nullptr, *tpf = nullptr;
    int *sperm = nullptr, *tperm = nullptr, *tboxs = nullptr, *sstart = nullptr;
    int *rowptr = nullptr, *src = nullptr;
    int *slice = nullptr;                 // slot of each 32-row slice (see launch_geom_rows)
    int64_t nslot = 0;                    // operator slots, padding included
    float2 *cf = nullptr;
    // apply scratch (grown on demand): staged RHS and outputs
    double2 *fin = nullptr, *din = nullptr, *uout = nullptr;
    size_t fin_n = 0, din_n = 0, uout_n = 0;
};

extern "C++" {
template <class T>
int geom_alloc(se2p_geom g, size_t count, T **out)
{
    void *p = nullptr;
    const size_t bytes = (count ? count : 1) * sizeof(T);
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(g->pl, SE2P_ERR_ALLOC, "geometry: cudaMalloc(%zu bytes) failed", bytes);
    }
    g->owned.push_back(p);
    g->bytes += bytes;
    *out = static_cast<T *>(p);
    return SE2P_OK;
}
}  // extern "C++"

static void geom_free(se2p_geom g)
{
    for (void *p : g->owned) cudaFree(p);
    g->owned.clear();
    g->bytes = 0;
}

// Grows one apply buffer (freeing the old one).
static int geom_grow(se2p_geom g, double2 **buf, size_t *have, size_t want)
{
    se2p_plan pl = g->pl;
    if (*have >= want && *buf) return SE2P_OK;
    if (*buf) {
        CK(cudaStreamSynchronize(pl->stream));
        for (auto it = g->owned.begin(); it != g->owned.end(); ++it)
            if (*it == *buf) {
                cudaFree(*it);
                g->owned.erase(it);
                g->bytes -= *have * sizeof(double2);
                break;
            }
        *buf = nullptr;
        *have = 0;
    }
    CKS(geom_alloc(g, want, buf));
    *have = want;
    return SE2P_OK;
}

static int geom_build(se2p_geom g, const double *psrc, const double *ptar, const double *n)
{
    se2p_plan pl = g->pl;
    cudaStream_t st = pl->stream;
    const se2p_params &p = g->prm;
    const int64_t ns = g->ns, nt = g->nt;
    const int nx = p.nside_x, ny = p.nside_y, nbox = nx * ny;
    const size_t nsz = (size_t)(ns > 0 ? ns : 1), ntz = (size_t)(nt > 0 ? nt : 1);
    CKS(geom_alloc(g, nsz, &g->ps));
    CKS(geom_alloc(g, ntz, &g->pt));
    if (ns > 0) CK(cudaMemcpyAsync(g->ps, psrc, 16 * (size_t)ns, cudaMemcpyDefault, st));
    if (nt > 0) CK(cudaMemcpyAsync(g->pt, ptar, 16 * (size_t)nt, cudaMemcpyDefault, st));
    if (g->dlp) {
        CKS(geom_alloc(g, nsz, &g->nr));
        if (ns > 0) CK(cudaMemcpyAsync(g->nr, n, 16 * (size_t)ns, cudaMemcpyDefault, st));
    }
    CKS(geom_alloc(g, nsz, &g->sp));
    CKS(geom_alloc(g, ntz, &g->tp));
    CKS(geom_alloc(g, nsz, &g->spf));
    CKS(geom_alloc(g, ntz, &g->tpf));
    CKS(geom_alloc(g, nsz, &g->sperm));
    CKS(geom_alloc(g, ntz, &g->tperm));
    CKS(geom_alloc(g, ntz, &g->tboxs));
    CKS(geom_alloc(g, (size_t)nbox + 1, &g->sstart));
    CKS(geom_alloc(g, ntz + 1, &g->rowptr));
    CKS(geom_alloc(g, (ntz + 31) / 32 + 1, &g->slice));
    // wrap, then sort into the real-space boxes
    double2 *ws = nullptr, *wt = nullptr;
    int *sbox, *srank, *tbox, *trank, *count, *tstart;
    CKS(ensure_t(pl, S_WPS, nsz, &ws));
    CKS(ensure_t(pl, S_WPT, ntz, &wt));
    CKS(ensure_t(pl, S_SBOX, nsz, &sbox));
    CKS(ensure_t(pl, S_SRANK, nsz, &srank));
    CKS(ensure_t(pl, S_TBOX, ntz, &tbox));
    CKS(ensure_t(pl, S_TRANK, ntz, &trank));
    CKS(ensure_t(pl, S_COUNT, (size_t)nbox, &count));
    CKS(ensure_t(pl, S_TSTART, (size_t)nbox + 1, &tstart));
    if (ns > 0) CK(launch_wrap(ns, g->ps, p.Lx, p.Ly, ws, st, pl->launches));
    if (nt > 0) CK(launch_wrap(nt, g->pt, p.Lx, p.Ly, wt, st, pl->launches));
    BinArgs bs{ws, ns, p.Lx, p.Ly, nx, ny, sbox, srank, count};
    CK(launch_bin(bs, g->sstart, nbox, g->sperm, nullptr, g->sp, g->spf, st, pl->launches));
    BinArgs bt{wt, nt, p.Lx, p.Ly, nx, ny, tbox, trank, count};
    CK(launch_bin(bt, tstart, nbox, g->tperm, g->tboxs, g->tp, g->tpf, st, pl->launches));

    RealArgs ra{};
    ra.sp = g->sp;
    ra.spf = g->spf;
    ra.sstart = g->sstart;
    ra.tp = g->tp;
    ra.tpf = g->tpf;
    ra.tbox = g->tboxs;
    ra.ntar = nt;
    ra.nx = nx;
    ra.ny = ny;
    ra.Lx = p.Lx;
    ra.Ly = p.Ly;
    ra.xi = p.xi;
    ra.xi2 = p.xi * p.xi;
    ra.cut2 = p.Lx * p.Ly / nx / ny;                  // mex_stokes_slp_real.cpp:127
    ra.cut2f = (float)ra.cut2;
    ra.xi2f = (float)(p.xi * p.xi);
    ra.inv_xi2 = 1.0 / (p.xi * p.xi);
    ra.pf = 2.0 * p.xi * p.xi;
    ra.zxm = (p.Lx * (double)(-nx)) / nx;
    ra.zxp = (p.Lx * (double)nx) / nx;
    ra.zym = (p.Ly * (double)(-ny)) / ny;
    ra.zyp = (p.Ly * (double)ny) / ny;
    ra.self_c = -1.288607832450766155 - std::log(p.xi);  // mex_stokes_slp_real.cpp:124
    CKS(gtab_device(pl, st, &ra.gtab));

    int *rowcnt = nullptr;
    CKS(ensure_t(pl, S_GCOUNT, ntz, &rowcnt));
    CK(launch_geom_rows(ra, g->slp, g->dlp, false, rowcnt, nullptr, nullptr, nullptr, nullptr,
                        st, pl->launches));
    if (nt > 0) CK(launch_scan(rowcnt, (int)nt, g->rowptr, st, pl->launches));
    else CK(cudaMemsetAsync(g->rowptr, 0, sizeof(int), st));
    int nnz = 0;
    CK(cudaMemcpyAsync(&nnz, g->rowptr + nt, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (nnz < 0) return fail(pl, SE2P_ERR_UNSUPPORTED, "geometry: more than 2^31-1 pairs");
    g->nnz = nnz;
    // slices of 32 rows, each padded to its longest row
    const int64_t nsl = (nt + 31) / 32;
    int nslot = 0;
    if (nt > 0) {
        CK(launch_geom_slices(g->rowptr, nt, rowcnt, st, pl->launches));
        CK(launch_scan(rowcnt, (int)nsl, g->slice, st, pl->launches));
        CK(cudaMemcpyAsync(&nslot, g->slice + nsl, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    if (nslot < 0) return fail(pl, SE2P_ERR_UNSUPPORTED, "geometry: more than 2^31-1 slots");
    g->nslot = nslot;
    const size_t nz = (size_t)(nslot > 0 ? nslot : 1);
    CKS(geom_alloc(g, nz, &g->src));
    CKS(geom_alloc(g, 7 * nz, &g->cf));
    int *tgt = nullptr;
    unsigned char *meta = nullptr;
    CKS(ensure_t(pl, S_GTGT, nz, &tgt));
    CKS(ensure_t(pl, S_GMETA, nz, &meta));
    CK(cudaMemsetAsync(tgt, 0xff, sizeof(int) * nz, st));   // padding slots: tgt = -1
    CK(launch_geom_rows(ra, g->slp, g->dlp, true, nullptr, g->slice, g->src, tgt, meta, st,
                        pl->launches));
    CK(launch_geom_coef(ra, g->slp, g->dlp, nslot, g->src, tgt, meta, g->cf, st, pl->launches));
    CK(cudaStreamSynchronize(st));
    return SE2P_OK;
}

// Whether the k space of a geometry's right-hand sides can run batched
// (geom_kspace_multi): the FP64 form with the integer spread and gather and
// the float-float FFT.
static bool geom_multi_ok(se2p_geom g, int *kY_out, double *kfac_out, int *mult_out)
{
    se2p_plan pl = g->pl;
    const se2p_params &p = g->prm;
    if (pl->precision != SE2P_PRECISION_FP64 || !fft_ff_ok(p.Mx, p.My)) return false;
    SpreadArgs sa;
    sa.Mx = p.Mx;
    sa.My = p.My;
    sa.P = p.P;
    sa.h = p.Lx / p.Mx;
    sa.w = p.w;
    sa.a = -2 * p.xi * p.xi / p.eta;
    int kY = 0, mult = 1;
    double kfac = 1.0;
    if (!spread_fixed_ok(sa, kY, kfac, mult) || kY != 0) return false;
    *kY_out = kY;
    *kfac_out = kfac;
    *mult_out = mult;
    return true;
}

// The k space of nr right-hand sides on a geometry's sorted points, in the
// FP64 form (geom_multi_ok): coef holds nr blocks of nc coefficients per
// sorted source (stride cstride doubles); uk receives per right-hand side r
// the gathered sums at uk + r (nout / 2) nt, kind after kind, sorted target
// order.  One spread launch covers all nr right-hand sides (each source's
// stencil origin and Gaussian factors formed once), then each one's forward
// transforms, filter and inverse transforms run into its own grids, and one
// gather launch covers them all (each target's factors formed once).  A
// right-hand side whose sources crowd too much for the integer sums, or whose
// values are not finite, takes the FP64 spread or gather as in run().
static int geom_kspace_multi(se2p_geom g, int nr, const double *coef, int64_t cstride,
                             cudaStream_t ks, double2 *uk)
{
    se2p_plan pl = g->pl;
    const se2p_params &p = g->prm;
    const int Mx = p.Mx, My = p.My, P = p.P;
    const size_t G = (size_t)Mx * My;
    const int nc = (g->slp ? 2 : 0) + (g->dlp ? 3 : 0);
    const int nout = (g->slp ? 2 : 0) + (g->dlp ? 2 : 0);
    const double h = p.Lx / Mx;
    int kY = 0, mult = 1;
    double kfac = 1.0;
    if (!geom_multi_ok(g, &kY, &kfac, &mult))
        return fail(pl, SE2P_ERR_UNSUPPORTED, "internal: batched k space");
    double *grid = nullptr, *e1 = nullptr, *ws = nullptr;
    cufftDoubleComplex *spec = nullptr, *zg = nullptr;
    unsigned long long *gmax = nullptr;
    CKS(ensure_t(pl, S_MGRID, G * nc * (size_t)nr, &grid));
    CKS(ensure_t(pl, S_SPEC, (size_t)Mx * (My / 2 + 1) * nc, &spec));
    CKS(ensure_t(pl, S_ZGRID, G * (size_t)((nc + 1) / 2), &zg));
    CKS(ensure_t(pl, S_E1, (size_t)P + 1, &e1));
    CKS(ensure_t(pl, S_MGMAX, (size_t)nr * kGmaxWords, &gmax));
    const int64_t bslot = spread_bound_slot(Mx, My, P);   // the bound slot in each set
    const int64_t bstride = spread_bound_words(Mx, My, P);
    CKS(ensure_t(pl, S_SBINS, (size_t)bstride * nr, &ws));
    // e1[j] = exp(-2 xi^2/eta h^2 j^2) (mex_stokes_slp_kspace.cpp:64-67)
    double e1h[kMaxP + 1];
    const double t = -2 * p.xi * p.xi / p.eta * h * h;
    for (int j = -P / 2; j <= P / 2; j++) e1h[j + P / 2] = std::exp(t * j * j);
    CK(cudaMemcpyAsync(e1, e1h, sizeof(double) * (P + 1), cudaMemcpyHostToDevice, ks));
    CK(cudaMemsetAsync(grid, 0, sizeof(double) * G * nc * nr, ks));
    CK(cudaMemsetAsync(gmax, 0, sizeof(unsigned long long) * kGmaxWords * nr, ks));

    SpreadArgs sa;
    sa.sp = g->sp;
    sa.coef = coef;
    sa.ns = g->ns;
    sa.grid = grid;
    sa.Mx = Mx;
    sa.My = My;
    sa.P = P;
    sa.Lhx = p.Lx / 2.0;
    sa.Lhy = p.Ly / 2.0;
    sa.h = h;
    sa.w = p.w;
    sa.a = -2 * p.xi * p.xi / p.eta;
    sa.e1 = e1;
    auto rhs_spread = [&](int r) {
        SpreadArgs sr = sa;
        sr.coef = coef + r * cstride;
        sr.grid = grid + (size_t)r * nc * G;
        sr.bound = reinterpret_cast<const unsigned long long *>(ws + r * bstride + bslot);
        return sr;
    };
    {
        StageTimer tm(pl, T_SPREAD, ks);
        for (int r = 0; r < nr; r++)
            CK(launch_spread_bound(rhs_spread(r), nc, kfac, mult, ws + r * bstride, ks, pl->launches));
        sa.bound = reinterpret_cast<const unsigned long long *>(ws + bslot);
        CK(launch_spread_fix_multi(sa, nc, kY, nr, cstride, (int64_t)(nc * G), (int)bstride, ks,
                                   pl->launches));
        for (int r = 0; r < nr; r++)                 // (the FP64 spread: returns at once unless crowded)
            CK(launch_spread(rhs_spread(r), nc, ks, pl->launches));
    }
    const int Bg = gather_fixed_bits(sa);
    FilterArgs fa;
    fa.spec = spec;
    fa.Mx = Mx;
    fa.My = My;
    fa.Lx = p.Lx;
    fa.Ly = p.Ly;
    fa.xi = p.xi;
    fa.eta = p.eta;
    fa.scale = 1.0 / ((double)Mx * (double)My);
    fa.slp_in = g->slp ? 0 : -1;
    fa.dlp_in = g->dlp ? (g->slp ? 2 : 0) : -1;
    fa.slp_out = 0;
    fa.dlp_out = g->slp ? 2 : 0;
    fa.transposed = 1;
    for (int r = 0; r < nr; r++) {
        double *gr = grid + (size_t)r * nc * G;
        const auto *fixb = reinterpret_cast<const unsigned long long *>(ws + r * bstride + bslot);
        {
            StageTimer tm(pl, T_FFT_FWD, ks);
            CKS(fft_fwd_1d(pl, ks, Mx, My, gr, nc, zg, spec, fixb, true));
        }
        {
            StageTimer tm(pl, T_FILTER, ks);
            CKS(filter_matrix(pl, fa, ks));
            CK(launch_filter(fa, ks, pl->launches));
        }
        {
            StageTimer tm(pl, T_FFT_INV, ks);
            CKS(fft_inv_1d(pl, ks, Mx, My, spec, nout, zg, gr, true, gmax + r * kGmaxWords));
        }
    }
    GatherArgs ga;
    ga.tp = g->tp;
    ga.nt = g->nt;
    ga.grid = grid;
    ga.Mx = Mx;
    ga.My = My;
    ga.P = P;
    ga.Lhx = p.Lx / 2.0;
    ga.Lhy = p.Ly / 2.0;
    ga.h = h;
    ga.w = p.w;
    ga.a = -2 * p.xi * p.xi / p.eta;
    double sc = 4 * p.xi * p.xi / p.eta;             // mex_stokes_slp_kspace.cpp:325-328
    sc = sc * sc * h * h / kPi;
    ga.scale = sc / (4 * kPi);
    ga.e1 = e1;
    ga.out = uk;
    ga.gmax = gmax;
    ga.Bg = Bg;
    // (in sorted order: the patch-major order of the single gather made this
    // one slower, 4.1 against 3.57 ms for one right-hand side and 18.2 against
    // 14.5 ms for four)
    StageTimer tm(pl, T_GATHER, ks);
    for (int r = 0; r < nr; r++)
        CK(launch_grid_to_fixed(grid + (size_t)r * nc * G, nout, (int64_t)G, gmax + r * kGmaxWords,
                                Bg, ks, pl->launches));
    const int64_t ostride = (int64_t)(nout / 2) * g->nt;
    CK(launch_gather_fix_multi(ga, nout, nr, (int64_t)(nc * G), ostride, ks, pl->launches));
    for (int r = 0; r < nr; r++) {                   // (the FP64 gather: returns at once unless non-finite)
        GatherArgs gr = ga;
        gr.grid = grid + (size_t)r * nc * G;
        gr.gmax = gmax + r * kGmaxWords;
        gr.out = uk + r * ostride;
        CK(launch_gather_fp64_fallback(gr, nout, ks, pl->launches));
    }
    return SE2P_OK;
}

int se2p_geom_create(se2p_plan pl, const se2p_params *prm, const double *psrc, int64_t ns,
                     const double *ptar, int64_t nt, const double *n, int kinds, se2p_geom *geom)
{
    if (!pl || !geom) return SE2P_ERR_ARG;
    *geom = nullptr;
    CKS(check_params(pl, prm));
    CKS(check_common(pl, psrc, ns, ptar, nt, prm->xi, prm->Lx, prm->Ly, ptar));
    if (kinds < 1 || kinds > 3) return fail(pl, SE2P_ERR_ARG, "kinds must be 1 (SLP), 2 (DLP) or 3");
    if ((kinds & 2) && ns > 0 && !n) return fail(pl, SE2P_ERR_ARG, "null n");
    DeviceGuard guard(pl->device);
    se2p_geom g = new se2p_geom_st;
    g->pl = pl;
    g->prm = *prm;
    g->slp = (kinds & 1) != 0;
    g->dlp = (kinds & 2) != 0;
    g->ns = ns;
    g->nt = nt;
    const int rc = geom_build(g, psrc, ptar, n);
    if (rc != SE2P_OK) {
        cudaStreamSynchronize(pl->stream);
        geom_free(g);
        delete g;
        return rc;
    }
    *geom = g;
    return SE2P_OK;
}

int se2p_geom_apply(se2p_geom g, int nrhs, const double *f_slp, const double *f_dlp,
                    double *u_slp, double *u_dlp)
{
    if (!g) return SE2P_ERR_ARG;
    se2p_plan pl = g->pl;
    DeviceGuard guard(pl->device);
    cudaStream_t st = pl->stream;
    const int64_t ns = g->ns, nt = g->nt;
    if (nrhs < 0) return fail(pl, SE2P_ERR_ARG, "negative nrhs");
    if (nrhs == 0 || nt == 0) return SE2P_OK;
    if (g->slp && ((ns > 0 && !f_slp) || !u_slp)) return fail(pl, SE2P_ERR_ARG, "null f_slp / u_slp");
    if (g->dlp && ((ns > 0 && !f_dlp) || !u_dlp)) return fail(pl, SE2P_ERR_ARG, "null f_dlp / u_dlp");
    const size_t nsz = (size_t)(ns > 0 ? ns : 1);
    // RHS in device memory, original order (one copy each, whatever their origin)
    if (g->slp) {
        CKS(geom_grow(g, &g->fin, &g->fin_n, (size_t)nrhs * nsz));
        if (ns > 0)
            CK(cudaMemcpyAsync(g->fin, f_slp, 16 * (size_t)ns * nrhs, cudaMemcpyDefault, st));
    }
    if (g->dlp) {
        CKS(geom_grow(g, &g->din, &g->din_n, (size_t)nrhs * nsz));
        if (ns > 0)
            CK(cudaMemcpyAsync(g->din, f_dlp, 16 * (size_t)ns * nrhs, cudaMemcpyDefault, st));
    }
    const int nk = (g->slp ? 1 : 0) + (g->dlp ? 1 : 0);
    CKS(geom_grow(g, &g->uout, &g->uout_n, (size_t)nk * nrhs * nt));
    double2 *uo_slp = g->uout, *uo_dlp = g->uout + (g->slp ? (size_t)nrhs * nt : 0);

    const int nc = (g->slp ? 2 : 0) + (g->dlp ? 3 : 0);
    // the stored operator reads five float-float coefficients per source and
    // right-hand side (SLP f; DLP S11, S12+S21, S22), stored per source for
    // the batch's right-hand sides together, [source][rhs][5]: one 40 B run
    // per right-hand side in one contiguous block per source
    const int ncf = nc;
    const int doff_ff = g->slp ? 2 : 0;
    constexpr int kBatch = 4;
    double *coef = nullptr;
    float2 *cff = nullptr;
    double2 *ur0 = nullptr, *ur1 = nullptr;
    CKS(ensure_t(pl, S_GCOEF, (size_t)kBatch * nc * nsz, &coef));
    CKS(ensure_t(pl, S_GCOEFF, (size_t)kBatch * ncf * nsz, &cff));
    if (g->slp) CKS(ensure_t(pl, S_GUR0, (size_t)kBatch * nt, &ur0));
    if (g->dlp) CKS(ensure_t(pl, S_GUR1, (size_t)kBatch * nt, &ur1));
    int mkY = 0, mmult = 1;
    double mkfac = 1.0;
    const bool multi = geom_multi_ok(g, &mkY, &mkfac, &mmult);
    for (int r0 = 0; r0 < nrhs && multi; r0 += kBatch) {
        // k space of the batch in one pass (geom_kspace_multi) on the plan's
        // stream, the stored real-space operator beside it on the side stream
        const int nb = std::min(kBatch, nrhs - r0);
        for (int r = 0; r < nb; r++) {
            const double2 *fs = g->slp ? g->fin + (size_t)(r0 + r) * ns : nullptr;
            const double2 *fd = g->dlp ? g->din + (size_t)(r0 + r) * ns : nullptr;
            double *cr = coef + (size_t)r * nc * nsz;
            CK(launch_src_coef(ns, g->sperm, fs, fd, g->nr, cr, nc, st, pl->launches));
            CK(launch_src_coef_ff(ns, cr, nc, g->slp, g->dlp, cff + (size_t)r * ncf, ncf,
                                  st, pl->launches, (int64_t)nb * ncf, false));
        }
        CK(cudaEventRecord(pl->fork, st));
        CK(cudaStreamWaitEvent(pl->side, pl->fork, 0));
        {
            StageTimer tm(pl, T_REAL, pl->side);
            CK(launch_geom_apply(g->slp, g->dlp, nt, g->nslot, g->rowptr, g->slice, g->src, g->cf,
                                 cff, nb * ncf, doff_ff, (int64_t)ncf, coef, nc, doff_ff,
                                 (int64_t)nc * (int64_t)nsz, nb, ur0, ur1, pl->side, pl->launches));
        }
        CK(cudaEventRecord(pl->join, pl->side));
        double2 *uk = nullptr, *zm = nullptr, *part = nullptr;
        const int nk2 = (g->slp ? 1 : 0) + (g->dlp ? 1 : 0);
        CKS(ensure_t(pl, S_MUK, (size_t)kBatch * nk2 * nt, &uk));
        // (on the plan's stream: on the high-priority stream beside the
        // operator product it ran 3 % slower, both being bound by L1 and L2)
        CKS(geom_kspace_multi(g, nb, coef, (int64_t)nc * (int64_t)nsz, st, uk));
        if (g->dlp) {
            CKS(ensure_t(pl, S_ZPART, (size_t)kZeroModeParts, &part));
            CKS(ensure_t(pl, S_MZM, (size_t)kBatch, &zm));
            StageTimer tm(pl, T_ZERO_MODE);
            for (int r = 0; r < nb; r++)             // sum over the caller's (unwrapped) sources
                CK(launch_zero_mode(ns, g->ps, g->din + (size_t)(r0 + r) * ns, g->nr,
                                    1.0 / (g->prm.Lx * g->prm.Ly), part, zm + r, st, pl->launches));
        }
        CK(cudaStreamWaitEvent(st, pl->join, 0));
        StageTimer tm(pl, T_ASSEMBLE);
        for (int r = 0; r < nb; r++) {
            const int rr = r0 + r;
            const double2 *ukr = uk + (size_t)r * nk2 * nt;
            if (g->slp)
                CK(launch_assemble(nt, 3, g->tperm, ur0 + (size_t)r * nt, ukr, nullptr,
                                   uo_slp + (size_t)rr * nt, nullptr, nullptr, st, pl->launches));
            if (g->dlp)
                CK(launch_assemble(nt, 4, g->tperm, ur1 + (size_t)r * nt, ukr + (g->slp ? nt : 0),
                                   zm + r, uo_dlp + (size_t)rr * nt, nullptr, nullptr, st,
                                   pl->launches));
        }
    }
    for (int r0 = 0; r0 < nrhs && !multi; r0 += kBatch) {
        const int nb = std::min(kBatch, nrhs - r0);
        // real space: float-float coefficients of each RHS, then the sparse product
        for (int r = 0; r < nb; r++) {
            const double2 *fs = g->slp ? g->fin + (size_t)(r0 + r) * ns : nullptr;
            const double2 *fd = g->dlp ? g->din + (size_t)(r0 + r) * ns : nullptr;
            double *cr = coef + (size_t)r * nc * nsz;
            CK(launch_src_coef(ns, g->sperm, fs, fd, g->nr, cr, nc, st, pl->launches));
            CK(launch_src_coef_ff(ns, cr, nc, g->slp, g->dlp, cff + (size_t)r * ncf, ncf,
                                  st, pl->launches, (int64_t)nb * ncf, false));
        }
        {
            StageTimer tm(pl, T_REAL);
            CK(launch_geom_apply(g->slp, g->dlp, nt, g->nslot, g->rowptr, g->slice, g->src, g->cf,
                                 cff, nb * ncf, doff_ff, (int64_t)ncf, coef, nc, doff_ff,
                                 (int64_t)nc * (int64_t)nsz, nb, ur0, ur1, st, pl->launches));
        }
        // k space (and the DLP zero mode and sign) per RHS through the drivers'
        // path, then the real-space part added in the caller's order
        for (int r = 0; r < nb; r++) {
            const int rr = r0 + r;
            Job J;
            job_from_params(J, &g->prm);
            J.real = false;
            J.slp = g->slp;
            J.dlp = g->dlp;
            J.zero_mode = g->dlp;
            J.reuse_sort = r0 + r > 0;               // same points as the first RHS's run
            Io io;
            io.psrc = reinterpret_cast<const double *>(g->ps);
            io.ptar = reinterpret_cast<const double *>(g->pt);
            io.f_slp = g->slp ? reinterpret_cast<const double *>(g->fin + (size_t)rr * ns) : nullptr;
            io.f_dlp = g->dlp ? reinterpret_cast<const double *>(g->din + (size_t)rr * ns) : nullptr;
            io.nrm = g->dlp ? reinterpret_cast<const double *>(g->nr) : nullptr;
            io.ns = ns;
            io.nt = nt;
            io.u_slp = g->slp ? reinterpret_cast<double *>(uo_slp + (size_t)rr * nt) : nullptr;
            io.u_dlp = g->dlp ? reinterpret_cast<double *>(uo_dlp + (size_t)rr * nt) : nullptr;
            io.mode_slp = 3;
            io.mode_dlp = 4;
            CKS(run(pl, J, io));
            if (g->slp)
                CK(launch_geom_add(nt, g->tperm, ur0 + (size_t)r * nt, false, uo_slp + (size_t)rr * nt,
                                   st, pl->launches));
            if (g->dlp)
                CK(launch_geom_add(nt, g->tperm, ur1 + (size_t)r * nt, true, uo_dlp + (size_t)rr * nt,
                                   st, pl->launches));
        }
    }
    if (g->slp)
        CK(cudaMemcpyAsync(u_slp, uo_slp, 16 * (size_t)nt * nrhs, cudaMemcpyDefault, st));
    if (g->dlp)
        CK(cudaMemcpyAsync(u_dlp, uo_dlp, 16 * (size_t)nt * nrhs, cudaMemcpyDefault, st));
    CK(cudaStreamSynchronize(st));
    return SE2P_OK;
}

int64_t se2p_geom_bytes(se2p_geom g) { return g ? (int64_t)g->bytes : 0; }

int64_t se2p_geom_pairs(se2p_geom g) { return g ? g->nnz : 0; }

int se2p_geom_destroy(se2p_geom g)
{
    if (!g) return SE2P_OK;
    DeviceGuard guard(g->pl->device);
    cudaStreamSynchronize(g->pl->stream);
    geom_free(g);
    delete g;
    return SE2P_OK;
}

int se2p_stokes_ewald_adjoint(se2p_plan pl, const se2p_params *prm, const double *psrc,
                              int64_t ns, const double *ptar, int64_t nt, const double *f_slp,
                              const double *f_dlp, const double *n, const double *w_slp,
                              const double *w_dlp, double *g_psrc, double *g_fslp,
                              double *g_fdlp, double *g_n)
{
    if (!pl) return SE2P_ERR_ARG;
    CKS(check_params(pl, prm));
    const bool slp = f_slp && w_slp, dlp = f_dlp && n && w_dlp;
    if (!slp && !dlp) return fail(pl, SE2P_ERR_ARG, "neither SLP (f_slp, w_slp) nor DLP (f_dlp, n, w_dlp) given");
    if (ns < 0 || nt < 0) return fail(pl, SE2P_ERR_ARG, "negative point count");
    if (ns > 0x7fffffff || nt > 0x7fffffff) return fail(pl, SE2P_ERR_UNSUPPORTED, "more than 2^31-1 points");
    if ((ns > 0 && !psrc) || (nt > 0 && !ptar)) return fail(pl, SE2P_ERR_ARG, "null point array");
    if (!(std::isfinite(prm->xi) && prm->xi > 0 && prm->Lx > 0 && prm->Ly > 0))
        return fail(pl, SE2P_ERR_ARG, "bad xi / box");
    Job J;
    job_from_params(J, prm);
    J.slp = slp;
    J.dlp = dlp;
    AdjIo io{psrc, ptar, f_slp, f_dlp, n, w_slp, w_dlp, ns, nt, g_psrc, g_fslp, g_fdlp, g_n};
    return run_adjoint(pl, J, io);
}

}  // extern "C"

// ============================================================================
// Allocation-free SLP real space (se2p_slp_real_noalloc)
//
// For callers that cannot call cudaMalloc (MATLAB MEX code whose GPU memory
// belongs to gpuArray's allocator; solver loops that must not allocate).  The
// working arrays of one call are carved from this fixed device array, which
// each GPU that loads the library keeps until exit.  In host code the names
// g_noalloc_scratch and g_noalloc_gtab are only host-side stand-ins: their
// device addresses come from cudaGetSymbolAddress, looked up on every call
// with the caller's device current (a host-side lookup), so that a context
// created anew -- after cudaDeviceReset, or MATLAB's reset(gpuDevice) -- is
// served with its own addresses.
// ============================================================================
static __device__ __align__(256) unsigned char g_noalloc_scratch[SE2P_NOALLOC_SCRATCH_BYTES];
// The E1 fit of the float-float pairs (the table gtab_device gives a plan),
// copied in on every call from the process's host copy.
static __device__ __align__(256) float4 g_noalloc_gtab[kGPieces * 3];

namespace {
size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

// Bytes of scratch one call needs (the carve order of se2p_slp_real_noalloc).
size_t noalloc_bytes(int64_t ns, int64_t nt, int64_t nbox)
{
    const size_t s = (size_t)(ns > 0 ? ns : 1), t = (size_t)nt, b = (size_t)nbox;
    return round256(4 * s) * 3 + round256(4 * t) * 4 + round256(4 * b) + 2 * round256(4 * (b + 1)) +
           round256(16 * s) + round256(16 * t) + round256(8 * s) + round256(8 * t) +
           round256(16 * s) + round256(16 * t) + round256(16 * s);
}

bool on_device(const void *p, int dev)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) &&
           at.device == dev && (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}
}  // namespace

extern "C" int se2p_slp_real_noalloc(const double *psrc, int64_t ns, const double *ptar,
                                     int64_t nt, const double *f, double xi, int nside_x,
                                     int nside_y, double Lx, double Ly, double *u,
                                     void *cuda_stream)
{
    if (ns < 0 || nt < 0 || nside_x < 1 || nside_y < 1) return SE2P_ERR_ARG;
    if (!(std::isfinite(xi) && xi > 0 && std::isfinite(Lx) && Lx > 0 && std::isfinite(Ly) && Ly > 0))
        return SE2P_ERR_ARG;
    if (nt == 0) return SE2P_OK;
    const int64_t nbox = (int64_t)nside_x * nside_y;
    if (ns > 0x7fffffff || nt > 0x7fffffff || nbox > (1 << 26) ||
        noalloc_bytes(ns, nt, nbox) > SE2P_NOALLOC_SCRATCH_BYTES)
        return SE2P_ERR_UNSUPPORTED;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return SE2P_ERR_CUDA;
    }
    if (!ptar || !u || !on_device(ptar, dev) || !on_device(u, dev)) return SE2P_ERR_ARG;
    if (ns > 0 && (!psrc || !f || !on_device(psrc, dev) || !on_device(f, dev))) return SE2P_ERR_ARG;
    const GFit &fit = gfit();
    if (!(fit.worst < 1e-14)) return SE2P_ERR_UNSUPPORTED;

    // Device addresses of the two file-scope arrays in the current context.
    void *sp_base = nullptr, *gt = nullptr;
    if (cudaGetSymbolAddress(&sp_base, g_noalloc_scratch) != cudaSuccess || !sp_base ||
        cudaGetSymbolAddress(&gt, g_noalloc_gtab) != cudaSuccess || !gt) {
        cudaGetLastError();
        return SE2P_ERR_CUDA;
    }
    unsigned char *base = static_cast<unsigned char *>(sp_base);
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    if (cudaMemcpyAsync(gt, fit.tab.data(), fit.tab.size() * sizeof(float), cudaMemcpyHostToDevice,
                        st) != cudaSuccess)
        return SE2P_ERR_CUDA;

    const size_t s1 = (size_t)(ns > 0 ? ns : 1), t1 = (size_t)nt;
    size_t off = 0;
    auto carve = [&](size_t bytes) {
        void *p = base + off;
        off += round256(bytes);
        return p;
    };
    int *sbox = (int *)carve(4 * s1), *srank = (int *)carve(4 * s1), *sperm = (int *)carve(4 * s1);
    int *tbox = (int *)carve(4 * t1), *trank = (int *)carve(4 * t1), *tperm = (int *)carve(4 * t1);
    int *tboxs = (int *)carve(4 * t1);
    int *count = (int *)carve(4 * (size_t)nbox);
    int *sstart = (int *)carve(4 * ((size_t)nbox + 1)), *tstart = (int *)carve(4 * ((size_t)nbox + 1));
    double2 *sp = (double2 *)carve(16 * s1), *tp = (double2 *)carve(16 * t1);
    float2 *spf = (float2 *)carve(8 * s1), *tpf = (float2 *)carve(8 * t1);
    double *coef = (double *)carve(16 * s1);
    double2 *ur = (double2 *)carve(16 * t1);
    float2 *coef_ff = (float2 *)carve(16 * s1);

    int64_t launches = 0;
    const double2 *ps = reinterpret_cast<const double2 *>(psrc);
    const double2 *pt = reinterpret_cast<const double2 *>(ptar);
    BinArgs bs{ps, ns, Lx, Ly, nside_x, nside_y, sbox, srank, count};
    if (launch_bin(bs, sstart, (int)nbox, sperm, nullptr, sp, spf, st, launches) != cudaSuccess)
        return SE2P_ERR_CUDA;
    BinArgs bt{pt, nt, Lx, Ly, nside_x, nside_y, tbox, trank, count};
    if (launch_bin(bt, tstart, (int)nbox, tperm, tboxs, tp, tpf, st, launches) != cudaSuccess)
        return SE2P_ERR_CUDA;
    if (launch_src_coef(ns, sperm, reinterpret_cast<const double2 *>(f), nullptr, nullptr, coef,
                        2, st, launches) != cudaSuccess)
        return SE2P_ERR_CUDA;
    if (launch_src_coef_ff(ns, coef, 2, true, false, coef_ff, 2, st, launches) != cudaSuccess)
        return SE2P_ERR_CUDA;
    // The same real-space arguments and form as se2p_slp_real on a plan of
    // the default precision (SE2P_PRECISION_FP64: far pairs in float-float).
    RealArgs ra{};
    ra.sp = sp;
    ra.spf = spf;
    ra.tpf = tpf;
    ra.coef = coef;
    ra.nc = 2;
    ra.doff = 0;
    ra.sstart = sstart;
    ra.tp = tp;
    ra.tbox = tboxs;
    ra.ntar = nt;
    ra.nx = nside_x;
    ra.ny = nside_y;
    ra.Lx = Lx;
    ra.Ly = Ly;
    ra.xi = xi;
    ra.xi2 = xi * xi;
    ra.cut2 = Lx * Ly / nside_x / nside_y;                 // mex_stokes_slp_real.cpp:127
    ra.cut2f = (float)ra.cut2;
    ra.xi2f = (float)(xi * xi);
    ra.inv_xi2 = 1.0 / (xi * xi);
    ra.pf = 2.0 * xi * xi;
    ra.zxm = (Lx * (double)(-nside_x)) / nside_x;
    ra.zxp = (Lx * (double)nside_x) / nside_x;
    ra.zym = (Ly * (double)(-nside_y)) / nside_y;
    ra.zyp = (Ly * (double)nside_y) / nside_y;
    ra.self_c = -1.288607832450766155 - std::log(xi);   // mex_stokes_slp_real.cpp:124
    ra.u_slp = ur;
    ra.u_dlp = nullptr;
    ra.counters = nullptr;
    ra.coef_ff = coef_ff;
    ra.ncf = 2;
    ra.doff_ff = 0;
    ra.gtab = static_cast<const float4 *>(gt);
    if (launch_real(ra, true, false, st, launches, kFormFF) != cudaSuccess) return SE2P_ERR_CUDA;
    if (launch_assemble(nt, 0, tperm, ur, nullptr, nullptr, reinterpret_cast<double2 *>(u), nullptr,
                        nullptr, st, launches) != cudaSuccess)
        return SE2P_ERR_CUDA;
    return SE2P_OK;
}
