// se2p_internal.cuh -- device helpers and kernel argument blocks shared by the
// spectral-Ewald kernels (se2p_kernels.cu) and the host orchestration
// (se2p_api.cu).  Everything here is sm_103a device code or plain structs.
#pragma once

#include <cuda_runtime.h>

#include "se2p_ff.cuh"
#include <cufft.h>
#include <stdint.h>

namespace se2p {

constexpr double kPi = 3.1415926535897932385;
// Largest stencil handled: P + 1 nodes per axis must fit one warp.
constexpr int kMaxP = 30;

// Real-space evaluation forms (k_real template argument).
constexpr int kFormFP64 = 0;   // every pair in FP64
constexpr int kFormF32 = 1;    // far pairs in FP32 (FP32-grid precision)
constexpr int kFormFF = 2;     // far pairs in float-float, near pairs in FP64

// Piecewise fit of g(x) = exp(x) E1(x) in the reference's Pade form on
// 1 <= x < 64: 64 pieces per octave, degree 6 in d = x - centre; per piece
// c0..c3 as float-float and c4..c6 as floats, 12 floats (3 float4).
constexpr int kGPiecesPerOctave = 64;
constexpr int kGOctaves = 6;
constexpr int kGPieces = kGPiecesPerOctave * kGOctaves;

// E1 Pade sets of the reference (PE/src/mex/StokesSLP/mex_stokes_slp_real.cpp:19-47)
// as (numerator, denominator) coefficient pairs, 11 pairs each, highest power
// first: 0 = far (x >= 16, in 1/x), 1 = mid (1 < x < 16, in 1/x), 2 = near
// (x <= 1, in x); far and near are padded with leading zeros.  One literal
// list for the device constant table and the host-side fits.
#define SE2P_E1_PADE \
    { \
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, \
     -17.70313744792479226930481672752649, -2.03222164752550948918496942496859, \
     -9.56230625623594754358691716333851, 24.24775264986217493401454703416675, \
     -0.99999982131078080094255255971802, 34.82867640350680460414878325536847, \
     -0.00000000083503088648841284312372, 11.56228921223568129050818242831156}, \
    {-1185.45720315201027667, -0.776491285282330997549, \
     -14751.4895786128450662, 1229.20784182403048905, \
     -54844.4587226402067411, 18455.4124737722049515, \
     -86273.1567711649528784, 86722.3403467334749201, \
     -66598.2652345418633509, 180329.498380501819718, \
     -27182.6254466733970467, 192104.047790227984431, \
     -6046.8250112711035463, 113057.05869159631492, \
     -724.581482791462469795, 38129.5594484818471461, \
     -43.3058660811817946037, 7417.37624454689546708, \
     -0.999999999999998811143, 809.193214954550328455, \
     -0.121013190657725568138e-18, 45.3058660811801465927}, \
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, \
     -0.000111507792921197858394, -0.528611029520217142048e-6, \
     -0.00399167106081113256961, 0.000131049900798434683324, \
     -0.0368031736257943745142, 0.00427347600017103698101, \
     -0.245088216639761496153, 0.056770677104207528384, \
     0.0320913665303559189999, 0.37091387659397013215, \
     0.0865197248079397976498, 1.0}}


// 2^(-j/64), j = 0..63, correctly rounded: the table of Tang's exp.
#define SE2P_EXP2_TAB64 \
    { \
    0x1.0000000000000p+0, \
    0x1.fa7c1819e90d8p-1, \
    0x1.f50765b6e4540p-1, \
    0x1.efa1bee615a27p-1, \
    0x1.ea4afa2a490dap-1, \
    0x1.e502ee78b3ff6p-1, \
    0x1.dfc97337b9b5fp-1, \
    0x1.da9e603db3285p-1, \
    0x1.d5818dcfba487p-1, \
    0x1.d072d4a07897cp-1, \
    0x1.cb720dcef9069p-1, \
    0x1.c67f12e57d14bp-1, \
    0x1.c199bdd85529cp-1, \
    0x1.bcc1e904bc1d2p-1, \
    0x1.b7f76f2fb5e47p-1, \
    0x1.b33a2b84f15fbp-1, \
    0x1.ae89f995ad3adp-1, \
    0x1.a9e6b5579fdbfp-1, \
    0x1.a5503b23e255dp-1, \
    0x1.a0c667b5de565p-1, \
    0x1.9c49182a3f090p-1, \
    0x1.97d829fde4e50p-1, \
    0x1.93737b0cdc5e5p-1, \
    0x1.8f1ae99157736p-1, \
    0x1.8ace5422aa0dbp-1, \
    0x1.868d99b4492edp-1, \
    0x1.82589994cce13p-1, \
    0x1.7e2f336cf4e62p-1, \
    0x1.7a11473eb0187p-1, \
    0x1.75feb564267c9p-1, \
    0x1.71f75e8ec5f74p-1, \
    0x1.6dfb23c651a2fp-1, \
    0x1.6a09e667f3bcdp-1, \
    0x1.6623882552225p-1, \
    0x1.6247eb03a5585p-1, \
    0x1.5e76f15ad2148p-1, \
    0x1.5ab07dd485429p-1, \
    0x1.56f4736b527dap-1, \
    0x1.5342b569d4f82p-1, \
    0x1.4f9b2769d2ca7p-1, \
    0x1.4bfdad5362a27p-1, \
    0x1.486a2b5c13cd0p-1, \
    0x1.44e086061892dp-1, \
    0x1.4160a21f72e2ap-1, \
    0x1.3dea64c123422p-1, \
    0x1.3a7db34e59ff7p-1, \
    0x1.371a7373aa9cbp-1, \
    0x1.33c08b26416ffp-1, \
    0x1.306fe0a31b715p-1, \
    0x1.2d285a6e4030bp-1, \
    0x1.29e9df51fdee1p-1, \
    0x1.26b4565e27cddp-1, \
    0x1.2387a6e756238p-1, \
    0x1.2063b88628cd6p-1, \
    0x1.1d4873168b9aap-1, \
    0x1.1a35beb6fcb75p-1, \
    0x1.172b83c7d517bp-1, \
    0x1.1429aaea92de0p-1, \
    0x1.11301d0125b51p-1, \
    0x1.0e3ec32d3d1a2p-1, \
    0x1.0b5586cf9890fp-1, \
    0x1.0874518759bc8p-1, \
    0x1.059b0d3158574p-1, \
    0x1.02c9a3e778061p-1 \
    }

// ---------------------------------------------------------------------------
// Never-contracted FP64 arithmetic.  Used wherever the reference's own
// rounding decides a discrete outcome: the box index of a point, the
// real-space cutoff test r2 < Lx*Ly/nside_x/nside_y and the grid-node snap.
// The reference is built for x86 SSE (no FMA), so each product and sum is
// rounded separately; a fused a*b+c could move a pair across the cutoff.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xdiv(double a, double b) { return __ddiv_rn(a, b); }

// Box of coordinate x: clamp(floor(nside*(x/L + 0.5)), 0, nside-1)
// (PE/src/mex/common/ewald_tools.cpp:28-33).
__device__ __forceinline__ int box1(double x, double L, int nside)
{
    double t = floor(xmul((double)nside, xadd(xdiv(x, L), 0.5)));
    int b = (int)t;  // saturating conversion; NaN -> 0, then clamped like x86's INT_MIN
    b = b < 0 ? 0 : b;
    return b >= nside ? nside - 1 : b;
}

// Stencil origin and in-cell offset of a point (FindClosestNode,
// PE/src/mex/common/ewald_tools.cpp:86-114).  Node index 0 sits at -L/2.
__device__ __forceinline__ void closest_node(double x, double y, double Lhx, double Lhy,
                                             double h, int P, int &mx, int &my,
                                             double &px, double &py)
{
    const double snap = 1e-13;
    double ox = xsub(x, xmul(h, floor(xdiv(x, h))));
    double oy = xsub(y, xmul(h, floor(xdiv(y, h))));
    double tx = xdiv(xadd(x, Lhx), h);
    double ty = xdiv(xadd(y, Lhy), h);
    const double half = (double)(P / 2);
    int ix = (int)xsub(floor(tx), half);
    int iy = (int)xsub(floor(ty), half);
    if (fabs(ox) < snap || fabs(xsub(ox, h)) < snap) ox = 0.0;
    if (fabs(oy) < snap || fabs(xsub(oy, h)) < snap) oy = 0.0;
    if (ox == 0.0 && remainder(xsub(tx, half), 1.0) < 0) ix++;
    if (oy == 0.0 && remainder(xsub(ty, half), 1.0) < 0) iy++;
    mx = ix; my = iy; px = ox; py = oy;
}

// ---------------------------------------------------------------------------
// E1 by the reference's three-regime Pade split
// (PE/src/mex/StokesSLP/mex_stokes_slp_real.cpp:19-47, :166-205).
// Coefficients are numerator/denominator pairs, highest power first; Horner
// runs in 1/x for x > 1 and in x for x <= 1.  e = exp(-x) is passed in.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double e1_pade(double x, double e)
{
    if (x >= 16.0) {
        const double r = 1.0 / x;
        double a = -17.70313744792479226930481672752649;
        double b = -2.03222164752550948918496942496859;
        a = fma(r, a, -9.56230625623594754358691716333851);
        b = fma(r, b, 24.24775264986217493401454703416675);
        a = fma(r, a, -0.99999982131078080094255255971802);
        b = fma(r, b, 34.82867640350680460414878325536847);
        a = fma(r, a, -0.00000000083503088648841284312372);
        b = fma(r, b, 11.56228921223568129050818242831156);
        return e * (r + a / (b + x));
    } else if (x > 1.0) {
        const double r = 1.0 / x;
        double a = -1185.45720315201027667;
        double b = -0.776491285282330997549;
        a = fma(r, a, -14751.4895786128450662);
        b = fma(r, b, 1229.20784182403048905);
        a = fma(r, a, -54844.4587226402067411);
        b = fma(r, b, 18455.4124737722049515);
        a = fma(r, a, -86273.1567711649528784);
        b = fma(r, b, 86722.3403467334749201);
        a = fma(r, a, -66598.2652345418633509);
        b = fma(r, b, 180329.498380501819718);
        a = fma(r, a, -27182.6254466733970467);
        b = fma(r, b, 192104.047790227984431);
        a = fma(r, a, -6046.8250112711035463);
        b = fma(r, b, 113057.05869159631492);
        a = fma(r, a, -724.581482791462469795);
        b = fma(r, b, 38129.5594484818471461);
        a = fma(r, a, -43.3058660811817946037);
        b = fma(r, b, 7417.37624454689546708);
        a = fma(r, a, -0.999999999999998811143);
        b = fma(r, b, 809.193214954550328455);
        a = fma(r, a, -0.121013190657725568138e-18);
        b = fma(r, b, 45.3058660811801465927);
        return e * (r + a / (b + x));
    }
    double a = -0.000111507792921197858394;
    double b = -0.528611029520217142048e-6;
    a = fma(x, a, -0.00399167106081113256961);
    b = fma(x, b, 0.000131049900798434683324);
    a = fma(x, a, -0.0368031736257943745142);
    b = fma(x, b, 0.00427347600017103698101);
    a = fma(x, a, -0.245088216639761496153);
    b = fma(x, b, 0.056770677104207528384);
    a = fma(x, a, 0.0320913665303559189999);
    b = fma(x, b, 0.37091387659397013215);
    a = fma(x, a, 0.0865197248079397976498);
    b = fma(x, b, 1.0);
    return a / b + x - log(x) - 0.66373538970947265625;
}

// ---------------------------------------------------------------------------
// Kernel argument blocks
// ---------------------------------------------------------------------------
struct BinArgs {
    const double2 *p;   // interleaved (x, y) per point
    int64_t n;
    double Lx, Ly;
    int nx, ny;
    int *box, *rank, *count;
};

struct RealArgs {
    const double2 *sp;    // sources, sorted by box
    const float2 *spf;    // the same rounded to FP32 (cutoff pre-test)
    const double *coef;   // nc coefficients per sorted source: SLP f at [0,1],
                          // DLP S = f (x) n as (S11, S12+S21, S22) at [doff, doff+3)
    int nc, doff;
    const int *sstart;    // box b's sources: [sstart[b], sstart[b+1])
    const double2 *tp;    // targets, sorted by box
    const float2 *tpf;
    const int *tbox;      // box of each sorted target
    int64_t ntar;
    int nx, ny;
    double Lx, Ly, xi, xi2, cut2, self_c;
    double inv_xi2, pf;   // 1/xi^2, 2 xi^2
    double zxm, zxp, zym, zyp;   // image shifts (L*(-+nside))/nside of the wrapped neighbours
    float cut2f, xi2f;
    double2 *u_slp;       // raw sums per sorted target (no 1/(4 pi))
    double2 *u_dlp;
    unsigned long long *counters;   // [candidates, SLP pairs, DLP pairs] (may be NULL)
    // float-float form only: per sorted source ncf coefficient pairs (SLP f1,
    // f2; DLP S11, S12+S21, S22, 3 S11 + S22, 3 S22 + S11 from doff_ff) and
    // the piecewise fit of the E1 Pade form (kGPieces x 3 float4)
    const float2 *coef_ff;
    int ncf, doff_ff;
    // FP32-grid form only: the low halves of the sorted positions (spf, tpf
    // being the high halves of float-float pairs), so that far-pair offsets
    // are formed exactly on the FP32 pipe
    const float2 *spl = nullptr, *tpl = nullptr;
    const float4 *gtab;
    // adjoint only: outer points are the forward sources (sp/spf/coef, boxes
    // obox), inner candidates the forward targets (cell list sstart, tp/tpf,
    // tbox) with weights wcoef = (w_slp, w_dlp) per target; 7 sums per source
    // go to gout.
    int64_t nouter;
    const int *obox;
    const double *wcoef;
    double *gout;
};

struct GatherAdjArgs {
    const double2 *sp;    // sorted forward sources
    int64_t ns;
    const double *coef;   // 5 per source: f1, f2, S11, S12+S21, S22
    const double *grid;   // 5 adjoint grids
    int Mx, My, P;
    double Lhx, Lhy, h, w, a, scale;
    const double *e1;
    double *out;          // 7 per source: 5 values, gradient x, y
    // float-float form (k_gather_adj_ff): the bit pattern of max |grid|
    // (from the inverse FFT's unpack) and room for the grids as float-float
    // planes; null for the FP64 gather alone
    unsigned long long *gmax = nullptr;
    float2 *gff = nullptr;
};

struct SpreadArgs {
    const double2 *sp;    // source positions
    const double *coef;   // NC coefficients per source
    int64_t ns;
    double *grid;         // NC grids, each Mx x My with y fastest
    int Mx, My, P;
    double Lhx, Lhy, h, w, a;   // a = -2 xi^2 / eta
    const double *e1;     // exp(a h^2 j^2), j = -P/2..P/2
    // Fixed-point form (k_spread_fix): the grids are int64 at scale 2^S, with S
    // derived from *bound (the bit pattern of a positive double bounding
    // every node's sum of |contributions|).
    const unsigned long long *bound = nullptr;
};

struct FilterArgs {
    cufftDoubleComplex *spec;   // component c at spec + c * Mx * (My/2+1)
    int Mx, My;
    double Lx, Ly, xi, eta, scale;   // scale = 1 / (Mx My)
    int slp_in, dlp_in;         // first spectrum of each kind (-1 = absent)
    int slp_out, dlp_out;       // where the 2 filtered spectra of each kind go
    int transposed = 0;         // spectra stored [c][ky][x] (x fastest) instead of [c][x][ky]
    // per-mode effective multipliers from k_filter_matrix_table (forward
    // filter only), or NULL: kFilterMat doubles per mode
    const double *mtab = nullptr;
};
// SLP (a, b, c): o1 = a h1 - b h2, o2 = -b h1 + c h2; DLP rows (B111, B112,
// B122) and (B211, B212, B222) times e t; Nyquist averaging, zero mode and
// 1/(Mx My) folded in.
constexpr int kFilterMat = 9;

struct GatherArgs {
    const double2 *tp;
    int64_t nt;
    const double *grid;   // NC grids (filtered, inverse transformed)
    int Mx, My, P;
    double Lhx, Lhy, h, w, a, scale;
    const double *e1;
    double2 *out;         // NC/2 outputs per target, [k * nt + t]
    // Fixed-point form (k_gather_fix): gmax[q] holds the bit pattern of
    // max |grid| over grids 2q and 2q+1 (from the unpack; kGmaxWords words),
    // and launch_grid_to_fixed has turned each grid into int64 at the scale
    // that its pair's gmax and Bg give.
    const unsigned long long *gmax = nullptr;
    int Bg = 0;
    // k_gather_fix: the order in which the sorted targets are visited (null:
    // sorted order), from launch_patch_order
    const int *order = nullptr;
};

// FP32-grid (mixed precision) k-space arguments (se2p_kernels_f32.cu).
struct SpreadArgsF {
    const double2 *sp;
    const double *coef;
    int64_t ns;
    float *grid;
    int Mx, My, P;
    double Lhx, Lhy, h, w, a;
};

struct FilterArgsF {
    float2 *spec;
    int Mx, My;
    double Lx, Ly, xi, eta;
    float scale;
    // from the host, as FP64 division is slow on the device: 1/(4 xi^2),
    // (1 - eta)/(4 xi^2) and the wavenumber steps 2 pi / L
    float c1, c2;
    double dkx, dky;
    int slp_in, dlp_in, slp_out, dlp_out;
};

struct GatherArgsF {
    const double2 *tp;
    int64_t nt;
    const float *grid;
    int Mx, My, P;
    double Lhx, Lhy, h, w, a, scale;
    double2 *out;
};

// ---------------------------------------------------------------------------
// Host launchers (se2p_kernels.cu).  Each returns the launch status.
// ---------------------------------------------------------------------------
cudaError_t launch_bin(const BinArgs &a, int *start, int nbox, int *perm, int *sorted_box,
                       double2 *sorted_pos, float2 *sorted_pos_f, cudaStream_t st,
                       int64_t &launches,
                       float2 *sorted_pos_lo = nullptr);
cudaError_t launch_src_coef(int64_t n, const int *perm, const double2 *f_slp,
                            const double2 *f_dlp, const double2 *nrm, double *coef, int nc,
                            cudaStream_t st, int64_t &launches);
// out: per source ostride float2 (ncf when 0) from out + ostride j; tails =
// false leaves out the DLP pair 3 S11 + S22, 3 S22 + S11 (the real-space
// kernels read it, the geometry's stored operator does not).
cudaError_t launch_src_coef_ff(int64_t n, const double *coef, int nc, bool slp, bool dlp,
                               float2 *out, int ncf, cudaStream_t st, int64_t &launches,
                               int64_t ostride = 0, bool tails = true);
cudaError_t launch_real(const RealArgs &a, bool slp, bool dlp, cudaStream_t st,
                        int64_t &launches, int form = kFormFP64);
// 2D real FFT through 1D complex passes (se2p_kernels.cu): pack real grid
// pairs as complex, split a y-transformed pair into half spectra, the inverse
// Hermitian join, and the final real/imaginary unpack.
cudaError_t launch_pack_real_pairs(const double *grid, int nc, int64_t G, double2 *z,
                                   cudaStream_t st, int64_t &launches);
// With gmax (kGmaxWords words, zeroed), also the largest |value| of each
// pair of grids, gmax[q] for grids 2q and 2q+1.
cudaError_t launch_unpack_real_pairs(const double2 *z, int nout, int64_t G, double *grid,
                                     cudaStream_t st, int64_t &launches,
                                     unsigned long long *gmax = nullptr);
// In place: each of the nout grids of G doubles becomes int64 round(g 2^Sg),
// max|g| 2^Sg < 2^Bg over its pair (gmax[c / 2]), unless a gmax word marks a
// non-finite value (then the grids stay as they are and the FP64 gather runs).
// Patch-major order of box-sorted targets (boxes by nx + bx, cell list
// tstart, box per sorted target tbox): patches of pw x ph boxes in row-major
// order, their boxes row-major, each box's targets in sorted order.  order
// gets nt entries; pcount and pstart nbox + 1 ints of scratch.
cudaError_t launch_patch_order(const int *tstart, const int *tbox, int64_t nt, int nx, int ny,
                               int pw, int ph, int *pcount, int *pstart, int *order,
                               cudaStream_t st, int64_t &launches);
cudaError_t launch_grid_to_fixed(double *grid, int nout, int64_t G, const unsigned long long *gmax,
                                 int Bg, cudaStream_t st, int64_t &launches);
// fold: the last pair of an odd nc holds plane nc-1's rows x (re) and x + Mx/2
// (im) as its rows x < Mx/2 (FftRowsFF::fold).
cudaError_t launch_split_half_spectra_t(const double2 *z, int nc, int Mx, int My, double2 *specT,
                                        cudaStream_t st, int64_t &launches, bool fold = false);
cudaError_t launch_join_half_spectra_t(const double2 *specT, int nout, int Mx, int My, double2 *z,
                                       cudaStream_t st, int64_t &launches);
// Float-float row FFTs (se2p_fft_ff.cu): unnormalised C2C of `rows`
// contiguous rows of L complex doubles, in place, sign -1 forward / +1
// inverse (cuFFT's convention).  Lengths 8^a 4^b 2^c 7^d 5^e 3^f up to
// kFftFFMaxLen; fft_rows_ff_plan says whether L is one.
constexpr int kFftFFMaxLen = 6144;
constexpr int kFftFFMaxStages = 16;
struct FftRowsFF {
    int L = 0, nst = 0, sign = -1;
    int radix[kFftFFMaxStages] = {};
    // ceil(2^32 / Ns) of each stage (Ns = product of the earlier radices):
    // j / Ns = umulhi(j, magic) exactly for j Ns < 2^32
    unsigned magic[kFftFFMaxStages] = {};
    // Optional fused pack (first forward pass) / unpack (last inverse pass):
    // row r = (pair q = r / Mx, x = r % Mx) is read from / written to two real
    // planes of G words, re = plane 2q, im = plane 2q+1 (zero / dropped when
    // 2q+1 >= npl), row x of a plane at x L.
    int Mx = 0;
    int64_t G = 0;
    const void *pack_in = nullptr;    // int64 planes at scale 2^S (bound), or doubles
    const unsigned long long *bound = nullptr;   // spread bound slot; null or all ones: doubles
    int npl_in = 0;
    // an odd plane count's last plane folded: its rows x and x + Mx/2 form
    // complex row x of its pair (Mx/2 rows instead of Mx half-empty ones)
    int fold = 0;
    double *unpack_out = nullptr;     // double planes
    int npl_out = 0;
    unsigned long long *gmax = nullptr;   // largest |value| unpacked per pair q (bit pattern), optional
};
bool fft_rows_ff_plan(int L, FftRowsFF &p);
void fft_rows_ff_twiddles(int L, float4 *host);   // exp(-2 pi i m/L), m < L, float-float
cudaError_t launch_fft_rows_ff(double2 *data, int64_t rows, const FftRowsFF &p, const float4 *tw,
                               cudaStream_t st, int64_t &launches);
// Real-space operator of a fixed geometry (se2p_geom.cu).
// Rows sliced by 32 targets: entry k of row t at slice[t / 32] + 32 k + t % 32
// (slice = exclusive scan of launch_geom_slices' slots per slice); the
// operator arrays hold slice[ceil(nt / 32)] slots, padding marked by tgt < 0.
cudaError_t launch_geom_rows(const RealArgs &a, bool slp, bool dlp, bool fill, int *rowcnt,
                             const int *slice, int *src, int *tgt, unsigned char *meta,
                             cudaStream_t st, int64_t &launches);
cudaError_t launch_geom_slices(const int *rowptr, int64_t nt, int *slen, cudaStream_t st,
                               int64_t &launches);
cudaError_t launch_geom_coef(const RealArgs &a, bool slp, bool dlp, int64_t nnz, int *src,
                             const int *tgt, const unsigned char *meta, float2 *cf,
                             cudaStream_t st, int64_t &launches);
cudaError_t launch_geom_apply(bool slp, bool dlp, int64_t nt, int64_t nnz, const int *rowptr,
                              const int *slice, const int *src, const float2 *cf,
                              const float2 *cff, int ncf,
                              int doff, int64_t rstride, const double *cfd_rhs, int nc,
                              int doffd, int64_t rstrided, int nr, double2 *ur_slp,
                              double2 *ur_dlp, cudaStream_t st, int64_t &launches);
cudaError_t launch_geom_add(int64_t n, const int *perm, const double2 *ur, bool dlp, double2 *u,
                            cudaStream_t st, int64_t &launches);
cudaError_t launch_scan(const int *count, int n, int *start, cudaStream_t st, int64_t &launches);
int sm_count();
cudaError_t launch_real_adj(const RealArgs &a, bool slp, bool dlp, cudaStream_t st,
                            int64_t &launches, int form = kFormFP64);
cudaError_t launch_sorted_pair(int64_t n, const int *perm, const double2 *a, const double2 *b,
                               double *out, cudaStream_t st, int64_t &launches);
cudaError_t launch_filter_adj(const FilterArgs &a, cudaStream_t st, int64_t &launches);
// With a.gff set (adj_gather_ff_ok), the float-float gather runs, and the
// FP64 one only when the grid holds a non-finite value.
bool adj_gather_ff_ok(double a, double h, double w, int P);
// iters coalesced 64-bit atomic adds per thread into a[0..n) (n >= 256 x 8 x
// SMs); *count = the atomics launched.
cudaError_t launch_probe_red64(unsigned long long *a, int64_t n, int iters, int64_t *count,
                               cudaStream_t st);
cudaError_t launch_gather_adj(const GatherAdjArgs &a, cudaStream_t st, int64_t &launches);
cudaError_t launch_adj_assemble(int64_t n, const int *perm, const double *gr, const double *gk,
                                const double *w, int64_t nt, double2 *part,
                                const double2 *praw, const double2 *fd, const double2 *nrm,
                                double inv_area, int slp, int dlp, double2 *g_pos,
                                double2 *g_fs, double2 *g_fd, double2 *g_n, cudaStream_t st,
                                int64_t &launches);
cudaError_t launch_spread_f32(const SpreadArgsF &a, int nc, int sms, cudaStream_t st,
                              int64_t &launches);
cudaError_t launch_filter_f32(const FilterArgsF &a, cudaStream_t st, int64_t &launches);
cudaError_t launch_gather_f32(const GatherArgsF &a, int nc, cudaStream_t st, int64_t &launches);
cudaError_t launch_spread(const SpreadArgs &a, int nc, cudaStream_t st, int64_t &launches);
// Fixed-point spread (se2p_kernels.cu): a bound on the grid values from
// per-bin sums of |coefficients|, then int64 accumulation into a.grid
// (reinterpreted as long long), and the pack that turns those grids into the
// complex pairs of the forward FFT.
// Bound-slot mark of the fixed-point spread: the FP64 spread ran instead and
// the grids hold doubles.
constexpr unsigned long long kFixedOff = ~0ull;      // above every finite bound

// The gather's grid maxima: one bit pattern per pair of output grids (SLP,
// DLP, and the adjoint's fifth grid), each grid scaled by its own pair's.
constexpr int kGmaxWords = 3;
__device__ __forceinline__ unsigned long long gmax_all(const unsigned long long *g)
{
    return max(g[0], max(g[1], g[2]));
}

// Scale S of the fixed-point spread's grids (int64 at 2^S, bound 2^S < 2^59),
// from the bit pattern of the positive bound.
__device__ __forceinline__ int fix_shift(unsigned long long bits)
{
    if (bits == kFixedOff) return 0;
    const int ex = (int)((bits >> 52) & 0x7ff);
    if (ex == 0 || ex == 0x7ff) return 0;            // zero (no sources) or not finite
    const int S = 59 - (ex - 1022);                  // bound < 2^(ex-1022)
    return S < -960 ? -960 : (S > 960 ? 960 : S);
}

// ws: spread_bound_words(Mx, My, P) doubles (the bins' sums of max_c |c|,
// their window along x, the bound slot at spread_bound_slot(Mx, My, P), then
// the bins' source counts and their window as ints).
// mult is the number of times one stencil can cover a node (> 1 when M <= P)
// and kfac = mult 2^(2 kY).  When the bound slot ends up all ones the FP64
// spread runs (launch it behind launch_spread_fix with a.bound set) and the
// grids hold doubles.
int64_t spread_bound_words(int Mx, int My, int P);
int64_t spread_bound_slot(int Mx, int My, int P);
cudaError_t launch_spread_bound(const SpreadArgs &a, int nc, double kfac, int mult, double *ws,
                                cudaStream_t st, int64_t &launches);
cudaError_t launch_spread_fix(const SpreadArgs &a, int nc, int kY, cudaStream_t st,
                              int64_t &launches);
// Many right-hand sides on one point set: k_spread_fix and k_gather_fix
// with the per-point Gaussian factors formed once for all nr of them
// (coefficients, grids, bound slots, outputs strided by right-hand side), and
// the FP64 gather alone (it runs where the grid holds a non-finite value).
cudaError_t launch_spread_fix_multi(const SpreadArgs &a, int nc, int kY, int nr, int64_t cstride,
                                    int64_t gstride, int bstride, cudaStream_t st,
                                    int64_t &launches);
cudaError_t launch_gather_fix_multi(const GatherArgs &a, int nc, int nr, int64_t gstride,
                                    int64_t ostride, cudaStream_t st, int64_t &launches);
cudaError_t launch_gather_fp64_fallback(const GatherArgs &a, int nc, cudaStream_t st,
                                        int64_t &launches);
cudaError_t launch_pack_fixed_pairs(const long long *grid, int nc, int64_t G,
                                    const unsigned long long *bound, double2 *z, cudaStream_t st,
                                    int64_t &launches);
cudaError_t launch_filter(const FilterArgs &a, cudaStream_t st, int64_t &launches);
cudaError_t launch_filter_matrix_table(const FilterArgs &a, double *mtab, cudaStream_t st,
                                       int64_t &launches);
cudaError_t launch_gather(const GatherArgs &a, int nc, cudaStream_t st, int64_t &launches);
cudaError_t launch_wrap(int64_t n, const double2 *p, double Lx, double Ly, double2 *out,
                        cudaStream_t st, int64_t &launches);
cudaError_t launch_zero_mode(int64_t n, const double2 *p, const double2 *f, const double2 *nrm,
                             double inv_area, double2 *part, double2 *zm, cudaStream_t st,
                             int64_t &launches);
cudaError_t launch_assemble(int64_t n, int mode, const int *perm, const double2 *ur,
                            const double2 *uk, const double2 *zm, double2 *u, double2 *ur_out,
                            double2 *uk_out, cudaStream_t st, int64_t &launches);
constexpr int kZeroModeParts = 304;

// g(x) = exp(x) E1(x) in the reference's Pade form (mid set below 16, far
// set from 16 on), from the piecewise fit gtab, for 1 < x < 64.  The piece
// follows from the head's exponent and top six mantissa bits; x = 16 with a
// negative tail belongs to the mid set's last piece.
__device__ __forceinline__ float2 ff_g_e1(float2 x, const float4 *__restrict__ gtab)
{
    const unsigned xb = __float_as_uint(x.x);
    int oct = (int)(xb >> 23) - 127;
    int m = (int)((xb >> 17) & 63u);
    if (x.x == 16.0f && x.y < 0.0f) {
        oct = 3;
        m = 63;
    }
    const float c = __uint_as_float(((unsigned)(oct + 127) << 23) | ((unsigned)m << 17) | (1u << 16));
    float dh, dl;
    fast_two_sum(x.x - c, x.y, dh, dl);           // x.x - c is exact (same binade)
    const float2 d = make_float2(dh, dl);
    const float4 *cf = gtab + 3 * (oct * kGPiecesPerOctave + m);
    const float4 A = __ldg(cf), B = __ldg(cf + 1), C = __ldg(cf + 2);
    const float t = fmaf(fmaf(C.z, dh, C.y), dh, C.x);
    float2 p = ff_add(make_float2(B.z, B.w), ff_mul_f(d, t));
    p = ff_add(make_float2(B.x, B.y), ff_mul(p, d));
    p = ff_add(make_float2(A.z, A.w), ff_mul(p, d));
    return ff_add(make_float2(A.x, A.y), ff_mul(p, d));
}

}  // namespace se2p
