// se2p_kernels.cu -- sm_103a kernels of the doubly-periodic spectral Ewald
// (SE) summation of the 2D Stokeslet (SLP) and stresslet (DLP).
//
// The reference (FastTools2D, PeriodicEwald/src/mex) runs these loops on the
// CPU with OpenMP; here each is a GB300 kernel.  GB300 issues about 2 FP64
// FMA per clock per SM, some 70 times fewer than FP32, so each stage of the
// default form runs in the narrowest arithmetic that keeps results within
// 1e-12 of the reference: real-space far pairs in float-float on the FP32
// pipe (near pairs, the self term and the cutoff decisions in FP64), the
// spread and gather as exact int64 sums of rounded products, the filter in
// FP64.  The all-FP64 versions of these kernels serve the FP64_NATIVE form
// and the fallbacks; they keep every FP64 warp instruction fully populated
// (accepted pairs compacted before the Pade/exp work, a flattened (P+1)^2
// stencil per spread source, one gather target per lane).
#include "se2p_internal.cuh"

#include <algorithm>

namespace se2p {

// ===========================================================================
// Binning: box index per point and a counting sort
// (PE/src/mex/common/ewald_tools.cpp:7-80).  The within-box order comes from
// atomics, so it is not the reference's input order; only FP64 summation
// order depends on it.
// ===========================================================================
__global__ void k_bin_count(BinArgs a)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const double2 q = a.p[i];
    const int b = box1(q.y, a.Ly, a.ny) * a.nx + box1(q.x, a.Lx, a.nx);
    a.box[i] = b;
    a.rank[i] = atomicAdd(&a.count[b], 1);
}

// Exclusive scan of count[0..n) into start[0..n], one block of 1024 threads,
// 8 consecutive items per thread per chunk.
__global__ void __launch_bounds__(1024) k_scan(const int *__restrict__ count, int n,
                                                 int *__restrict__ start)
{
    __shared__ int warp_tot[32];
    __shared__ int carry_s;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) carry_s = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 8192) {
        int v[8], sum = 0;
        const int i0 = base + tid * 8;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            v[k] = (i0 + k < n) ? count[i0 + k] : 0;
            sum += v[k];
        }
        int incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(~0u, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int w = warp_tot[lane], wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(~0u, wi, o);
                if (lane >= o) wi += t;
            }
            warp_tot[lane] = wi - w;  // exclusive prefix of warp totals
        }
        __syncthreads();
        int run = carry_s + warp_tot[wid] + incl - sum;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            if (i0 + k < n) start[i0 + k] = run;
            run += v[k];
        }
        __syncthreads();
        if (tid == 1023) carry_s = run;
        __syncthreads();
    }
    if (tid == 0) start[n] = carry_s;
}

// Sorted slot of point i; writes the permutation and the sorted copies.
__global__ void k_bin_place(int64_t n, const int *__restrict__ box, const int *__restrict__ rank,
                            const int *__restrict__ start, int *__restrict__ perm,
                            int *__restrict__ sorted_box, const double2 *__restrict__ p,
                            double2 *__restrict__ sp, float2 *__restrict__ spf,
                            float2 *__restrict__ spl)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = box[i];
    const int j = start[b] + rank[i];
    perm[j] = (int)i;
    if (sorted_box) sorted_box[j] = b;
    const double2 q = p[i];
    sp[j] = q;
    const float hx = (float)q.x, hy = (float)q.y;
    if (spf) spf[j] = make_float2(hx, hy);
    // q - hi is exact in FP64; its rounding to FP32 leaves hi + lo within
    // 2^-48 |q| of q
    if (spl) spl[j] = make_float2((float)(q.x - (double)hx), (float)(q.y - (double)hy));
}

// Per-source coefficients in sorted order, nc per source: SLP f (f1, f2),
// then DLP S = f (x) n as (S11, S12+S21, S22)
// (PE/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:81-91; S12 and S21 only ever
// enter as their sum, in the real-space contraction and as H2+H3 in the
// DLP filter).  The same array is the spread's per-grid weights.
__global__ void k_src_coef(int64_t n, const int *__restrict__ perm,
                           const double2 *__restrict__ f_slp, const double2 *__restrict__ f_dlp,
                           const double2 *__restrict__ nrm, double *__restrict__ coef, int nc)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int i = perm[j];
    double *c = coef + (int64_t)nc * j;
    if (f_slp) {
        const double2 f = f_slp[i];
        c[0] = f.x;
        c[1] = f.y;
        c += 2;
    }
    if (f_dlp) {
        const double2 f = f_dlp[i], m = nrm[i];
        c[0] = f.x * m.x;
        c[1] = f.x * m.y + f.y * m.x;
        c[2] = f.y * m.y;
    }
}

// Float-float copy of the sorted coefficients for the far pairs of the FP64
// form: SLP f1, f2; DLP S11, S12+S21, S22 and the combinations 3 S11 + S22,
// 3 S22 + S11 of the stresslet contraction (formed in FP64, then split).
__global__ void k_src_coef_ff(int64_t n, const double *__restrict__ coef, int nc, int slp,
                              int dlp, float2 *__restrict__ out, int64_t ostride, int tails)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double *c = coef + (int64_t)nc * j;
    float2 *o = out + ostride * j;
    if (slp) {
        o[0] = ff_split(c[0]);
        o[1] = ff_split(c[1]);
        c += 2;
        o += 2;
    }
    if (dlp) {
        o[0] = ff_split(c[0]);
        o[1] = ff_split(c[1]);
        o[2] = ff_split(c[2]);
        if (tails) {
            o[3] = ff_split(fma(3.0, c[0], c[2]));
            o[4] = ff_split(fma(3.0, c[2], c[0]));
        }
    }
}

// Sorted copy of two per-point 2-vectors (either may be NULL -> zeros):
// out[4 j .. 4 j + 3] = (a[perm[j]], b[perm[j]]).
__global__ void k_sorted_pair(int64_t n, const int *__restrict__ perm,
                              const double2 *__restrict__ a, const double2 *__restrict__ b,
                              double *__restrict__ out)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int i = perm[j];
    const double2 x = a ? a[i] : make_double2(0.0, 0.0);
    const double2 y = b ? b[i] : make_double2(0.0, 0.0);
    double *o = out + 4 * j;
    o[0] = x.x;
    o[1] = x.y;
    o[2] = y.x;
    o[3] = y.y;
}

// ===========================================================================
// Real-space pair sums (PE/src/mex/StokesSLP/mex_stokes_slp_real.cpp:131-333,
// PE/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:103-187), SLP and DLP fused.
//
// One warp walks a sequence of targets.  For each target the candidate
// sources of its own box (every pair, no cutoff) and its 8 periodic
// neighbour boxes (pairs with r2 < Lx*Ly/nside_x/nside_y) form one list,
// scanned 32 at a time.  The cutoff test runs in FP32 with a rigorous
// rounding-error band; only candidates inside the band take the reference's
// exact FP64 test, separately for the SLP offset s-(t-z) and the DLP offset
// (s-t)+z.  Accepted pairs go into a per-warp FIFO that carries over from one
// target to the next, so the FP64 pair evaluation always runs on 32 lanes.
// Each lane keeps register sums tagged with the target they belong to; when
// its next pair is for a later target, the lanes flush with a segmented
// warp reduction into a small ring of per-target accumulators, and a target
// is written out once every lane has moved past it.
//
// Per pair the SLP and DLP share one exp(-xi^2 r^2) (table-driven, Tang's
// method) and one reciprocal 1/r2 (rcp.approx + Newton).  E1 uses the
// reference's three Pade forms through one Horner loop whose coefficient
// set is chosen per lane (shorter forms padded with leading zeros, which
// leaves their values unchanged), so only the log of the near form diverges.
// The DLP contraction is regrouped as fb x_i (x.S.x) + 2 xi^2 (...),
// algebraically equal to the reference's T_ijk S_jk.
// ===========================================================================
constexpr int kRealWarps = 4;
constexpr int kRing = 32;     // targets in flight per warp
__constant__ int c_nb_dx[9] = {0, -1, -1, -1, 0, 0, 1, 1, 1};
__constant__ int c_nb_dy[9] = {0, -1, 0, 1, -1, 1, -1, 0, 1};

// 2^(-j/64), j = 0..63, correctly rounded (table in se2p_internal.cuh).
__constant__ double c_exp_tab[64] = SE2P_EXP2_TAB64;

// The three E1 Pade sets (layout in se2p_internal.cuh).
__constant__ double c_e1[3][22] = SE2P_E1_PADE;

// exp(-x) for x >= 0 by Tang's table-driven method (P. T. P. Tang, "Table-
// driven implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989): x = (n/64) ln 2 + r, |r| <= ln2/128,
// exp(-x) = 2^-(n>>6) * 2^-((n&63)/64) * exp(-r) with a degree-5 Taylor
// polynomial (truncation < 4e-17).  ln2/64 is split Cody-Waite style (36-bit
// head).  Returns 0 from x = 704 on and propagates NaN.
__device__ __forceinline__ double exp_neg(double x, const double *tab)
{
    const double kShift = 6755399441055744.0;   // 1.5 * 2^52
    const double t = fma(x, 0x1.71547652b82fep+6, kShift);
    const int n = __double2loint(t);
    const double kd = t - kShift;
    double r = fma(-kd, 0x1.62e42fefa0000p-7, x);
    r = fma(-kd, 0x1.cf79abc9e3b3ap-46, r);
    double p = fma(-r, 1.0 / 120.0, 1.0 / 24.0);
    p = fma(-r, p, 1.0 / 6.0);
    p = fma(-r, p, 0.5);
    p = fma(-r, p, 1.0);
    p = fma(-r, p, 1.0);
    if (__double2hiint(x) >= 0x40860000) return x == x ? 0.0 : x;   // x >= 704, inf, NaN
    const double scale = __hiloint2double((1023 - (n >> 6)) << 20, 0);
    return p * tab[n & 63] * scale;
}

// 1/a by the hardware approximation plus two Newton-Raphson steps
// (r <- r + r (1 - a r)); each step doubles the correct bits.
__device__ __forceinline__ double rcp_nr(double a)
{
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(a));
    double e = fma(-a, r, 1.0);
    r = fma(r, e, r);
    e = fma(-a, r, 1.0);
    return fma(r, e, r);
}

struct RealWarp {
    int2 q[2][64];              // pair FIFOs: [0] main, [1] near field (x <= 1)
                                // entry = (sorted source, slot | k << 8 | flags << 12)
    double acc[kRing][4];       // per-target sums: SLP u1, u2, DLP u1, u2
    float2 accf[kRing][4];      // the same from float-float pairs (FP64 form, queue 0)
    double2 tpos[kRing];
    int2 tbxy[kRing];           // the target's box as (column, row)
    int tidx[kRing];
    unsigned tend[2][kRing];    // FIFO position after the target's last pair (mod 2^32)
    int nbs[9], nbp[10];        // neighbour box: first sorted source, list prefix
    int curbox;                 // the box those describe (-1: none yet)
    int2 curbxy;                // and its (column, row)
    double2 nbz[9];
    float2 nbzf[9];
    float2 nbe[9];              // 2^-22 (|t| + |z|) per neighbour box (the pre-test band)
};

// Segmented warp reduction of (v0..v3) by nondecreasing key; the last lane
// of each segment with a real key adds its sum into ring slot key % kRing.
__device__ __forceinline__ void seg_flush(RealWarp &W, int lane, int key, double v0, double v1,
                                          double v2, double v3)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int ko = __shfl_up_sync(~0u, key, o);
        const double a0 = __shfl_up_sync(~0u, v0, o), a1 = __shfl_up_sync(~0u, v1, o);
        const double a2 = __shfl_up_sync(~0u, v2, o), a3 = __shfl_up_sync(~0u, v3, o);
        if (lane >= o && ko == key) {
            v0 += a0; v1 += a1; v2 += a2; v3 += a3;
        }
    }
    const int kn = __shfl_down_sync(~0u, key, 1);
    if (key >= 0 && key != 0x7fffffff && (lane == 31 || kn != key)) {
        double *a = W.acc[key % kRing];
        a[0] += v0; a[1] += v1; a[2] += v2; a[3] += v3;
    }
    __syncwarp();
}

// seg_flush for float-float sums (queue 0 of the FP64 form), into W.accf.
// The tree adds the heads with TwoSum and carries tails and TwoSum errors
// in the second float unnormalised; each segment's total is normalised once
// before it joins the slot's accumulator.
__device__ __forceinline__ void seg_flush_ff(RealWarp &W, int lane, int key, float2 v0, float2 v1,
                                             float2 v2, float2 v3)
{
    float2 v[4] = {v0, v1, v2, v3};
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int ko = __shfl_up_sync(~0u, key, o);
        float2 a[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            a[k].x = __shfl_up_sync(~0u, v[k].x, o);
            a[k].y = __shfl_up_sync(~0u, v[k].y, o);
        }
        if (lane >= o && ko == key) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                float s, e;
                two_sum(v[k].x, a[k].x, s, e);
                v[k] = make_float2(s, v[k].y + a[k].y + e);
            }
        }
    }
    const int kn = __shfl_down_sync(~0u, key, 1);
    if (key >= 0 && key != 0x7fffffff && (lane == 31 || kn != key)) {
        float2 *acc = W.accf[key % kRing];
#pragma unroll
        for (int k = 0; k < 4; k++) acc[k] = ff_add(acc[k], ff_norm(v[k].x, v[k].y));
    }
    __syncwarp();
}

// seg_flush for the FP32-grid form's float sums: the tree adds in float
// (the lanes' own sums are float already), and each segment's total joins
// the slot's float-float accumulator.
__device__ __forceinline__ void seg_flush_f(RealWarp &W, int lane, int key, float v0, float v1,
                                            float v2, float v3)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int ko = __shfl_up_sync(~0u, key, o);
        const float a0 = __shfl_up_sync(~0u, v0, o), a1 = __shfl_up_sync(~0u, v1, o);
        const float a2 = __shfl_up_sync(~0u, v2, o), a3 = __shfl_up_sync(~0u, v3, o);
        if (lane >= o && ko == key) {
            v0 += a0; v1 += a1; v2 += a2; v3 += a3;
        }
    }
    const int kn = __shfl_down_sync(~0u, key, 1);
    if (key >= 0 && key != 0x7fffffff && (lane == 31 || kn != key)) {
        float2 *a = W.accf[key % kRing];
        a[0] = ff_add_f(a[0], v0); a[1] = ff_add_f(a[1], v1);
        a[2] = ff_add_f(a[2], v2); a[3] = ff_add_f(a[3], v3);
    }
    __syncwarp();
}

template <bool SLP, bool DLP>
__device__ __forceinline__ void real_pair(const RealArgs &a, const RealWarp &W, int2 e,
                                          const double *tab, const double *e1s, double &s1,
                                          double &s2, double &d1, double &d2)
{
    const int s = e.x, slot = e.y & 0xff, k = (e.y >> 8) & 0xf, fl = e.y >> 12;
    const double2 S = a.sp[s];
    const double2 T = W.tpos[slot];
    // image shift of neighbour k: 0 or the reference's (L*(+-nside))/nside
    const int2 tb = W.tbxy[slot];
    const int ux = tb.x + c_nb_dx[k], uy = tb.y + c_nb_dy[k];
    // Without a periodic image both offset forms are exactly s - t; across an
    // image (rare) the SLP form s-(t-z) and the DLP form (s-t)+z are formed
    // separately and each kernel keeps its own r2, as the reference does.
    const bool img = ux < 0 || ux >= a.nx || uy < 0 || uy >= a.ny;
    double x1 = S.x - T.x, x2 = S.y - T.y, dxs = x1, dys = x2;
    if (img) {
        const double zx = ux < 0 ? a.zxm : (ux >= a.nx ? a.zxp : 0.0);
        const double zy = uy < 0 ? a.zym : (uy >= a.ny ? a.zyp : 0.0);
        x1 += zx;
        x2 += zy;
        dxs = S.x - (T.x - zx);
        dys = S.y - (T.y - zy);
    }
    const double r2 = fma(dxs, dxs, dys * dys);
    const double x = r2 * a.xi2;
    const double ex = exp_neg(x, tab);
    const double ir2 = rcp_nr(r2);
    // E1 (unified Horner over the three Pade forms)
    const int set = x >= 16.0 ? 0 : (x > 1.0 ? 1 : 2);
    const double *c = e1s + 22 * set;
    const double z = set == 2 ? x : ir2 * a.inv_xi2;
    double pa = c[0], pb = c[1];
#pragma unroll
    for (int i = 2; i < 22; i += 2) {
        pa = fma(z, pa, c[i]);
        pb = fma(z, pb, c[i + 1]);
    }
    const double den = set == 2 ? pb : pb + x;
    const double qv = pa * rcp_nr(den);
    double E;
    if (set == 2) E = qv + x - log(x) - 0.66373538970947265625;
    else E = ex * (z + qv);
    if (SLP && (fl & 1)) {
        const double f1 = a.coef[(int64_t)a.nc * s], f2 = a.coef[(int64_t)a.nc * s + 1];
        const double h = 0.5 * E, g = ex * ir2;
        const double gq = g * fma(dxs, f2, -dys * f1);
        s1 = fma(h, f1, fma(gq, dys, s1));
        s2 = fma(h, f2, fma(-gq, dxs, s2));
    }
    if (DLP && (fl & 2)) {
        const double *Sc = a.coef + (int64_t)a.nc * s + a.doff;
        const double S11 = Sc[0], S1221 = Sc[1], S22 = Sc[2];
        double xd = x, exd = ex, ird = ir2;
        if (img) {                             // offsets can differ only across an image
            const double r2d = fma(x1, x1, x2 * x2);
            if (r2d != r2) {
                xd = r2d * a.xi2;
                exd = exp_neg(xd, tab);
                ird = rcp_nr(r2d);
            }
        }
        const double fb = -4.0 * (1.0 + xd) * ird * ird;
        const double Q = fma(x1 * x1, S11, fma(x1 * x2, S1221, x2 * x2 * S22));
        const double A1 = fma(x1, fma(3.0, S11, S22), x2 * S1221);
        const double A2 = fma(x2, fma(3.0, S22, S11), x1 * S1221);
        const double fq = fb * Q, pf = a.pf;
        d1 = fma(exd, fma(fq, x1, pf * A1), d1);
        d2 = fma(exd, fma(fq, x2, pf * A2), d2);
    }
}

// The E1 Pade sets in FP32, same layout as c_e1.
__constant__ float c_e1f[3][22] = {
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
     -17.70313744792479226930481672752649f, -2.03222164752550948918496942496859f,
     -9.56230625623594754358691716333851f, 24.24775264986217493401454703416675f,
     -0.99999982131078080094255255971802f, 34.82867640350680460414878325536847f,
     -0.00000000083503088648841284312372f, 11.56228921223568129050818242831156f},
    {-1185.45720315201027667f, -0.776491285282330997549f, -14751.4895786128450662f,
     1229.20784182403048905f, -54844.4587226402067411f, 18455.4124737722049515f,
     -86273.1567711649528784f, 86722.3403467334749201f, -66598.2652345418633509f,
     180329.498380501819718f, -27182.6254466733970467f, 192104.047790227984431f,
     -6046.8250112711035463f, 113057.05869159631492f, -724.581482791462469795f,
     38129.5594484818471461f, -43.3058660811817946037f, 7417.37624454689546708f,
     -0.999999999999998811143f, 809.193214954550328455f, -0.121013190657725568138e-18f,
     45.3058660811801465927f},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
     -0.000111507792921197858394f, -0.528611029520217142048e-6f,
     -0.00399167106081113256961f, 0.000131049900798434683324f,
     -0.0368031736257943745142f, 0.00427347600017103698101f,
     -0.245088216639761496153f, 0.056770677104207528384f,
     0.0320913665303559189999f, 0.37091387659397013215f,
     0.0865197248079397976498f, 1.0f}};

// A pair in FP32 (mixed-precision form, far pairs): the offsets are formed in
// FP64 in each kernel's own order, then everything runs in FP32.
template <bool SLP, bool DLP>
__device__ __forceinline__ void real_pair_f32(const RealArgs &a, const RealWarp &W,
                                              const float4 *tposff, int2 e,
                                              const float *e1f, const float4 &zxf,
                                              const float4 &zyf, float &s1, float &s2, float &d1,
                                              float &d2)
{
    const int s = e.x, slot = e.y & 0xff, k = (e.y >> 8) & 0xf, fl = e.y >> 12;
    const int2 tb = W.tbxy[slot];
    const int ux = tb.x + c_nb_dx[k], uy = tb.y + c_nb_dy[k];
    // The offset s - t + z from float-float positions, on the FP32 pipe: the
    // TwoSum of the high halves is exact, the image shift z (zxf = (z-.hi,
    // z-.lo, z+.hi, z+.lo)) cancels its head exactly (Sterbenz: the two are
    // within a factor of 2 across a periodic image), and the low-order terms
    // follow; one rounding to FP32 at the end.
    const float2 Sh = a.spf[s], Sl = a.spl[s];
    const float4 Tq = tposff[slot];
    const float2 zx = ux < 0 ? make_float2(zxf.x, zxf.y)
                             : (ux >= a.nx ? make_float2(zxf.z, zxf.w) : make_float2(0.f, 0.f));
    const float2 zy = uy < 0 ? make_float2(zyf.x, zyf.y)
                             : (uy >= a.ny ? make_float2(zyf.z, zyf.w) : make_float2(0.f, 0.f));
    float px, ex, py, ey;
    two_sum(Sh.x, -Tq.x, px, ex);
    two_sum(Sh.y, -Tq.y, py, ey);
    const float x1 = (px + zx.x) + ((ex + (Sl.x - Tq.z)) + zx.y);
    const float x2 = (py + zy.x) + ((ey + (Sl.y - Tq.w)) + zy.y);
    const float dxs = x1, dys = x2;
    const float xi2 = a.xi2f;
    if (SLP && (fl & 1)) {
        const float r2 = fmaf(dxs, dxs, dys * dys);
        const float x = r2 * xi2;
        const float ex = __expf(-x);
        const float ir2 = __frcp_rn(r2);
        const int set = x >= 16.f ? 0 : (x > 1.f ? 1 : 2);
        const float *c = e1f + 22 * set;
        const float z = set == 2 ? x : ir2 * (float)a.inv_xi2;
        float pa = c[0], pb = c[1];
#pragma unroll
        for (int i = 2; i < 22; i += 2) {
            pa = fmaf(z, pa, c[i]);
            pb = fmaf(z, pb, c[i + 1]);
        }
        const float E = set == 2 ? __fdividef(pa, pb) + x - __logf(x) - 0.66373538970947265625f
                                 : ex * (z + __fdividef(pa, pb + x));
        // coefficients: the high halves of the float-float copy (no FP64-rate conversion)
        const float f1 = a.coef_ff[(int64_t)a.ncf * s].x, f2 = a.coef_ff[(int64_t)a.ncf * s + 1].x;
        const float h = 0.5f * E, gq = ex * ir2 * fmaf(dxs, f2, -dys * f1);
        s1 = fmaf(h, f1, fmaf(gq, dys, s1));
        s2 = fmaf(h, f2, fmaf(-gq, dxs, s2));
    }
    if (DLP && (fl & 2)) {
        const float2 *Sc = a.coef_ff + (int64_t)a.ncf * s + a.doff_ff;
        const float S11 = Sc[0].x, S1221 = Sc[1].x, S22 = Sc[2].x;
        const float T1 = Sc[3].x, T2 = Sc[4].x;   // 3 S11 + S22, 3 S22 + S11
        const float r2 = fmaf(x1, x1, x2 * x2);
        const float x = r2 * xi2;
        const float ex = __expf(-x);
        const float ir2 = __frcp_rn(r2);
        const float fb = -4.f * (1.f + x) * ir2 * ir2;
        const float Q = fmaf(x1 * x1, S11, fmaf(x1 * x2, S1221, x2 * x2 * S22));
        const float A1 = fmaf(x1, T1, x2 * S1221);
        const float A2 = fmaf(x2, T2, x1 * S1221);
        const float fq = fb * Q, pf = 2.f * xi2;
        d1 = fmaf(ex, fmaf(fq, x1, pf * A1), d1);
        d2 = fmaf(ex, fmaf(fq, x2, pf * A2), d2);
    }
}

// A pair in float-float (FP64 form, far pairs 1 < xi^2 r^2 < 64): the offset
// is formed in FP64 (s - t, plus the image shift), split, and everything
// after runs on the FP32 pipe: r^2, x = xi^2 r^2, exp(-x) (Tang), 1/r^2
// (Newton), E1 = exp(-x) g(x), and the SLP / DLP contractions of real_pair.
template <bool SLP, bool DLP>
__device__ __forceinline__ void real_pair_ff(const RealArgs &a, const RealWarp &W, int2 e,
                                             const float2 *tabff, float2 xi2, float2 pf,
                                             float2 &s1, float2 &s2, float2 &d1, float2 &d2)
{
    const int s = e.x, slot = e.y & 0xff, k = (e.y >> 8) & 0xf, fl = e.y >> 12;
    const double2 S = a.sp[s];
    const double2 T = W.tpos[slot];
    // image shift of neighbour k of this pair's target (the FIFO outlives W.nbz)
    const int2 tb = W.tbxy[slot];
    const int ux = tb.x + c_nb_dx[k], uy = tb.y + c_nb_dy[k];
    double dx = S.x - T.x, dy = S.y - T.y;
    if (ux < 0 || ux >= a.nx || uy < 0 || uy >= a.ny) {   // across a periodic image
        dx += ux < 0 ? a.zxm : (ux >= a.nx ? a.zxp : 0.0);
        dy += uy < 0 ? a.zym : (uy >= a.ny ? a.zyp : 0.0);
    }
    const float2 x1 = ff_split(dx), x2 = ff_split(dy);
    const float2 r2 = ff_add(ff_sqr(x1), ff_sqr(x2));
    const float2 x = ff_mul(r2, xi2);
    const float2 ex = ff_exp_neg(x, tabff);
    const float2 ir2 = ff_rcp(r2);
    const float2 *cf = a.coef_ff + (int64_t)a.ncf * s;
    if (SLP && (fl & 1)) {
        const float2 f1 = cf[0], f2 = cf[1];
        const float2 h = ff_scale(ff_mul(ex, ff_g_e1(x, a.gtab)), 0.5f);
        const float2 gq = ff_mul(ff_mul(ex, ir2), ff_dot2(x1, f2, ff_neg(x2), f1));
        // the lane's sums as Dot2 accumulators (running float sum, float
        // compensation): each product's exact head and error go straight in,
        // and the pair renormalises the sum once (a lane may sum hundreds of
        // pairs of one target where the boxes are large)
        ff_dot_acc(h, f1, s1.x, s1.y);
        ff_dot_acc(gq, x2, s1.x, s1.y);
        ff_dot_acc(h, f2, s2.x, s2.y);
        ff_dot_acc(ff_neg(gq), x1, s2.x, s2.y);
        s1 = ff_norm(s1.x, s1.y);
        s2 = ff_norm(s2.x, s2.y);
    }
    if (DLP && (fl & 2)) {
        const float2 *Sc = cf + a.doff_ff;
        const float2 S11 = Sc[0], S1221 = Sc[1], S22 = Sc[2], T1 = Sc[3], T2 = Sc[4];
        const float2 fb = ff_scale(ff_mul(ff_add_f(x, 1.0f), ff_sqr(ir2)), -4.0f);
        const float2 Q = ff_dot3(ff_sqr(x1), S11, ff_mul(x1, x2), S1221, ff_sqr(x2), S22);
        const float2 A1 = ff_dot2(x1, T1, x2, S1221);
        const float2 A2 = ff_dot2(x2, T2, x1, S1221);
        const float2 fq = ff_mul(fb, Q);
        const float2 efq = ff_mul(ex, fq), epf = ff_mul(ex, pf);
        ff_dot_acc(efq, x1, d1.x, d1.y);
        ff_dot_acc(epf, A1, d1.x, d1.y);
        ff_dot_acc(efq, x2, d2.x, d2.y);
        ff_dot_acc(epf, A2, d2.x, d2.y);
        d1 = ff_norm(d1.x, d1.y);
        d2 = ff_norm(d2.x, d2.y);
    }
}

// Lane-side state of one pair FIFO.
struct PairQueue {
    int qn;               // entries queued (warp-uniform)
    unsigned enq, proc;   // entries enqueued / processed so far, mod 2^32 (warp-uniform)
    int tag;              // sequence number of the target this lane's sums belong to
    double s1, s2, d1, d2;
    float f1, f2, g1, g2; // FP32 sums of the mixed-precision form
    float2 h1, h2, k1, k2; // float-float sums of the FP64 form's far pairs
};

#ifndef SE2P_REAL_MINB
#define SE2P_REAL_MINB 6
#endif
template <bool SLP, bool DLP, int FORM>
__global__ void __launch_bounds__(kRealWarps * 32, SE2P_REAL_MINB) k_real(RealArgs a)
{
    constexpr bool MIXED = FORM == kFormF32;
    constexpr bool FF = FORM == kFormFF;
    // Shared arrays of one form only are sized 1 in the others: the
    // float-float form's 6 blocks per SM then fit the 132 KB shared-memory
    // carve-out, which leaves more of the SM's L1 to the source reads.
    __shared__ RealWarp warps[kRealWarps];
    __shared__ double tab[64];
    __shared__ float2 tabff[FF ? 64 : 1];
    __shared__ double e1s[66];
    __shared__ float e1f[MIXED ? 66 : 1];
    // FP32-grid form: target positions as float-float (hi.x, hi.y, lo.x, lo.y)
    __shared__ float4 tposff_s[kRealWarps][MIXED ? kRing : 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float4 *tposff = tposff_s[wid];
    for (int i = threadIdx.x; i < 64; i += blockDim.x) {
        tab[i] = c_exp_tab[i];
        if (FF) tabff[i] = ff_split(c_exp_tab[i]);
    }
    const float2 xi2ff = ff_split(a.xi2), pfff = ff_split(a.pf);
    // image shifts as float-float, for the FP32-grid form's offsets
    const float2 zmx = ff_split(a.zxm), zpx = ff_split(a.zxp);
    const float2 zmy = ff_split(a.zym), zpy = ff_split(a.zyp);
    const float4 zxf = make_float4(zmx.x, zmx.y, zpx.x, zpx.y);
    const float4 zyf = make_float4(zmy.x, zmy.y, zpy.x, zpy.y);
    // Queue 0 (the fast pairs): float-float pairs 1 < x < 64 with margins
    // for the FP32 pre-test; FP32-grid form, x > 1 (near pairs, E1 at small
    // argument, stay FP64 in both forms).
    const float xlo = FF ? 1.0001f : 1.0f, xhi = FF ? 63.9f : INFINITY;
    for (int i = threadIdx.x; i < 66; i += blockDim.x) {
        e1s[i] = (&c_e1[0][0])[i];
        if (MIXED) e1f[i] = (&c_e1f[0][0])[i];
    }
    __syncthreads();
    RealWarp &W = warps[wid];

    int head = 0, nfl = 0, gseq = 0;   // ring head slot, targets in flight, targets started
    PairQueue Q[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
        Q[j].qn = 0; Q[j].enq = 0; Q[j].proc = 0; Q[j].tag = -1;
        Q[j].s1 = Q[j].s2 = Q[j].d1 = Q[j].d2 = 0.0;
        Q[j].f1 = Q[j].f2 = Q[j].g1 = Q[j].g2 = 0.f;
        Q[j].h1 = Q[j].h2 = Q[j].k1 = Q[j].k2 = make_float2(0.f, 0.f);
    }

    // Evaluate the first cnt pairs of FIFO j (lanes >= cnt idle); lanes whose
    // sums belong to another target flush first.
    auto batch = [&](int j, int cnt) {
        PairQueue &P = Q[j];
        const int2 e = lane < cnt ? W.q[j][lane] : make_int2(0, -1);
        __syncwarp();
        if (lane < P.qn - cnt) W.q[j][lane] = W.q[j][lane + cnt];
        P.qn -= cnt;
        P.proc += cnt;
        int eseq = -1;
        if (e.y >= 0) eseq = gseq - nfl + (((e.y & 0xff) - head + kRing) % kRing);
        const bool fl = P.tag >= 0 && (lane >= cnt || P.tag != eseq);
        const bool f32 = MIXED && j == 0;
        const bool ffp = FF && j == 0;
        if (__any_sync(~0u, fl)) {
            const float2 z = make_float2(0.f, 0.f);
            if (ffp) {
                seg_flush_ff(W, lane, P.tag, fl ? P.h1 : z, fl ? P.h2 : z, fl ? P.k1 : z,
                             fl ? P.k2 : z);
            } else if (f32) {
                seg_flush_f(W, lane, P.tag, fl ? P.f1 : 0.f, fl ? P.f2 : 0.f, fl ? P.g1 : 0.f,
                            fl ? P.g2 : 0.f);
            } else {
                seg_flush(W, lane, P.tag, fl ? P.s1 : 0.0, fl ? P.s2 : 0.0, fl ? P.d1 : 0.0,
                          fl ? P.d2 : 0.0);
            }
            if (fl) {
                P.s1 = P.s2 = P.d1 = P.d2 = 0.0;
                P.f1 = P.f2 = P.g1 = P.g2 = 0.f;
                P.h1 = P.h2 = P.k1 = P.k2 = make_float2(0.f, 0.f);
                P.tag = -1;
            }
        }
        if (lane < cnt) {
            if (f32) real_pair_f32<SLP, DLP>(a, W, tposff, e, e1f, zxf, zyf, P.f1, P.f2, P.g1, P.g2);
            else if (ffp)
                real_pair_ff<SLP, DLP>(a, W, e, tabff, xi2ff, pfff, P.h1, P.h2, P.k1, P.k2);
            else real_pair<SLP, DLP>(a, W, e, tab, e1s, P.s1, P.s2, P.d1, P.d2);
            P.tag = eseq;
        }
    };
    // Retire finished targets in order (all of them after a full flush).
    auto retire = [&](bool all) {
        while (nfl > 0 && (all || ((int)(Q[0].proc - W.tend[0][head]) >= 32 &&
                                   (int)(Q[1].proc - W.tend[1][head]) >= 32))) {
            if (lane < 4 && (lane < 2 ? SLP : DLP)) {
                const int64_t t = W.tidx[head];
                double v = W.acc[head][lane];
                if (FF || MIXED) v += ff_to_double(W.accf[head][lane]);
                double *u = reinterpret_cast<double *>(lane < 2 ? a.u_slp : a.u_dlp);
                u[2 * t + (lane & 1)] = v;
            }
            head = (head + 1) % kRing;
            nfl--;
        }
        __syncwarp();
    };
    auto drain = [&]() {
#pragma unroll
        for (int j = 0; j < 2; j++) {
            batch(j, Q[j].qn);
            const int key = Q[j].tag >= 0 ? Q[j].tag : 0x7fffffff;
            if (MIXED && j == 0)
                seg_flush_f(W, lane, key, Q[j].f1, Q[j].f2, Q[j].g1, Q[j].g2);
            else if (FF && j == 0)
                seg_flush_ff(W, lane, key, Q[j].h1, Q[j].h2, Q[j].k1, Q[j].k2);
            else
                seg_flush(W, lane, key, Q[j].s1, Q[j].s2, Q[j].d1, Q[j].d2);
            Q[j].s1 = Q[j].s2 = Q[j].d1 = Q[j].d2 = 0.0;
            Q[j].f1 = Q[j].f2 = Q[j].g1 = Q[j].g2 = 0.f;
            Q[j].h1 = Q[j].h2 = Q[j].k1 = Q[j].k2 = make_float2(0.f, 0.f);
            Q[j].tag = -1;
        }
        retire(true);
    };

    // Each block takes one contiguous run of the box-sorted targets, and its
    // warps interleave over it: a warp's consecutive targets mostly share a
    // box (so its neighbour-box set is built once per box), and the block's
    // warps read the same sources at the same time.
    // (the cell lists hold int indices, so ntar < 2^31)
    const int per = (int)((a.ntar + gridDim.x - 1) / gridDim.x);
    const int t_end = (int)min(a.ntar, (int64_t)blockIdx.x * per + per);
    if (lane == 0) W.curbox = -1;
    __syncwarp();
    for (int t = (int)blockIdx.x * per + wid; t < t_end; t += kRealWarps) {
        if (nfl == kRing) drain();
        const int slot = (head + nfl) % kRing;
        nfl++;
        gseq++;
        const int tb = a.tbox[t];
        const double2 T = a.tp[t];
        const float2 Tf = a.tpf[t];
        const bool newbox = tb != W.curbox;                // (warp-uniform)
        if (newbox) {
            __syncwarp();
            if (lane == 0) {
                W.curbox = tb;
                W.curbxy = make_int2(tb % a.nx, tb / a.nx);
            }
            __syncwarp();
        }
        const int2 cur_bxy = W.curbxy;
        if (lane < 4) {
            W.acc[slot][lane] = 0.0;
            W.accf[slot][lane] = make_float2(0.f, 0.f);
        }
        if (lane == 0) {
            W.tpos[slot] = T;
            W.tbxy[slot] = cur_bxy;
            W.tidx[slot] = t;
            if (MIXED) {
                const float2 tl = a.tpl[t];
                tposff[slot] = make_float4(Tf.x, Tf.y, tl.x, tl.y);
            }
        }
        // neighbour boxes: first source, counts -> list prefix, image shift
        // (once per box), and the pre-test band, which depends on the target
        if (newbox) {
            int cntk = 0;
            if (lane < 9) {
                const int ux = cur_bxy.x + c_nb_dx[lane], uy = cur_bxy.y + c_nb_dy[lane];
                const int wx = (ux + a.nx) % a.nx, wy = (uy + a.ny) % a.ny;
                const int sb = wy * a.nx + wx;
                const int b0 = a.sstart[sb];
                cntk = a.sstart[sb + 1] - b0;
                W.nbs[lane] = b0;
                const double zx = ux < 0 ? a.zxm : (ux >= a.nx ? a.zxp : 0.0);
                const double zy = uy < 0 ? a.zym : (uy >= a.ny ? a.zyp : 0.0);
                W.nbz[lane] = make_double2(zx, zy);
                W.nbzf[lane] = make_float2((float)zx, (float)zy);
            }
            int incl = cntk;
#pragma unroll
            for (int o = 1; o < 16; o <<= 1) {
                const int v = __shfl_up_sync(~0u, incl, o);
                if (lane >= o) incl += v;
            }
            if (lane < 9) W.nbp[lane + 1] = incl;
            if (lane == 0) W.nbp[0] = 0;
            __syncwarp();
        }
        if (lane < 9) {
            const float2 zf = W.nbzf[lane];
            W.nbe[lane] = make_float2(0x1p-22f * (fabsf(Tf.x) + fabsf(zf.x)),
                                      0x1p-22f * (fabsf(Tf.y) + fabsf(zf.y)));
        }
        __syncwarp();
        const int total = W.nbp[9];
        unsigned nslp = 0, ndlp = 0;
        int kc = 0;   // neighbour box of this lane's candidate (v only grows)
        for (int v0 = 0; v0 < total; v0 += 32) {
            const int v = v0 + lane;
            int fl = 0, s = 0, k = kc;
            bool nearp = false;
            if (v < total) {
                while (v >= W.nbp[k + 1]) k++;
                kc = k;
                s = W.nbs[k] + (v - W.nbp[k]);
                if (k == 0) {
                    // own box, no cutoff.  Distinct FP32 images imply an FP64
                    // r2 > 0 (the offset is then >= 2^-150, its square normal),
                    // so only r2f == 0 (or NaN) needs the reference's exact r2.
                    const float2 Sf = a.spf[s];
                    const float dxf = Tf.x - Sf.x, dyf = Tf.y - Sf.y;
                    float r2f = dxf * dxf + dyf * dyf;
                    bool self = false;
                    if (!(r2f > 0.0f)) {
                        const double2 S = a.sp[s];
                        const double dx = xsub(T.x, S.x), dy = xsub(T.y, S.y);
                        const double r2 = xadd(xmul(dx, dx), xmul(dy, dy));
                        self = r2 == 0.0;
                        r2f = (float)r2;
                    }
                    if (self) {
                        // SLP self term (mex_stokes_slp_real.cpp:161-163); DLP skips r2 == 0.
                        if (SLP) {
                            const double *f = a.coef + (int64_t)a.nc * s;
                            atomicAdd(&W.acc[slot][0], a.self_c * f[0]);
                            atomicAdd(&W.acc[slot][1], a.self_c * f[1]);
                        }
                    } else {
                        fl = 3;
                        const float xf = r2f * a.xi2f;
                        nearp = !(xf > xlo && xf < xhi);
                    }
                } else {
                    const float2 Sf = a.spf[s];
                    const float2 zf = W.nbzf[k];
                    const float dxf = Sf.x - (Tf.x - zf.x), dyf = Sf.y - (Tf.y - zf.y);
                    const float r2f = dxf * dxf + dyf * dyf;
                    // |r2f - r2| bound for both offset forms (3 roundings per
                    // coordinate, then squaring and summing), doubled.
                    const float2 nbe = W.nbe[k];
                    const float ex = fmaf(0x1p-22f, fabsf(Sf.x), nbe.x);
                    const float ey = fmaf(0x1p-22f, fabsf(Sf.y), nbe.y);
                    const float band = 2.0f * (ex * (2.0f * fabsf(dxf) + ex) +
                                               ey * (2.0f * fabsf(dyf) + ey) + 0x1p-22f * r2f);
                    const float xf = r2f * a.xi2f;
                    nearp = !(xf > xlo && xf < xhi);
                    if (r2f + band < a.cut2f) {
                        fl = 3;
                    } else if (!(r2f - band >= a.cut2f)) {
                        // near the cutoff (or non-finite): the reference's exact tests
                        const double2 S = a.sp[s];
                        const double2 z = W.nbz[k];
                        if (SLP) {
                            const double dx = xsub(S.x, xsub(T.x, z.x));
                            const double dy = xsub(S.y, xsub(T.y, z.y));
                            if (xadd(xmul(dx, dx), xmul(dy, dy)) < a.cut2) fl |= 1;
                        }
                        if (DLP) {
                            const double x1 = xadd(xsub(S.x, T.x), z.x);
                            const double x2 = xadd(xsub(S.y, T.y), z.y);
                            if (xadd(xmul(x1, x1), xmul(x2, x2)) < a.cut2) fl |= 2;
                        }
                    }
                }
            }
            if (!SLP) fl &= 2;
            if (!DLP) fl &= 1;
            if (a.counters) {                        // (warp-uniform)
                nslp += __popc(__ballot_sync(~0u, (fl & 1) != 0));
                ndlp += __popc(__ballot_sync(~0u, (fl & 2) != 0));
            }
            const int2 ent = make_int2(s, slot | (k << 8) | (fl << 12));
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const bool mine = fl != 0 && nearp == (j == 1);
                const unsigned m = __ballot_sync(~0u, mine);
                if (mine) W.q[j][Q[j].qn + __popc(m & ((1u << lane) - 1u))] = ent;
                Q[j].qn += __popc(m);
                Q[j].enq += __popc(m);
            }
            __syncwarp();
            if (Q[0].qn >= 32) batch(0, 32);
            if (Q[1].qn >= 32) batch(1, 32);
        }
        if (lane == 0) {
            W.tend[0][slot] = Q[0].enq;
            W.tend[1][slot] = Q[1].enq;
            if (a.counters) {                        // (diagnostic counts, per target)
                atomicAdd(a.counters, (unsigned long long)total);
                if (SLP) atomicAdd(a.counters + 1, (unsigned long long)nslp);
                if (DLP) atomicAdd(a.counters + 2, (unsigned long long)ndlp);
            }
        }
        __syncwarp();
        retire(false);
    }
    drain();
}

template __global__ void k_real<true, false, kFormFP64>(RealArgs);
template __global__ void k_real<false, true, kFormFP64>(RealArgs);
template __global__ void k_real<true, true, kFormFP64>(RealArgs);
template __global__ void k_real<true, false, kFormF32>(RealArgs);
template __global__ void k_real<false, true, kFormF32>(RealArgs);
template __global__ void k_real<true, true, kFormF32>(RealArgs);
template __global__ void k_real<true, false, kFormFF>(RealArgs);
template __global__ void k_real<false, true, kFormFF>(RealArgs);
template __global__ void k_real<true, true, kFormFF>(RealArgs);

// ===========================================================================
// Real-space adjoint (source-centric).
//
// For J = sum_t w_slp(t).u_slp(t) + w_dlp(t).u_dlp(t) the real-space part
// contributes, per forward source s and every pair (t, s) of the forward's
// own pair set (same boxes, same exact cutoff arithmetic, same image shift z
// of the source seen from the target's box):
//   SLP  dJ/df_s   += A(d) w_t                 (A symmetric: the forward kernel)
//        dJ/dy_s   += grad_d [w_t^T A(d) f_s],  E1'(x) = -exp(-x)/x
//   DLP  dJ/dS_s   += d(w_t . v(d; S))/dS       (S = (S11, S12+S21, S22))
//        dJ/dy_s   -= grad_d [w_t . v(d; S_s)]  (the DLP enters u with a minus)
// with d = y_s + z - x_t in each kernel's own rounding order.  One warp per
// forward source walks the 3x3 neighbourhood of forward targets through the
// same two pair FIFOs as k_real; lanes keep 7 sums per source.
// ===========================================================================
constexpr int kAdjVals = 7;   // gf1, gf2, gS11, gS1221, gS22, gy1, gy2

constexpr int kAdjWarps = 4;   // warps per block of k_real_adj (shared memory per warp ~6.5 KB)

struct AdjWarp {
    int2 q[2][64];
    double acc[kRing][kAdjVals + 1];
    float2 accf[kRing][kAdjVals];    // the same from float-float pairs (FP64 form, queue 0)
    double2 pos[kRing];
    int2 bxy[kRing];            // the source's box as (column, row)
    long long idx[kRing];
    long long tend[2][kRing];
    int nbs[9], nbp[10];
    double2 nbz[9];
    float2 nbzf[9];
};

template <int NV, class Acc>
__device__ __forceinline__ void seg_flush_n(Acc &accs, int lane, int key, double *v)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int ko = __shfl_up_sync(~0u, key, o);
        double a[NV];
#pragma unroll
        for (int i = 0; i < NV; i++) a[i] = __shfl_up_sync(~0u, v[i], o);
        if (lane >= o && ko == key) {
#pragma unroll
            for (int i = 0; i < NV; i++) v[i] += a[i];
        }
    }
    const int kn = __shfl_down_sync(~0u, key, 1);
    if (key >= 0 && key != 0x7fffffff && (lane == 31 || kn != key)) {
        double *a = accs[key % kRing];
#pragma unroll
        for (int i = 0; i < NV; i++) a[i] += v[i];
    }
    __syncwarp();
}

// seg_flush_n for float-float sums, into the float-float ring.
template <int NV, class Acc>
__device__ __forceinline__ void seg_flush_n_ff(Acc &accs, int lane, int key, float2 *v)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int ko = __shfl_up_sync(~0u, key, o);
        float2 a[NV];
#pragma unroll
        for (int i = 0; i < NV; i++) {
            a[i].x = __shfl_up_sync(~0u, v[i].x, o);
            a[i].y = __shfl_up_sync(~0u, v[i].y, o);
        }
        if (lane >= o && ko == key) {
            // heads by TwoSum, tails and errors carried unnormalised (as in seg_flush_ff)
#pragma unroll
            for (int i = 0; i < NV; i++) {
                float s, e;
                two_sum(v[i].x, a[i].x, s, e);
                v[i] = make_float2(s, v[i].y + a[i].y + e);
            }
        }
    }
    const int kn = __shfl_down_sync(~0u, key, 1);
    if (key >= 0 && key != 0x7fffffff && (lane == 31 || kn != key)) {
        float2 *a = accs[key % kRing];
#pragma unroll
        for (int i = 0; i < NV; i++) a[i] = ff_add(a[i], ff_norm(v[i].x, v[i].y));
    }
    __syncwarp();
}

template <bool SLP, bool DLP>
__device__ __forceinline__ void adj_pair(const RealArgs &a, const AdjWarp &W, int2 e,
                                         const double *tab, const double *e1s, double *g)
{
    const int t = e.x, slot = e.y & 0xff, k = (e.y >> 8) & 0xf, fl = e.y >> 12;
    const double2 T = a.tp[t];                  // forward target (inner point)
    const double2 S = W.pos[slot];              // forward source (outer point)
    // image shift of the source seen from the target's box: the target sits
    // in box wrap(source box + offset k), so the unwrapped source box
    // (target box - offset k) lies below 0 exactly when source box + offset
    // reached past the last box, and beyond it when that went below 0
    const int2 b = W.bxy[slot];
    const int tx = b.x + c_nb_dx[k], ty = b.y + c_nb_dy[k];
    const double zx = tx >= a.nx ? a.zxm : (tx < 0 ? a.zxp : 0.0);
    const double zy = ty >= a.ny ? a.zym : (ty < 0 ? a.zyp : 0.0);
    const double x1 = (S.x - T.x) + zx, x2 = (S.y - T.y) + zy;          // DLP form
    const double d1 = S.x - (T.x - zx), d2 = S.y - (T.y - zy);          // SLP form
    const double *wt = a.wcoef + 4 * (int64_t)t;                         // w_slp, w_dlp of t
    const double *cs = a.coef + (int64_t)a.nc * W.idx[slot];            // outer coefficients
    if (SLP && (fl & 1)) {
        const double r2 = fma(d1, d1, d2 * d2);
        const double x = r2 * a.xi2;
        const double ex = exp_neg(x, tab);
        const double ir2 = rcp_nr(r2);
        const int set = x >= 16.0 ? 0 : (x > 1.0 ? 1 : 2);
        const double *c = e1s + 22 * set;
        const double z = set == 2 ? x : ir2 * a.inv_xi2;
        double pa = c[0], pb = c[1];
#pragma unroll
        for (int i = 2; i < 22; i += 2) {
            pa = fma(z, pa, c[i]);
            pb = fma(z, pb, c[i + 1]);
        }
        const double den = set == 2 ? pb : pb + x;
        const double qv = pa * rcp_nr(den);
        const double E = set == 2 ? qv + x - log(x) - 0.66373538970947265625 : ex * (z + qv);
        const double w1 = wt[0], w2 = wt[1], f1 = cs[0], f2 = cs[1];
        const double h = 0.5 * E, gg = ex * ir2;
        const double gq = gg * fma(d1, w2, -d2 * w1);
        g[0] = fma(h, w1, fma(gq, d2, g[0]));
        g[1] = fma(h, w2, fma(-gq, d1, g[1]));
        // grad_d [w^T A(d) f]
        const double aa = fma(d1, w1, d2 * w2), bb = fma(d1, f1, d2 * f2), cc = fma(w1, f1, w2 * f2);
        const double ab = aa * bb;
        const double kap = ex * (-cc * ir2 - 2.0 * a.xi2 * fma(ab, ir2, -cc) - 2.0 * ab * ir2 * ir2);
        g[5] = fma(kap, d1, fma(gg, fma(bb, w1, aa * f1), g[5]));
        g[6] = fma(kap, d2, fma(gg, fma(bb, w2, aa * f2), g[6]));
    }
    if (DLP && (fl & 2)) {
        const double r2 = fma(x1, x1, x2 * x2);
        const double x = r2 * a.xi2;
        const double ex = exp_neg(x, tab);
        const double ir2 = rcp_nr(r2);
        const double w1 = wt[2], w2 = wt[3];
        const double *Sc = cs + a.doff;
        const double S11 = Sc[0], S1221 = Sc[1], S22 = Sc[2];
        const double fb = -4.0 * (1.0 + x) * ir2 * ir2;
        const double fbp = 4.0 * (2.0 + x) * ir2 * ir2 * ir2;     // d fb / d r2
        const double pf = a.pf;
        const double wd = fma(w1, x1, w2 * x2);
        // d(w.v)/dS
        const double fw = fb * wd;
        g[2] = fma(ex, fma(fw * x1, x1, pf * fma(3.0 * w1, x1, w2 * x2)), g[2]);
        g[3] = fma(ex, fma(fw * x1, x2, pf * fma(w1, x2, w2 * x1)), g[3]);
        g[4] = fma(ex, fma(fw * x2, x2, pf * fma(w1, x1, 3.0 * w2 * x2)), g[4]);
        // grad_d [w.v(d; S)], subtracted (the DLP enters u_dlp with a minus)
        const double B11 = fma(3.0, S11, S22), B22 = fma(3.0, S22, S11);
        const double Q = fma(x1 * x1, S11, fma(x1 * x2, S1221, x2 * x2 * S22));
        const double A1 = fma(B11, x1, S1221 * x2), A2 = fma(S1221, x1, B22 * x2);
        const double wA = fma(w1, A1, w2 * A2);
        const double Bw1 = fma(B11, w1, S1221 * w2), Bw2 = fma(S1221, w1, B22 * w2);
        const double Sd1 = fma(2.0 * S11, x1, S1221 * x2), Sd2 = fma(S1221, x1, 2.0 * S22 * x2);
        const double radial = -2.0 * a.xi2 * fma(fb * Q, wd, pf * wA) + 2.0 * fbp * Q * wd;
        const double fbQ = fb * Q, fbw = fb * wd;
        g[5] -= ex * (radial * x1 + fbw * Sd1 + fbQ * w1 + pf * Bw1);
        g[6] -= ex * (radial * x2 + fbw * Sd2 + fbQ * w2 + pf * Bw2);
    }
}

// adj_pair in float-float for the far pairs (1 < xi^2 r^2 < 64) of the FP64
// form: same terms, same pair, evaluated as in real_pair_ff.
template <bool SLP, bool DLP>
__device__ __forceinline__ void adj_pair_ff(const RealArgs &a, const AdjWarp &W, int2 e,
                                            const float2 *tabff, float2 xi2, float2 pf,
                                            float2 *g)
{
    const int t = e.x, slot = e.y & 0xff, k = (e.y >> 8) & 0xf, fl = e.y >> 12;
    const double2 T = a.tp[t];
    const double2 S = W.pos[slot];
    // (the image shift as in adj_pair)
    const int2 b = W.bxy[slot];
    const int tx = b.x + c_nb_dx[k], ty = b.y + c_nb_dy[k];
    const double zx = tx >= a.nx ? a.zxm : (tx < 0 ? a.zxp : 0.0);
    const double zy = ty >= a.ny ? a.zym : (ty < 0 ? a.zyp : 0.0);
    const float2 x1 = ff_split((S.x - T.x) + zx), x2 = ff_split((S.y - T.y) + zy);
    const float2 r2 = ff_add(ff_sqr(x1), ff_sqr(x2));
    const float2 x = ff_mul(r2, xi2);
    const float2 ex = ff_exp_neg(x, tabff);
    const float2 ir2 = ff_rcp(r2);
    const double *wt = a.wcoef + 4 * (int64_t)t;
    const double *cs = a.coef + (int64_t)a.nc * W.idx[slot];
    if (SLP && (fl & 1)) {
        const float2 w1 = ff_split(wt[0]), w2 = ff_split(wt[1]);
        const float2 f1 = ff_split(cs[0]), f2 = ff_split(cs[1]);
        const float2 h = ff_scale(ff_mul(ex, ff_g_e1(x, a.gtab)), 0.5f);
        const float2 gg = ff_mul(ex, ir2);
        const float2 gq = ff_mul(gg, ff_sub(ff_mul(x1, w2), ff_mul(x2, w1)));
        g[0] = ff_add(g[0], ff_add(ff_mul(h, w1), ff_mul(gq, x2)));
        g[1] = ff_add(g[1], ff_sub(ff_mul(h, w2), ff_mul(gq, x1)));
        const float2 aa = ff_add(ff_mul(x1, w1), ff_mul(x2, w2));
        const float2 bb = ff_add(ff_mul(x1, f1), ff_mul(x2, f2));
        const float2 cc = ff_add(ff_mul(w1, f1), ff_mul(w2, f2));
        const float2 ab = ff_mul(aa, bb);
        const float2 abr = ff_mul(ab, ir2);
        // kap = ex (-cc ir2 - 2 xi2 (ab ir2 - cc) - 2 ab ir2^2)
        float2 kp = ff_neg(ff_mul(cc, ir2));
        kp = ff_sub(kp, ff_scale(ff_mul(xi2, ff_sub(abr, cc)), 2.0f));
        kp = ff_sub(kp, ff_scale(ff_mul(abr, ir2), 2.0f));
        const float2 kap = ff_mul(ex, kp);
        g[5] = ff_add(g[5], ff_add(ff_mul(kap, x1),
                                   ff_mul(gg, ff_add(ff_mul(bb, w1), ff_mul(aa, f1)))));
        g[6] = ff_add(g[6], ff_add(ff_mul(kap, x2),
                                   ff_mul(gg, ff_add(ff_mul(bb, w2), ff_mul(aa, f2)))));
    }
    if (DLP && (fl & 2)) {
        const float2 w1 = ff_split(wt[2]), w2 = ff_split(wt[3]);
        const double *Sc = cs + a.doff;
        const float2 S11 = ff_split(Sc[0]), S1221 = ff_split(Sc[1]), S22 = ff_split(Sc[2]);
        const float2 ir4 = ff_sqr(ir2);
        const float2 fb = ff_scale(ff_mul(ff_add_f(x, 1.0f), ir4), -4.0f);
        const float2 fbp = ff_scale(ff_mul(ff_add_f(x, 2.0f), ff_mul(ir4, ir2)), 4.0f);
        const float2 wd = ff_add(ff_mul(w1, x1), ff_mul(w2, x2));
        const float2 fw = ff_mul(fb, wd);
        const float2 fwx1 = ff_mul(fw, x1), fwx2 = ff_mul(fw, x2);
        const float2 w1x1 = ff_mul(w1, x1), w2x2 = ff_mul(w2, x2);
        const float2 w1x2 = ff_mul(w1, x2), w2x1 = ff_mul(w2, x1);
        // d(w.v)/dS
        g[2] = ff_add(g[2], ff_mul(ex, ff_add(ff_mul(fwx1, x1),
                                              ff_mul(pf, ff_add(ff_mul_f(w1x1, 3.0f), w2x2)))));
        g[3] = ff_add(g[3], ff_mul(ex, ff_add(ff_mul(fwx1, x2), ff_mul(pf, ff_add(w1x2, w2x1)))));
        g[4] = ff_add(g[4], ff_mul(ex, ff_add(ff_mul(fwx2, x2),
                                              ff_mul(pf, ff_add(w1x1, ff_mul_f(w2x2, 3.0f))))));
        // grad_d [w.v(d; S)], subtracted
        const float2 B11 = ff_add(ff_mul_f(S11, 3.0f), S22), B22 = ff_add(ff_mul_f(S22, 3.0f), S11);
        const float2 Q = ff_add(ff_add(ff_mul(ff_sqr(x1), S11), ff_mul(ff_mul(x1, x2), S1221)),
                                ff_mul(ff_sqr(x2), S22));
        const float2 A1 = ff_add(ff_mul(B11, x1), ff_mul(S1221, x2));
        const float2 A2 = ff_add(ff_mul(S1221, x1), ff_mul(B22, x2));
        const float2 wA = ff_add(ff_mul(w1, A1), ff_mul(w2, A2));
        const float2 Bw1 = ff_add(ff_mul(B11, w1), ff_mul(S1221, w2));
        const float2 Bw2 = ff_add(ff_mul(S1221, w1), ff_mul(B22, w2));
        const float2 Sd1 = ff_add(ff_scale(ff_mul(S11, x1), 2.0f), ff_mul(S1221, x2));
        const float2 Sd2 = ff_add(ff_mul(S1221, x1), ff_scale(ff_mul(S22, x2), 2.0f));
        const float2 fbQ = ff_mul(fb, Q);
        const float2 radial = ff_add(ff_scale(ff_mul(xi2, ff_add(ff_mul(fbQ, wd), ff_mul(pf, wA))), -2.0f),
                                     ff_scale(ff_mul(ff_mul(fbp, Q), wd), 2.0f));
        const float2 r1 = ff_add(ff_add(ff_mul(radial, x1), ff_mul(fw, Sd1)),
                                 ff_add(ff_mul(fbQ, w1), ff_mul(pf, Bw1)));
        const float2 r2b = ff_add(ff_add(ff_mul(radial, x2), ff_mul(fw, Sd2)),
                                  ff_add(ff_mul(fbQ, w2), ff_mul(pf, Bw2)));
        g[5] = ff_sub(g[5], ff_mul(ex, r1));
        g[6] = ff_sub(g[6], ff_mul(ex, r2b));
    }
}

template <bool SLP, bool DLP, int FORM>
__global__ void __launch_bounds__(kAdjWarps * 32, 5) k_real_adj(RealArgs a)
{
    constexpr bool FF = FORM == kFormFF;
    __shared__ AdjWarp warps[kAdjWarps];
    __shared__ double tab[64];
    __shared__ float2 tabff[64];
    __shared__ double e1s[66];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < 64; i += blockDim.x) {
        tab[i] = c_exp_tab[i];
        tabff[i] = ff_split(c_exp_tab[i]);
    }
    for (int i = threadIdx.x; i < 66; i += blockDim.x) e1s[i] = (&c_e1[0][0])[i];
    __syncthreads();
    const float2 xi2ff = ff_split(a.xi2), pfff = ff_split(a.pf);
    // queue 0: far pairs (float-float in the FF form), queue 1: the rest in FP64
    const float xlo = FF ? 1.0001f : 1.0f, xhi = FF ? 63.9f : INFINITY;
    AdjWarp &W = warps[wid];
    const int64_t nw = (int64_t)gridDim.x * kAdjWarps;
    int head = 0, nfl = 0, gseq = 0;
    int qn[2] = {0, 0}, tag[2] = {-1, -1};
    long long enq[2] = {0, 0}, proc[2] = {0, 0};
    double v[2][kAdjVals];
    float2 vf[kAdjVals];
#pragma unroll
    for (int i = 0; i < kAdjVals; i++) vf[i] = make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
        for (int i = 0; i < kAdjVals; i++) v[j][i] = 0.0;

    auto batch = [&](int j, int cnt) {
        const int2 e = lane < cnt ? W.q[j][lane] : make_int2(0, -1);
        __syncwarp();
        if (lane < qn[j] - cnt) W.q[j][lane] = W.q[j][lane + cnt];
        qn[j] -= cnt;
        proc[j] += cnt;
        int eseq = -1;
        if (e.y >= 0) eseq = gseq - nfl + (((e.y & 0xff) - head + kRing) % kRing);
        const bool fl = tag[j] >= 0 && (lane >= cnt || tag[j] != eseq);
        const bool ffq = FF && j == 0;
        if (__any_sync(~0u, fl)) {
            if (ffq) {
                float2 tf[kAdjVals];
#pragma unroll
                for (int i = 0; i < kAdjVals; i++) tf[i] = fl ? vf[i] : make_float2(0.f, 0.f);
                seg_flush_n_ff<kAdjVals>(W.accf, lane, tag[j], tf);
            } else {
                double tmp[kAdjVals];
#pragma unroll
                for (int i = 0; i < kAdjVals; i++) tmp[i] = fl ? v[j][i] : 0.0;
                seg_flush_n<kAdjVals>(W.acc, lane, tag[j], tmp);
            }
            if (fl) {
#pragma unroll
                for (int i = 0; i < kAdjVals; i++) {
                    v[j][i] = 0.0;
                    if (ffq) vf[i] = make_float2(0.f, 0.f);   // vf holds queue 0 only
                }
                tag[j] = -1;
            }
        }
        if (lane < cnt) {
            if (ffq) adj_pair_ff<SLP, DLP>(a, W, e, tabff, xi2ff, pfff, vf);
            else adj_pair<SLP, DLP>(a, W, e, tab, e1s, v[j]);
            tag[j] = eseq;
        }
    };
    auto retire = [&](bool all) {
        while (nfl > 0 && (all || (proc[0] >= W.tend[0][head] + 32 &&
                                   proc[1] >= W.tend[1][head] + 32))) {
            if (lane < kAdjVals) {
                double v = W.acc[head][lane];
                if (FF) v += ff_to_double(W.accf[head][lane]);
                a.gout[kAdjVals * W.idx[head] + lane] = v;
            }
            head = (head + 1) % kRing;
            nfl--;
        }
        __syncwarp();
    };
    auto drain = [&]() {
#pragma unroll
        for (int j = 0; j < 2; j++) {
            batch(j, qn[j]);
            const int key = tag[j] >= 0 ? tag[j] : 0x7fffffff;
            if (FF && j == 0) {
                seg_flush_n_ff<kAdjVals>(W.accf, lane, key, vf);
            } else {
                seg_flush_n<kAdjVals>(W.acc, lane, key, v[j]);
            }
#pragma unroll
            for (int i = 0; i < kAdjVals; i++) {
                v[j][i] = 0.0;
                vf[i] = make_float2(0.f, 0.f);
            }
            tag[j] = -1;
        }
        retire(true);
    };

    // outer loop over forward sources (sorted), inner candidates are forward targets
    for (int64_t s = (int64_t)blockIdx.x * kAdjWarps + wid; s < a.nouter; s += nw) {
        if (nfl == kRing) drain();
        const int slot = (head + nfl) % kRing;
        nfl++;
        gseq++;
        const int sbx = a.obox[s];
        const double2 Sp = a.sp[s];
        const float2 Sf = a.spf[s];
        if (lane < kAdjVals + 1) W.acc[slot][lane] = 0.0;
        if (lane < kAdjVals) W.accf[slot][lane] = make_float2(0.f, 0.f);
        if (lane == 0) {
            W.pos[slot] = Sp;
            W.bxy[slot] = make_int2(sbx % a.nx, sbx / a.nx);
            W.idx[slot] = s;
        }
        int cntk = 0;
        if (lane < 9) {
            // target box at offset k from the source box
            const int ux = sbx % a.nx + c_nb_dx[lane], uy = sbx / a.nx + c_nb_dy[lane];
            const int wx = (ux + a.nx) % a.nx, wy = (uy + a.ny) % a.ny;
            const int tb = wy * a.nx + wx;
            const int b0 = a.sstart[tb];           // target cell list
            cntk = a.sstart[tb + 1] - b0;
            W.nbs[lane] = b0;
            // source image shift seen from that target box (box tb, offset -k)
            const int vx = wx - c_nb_dx[lane], vy = wy - c_nb_dy[lane];
            const double zx = vx < 0 ? a.zxm : (vx >= a.nx ? a.zxp : 0.0);
            const double zy = vy < 0 ? a.zym : (vy >= a.ny ? a.zyp : 0.0);
            W.nbz[lane] = make_double2(zx, zy);
            W.nbzf[lane] = make_float2((float)zx, (float)zy);
        }
        int incl = cntk;
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) {
            const int vv = __shfl_up_sync(~0u, incl, o);
            if (lane >= o) incl += vv;
        }
        if (lane < 9) W.nbp[lane + 1] = incl;
        if (lane == 0) W.nbp[0] = 0;
        __syncwarp();
        const int total = W.nbp[9];
        int kc = 0;   // neighbour box of this lane's candidate (vi only grows)
        for (int v0 = 0; v0 < total; v0 += 32) {
            const int vi = v0 + lane;
            int fl = 0, t = 0, k = kc;
            bool nearp = false;
            if (vi < total) {
                while (vi >= W.nbp[k + 1]) k++;
                kc = k;
                t = W.nbs[k] + (vi - W.nbp[k]);
                if (k == 0) {
                    const double2 T = a.tp[t];
                    const double dx = xsub(T.x, Sp.x), dy = xsub(T.y, Sp.y);
                    const double r2 = xadd(xmul(dx, dx), xmul(dy, dy));
                    if (r2 == 0.0) {
                        // SLP self term: d/df of self_c f.w (mex_stokes_slp_real.cpp:161-163)
                        if (SLP) {
                            atomicAdd(&W.acc[slot][0], a.self_c * a.wcoef[4 * (int64_t)t]);
                            atomicAdd(&W.acc[slot][1], a.self_c * a.wcoef[4 * (int64_t)t + 1]);
                        }
                    } else {
                        fl = 3;
                        const float xf = (float)r2 * a.xi2f;
                        nearp = !(xf > xlo && xf < xhi);
                    }
                } else {
                    const float2 Tf = a.tpf[t];
                    const float2 zf = W.nbzf[k];
                    const float dxf = Sf.x - (Tf.x - zf.x), dyf = Sf.y - (Tf.y - zf.y);
                    const float r2f = dxf * dxf + dyf * dyf;
                    const float ex = 0x1p-22f * (fabsf(Sf.x) + fabsf(Tf.x) + fabsf(zf.x));
                    const float ey = 0x1p-22f * (fabsf(Sf.y) + fabsf(Tf.y) + fabsf(zf.y));
                    const float band = 2.0f * (ex * (2.0f * fabsf(dxf) + ex) +
                                               ey * (2.0f * fabsf(dyf) + ey) + 0x1p-22f * r2f);
                    const float xf = r2f * a.xi2f;
                    nearp = !(xf > xlo && xf < xhi);
                    if (r2f + band < a.cut2f) {
                        fl = 3;
                    } else if (!(r2f - band >= a.cut2f)) {
                        const double2 T = a.tp[t];
                        const double2 z = W.nbz[k];
                        if (SLP) {
                            const double dx = xsub(Sp.x, xsub(T.x, z.x));
                            const double dy = xsub(Sp.y, xsub(T.y, z.y));
                            if (xadd(xmul(dx, dx), xmul(dy, dy)) < a.cut2) fl |= 1;
                        }
                        if (DLP) {
                            const double x1 = xadd(xsub(Sp.x, T.x), z.x);
                            const double x2 = xadd(xsub(Sp.y, T.y), z.y);
                            if (xadd(xmul(x1, x1), xmul(x2, x2)) < a.cut2) fl |= 2;
                        }
                    }
                }
            }
            if (!SLP) fl &= 2;
            if (!DLP) fl &= 1;
            const int2 ent = make_int2(t, slot | (k << 8) | (fl << 12));
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const bool mine = fl != 0 && nearp == (j == 1);
                const unsigned m = __ballot_sync(~0u, mine);
                if (mine) W.q[j][qn[j] + __popc(m & ((1u << lane) - 1u))] = ent;
                qn[j] += __popc(m);
                enq[j] += __popc(m);
            }
            __syncwarp();
            if (qn[0] >= 32) batch(0, 32);
            if (qn[1] >= 32) batch(1, 32);
        }
        if (lane == 0) {
            W.tend[0][slot] = enq[0];
            W.tend[1][slot] = enq[1];
        }
        __syncwarp();
        retire(false);
    }
    drain();
}

template __global__ void k_real_adj<true, false, kFormFP64>(RealArgs);
template __global__ void k_real_adj<false, true, kFormFP64>(RealArgs);
template __global__ void k_real_adj<true, true, kFormFP64>(RealArgs);
template __global__ void k_real_adj<true, false, kFormFF>(RealArgs);
template __global__ void k_real_adj<false, true, kFormFF>(RealArgs);
template __global__ void k_real_adj<true, true, kFormFF>(RealArgs);

// ===========================================================================
// Gaussian spread (fast Gaussian gridding; PE/src/mex/StokesSLP/
// mex_stokes_slp_kspace.cpp:64-130, PE/src/mex/StokesDLP/
// mex_stokes_dlp_kspace.cpp:79-150).
//
// Node (mx+i, my+j) of a source gets c * Wx[i] * Wy[j] with
//   Wx[i] = exp(a(px^2+py^2+2w px)) exp(2 a w py) e1[i] e3x^i,
//   Wy[j] = e1[j] e3y^j,  e1[j] = exp(a h^2 (j-P/2)^2), a = -2 xi^2/eta.
// A warp takes 32 sources; each lane computes its source's exponentials,
// then for every source of the batch the warp builds Wx, Wy with product
// scans across lanes (lane i holds e3^i) and walks the flattened (P+1)^2
// stencil, 32 nodes per step, adding into the global grids with FP64
// atomics (executed in L2, off the SM's FP64 pipe).
// ===========================================================================
constexpr int kSpreadWarps = 8;
// Bit patterns of |g| at or above this are infinities and NaNs.
constexpr unsigned long long kGridNonFinite = 0x7ff0000000000000ull;

__device__ __forceinline__ int wrap_index(int i, int M)
{
    i %= M;
    return i < 0 ? i + M : i;
}

template <int NC>
__global__ void __launch_bounds__(kSpreadWarps * 32) k_spread(SpreadArgs a)
{
    // behind k_spread_fix: runs only when the bound slot says kFixedOff
    if (a.bound && *a.bound != kFixedOff) return;
    __shared__ double wsh[kSpreadWarps][NC + 1][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P1 = a.P + 1, NN = P1 * P1;
    const size_t G = (size_t)a.Mx * a.My;
    const int64_t nw = (int64_t)gridDim.x * kSpreadWarps;
    for (int64_t base = ((int64_t)blockIdx.x * kSpreadWarps + wid) * 32; base < a.ns;
         base += nw * 32) {
        const int64_t sl = base + lane;
        int mx = 0, my = 0;
        double A = 0.0, e3x = 1.0, e3y = 1.0;
        double cf[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) cf[c] = 0.0;
        if (sl < a.ns) {
            const double2 S = a.sp[sl];
            double px, py;
            closest_node(S.x, S.y, a.Lhx, a.Lhy, a.h, a.P, mx, my, px, py);
            const double ex = exp(a.a * (px * px + py * py + 2.0 * a.w * px));
            const double e4y = exp(2.0 * a.a * a.w * py);
            e3x = exp(-2.0 * a.a * a.h * px);
            e3y = exp(-2.0 * a.a * a.h * py);
            A = ex * e4y;
#pragma unroll
            for (int c = 0; c < NC; c++) cf[c] = a.coef[NC * sl + c];
        }
        const int cnt = (int)min((int64_t)32, a.ns - base);
        for (int j = 0; j < cnt; j++) {
            const int smx = __shfl_sync(~0u, mx, j), smy = __shfl_sync(~0u, my, j);
            const double sA = __shfl_sync(~0u, A, j);
            const double b3x = __shfl_sync(~0u, e3x, j), b3y = __shfl_sync(~0u, e3y, j);
            double px_ = lane >= 1 ? b3x : 1.0;
            double py_ = lane >= 1 ? b3y : 1.0;
            double sc[NC];
#pragma unroll
            for (int c = 0; c < NC; c++) sc[c] = __shfl_sync(~0u, cf[c], j);
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double tx = __shfl_up_sync(~0u, px_, o);
                const double ty = __shfl_up_sync(~0u, py_, o);
                if (lane >= o) {
                    px_ *= tx;
                    py_ *= ty;
                }
            }
            if (lane < P1) {
                const double e1v = a.e1[lane];
                const double wx = sA * e1v * px_;
#pragma unroll
                for (int c = 0; c < NC; c++) wsh[wid][c][lane] = sc[c] * wx;
                wsh[wid][NC][lane] = e1v * py_;
            }
            __syncwarp();
            for (int qd = lane; qd < NN; qd += 32) {
                const int i = qd / P1, jj = qd - i * P1;
                const int col = wrap_index(smx + i, a.Mx), row = wrap_index(smy + jj, a.My);
                const double wy = wsh[wid][NC][jj];
                double *g = a.grid + (size_t)col * a.My + row;
#pragma unroll
                for (int c = 0; c < NC; c++) atomicAdd(g + c * G, wsh[wid][c][i] * wy);
            }
            __syncwarp();
        }
    }
}

template __global__ void k_spread<2>(SpreadArgs);
template __global__ void k_spread<4>(SpreadArgs);
template __global__ void k_spread<3>(SpreadArgs);
template __global__ void k_spread<5>(SpreadArgs);

// ===========================================================================
// Fixed-point spread (FP64 form).
//
// The FP64 spread above is bound by the FP64 pipe (one DMUL per node and
// component, 1.6 per clock per SM on GB300) and by FP64 atomics in L2.  Here
// each contribution c Wx[i] Wy[j] is formed in integer arithmetic and added
// with 64-bit integer atomics.  The source's Gaussian is split into its exact
// x and y factors, X[i] = exp(a (px - h (i - P/2))^2) and the same for y, both
// <= 1 when w = h P/2 (otherwise <= wf = exp(2 |a| h |w - h P/2|), which the
// caller folds in as 2^kY).  The kernel stores Xc[i] = round(c X[i] 2^(S+3+kY))
// and Y[j] = round(Y[j] 2^(62-kY)) as int64; the high 64 bits of Xc[i] Y[j]
// are q = floor(2 c X Y 2^S), and the node receives (q + 1) >> 1, c X Y 2^S
// rounded to the nearest integer.  (A plain floor would add a bias of -1/2
// unit per contribution, which the k-space sums amplify where sources
// cluster.)  The grid is int64 at scale 2^S, S chosen so that 2^S times a
// bound on every node's sum of |contributions| is below 2^59: no partial sum
// can overflow, the sum is exact and independent of the order of the atomics
// (the grid is bitwise reproducible), and each contribution is off by at most
// 3/4 unit of 2^-S, with no bias.
//
// The bound (k_spread_bin_sum, k_bound_x, k_bound_y_max): bins of kBoundBin
// x kBoundBin nodes hold the sums over their sources of max_c |c|.  A source
// at node coordinate t gives a node at distance d (in nodes) the factor
// X Y = exp(a h^2 dx^2) exp(a h^2 dy^2) (times at most 2^(2 kY) when w differs
// from h P/2), and reaches only |d| <= P/2 + 1.  Between a source's bin and a
// node's bin k bins apart the distance is at least (k - 1) kBoundBin (one bin
// less when kBoundBin does not divide M, where the last bin is short), so the
// bin sums weighted by those largest factors, a separable window of 2R + 1
// bins per axis, bound every node's sum; its largest value, times 2^(2 kY)
// and the number of times one stencil covers a node when M <= P, is the
// bound, about 5 times the largest node sum on uniform points.  (Bins of P+2
// nodes with every factor taken as 1 gave about 170 times it.  The unit 2^-S
// scales with the bound, and its rounding noise, white on the grid, is
// amplified by the deconvolution of the Gaussian in the filter: at eta = 3.3
// it reached 3e-13 of the k-space velocity.)  Where the window would wrap
// onto itself (grids under 2R + 1 bins) every bin counts with factor 1.
//
// The unit 2^-S is fixed by that bound, i.e. by sum |c|, while FP64 atomics
// round relative to the partial sums, which grow like sqrt(n) when the signs
// of the coefficients vary.  Each node's error is about n 2^-59 of its value
// here against sqrt(n) 2^-53 there, n the number of stencils covering it: the
// integer sums are the more accurate below n ~ 2^11 and lose beyond.  So when
// some window holds more than kFixedMaxCover sources (stencil covers),
// k_bound_y_max marks the bound slot kFixedOff, the integer spreads return at
// once and the FP64 spread (launched behind them) runs instead; the pack reads
// the same mark.  The choice costs no host synchronisation.
// ===========================================================================
constexpr int kFixedMaxCover = 1 << 14;

// High 64 bits of the 128-bit product a b, for signed a and 0 <= b < 2^63
// (b a Gaussian factor): the unsigned high product of a's bit pattern, less b
// where a is negative (two's complement).  Equal to __mul64hi(a, b), without
// the correction for a negative b.  (The integer spread gains 0.2 ms from it;
// the integer gather runs slightly faster with __mul64hi and keeps it.)
__device__ __forceinline__ long long mulhi_s_u(long long a, long long b)
{
    const long long h = (long long)__umul64hi((unsigned long long)a, (unsigned long long)b);
    return a < 0 ? h - b : h;
}


constexpr int kBoundBin = 4;      // nodes per bound bin and axis
constexpr int kBoundMaxR = 15;

// Bound bins along an axis of M nodes.
static int spread_bins(int M) { return (M + kBoundBin - 1) / kBoundBin; }

int64_t spread_bound_words(int Mx, int My, int P)
{
    (void)P;
    return 3 * (int64_t)spread_bins(Mx) * spread_bins(My) + 1;
}

int64_t spread_bound_slot(int Mx, int My, int P)
{
    (void)P;
    return 2 * (int64_t)spread_bins(Mx) * spread_bins(My);
}

// One axis of the bound's window: bins within R of a node's bin, and the
// largest Gaussian factor a source k bins away can give it (full: every bin,
// factor 1).
struct BoundAxis {
    int nb, R, full;
    double w[kBoundMaxR + 1];
};

static BoundAxis bound_axis(int M, int P, double a, double h)
{
    BoundAxis ax{};
    ax.nb = spread_bins(M);
    const int slack = M % kBoundBin ? 1 : 0;
    const int R = (P / 2 + 1) / kBoundBin + 1 + slack;
    if (2 * R + 1 > ax.nb || R > kBoundMaxR) {
        ax.full = 1;
        return ax;
    }
    ax.R = R;
    for (int k = 0; k <= R; k++) {
        const double d = (double)std::max(0, (k - 1 - slack) * kBoundBin);
        ax.w[k] = std::exp(a * h * h * d * d) * (1.0 + 1e-12);
    }
    return ax;
}

// (A NaN or infinite coefficient marks the bound kFixedOff: the FP64 spread
// carries it into the grid as the reference does.)
__global__ void k_spread_bin_sum(SpreadArgs a, int nc, int nbx, int nby, double *__restrict__ bins,
                                 int *__restrict__ cnt, unsigned long long *__restrict__ bound)
{
    const double inv_h = 1.0 / a.h;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < a.ns;
         s += (int64_t)gridDim.x * blockDim.x) {
        double m = 0.0;
        bool finite = true;
        for (int c = 0; c < nc; c++) {
            const double v = fabs(a.coef[(int64_t)nc * s + c]);
            finite = finite && v <= 1.7976931348623157e308;
            m = fmax(m, v);
        }
        if (!finite) atomicMax(bound, kFixedOff);
        if (!(m > 0.0)) continue;
        const double2 S = a.sp[s];
        // the node cell holding the source, t in [cx, cx + 1) (mod M)
        const int cx = wrap_index((int)floor((S.x + a.Lhx) * inv_h), a.Mx);
        const int cy = wrap_index((int)floor((S.y + a.Lhy) * inv_h), a.My);
        const int bx = cx / kBoundBin, by = cy / kBoundBin;
        atomicAdd(&bins[(int64_t)bx * nby + by], m);
        atomicAdd(&cnt[(int64_t)bx * nby + by], 1);
    }
}

// The window along x: t = sum_k bins[bx + k] w[|k|], tc the plain count.
__global__ void k_bound_x(const double *__restrict__ bins, const int *__restrict__ cnt,
                          BoundAxis ax, int nby, double *__restrict__ t, int *__restrict__ tc)
{
    const int nbx = ax.nb;
    const int64_t nb = (int64_t)nbx * nby;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int bx = (int)(i / nby), by = (int)(i - (int64_t)bx * nby);
        double s = 0.0;
        int c = 0;
        if (ax.full) {
            for (int k = 0; k < nbx; k++) {
                s += bins[(int64_t)k * nby + by];
                c += cnt[(int64_t)k * nby + by];
            }
        } else {
            for (int k = -ax.R; k <= ax.R; k++) {
                int x = bx + k;
                x = x < 0 ? x + nbx : (x >= nbx ? x - nbx : x);
                s = fma(bins[(int64_t)x * nby + by], ax.w[k < 0 ? -k : k], s);
                c += cnt[(int64_t)x * nby + by];
            }
        }
        t[i] = s;
        tc[i] = c;
    }
}

// The window along y, and the largest value over the bins.
__global__ void k_bound_y_max(const double *__restrict__ t, const int *__restrict__ tc,
                              BoundAxis ay, int nbx, double kfac, int mult,
                              unsigned long long *__restrict__ bound)
{
    const int nby = ay.nb;
    const int64_t nb = (int64_t)nbx * nby;
    double best = 0.0;
    int64_t crowd = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int bx = (int)(i / nby), by = (int)(i - (int64_t)bx * nby);
        const double *row = t + (int64_t)bx * nby;
        const int *rowc = tc + (int64_t)bx * nby;
        double s = 0.0;
        int64_t c = 0;
        if (ay.full) {
            for (int k = 0; k < nby; k++) {
                s += row[k];
                c += rowc[k];
            }
        } else {
            for (int k = -ay.R; k <= ay.R; k++) {
                int y = by + k;
                y = y < 0 ? y + nby : (y >= nby ? y - nby : y);
                s = fma(row[y], ay.w[k < 0 ? -k : k], s);
                c += rowc[y];
            }
        }
        best = fmax(best, s);
        crowd = max(crowd, c);
    }
    for (int o = 16; o > 0; o >>= 1) {
        best = fmax(best, __shfl_xor_sync(~0u, best, o));
        crowd = max(crowd, __shfl_xor_sync(~0u, crowd, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (crowd * mult > kFixedMaxCover)
            atomicMax(bound, kFixedOff);
        else if (best > 0.0)      // positive doubles order as their bit patterns
            atomicMax(bound, (unsigned long long)__double_as_longlong(best * kfac));
    }
}

template <int NC>
__global__ void __launch_bounds__(kSpreadWarps * 32, 4) k_spread_fix(SpreadArgs a, int kY)
{
    __shared__ long long xsh[kSpreadWarps][NC][32];
    __shared__ long long ysh[kSpreadWarps][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P1 = a.P + 1, NN = P1 * P1;            // P1 <= 31
    const size_t G = (size_t)a.Mx * a.My;
    const unsigned long long bnd = *a.bound;
    if (bnd == kFixedOff) return;                    // the FP64 spread runs instead
    const int S = fix_shift(bnd);
    const double sx = ldexp(1.0, S + 3 + kY), sy = ldexp(1.0, 62 - kY);
    // (i, j) of flattened stencil entry q = lane + 32 k, stepped without division
    const int di = 32 / P1, dj = 32 - di * P1, i0 = lane / P1, j0 = lane - i0 * P1;
    const bool once = a.Mx > a.P && a.My > a.P;      // a stencil wraps at most once
    long long *grid = reinterpret_cast<long long *>(a.grid);
    const int64_t nw = (int64_t)gridDim.x * kSpreadWarps;
    // Batch k of warp w holds the sources k 32 nw + w + lane nw: all warps
    // walk the box-sorted sources together, nw apart, so the grid band they
    // update at any time spans about nw sources' stencils and stays in L2
    // (32 consecutive sources per warp kept a third of the grids live).
    const int64_t sstep = nw;
    for (int64_t base = (int64_t)blockIdx.x * kSpreadWarps + wid; base < a.ns; base += nw * 32) {
        const int64_t sl = base + (int64_t)lane * sstep;
        int mx = 0, my = 0;
        double Ax = 0.0, Ay = 0.0, e3x = 1.0, e3y = 1.0;
        double cf[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) cf[c] = 0.0;
        if (sl < a.ns) {
            const double2 Sp = a.sp[sl];
            double px, py;
            closest_node(Sp.x, Sp.y, a.Lhx, a.Lhy, a.h, a.P, mx, my, px, py);
            Ax = exp(a.a * (px * px + 2.0 * a.w * px)) * sx;
            Ay = exp(a.a * (py * py + 2.0 * a.w * py)) * sy;
            e3x = exp(-2.0 * a.a * a.h * px);
            e3y = exp(-2.0 * a.a * a.h * py);
#pragma unroll
            for (int c = 0; c < NC; c++) cf[c] = a.coef[NC * sl + c];
        }
        const int cnt = (int)min((int64_t)32, (a.ns - base + sstep - 1) / sstep);   // lanes holding one
        for (int j = 0; j < cnt; j++) {
            const int smx = __shfl_sync(~0u, mx, j), smy = __shfl_sync(~0u, my, j);
            const double sAx = __shfl_sync(~0u, Ax, j), sAy = __shfl_sync(~0u, Ay, j);
            const double b3x = __shfl_sync(~0u, e3x, j), b3y = __shfl_sync(~0u, e3y, j);
            double px_ = lane >= 1 ? b3x : 1.0;
            double py_ = lane >= 1 ? b3y : 1.0;
            double sc[NC];
#pragma unroll
            for (int c = 0; c < NC; c++) sc[c] = __shfl_sync(~0u, cf[c], j);
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double tx = __shfl_up_sync(~0u, px_, o);
                const double ty = __shfl_up_sync(~0u, py_, o);
                if (lane >= o) {
                    px_ *= tx;
                    py_ *= ty;
                }
            }
            if (lane < P1) {
                const double e1v = a.e1[lane];
                const double X = sAx * e1v * px_;
#pragma unroll
                for (int c = 0; c < NC; c++) xsh[wid][c][lane] = __double2ll_rn(sc[c] * X);
                ysh[wid][lane] = __double2ll_rn(sAy * e1v * py_);
            }
            __syncwarp();
            const int c0 = wrap_index(smx, a.Mx), r0 = wrap_index(smy, a.My);
            int i = i0, jj = j0;
            for (int qd = lane; qd < NN; qd += 32) {
                int col = c0 + i, row = r0 + jj;
                if (once) {
                    col = col >= a.Mx ? col - a.Mx : col;
                    row = row >= a.My ? row - a.My : row;
                } else {
                    col %= a.Mx;
                    row %= a.My;
                }
                const long long y = ysh[wid][jj];
                unsigned long long *g =
                    reinterpret_cast<unsigned long long *>(grid + (size_t)col * a.My + row);
#pragma unroll
                for (int c = 0; c < NC; c++)
                    atomicAdd(g + c * G,
                              (unsigned long long)((mulhi_s_u(xsh[wid][c][i], y) + 1) >> 1));
                i += di;
                jj += dj;
                if (jj >= P1) {
                    jj -= P1;
                    i++;
                }
            }
            __syncwarp();
        }
    }
}

template __global__ void k_spread_fix<2>(SpreadArgs, int);
template __global__ void k_spread_fix<3>(SpreadArgs, int);
template __global__ void k_spread_fix<4>(SpreadArgs, int);
template __global__ void k_spread_fix<5>(SpreadArgs, int);

// k_spread_fix for nr right-hand sides on one point set (many densities per
// geometry): the stencil origin, exponentials and factor scans of a source
// are formed once, then each right-hand side r spreads its NC coefficients
// (a.coef + r cstride, NC per source) into its own grids (a.grid + r gstride
// words) at its own scale (bound slot a.bound[r bstride]).  A right-hand side
// whose slot is kFixedOff is left to the FP64 spread.  The grids are the same
// integers k_spread_fix gives for each right-hand side alone.
template <int NC>
__global__ void __launch_bounds__(kSpreadWarps * 32, 4) k_spread_fix_multi(SpreadArgs a, int kY, int nr,
                                                                        int64_t cstride,
                                                                        int64_t gstride, int bstride)
{
    __shared__ long long xsh[kSpreadWarps][NC][32];
    __shared__ long long ysh[kSpreadWarps][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P1 = a.P + 1, NN = P1 * P1;            // P1 <= 31
    const size_t G = (size_t)a.Mx * a.My;
    const double sy = ldexp(1.0, 62 - kY);
    const int di = 32 / P1, dj = 32 - di * P1, i0 = lane / P1, j0 = lane - i0 * P1;
    const bool once = a.Mx > a.P && a.My > a.P;      // a stencil wraps at most once
    const int64_t nw = (int64_t)gridDim.x * kSpreadWarps;
    // Batch k of warp w holds the sources k 32 nw + w + lane nw: all warps
    // walk the box-sorted sources together, nw apart, so the grid band they
    // update at any time spans about nw sources' stencils and stays in L2
    // (32 consecutive sources per warp kept a third of the grids live).
    const int64_t sstep = nw;
    for (int64_t base = (int64_t)blockIdx.x * kSpreadWarps + wid; base < a.ns; base += nw * 32) {
        const int64_t sl = base + (int64_t)lane * sstep;
        int mx = 0, my = 0;
        double Ax = 0.0, Ay = 0.0, e3x = 1.0, e3y = 1.0;
        if (sl < a.ns) {
            const double2 Sp = a.sp[sl];
            double px, py;
            closest_node(Sp.x, Sp.y, a.Lhx, a.Lhy, a.h, a.P, mx, my, px, py);
            Ax = exp(a.a * (px * px + 2.0 * a.w * px));
            Ay = exp(a.a * (py * py + 2.0 * a.w * py)) * sy;
            e3x = exp(-2.0 * a.a * a.h * px);
            e3y = exp(-2.0 * a.a * a.h * py);
        }
        const int cnt = (int)min((int64_t)32, (a.ns - base + sstep - 1) / sstep);   // lanes holding one
        for (int j = 0; j < cnt; j++) {
            const int smx = __shfl_sync(~0u, mx, j), smy = __shfl_sync(~0u, my, j);
            const double sAx = __shfl_sync(~0u, Ax, j), sAy = __shfl_sync(~0u, Ay, j);
            const double b3x = __shfl_sync(~0u, e3x, j), b3y = __shfl_sync(~0u, e3y, j);
            double px_ = lane >= 1 ? b3x : 1.0;
            double py_ = lane >= 1 ? b3y : 1.0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double tx = __shfl_up_sync(~0u, px_, o);
                const double ty = __shfl_up_sync(~0u, py_, o);
                if (lane >= o) {
                    px_ *= tx;
                    py_ *= ty;
                }
            }
            double X = 0.0;
            if (lane < P1) {
                const double e1v = a.e1[lane];
                X = sAx * e1v * px_;
                ysh[wid][lane] = __double2ll_rn(sAy * e1v * py_);
            }
            const int c0 = wrap_index(smx, a.Mx), r0 = wrap_index(smy, a.My);
            for (int r = 0; r < nr; r++) {
                const unsigned long long bnd = a.bound[(int64_t)r * bstride];
                if (bnd == kFixedOff) continue;      // (uniform) this one runs the FP64 spread
                // the scale is a power of two, so X sx rounds as k_spread_fix's factors do
                const double Xs = X * ldexp(1.0, fix_shift(bnd) + 3 + kY);
                __syncwarp();
                if (lane < P1) {
                    const double *cf = a.coef + r * cstride + (int64_t)NC * (base + (int64_t)j * sstep);
#pragma unroll
                    for (int c = 0; c < NC; c++) xsh[wid][c][lane] = __double2ll_rn(cf[c] * Xs);
                }
                __syncwarp();
                long long *grid = reinterpret_cast<long long *>(a.grid) + r * gstride;
                int i = i0, jj = j0;
                for (int qd = lane; qd < NN; qd += 32) {
                    int col = c0 + i, row = r0 + jj;
                    if (once) {
                        col = col >= a.Mx ? col - a.Mx : col;
                        row = row >= a.My ? row - a.My : row;
                    } else {
                        col %= a.Mx;
                        row %= a.My;
                    }
                    const long long y = ysh[wid][jj];
                    unsigned long long *g =
                        reinterpret_cast<unsigned long long *>(grid + (size_t)col * a.My + row);
#pragma unroll
                    for (int c = 0; c < NC; c++)
                        atomicAdd(g + c * G,
                                  (unsigned long long)((mulhi_s_u(xsh[wid][c][i], y) + 1) >> 1));
                    i += di;
                    jj += dj;
                    if (jj >= P1) {
                        jj -= P1;
                        i++;
                    }
                }
            }
            __syncwarp();
        }
    }
}

template __global__ void k_spread_fix_multi<2>(SpreadArgs, int, int, int64_t, int64_t, int);
template __global__ void k_spread_fix_multi<3>(SpreadArgs, int, int, int64_t, int64_t, int);
template __global__ void k_spread_fix_multi<5>(SpreadArgs, int, int, int64_t, int64_t, int);



// ===========================================================================
// 2D real FFT as two 1D complex passes (FP64 form).
//
// cuFFT's batched 1D R2C of length 2688 runs at half the rate of its C2C of
// the same length, and its 2D plans run the second dimension strided, so the
// real grids are transformed as complex pairs: z = a + i b for grids
// (2p, 2p+1), C2C along y (contiguous rows), split by Hermitian symmetry into
// the half spectra A(ky) = (Z(ky) + conj Z(-ky))/2, B(ky) = (Z(ky) -
// conj Z(-ky))/(2i) for ky = 0..My/2, stored transposed ([c][ky][x]) so that
// the C2C along x again runs on contiguous rows -- the D2Z result, transposed.
// The inverse mirrors it: C2C along x, Hermitian extension in ky with the
// transpose back and packing z = A + i B, C2C along y, real and imaginary
// parts -- the Z2D result (unnormalised, as cuFFT's).
// ===========================================================================
__device__ __forceinline__ void k_pack_real_pairs_body(const double *__restrict__ grid, int nc,
                                                       int64_t G, double2 *__restrict__ z)
{
    const int ncg = (nc + 1) / 2;
    const int64_t n = (int64_t)ncg * G;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(i / G);
        const int64_t e = i - (int64_t)p * G;
        const double re = grid[(int64_t)(2 * p) * G + e];
        const double im = 2 * p + 1 < nc ? grid[(int64_t)(2 * p + 1) * G + e] : 0.0;
        z[i] = make_double2(re, im);
    }
}

__global__ void k_pack_real_pairs(const double *__restrict__ grid, int nc, int64_t G,
                                  double2 *__restrict__ z)
{
    k_pack_real_pairs_body(grid, nc, G, z);
}

// The same pack from the fixed-point grids of k_spread_fix (value 2^-S v).
__global__ void k_pack_fixed_pairs(const long long *__restrict__ grid, int nc, int64_t G,
                                   const unsigned long long *__restrict__ bound,
                                   double2 *__restrict__ z)
{
    if (*bound == kFixedOff) {                       // the grids hold doubles
        k_pack_real_pairs_body(reinterpret_cast<const double *>(grid), nc, G, z);
        return;
    }
    const double inv = ldexp(1.0, -fix_shift(*bound));
    const int ncg = (nc + 1) / 2;
    const int64_t n = (int64_t)ncg * G;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(i / G);
        const int64_t e = i - (int64_t)p * G;
        const double re = (double)grid[(int64_t)(2 * p) * G + e] * inv;
        const double im = 2 * p + 1 < nc ? (double)grid[(int64_t)(2 * p + 1) * G + e] * inv : 0.0;
        z[i] = make_double2(re, im);
    }
}

// With gmax, also the largest |value| as a bit pattern (non-finite values
// order above every finite one), for the fixed-point gather.
__global__ void k_unpack_real_pairs(const double2 *__restrict__ z, int nout, int64_t G,
                                    double *__restrict__ grid, unsigned long long *gmax)
{
    const int npair = (nout + 1) / 2;
    const int64_t n = (int64_t)npair * G;
    unsigned long long m[kGmaxWords] = {0, 0, 0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(i / G);
        const int64_t e = i - (int64_t)p * G;
        const double2 v = z[i];
        grid[(int64_t)(2 * p) * G + e] = v.x;
        unsigned long long mp = (unsigned long long)__double_as_longlong(fabs(v.x));
        if (2 * p + 1 < nout) {
            grid[(int64_t)(2 * p + 1) * G + e] = v.y;
            mp = max(mp, (unsigned long long)__double_as_longlong(fabs(v.y)));
        }
#pragma unroll
        for (int q = 0; q < kGmaxWords; q++)
            if (q == p) m[q] = max(m[q], mp);
    }
    if (gmax) {
#pragma unroll
        for (int q = 0; q < kGmaxWords; q++) {
            unsigned long long v = m[q];
            for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(~0u, v, o));
            if ((threadIdx.x & 31) == 0 && v) atomicMax(gmax + q, v);
        }
    }
}

// The same split and join with the half spectra stored transposed,
// specT[c][ky][x] (x fastest), so that the x transforms run on contiguous
// rows.  32 x 32 tiles through shared memory keep both sides coalesced.
constexpr int kTT = 32;

__global__ void __launch_bounds__(256) k_split_half_spectra_t(const double2 *__restrict__ z,
                                                              int nc, int Mx, int My,
                                                              double2 *__restrict__ specT,
                                                              int fold)
{
    __shared__ double2 sa[kTT][kTT + 1], sb[kTT][kTT + 1];
    const int H1 = My / 2 + 1;
    const int64_t G = (int64_t)Mx * My, HT = (int64_t)H1 * Mx;
    const int ky0 = blockIdx.x * kTT, x0 = blockIdx.y * kTT, p = blockIdx.z;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
    const double2 *zp = z + (int64_t)p * G;
    // a folded pair: rows x < Mx/2 hold plane 2p's rows x and x + Mx/2
    const bool folded = fold && 2 * p + 1 == nc;
    const int xend = folded ? Mx / 2 : Mx;
    // load: lanes along ky
    for (int r = ty; r < kTT; r += 8) {
        const int x = x0 + r, ky = ky0 + tx;
        if (x < xend && ky < H1) {
            const double2 zk = zp[(int64_t)x * My + ky];
            const double2 zm = zp[(int64_t)x * My + (ky == 0 ? 0 : My - ky)];
            sa[tx][r] = make_double2(0.5 * (zk.x + zm.x), 0.5 * (zk.y - zm.y));
            sb[tx][r] = make_double2(0.5 * (zk.y + zm.y), 0.5 * (zm.x - zk.x));
        }
    }
    __syncthreads();
    // store: lanes along x
    for (int r = ty; r < kTT; r += 8) {
        const int ky = ky0 + r, x = x0 + tx;
        if (x < xend && ky < H1) {
            specT[(int64_t)(2 * p) * HT + (int64_t)ky * Mx + x] = sa[r][tx];
            if (folded)
                specT[(int64_t)(2 * p) * HT + (int64_t)ky * Mx + x + Mx / 2] = sb[r][tx];
            else if (2 * p + 1 < nc)
                specT[(int64_t)(2 * p + 1) * HT + (int64_t)ky * Mx + x] = sb[r][tx];
        }
    }
}

__global__ void __launch_bounds__(256) k_join_half_spectra_t(const double2 *__restrict__ specT,
                                                             int nout, int Mx, int My,
                                                             double2 *__restrict__ z)
{
    __shared__ double2 sa[kTT][kTT + 1], sb[kTT][kTT + 1];
    const int H1 = My / 2 + 1;
    const int64_t G = (int64_t)Mx * My, HT = (int64_t)H1 * Mx;
    const int ky0 = blockIdx.x * kTT, x0 = blockIdx.y * kTT, p = blockIdx.z;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const bool hasb = 2 * p + 1 < nout;
    // load: lanes along x, one (mirrored) ky row per step
    for (int r = ty; r < kTT; r += 8) {
        const int ky = ky0 + r, x = x0 + tx;
        if (x < Mx && ky < My) {
            const bool hi = ky > My / 2;
            const int64_t src = (int64_t)(hi ? My - ky : ky) * Mx + x;
            double2 a = specT[(int64_t)(2 * p) * HT + src];
            double2 b = hasb ? specT[(int64_t)(2 * p + 1) * HT + src] : make_double2(0.0, 0.0);
            if (hi) {
                a.y = -a.y;
                b.y = -b.y;
            }
            sa[r][tx] = a;
            sb[r][tx] = b;
        }
    }
    __syncthreads();
    // store: lanes along ky
    for (int r = ty; r < kTT; r += 8) {
        const int x = x0 + r, ky = ky0 + tx;
        if (x < Mx && ky < My) {
            const double2 a = sa[tx][r], b = sb[tx][r];
            z[(int64_t)p * G + (int64_t)x * My + ky] = make_double2(a.x - b.y, a.y + b.x);
        }
    }
}

// ===========================================================================
// k-space filter on the half spectrum (R2C layout Mx x (My/2+1)).
//
// The reference transforms real grids with a full complex fft2, applies the
// filter to every mode, inverse-transforms and keeps Re (SLP,
// mex_stokes_slp_kspace.cpp:189-241) or Im (DLP, mex_stokes_dlp_kspace.cpp:
// 219-305) of the result.  Its frequency map sends index M/2 to +M/2, so on
// the Nyquist row/column the filtered spectrum is not Hermitian.  A C2R
// transform reproduces Re(ifft2(G)) exactly when fed the Hermitian part
// (G(k) + conj G(-k))/2; since H(-k) = conj H(k) for real grids this is the
// filter averaged over k and its index partner -k mod M.  Off the Nyquist
// lines the SLP filter is even and the DLP filter odd in k, so the average
// is the plain filter.  Im is taken as Re of -i G.  The 1/(Mx My) of MATLAB's
// ifft2 is folded in, and the zero mode is set to 0.
// ===========================================================================
__device__ __forceinline__ double kfreq(int j, int M, double L)
{
    return 2.0 * kPi / L * (double)(j <= M / 2 ? j : j - M);
}

// Per-mode scalar factors of the two filters; they depend on |k|^2 only.
// SLP: (1/K^4 + 1/(4 xi^2 K^2)) exp(-(1-eta) K^2/(4 xi^2))  (mex_stokes_slp_kspace.cpp:200)
// DLP: exp(-(1-eta) K^2/(4 xi^2))/K^4 (1 + K^2/(4 xi^2))   (mex_stokes_dlp_kspace.cpp:232-233)
__device__ __forceinline__ double slp_factor(double K2, double xi, double eta)
{
    return (1.0 / (K2 * K2) + 0.25 / (K2 * xi * xi)) * exp(-0.25 * (1 - eta) / (xi * xi) * K2);
}

__device__ __forceinline__ double dlp_factor(double K2, double xi, double eta)
{
    const double e = exp(-0.25 * (1 - eta) / (xi * xi) * K2) / K2 / K2;
    const double t = 1 + 0.25 * K2 / xi / xi;
    return e * t;
}

// SLP filter (mex_stokes_slp_kspace.cpp:197-208) applied to (h1, h2); e < 0
// means "compute the factor here".
__device__ __forceinline__ void slp_mode(double k1, double k2, double xi, double eta,
                                         double2 h1, double2 h2, double2 &o1, double2 &o2,
                                         double e = -1.0)
{
    const double K2 = k1 * k1 + k2 * k2;
    if (e < 0.0) e = slp_factor(K2, xi, eta);
    o1.x = k2 * (k2 * h1.x - k1 * h2.x) * e;
    o1.y = k2 * (k2 * h1.y - k1 * h2.y) * e;
    o2.x = k1 * (k1 * h2.x - k2 * h1.x) * e;
    o2.y = k1 * (k1 * h2.y - k2 * h1.y) * e;
}

// DLP filter (mex_stokes_dlp_kspace.cpp:228-251) applied to (h1, h2+h3, h4).
__device__ __forceinline__ void dlp_mode(double k1, double k2, double xi, double eta,
                                         double2 h1, double2 h23, double2 h4, double2 &o1,
                                         double2 &o2, double et = -1.0)
{
    const double K2 = k1 * k1 + k2 * k2;
    if (et < 0.0) et = dlp_factor(K2, xi, eta);
    const double B111 = 3.0 * k1 * K2 - 2.0 * k1 * k1 * k1;
    const double B112 = k2 * K2 - 2.0 * k1 * k1 * k2;
    const double B122 = k1 * K2 - 2.0 * k1 * k2 * k2;
    const double B211 = k2 * K2 - 2.0 * k2 * k1 * k1;
    const double B212 = k1 * K2 - 2.0 * k2 * k1 * k2;
    const double B222 = 3.0 * k2 * K2 - 2.0 * k2 * k2 * k2;
    o1.x = et * (B111 * h1.x + B112 * h23.x + B122 * h4.x);
    o1.y = et * (B111 * h1.y + B112 * h23.y + B122 * h4.y);
    o2.x = et * (B211 * h1.x + B212 * h23.x + B222 * h4.x);
    o2.y = et * (B211 * h1.y + B212 * h23.y + B222 * h4.y);
}

__global__ void k_filter(FilterArgs a)
{
    const int H = a.My / 2 + 1;
    const int64_t G = (int64_t)a.Mx * H;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= G) return;
    int jx, jy;
    if (a.transposed) {
        jy = (int)(idx / a.Mx);
        jx = (int)(idx - (int64_t)jy * a.Mx);
    } else {
        jx = (int)(idx / H);
        jy = (int)(idx - (int64_t)jx * H);
    }
    double2 *sp = reinterpret_cast<double2 *>(a.spec);
    if (a.mtab) {
        // the cached effective multipliers (k_filter_matrix_table)
        const double *m = a.mtab + (int64_t)kFilterMat * idx;
        if (a.slp_in >= 0) {
            const double2 h1 = sp[a.slp_in * G + idx], h2 = sp[(a.slp_in + 1) * G + idx];
            const double ma = m[0], mb = m[1], mc = m[2];
            sp[a.slp_out * G + idx] = make_double2(fma(ma, h1.x, -mb * h2.x), fma(ma, h1.y, -mb * h2.y));
            sp[(a.slp_out + 1) * G + idx] =
                make_double2(fma(mc, h2.x, -mb * h1.x), fma(mc, h2.y, -mb * h1.y));
        }
        if (a.dlp_in >= 0) {
            const double2 h1 = sp[a.dlp_in * G + idx], h23 = sp[(a.dlp_in + 1) * G + idx];
            const double2 h4 = sp[(a.dlp_in + 2) * G + idx];
            const double2 t1 = make_double2(fma(m[3], h1.x, fma(m[4], h23.x, m[5] * h4.x)),
                                            fma(m[3], h1.y, fma(m[4], h23.y, m[5] * h4.y)));
            const double2 t2 = make_double2(fma(m[6], h1.x, fma(m[7], h23.x, m[8] * h4.x)),
                                            fma(m[6], h1.y, fma(m[7], h23.y, m[8] * h4.y)));
            sp[a.dlp_out * G + idx] = make_double2(t1.y, -t1.x);            // -i
            sp[(a.dlp_out + 1) * G + idx] = make_double2(t2.y, -t2.x);
        }
        return;
    }
    const bool zero = (jx == 0 && jy == 0);
    const bool nyq = (jx == a.Mx / 2) || (jy == a.My / 2);
    const double k1 = kfreq(jx, a.Mx, a.Lx), k2 = kfreq(jy, a.My, a.Ly);
    // Index partner -j mod M: frequency negated except on the Nyquist index.
    const double k1p = (jx == a.Mx / 2) ? k1 : -k1;
    const double k2p = (jy == a.My / 2) ? k2 : -k2;
    const double sc = a.scale;
    double2 so1, so2, do1, do2;
    // (without the cached multipliers: the factors computed here)
    const double2 ft = make_double2(-1.0, -1.0);
    if (a.slp_in >= 0) {
        const double2 h1 = sp[a.slp_in * G + idx], h2 = sp[(a.slp_in + 1) * G + idx];
        slp_mode(k1, k2, a.xi, a.eta, h1, h2, so1, so2, ft.x);
        if (nyq) {
            double2 p1, p2;
            slp_mode(k1p, k2p, a.xi, a.eta, h1, h2, p1, p2, ft.x);
            so1.x = 0.5 * (so1.x + p1.x); so1.y = 0.5 * (so1.y + p1.y);
            so2.x = 0.5 * (so2.x + p2.x); so2.y = 0.5 * (so2.y + p2.y);
        }
        so1.x *= sc; so1.y *= sc; so2.x *= sc; so2.y *= sc;
        if (zero) so1 = so2 = make_double2(0.0, 0.0);
    }
    if (a.dlp_in >= 0) {
        const double2 h1 = sp[a.dlp_in * G + idx], h23 = sp[(a.dlp_in + 1) * G + idx];
        const double2 h4 = sp[(a.dlp_in + 2) * G + idx];
        dlp_mode(k1, k2, a.xi, a.eta, h1, h23, h4, do1, do2, ft.y);
        if (nyq) {
            double2 p1, p2;
            dlp_mode(k1p, k2p, a.xi, a.eta, h1, h23, h4, p1, p2, ft.y);
            do1.x = 0.5 * (do1.x - p1.x); do1.y = 0.5 * (do1.y - p1.y);
            do2.x = 0.5 * (do2.x - p2.x); do2.y = 0.5 * (do2.y - p2.y);
        }
        // -i * G, scaled
        do1 = make_double2(do1.y * sc, -do1.x * sc);
        do2 = make_double2(do2.y * sc, -do2.x * sc);
        if (zero) do1 = do2 = make_double2(0.0, 0.0);
    }
    if (a.slp_in >= 0) {
        sp[a.slp_out * G + idx] = so1;
        sp[(a.slp_out + 1) * G + idx] = so2;
    }
    if (a.dlp_in >= 0) {
        sp[a.dlp_out * G + idx] = do1;
        sp[(a.dlp_out + 1) * G + idx] = do2;
    }
}

// Per-mode effective multipliers of k_filter (its arithmetic, once per
// parameter set): the SLP matrix e [[k2^2, -k1 k2], [-k1 k2, k1^2]] and the
// DLP rows e t (B1., B2.), averaged with the index partner on the Nyquist
// lines (even for the SLP, odd for the DLP), times 1/(Mx My); zero at k = 0.
__global__ void k_filter_matrix_table(FilterArgs a, double *__restrict__ mtab)
{
    const int H = a.My / 2 + 1;
    const int64_t G = (int64_t)a.Mx * H;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= G) return;
    int jx, jy;
    if (a.transposed) {
        jy = (int)(idx / a.Mx);
        jx = (int)(idx - (int64_t)jy * a.Mx);
    } else {
        jx = (int)(idx / H);
        jy = (int)(idx - (int64_t)jx * H);
    }
    double *m = mtab + (int64_t)kFilterMat * idx;
    if (jx == 0 && jy == 0) {
        for (int i = 0; i < kFilterMat; i++) m[i] = 0.0;
        return;
    }
    const bool nyq = (jx == a.Mx / 2) || (jy == a.My / 2);
    const double k1 = kfreq(jx, a.Mx, a.Lx), k2 = kfreq(jy, a.My, a.Ly);
    const double k1p = (jx == a.Mx / 2) ? k1 : -k1;
    const double k2p = (jy == a.My / 2) ? k2 : -k2;
    const double K2 = k1 * k1 + k2 * k2;
    const double sc = a.scale;
    const double e = slp_factor(K2, a.xi, a.eta), et = dlp_factor(K2, a.xi, a.eta);
    // SLP
    double b = k1 * k2;
    if (nyq) b = 0.5 * (b + k1p * k2p);
    m[0] = k2 * k2 * e * sc;
    m[1] = b * e * sc;
    m[2] = k1 * k1 * e * sc;
    // DLP (mex_stokes_dlp_kspace.cpp:228-251)
    double B[6], Bp[6];
    auto bmat = [](double q1, double q2, double Q2, double *o) {
        o[0] = 3.0 * q1 * Q2 - 2.0 * q1 * q1 * q1;
        o[1] = q2 * Q2 - 2.0 * q1 * q1 * q2;
        o[2] = q1 * Q2 - 2.0 * q1 * q2 * q2;
        o[3] = q2 * Q2 - 2.0 * q2 * q1 * q1;
        o[4] = q1 * Q2 - 2.0 * q2 * q1 * q2;
        o[5] = 3.0 * q2 * Q2 - 2.0 * q2 * q2 * q2;
    };
    bmat(k1, k2, K2, B);
    if (nyq) {
        bmat(k1p, k2p, K2, Bp);
        for (int i = 0; i < 6; i++) B[i] = 0.5 * (B[i] - Bp[i]);
    }
    for (int i = 0; i < 6; i++) m[3 + i] = et * B[i] * sc;
}

// ===========================================================================
// Gather (PE/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:264-329 and
// PE/src/mex/StokesDLP/mex_stokes_dlp_kspace.cpp:334-400): one lane per
// target; per stencil column the NC grid values are reduced against Wy, then
// weighted by Wx.  Output k of target t holds grids 2k, 2k+1, times scale.
// ===========================================================================
template <int NC, int PT>
__global__ void __launch_bounds__(256) k_gather(GatherArgs a)
{
    // behind k_gather_fix: runs only when a grid held a non-finite value
    if (a.gmax && gmax_all(a.gmax) < kGridNonFinite) return;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.nt;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int P = PT > 0 ? PT : a.P;
        const size_t G = (size_t)a.Mx * a.My;
        const double2 T = a.tp[t];
        int mx, my;
        double px, py;
        closest_node(T.x, T.y, a.Lhx, a.Lhy, a.h, P, mx, my, px, py);
        const double ex = exp(a.a * (px * px + py * py + 2.0 * a.w * px));
        const double e4y = exp(2.0 * a.a * a.w * py);
        const double e3x = exp(-2.0 * a.a * a.h * px);
        const double e3y = exp(-2.0 * a.a * a.h * py);
        double wy[(PT > 0 ? PT : kMaxP) + 1];
        {
            double ey = 1.0;
    #pragma unroll
            for (int j = 0; j <= (PT > 0 ? PT : kMaxP); j++) {
                if (j <= P) {
                    wy[j] = a.e1[j] * ey;
                    ey *= e3y;
                }
            }
        }
        double acc[NC];
    #pragma unroll
        for (int c = 0; c < NC; c++) acc[c] = 0.0;
        const bool rows_inside = my >= 0 && my + P < a.My;
        double xf = ex * e4y;
        for (int i = 0; i <= P; i++) {
            const double *g = a.grid + (size_t)wrap_index(mx + i, a.Mx) * a.My;
            double tc[NC];
    #pragma unroll
            for (int c = 0; c < NC; c++) tc[c] = 0.0;
            if (rows_inside) {
                const double *gr = g + my;
    #pragma unroll
                for (int j = 0; j <= (PT > 0 ? PT : kMaxP); j++) {
                    if (j <= P) {
    #pragma unroll
                        for (int c = 0; c < NC; c++) tc[c] = fma(wy[j], __ldg(gr + c * G + j), tc[c]);
                    }
                }
            } else {
    #pragma unroll
                for (int j = 0; j <= (PT > 0 ? PT : kMaxP); j++) {
                    if (j <= P) {
                        const int row = wrap_index(my + j, a.My);
    #pragma unroll
                        for (int c = 0; c < NC; c++) tc[c] = fma(wy[j], __ldg(g + c * G + row), tc[c]);
                    }
                }
            }
            const double wx = xf * a.e1[i];
            xf *= e3x;
    #pragma unroll
            for (int c = 0; c < NC; c++) acc[c] = fma(wx, tc[c], acc[c]);
        }
    #pragma unroll
        for (int k = 0; k < NC / 2; k++)
            a.out[k * a.nt + t] = make_double2(acc[2 * k] * a.scale, acc[2 * k + 1] * a.scale);
    }
}

template __global__ void k_gather<2, 24>(GatherArgs);
template __global__ void k_gather<4, 24>(GatherArgs);
template __global__ void k_gather<2, 12>(GatherArgs);
template __global__ void k_gather<4, 12>(GatherArgs);
template __global__ void k_gather<2, 0>(GatherArgs);
template __global__ void k_gather<4, 0>(GatherArgs);

// ===========================================================================
// Fixed-point gather (FP64 form).
//
// The FP64 gather above issues one DFMA per stencil node and component and
// is bound by the FP64 pipe.  Here the sums run in int64 registers.  After
// the inverse FFT the grids become g' = round(g 2^Sg) (k_grid_to_fixed), Sg
// chosen from the largest |g| of the grid's output pair (SLP, DLP) so that
// |g'| < 2^Bg; the target's Gaussian
// factors are Yq[j] = round(Y[j] 2^62) and Xq[i] = round(X[i] 2^62) with
// X[i] = exp(a (px - h (i - P/2))^2) and Y the same in y, as in the fixed
// spread.  A column sums the high 64 bits of g' Yq[j], floor(g Y 2^(Sg-2)),
// and the target sums the high 64 bits of column * Xq[i]: sum g X Y at scale
// 2^(Sg-4).  Each floor is off by -1/2 unit on average, which the sums take
// back by starting from P/2 + 1 (P + 1 floors each).  Bg = 64 - log2(SX SY),
// SX and SY the largest sums of the x and y factors over a stencil (host), so
// no sum can overflow.  Every product is within one unit of 2^-(Sg-4), and a
// unit is about SX SY 2^-60 max|g|: finer than the FP64 gather's roundings
// relative to its partial sums unless max|g| is far above the grid values
// near the target, which the normwise error measure does not see.
// A NaN or infinity in the grid (non-finite inputs) sets gmax to a
// non-finite pattern; then the grid stays double and the FP64 gather runs.
// ===========================================================================

// Blocks of kGatherThreads, 512 / kGatherThreads per SM (128 registers).
// With the targets in patch-major order (launch_patch_order) a block's
// targets in flight form a compact patch of boxes, whose grid lines the
// block's warps share in L1.  At 2^20 targets, M = 2688, 15-node boxes:
// 3.17 ms with 3 x 3-box patches against 3.29 ms in box-sorted order (2 x 2:
// 3.29, 4 x 4: 3.27, 5 x 5: 3.35 ms); one 512-thread block per SM, 3.26 ms.
#ifndef SE2P_GATHER_THREADS
#define SE2P_GATHER_THREADS 256
#endif
constexpr int kGatherThreads = SE2P_GATHER_THREADS;

// Sg with max|g| 2^Sg < 2^Bg, from the bit pattern of max|g|.
__device__ __forceinline__ int grid_shift(unsigned long long gb, int Bg)
{
    if (gb == 0) return 0;
    const int e = (int)((gb >> 52) & 0x7ff) - 1022;  // max|g| < 2^e
    const int S = Bg - e;
    return S < -960 ? -960 : (S > 960 ? 960 : S);
}

// Grid c = blockIdx.y at its pair's scale.
__global__ void k_grid_to_fixed(double *__restrict__ grid, int64_t G,
                                const unsigned long long *__restrict__ gmax, int Bg)
{
    if (gmax_all(gmax) >= kGridNonFinite) return;
    const int c = blockIdx.y;
    const double s = ldexp(1.0, grid_shift(gmax[c / 2], Bg));
    double *g = grid + (int64_t)c * G;
    long long *q = reinterpret_cast<long long *>(g);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < G;
         i += (int64_t)gridDim.x * blockDim.x)
        q[i] = __double2ll_rn(g[i] * s);
}

template <int NC, int PT>
__global__ void __launch_bounds__(kGatherThreads, 512 / kGatherThreads) k_gather_fix(GatherArgs a)
{
    if (gmax_all(a.gmax) >= kGridNonFinite) return;
    const int P = PT > 0 ? PT : a.P;
    double outs[NC / 2];
#pragma unroll
    for (int k = 0; k < NC / 2; k++) {
        const unsigned long long gb = a.gmax[k];
        outs[k] = gb == 0 ? 0.0 : ldexp(a.scale, 4 - grid_shift(gb, a.Bg));
    }
    const long long bias = P / 2 + 1;
    const long long *grid = reinterpret_cast<const long long *>(a.grid);
    const size_t G = (size_t)a.Mx * a.My;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < a.nt;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = a.order ? (int64_t)a.order[k] : k;
        const double2 T = a.tp[t];
        int mx, my;
        double px, py;
        closest_node(T.x, T.y, a.Lhx, a.Lhy, a.h, P, mx, my, px, py);
        const double ax = exp(a.a * (px * px + 2.0 * a.w * px)) * 0x1p62;
        const double ay = exp(a.a * (py * py + 2.0 * a.w * py)) * 0x1p62;
        const double e3x = exp(-2.0 * a.a * a.h * px);
        const double e3y = exp(-2.0 * a.a * a.h * py);
        long long yq[(PT > 0 ? PT : kMaxP) + 1];
        {
            double ey = ay;
#pragma unroll
            for (int j = 0; j <= (PT > 0 ? PT : kMaxP); j++) {
                if (j <= P) {
                    yq[j] = __double2ll_rn(a.e1[j] * ey);
                    ey *= e3y;
                }
            }
        }
        long long acc[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) acc[c] = bias;
        const bool rows_inside = my >= 0 && my + P < a.My;
        double xf = ax;
        for (int i = 0; i <= P; i++) {
            const long long *g = grid + (size_t)wrap_index(mx + i, a.Mx) * a.My;
            long long tc[NC];
#pragma unroll
            for (int c = 0; c < NC; c++) tc[c] = bias;
            if (rows_inside) {
                const long long *gr = g + my;
#pragma unroll
                for (int j = 0; j <= (PT > 0 ? PT : kMaxP); j++) {
                    if (j <= P) {
#pragma unroll
                        for (int c = 0; c < NC; c++) tc[c] += __mul64hi(__ldg(gr + c * G + j), yq[j]);
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j <= (PT > 0 ? PT : kMaxP); j++) {
                    if (j <= P) {
                        const int row = wrap_index(my + j, a.My);
#pragma unroll
                        for (int c = 0; c < NC; c++) tc[c] += __mul64hi(__ldg(g + c * G + row), yq[j]);
                    }
                }
            }
            const long long xq = __double2ll_rn(xf * a.e1[i]);
            xf *= e3x;
#pragma unroll
            for (int c = 0; c < NC; c++) acc[c] += __mul64hi(tc[c], xq);
        }
#pragma unroll
        for (int k = 0; k < NC / 2; k++)
            a.out[k * a.nt + t] =
                make_double2((double)acc[2 * k] * outs[k], (double)acc[2 * k + 1] * outs[k]);
    }
}
template __global__ void k_gather_fix<2, 24>(GatherArgs);
template __global__ void k_gather_fix<4, 24>(GatherArgs);
template __global__ void k_gather_fix<2, 12>(GatherArgs);
template __global__ void k_gather_fix<4, 12>(GatherArgs);
template __global__ void k_gather_fix<2, 0>(GatherArgs);
template __global__ void k_gather_fix<4, 0>(GatherArgs);

// k_gather_fix for nr right-hand sides on one point set: a target's stencil
// origin and Gaussian factors are formed once, then each right-hand side r
// gathers its NC fixed-point grids (a.grid + r gstride words, scales from
// a.gmax + r kGmaxWords) into a.out + r ostride.  A right-hand side whose
// grids held a non-finite value is left to the FP64 gather.
template <int NC, int PT>
__global__ void __launch_bounds__(256, 2) k_gather_fix_multi(GatherArgs a, int nr, int64_t gstride,
                                                             int64_t ostride)
{
    const int P = PT > 0 ? PT : a.P;
    const long long bias = P / 2 + 1;
    const size_t G = (size_t)a.Mx * a.My;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.nt;
         t += (int64_t)gridDim.x * blockDim.x) {
        const double2 T = a.tp[t];
        int mx, my;
        double px, py;
        closest_node(T.x, T.y, a.Lhx, a.Lhy, a.h, P, mx, my, px, py);
        const double ax = exp(a.a * (px * px + 2.0 * a.w * px)) * 0x1p62;
        const double ay = exp(a.a * (py * py + 2.0 * a.w * py)) * 0x1p62;
        const double e3x = exp(-2.0 * a.a * a.h * px);
        const double e3y = exp(-2.0 * a.a * a.h * py);
        long long yq[(PT > 0 ? PT : kMaxP) + 1];
        {
            double ey = ay;
#pragma unroll
            for (int j = 0; j <= (PT > 0 ? PT : kMaxP); j++) {
                if (j <= P) {
                    yq[j] = __double2ll_rn(a.e1[j] * ey);
                    ey *= e3y;
                }
            }
        }
        const bool rows_inside = my >= 0 && my + P < a.My;
        for (int r = 0; r < nr; r++) {
            const unsigned long long *gm = a.gmax + r * kGmaxWords;
            if (gmax_all(gm) >= kGridNonFinite) continue;   // this one runs the FP64 gather
            double outs[NC / 2];
#pragma unroll
            for (int k = 0; k < NC / 2; k++)
                outs[k] = gm[k] == 0 ? 0.0 : ldexp(a.scale, 4 - grid_shift(gm[k], a.Bg));
            const long long *grid = reinterpret_cast<const long long *>(a.grid) + r * gstride;
            long long acc[NC];
#pragma unroll
            for (int c = 0; c < NC; c++) acc[c] = bias;
            double xf = ax;
            for (int i = 0; i <= P; i++) {
                const long long *g = grid + (size_t)wrap_index(mx + i, a.Mx) * a.My;
                long long tc[NC];
#pragma unroll
                for (int c = 0; c < NC; c++) tc[c] = bias;
                if (rows_inside) {
                    const long long *gr = g + my;
#pragma unroll
                    for (int j = 0; j <= (PT > 0 ? PT : kMaxP); j++) {
                        if (j <= P) {
#pragma unroll
                            for (int c = 0; c < NC; c++) tc[c] += __mul64hi(__ldg(gr + c * G + j), yq[j]);
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j <= (PT > 0 ? PT : kMaxP); j++) {
                        if (j <= P) {
                            const int row = wrap_index(my + j, a.My);
#pragma unroll
                            for (int c = 0; c < NC; c++) tc[c] += __mul64hi(__ldg(g + c * G + row), yq[j]);
                        }
                    }
                }
                const long long xq = __double2ll_rn(xf * a.e1[i]);
                xf *= e3x;
#pragma unroll
                for (int c = 0; c < NC; c++) acc[c] += __mul64hi(tc[c], xq);
            }
            double2 *out = a.out + r * ostride;
#pragma unroll
            for (int k = 0; k < NC / 2; k++)
                out[k * a.nt + t] =
                    make_double2((double)acc[2 * k] * outs[k], (double)acc[2 * k + 1] * outs[k]);
        }
    }
}
template __global__ void k_gather_fix_multi<2, 24>(GatherArgs, int, int64_t, int64_t);
template __global__ void k_gather_fix_multi<4, 24>(GatherArgs, int, int64_t, int64_t);
template __global__ void k_gather_fix_multi<2, 0>(GatherArgs, int, int64_t, int64_t);
template __global__ void k_gather_fix_multi<4, 0>(GatherArgs, int, int64_t, int64_t);


// ===========================================================================
// k-space adjoint.
//
// The SLP operator grid -> filtered grid is a real circulant with an even,
// symmetric multiplier, so it is its own transpose: the adjoint spreads w at
// the targets and runs the same filter.  The DLP operator has the odd
// multiplier m(k) = -i c(k); its transpose has m(-k) = -m(k), and the minus
// sign with which the DLP enters u cancels that, so the adjoint applies the
// transposed 3x2 coefficient matrix with the same -i factor.  Spectra: 0,1 =
// SLP (in and out), 2,3 = DLP in, 2,3,4 = DLP out.
// ===========================================================================
__device__ __forceinline__ void dlp_matrix(double k1, double k2, double xi, double eta,
                                           double m[2][3])
{
    const double K2 = k1 * k1 + k2 * k2;
    const double e = exp(-0.25 * (1 - eta) / (xi * xi) * K2) / K2 / K2;
    const double et = e * (1 + 0.25 * K2 / xi / xi);
    m[0][0] = et * (3.0 * k1 * K2 - 2.0 * k1 * k1 * k1);
    m[0][1] = et * (k2 * K2 - 2.0 * k1 * k1 * k2);
    m[0][2] = et * (k1 * K2 - 2.0 * k1 * k2 * k2);
    m[1][0] = et * (k2 * K2 - 2.0 * k2 * k1 * k1);
    m[1][1] = et * (k1 * K2 - 2.0 * k2 * k1 * k2);
    m[1][2] = et * (3.0 * k2 * K2 - 2.0 * k2 * k2 * k2);
}

__global__ void k_filter_adj(FilterArgs a)
{
    const int H = a.My / 2 + 1;
    const int64_t G = (int64_t)a.Mx * H;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= G) return;
    int jx, jy;
    if (a.transposed) {
        jy = (int)(idx / a.Mx);
        jx = (int)(idx - (int64_t)jy * a.Mx);
    } else {
        jx = (int)(idx / H);
        jy = (int)(idx - (int64_t)jx * H);
    }
    double2 *sp = reinterpret_cast<double2 *>(a.spec);
    if (a.mtab) {
        // the forward filter's cached multipliers: the SLP matrix (symmetric)
        // and the DLP rows applied transposed, with the same -i
        const double *m = a.mtab + (int64_t)kFilterMat * idx;
        if (a.slp_in >= 0) {
            const double2 h1 = sp[a.slp_in * G + idx], h2 = sp[(a.slp_in + 1) * G + idx];
            sp[a.slp_out * G + idx] =
                make_double2(fma(m[0], h1.x, -m[1] * h2.x), fma(m[0], h1.y, -m[1] * h2.y));
            sp[(a.slp_out + 1) * G + idx] =
                make_double2(fma(m[2], h2.x, -m[1] * h1.x), fma(m[2], h2.y, -m[1] * h1.y));
        }
        if (a.dlp_in >= 0) {
            const double2 p1 = sp[a.dlp_in * G + idx], p2 = sp[(a.dlp_in + 1) * G + idx];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double re = fma(m[3 + c], p1.x, m[6 + c] * p2.x);
                const double im = fma(m[3 + c], p1.y, m[6 + c] * p2.y);
                sp[(a.dlp_out + c) * G + idx] = make_double2(im, -re);
            }
        }
        return;
    }
    const bool zero = (jx == 0 && jy == 0);
    const bool nyq = (jx == a.Mx / 2) || (jy == a.My / 2);
    const double k1 = kfreq(jx, a.Mx, a.Lx), k2 = kfreq(jy, a.My, a.Ly);
    const double k1p = (jx == a.Mx / 2) ? k1 : -k1;
    const double k2p = (jy == a.My / 2) ? k2 : -k2;
    const double sc = a.scale;
    if (a.slp_in >= 0) {
        double2 o1, o2;
        const double2 h1 = sp[a.slp_in * G + idx], h2 = sp[(a.slp_in + 1) * G + idx];
        const double fe = -1.0;                      // computed in slp_mode
        slp_mode(k1, k2, a.xi, a.eta, h1, h2, o1, o2, fe);
        if (nyq) {
            double2 p1, p2;
            slp_mode(k1p, k2p, a.xi, a.eta, h1, h2, p1, p2, fe);
            o1.x = 0.5 * (o1.x + p1.x); o1.y = 0.5 * (o1.y + p1.y);
            o2.x = 0.5 * (o2.x + p2.x); o2.y = 0.5 * (o2.y + p2.y);
        }
        if (zero) o1 = o2 = make_double2(0.0, 0.0);
        sp[a.slp_out * G + idx] = make_double2(o1.x * sc, o1.y * sc);
        sp[(a.slp_out + 1) * G + idx] = make_double2(o2.x * sc, o2.y * sc);
    }
    if (a.dlp_in >= 0) {
        const double2 p1 = sp[a.dlp_in * G + idx], p2 = sp[(a.dlp_in + 1) * G + idx];
        double m[2][3];
        dlp_matrix(k1, k2, a.xi, a.eta, m);
        if (nyq) {
            double mp[2][3];
            dlp_matrix(k1p, k2p, a.xi, a.eta, mp);
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int c = 0; c < 3; c++) m[i][c] = 0.5 * (m[i][c] - mp[i][c]);
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            // -i (m_0c p1 + m_1c p2), scaled
            const double re = m[0][c] * p1.x + m[1][c] * p2.x;
            const double im = m[0][c] * p1.y + m[1][c] * p2.y;
            sp[(a.dlp_out + c) * G + idx] = zero ? make_double2(0.0, 0.0)
                                                 : make_double2(im * sc, -re * sc);
        }
    }
}

// Gather at the forward sources of the adjoint grids, with the gradient of
// the Gaussian weights: for coefficients c_k (f1, f2, S11, S12+S21, S22)
//   val_k = s sum_n W_n Phi_k(n),  grad = s sum_n grad_y W_n sum_k c_k Phi_k(n)
// where d/dp of the weight exponent a(p^2 + 2wp) + a h^2 (i-P/2)^2 - 2ahpi is
// 2a (p + w - h i).  Output: 7 values per sorted source.
template <int PT>
__global__ void __launch_bounds__(256) k_gather_adj(GatherAdjArgs a)
{
    // behind k_gather_adj_ff: runs only when a grid held a non-finite value
    if (a.gff && gmax_all(a.gmax) < kGridNonFinite) return;
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.ns) return;
    const int P = PT > 0 ? PT : a.P;
    const size_t G = (size_t)a.Mx * a.My;
    const double2 S = a.sp[s];
    int mx, my;
    double px, py;
    closest_node(S.x, S.y, a.Lhx, a.Lhy, a.h, P, mx, my, px, py);
    const double ex = exp(a.a * (px * px + py * py + 2.0 * a.w * px));
    const double e4y = exp(2.0 * a.a * a.w * py);
    const double e3x = exp(-2.0 * a.a * a.h * px);
    const double e3y = exp(-2.0 * a.a * a.h * py);
    constexpr int PM = (PT > 0 ? PT : kMaxP) + 1;
    double wy[PM], wyd[PM];
    {
        double ey = 1.0;
#pragma unroll
        for (int j = 0; j < PM; j++) {
            if (j <= P) {
                wy[j] = a.e1[j] * ey;
                wyd[j] = wy[j] * 2.0 * a.a * (py + a.w - a.h * j);
                ey *= e3y;
            }
        }
    }
    double c[5];
#pragma unroll
    for (int k = 0; k < 5; k++) c[k] = a.coef[5 * s + k];
    double acc[5] = {0, 0, 0, 0, 0}, gx = 0.0, gy = 0.0;
    const bool rows_inside = my >= 0 && my + P < a.My;
    double xf = ex * e4y;
    for (int i = 0; i <= P; i++) {
        const double *g = a.grid + (size_t)wrap_index(mx + i, a.Mx) * a.My;
        // per component the column sums with wy and wyd (10 DFMA per node);
        // the wyd sums meet the coefficients once per column
        double tc[5] = {0, 0, 0, 0, 0}, td[5] = {0, 0, 0, 0, 0};
#pragma unroll
        for (int j = 0; j < PM; j++) {
            if (j <= P) {
                const int row = rows_inside ? my + j : wrap_index(my + j, a.My);
#pragma unroll
                for (int k = 0; k < 5; k++) {
                    const double v = __ldg(g + k * G + row);
                    tc[k] = fma(wy[j], v, tc[k]);
                    td[k] = fma(wyd[j], v, td[k]);
                }
            }
        }
        double u = 0.0;
#pragma unroll
        for (int k = 0; k < 5; k++) u = fma(c[k], td[k], u);
        const double wx = xf * a.e1[i];
        const double wxd = wx * 2.0 * a.a * (px + a.w - a.h * i);
        xf *= e3x;
        double ct = 0.0;
#pragma unroll
        for (int k = 0; k < 5; k++) {
            acc[k] = fma(wx, tc[k], acc[k]);
            ct = fma(c[k], tc[k], ct);
        }
        gx = fma(wxd, ct, gx);
        gy = fma(wx, u, gy);
    }
    double *o = a.out + 7 * s;
#pragma unroll
    for (int k = 0; k < 5; k++) o[k] = acc[k] * a.scale;
    o[5] = gx * a.scale;
    o[6] = gy * a.scale;
}

template __global__ void k_gather_adj<24>(GatherAdjArgs);
template __global__ void k_gather_adj<0>(GatherAdjArgs);

// ---------------------------------------------------------------------------
// The adjoint gather in float-float arithmetic (FP64 form).
//
// k_gather_adj spends 10 DFMA per stencil node, at GB300's FP64 rate, and
// its 255 registers leave one block per SM.  Here a warp takes one source
// at a time with lane = stencil row j: per column i the lanes load the five
// grid values of their rows (consecutive, so the loads coalesce) and keep
//   A_k(j) = sum_i wx_i g_k(i, j),   B_k(j) = sum_i wx'_i g_k(i, j)
// in float-float (wx' the x derivative of the weight).  Then
//   value_k = sum_j wy_j A_k(j),  grad_x = sum_j wy_j sum_k c_k B_k(j),
//   grad_y = sum_j wy'_j sum_k c_k A_k(j),
// the same sums as k_gather_adj in another order, with warp reductions over
// the rows.  The weights come from float-float product scans across lanes
// (lane i holds e3^i) of the per-source factors, which the lanes form in
// FP64 for 32 sources at a time; the grids are read as float-float planes
// scaled by a power of two from the grid maximum (k_grid_to_ff), and the
// coefficients by their own power of two, so that float's exponent range
// holds every factor (adj_gather_ff_ok bounds the weights' exponents).
// The sums carry about 1e-13 relative error (the tests hold the float-float
// adjoint to 1e-11 of the all-FP64 one), far below the adjoint's
// finite-difference checks.
// ---------------------------------------------------------------------------
constexpr int kAdjFFWarps = 8;

// 2^sg brings max |grid| below 1.
__device__ __forceinline__ int ff_grid_shift(unsigned long long gb)
{
    if (gb == 0) return 0;
    return -((int)((gb >> 52) & 0x7ff) - 1022);
}

__global__ void k_grid_to_ff(const double *__restrict__ grid, int64_t n,
                             const unsigned long long *__restrict__ gmax, float2 *__restrict__ out)
{
    const unsigned long long gb = gmax_all(gmax);    // one scale for the five grids
    if (gb >= kGridNonFinite) return;
    const double sc = ldexp(1.0, ff_grid_shift(gb));
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = ff_split(grid[i] * sc);
}

// acc + w * v, all float-float.
__device__ __forceinline__ float2 ff_fma(float2 w, float2 v, float2 acc)
{
    const float p = w.x * v.x;
    float e = fmaf(w.x, v.x, -p);
    e = fmaf(w.x, v.y, e);
    e = fmaf(w.y, v.x, e);
    float s, t;
    two_sum(acc.x, p, s, t);
    t += e + acc.y;
    float h, l;
    fast_two_sum(s, t, h, l);
    return make_float2(h, l);
}

__device__ __forceinline__ float2 shfl_ff(float2 v, int src)
{
    return make_float2(__shfl_sync(~0u, v.x, src), __shfl_sync(~0u, v.y, src));
}

__device__ __forceinline__ float2 shfl_up_ff(float2 v, int o)
{
    return make_float2(__shfl_up_sync(~0u, v.x, o), __shfl_up_sync(~0u, v.y, o));
}

__device__ __forceinline__ float2 shfl_xor_ff(float2 v, int o)
{
    return make_float2(__shfl_xor_sync(~0u, v.x, o), __shfl_xor_sync(~0u, v.y, o));
}

template <int PT>
__global__ void __launch_bounds__(kAdjFFWarps * 32, 2) k_gather_adj_ff(GatherAdjArgs a)
{
    const unsigned long long gb = gmax_all(a.gmax);
    if (gb >= kGridNonFinite) return;                // the FP64 gather runs instead
    const int sg = ff_grid_shift(gb);
    const int P = PT > 0 ? PT : a.P, P1 = P + 1;     // P1 <= 31
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const size_t G = (size_t)a.Mx * a.My;
    const float2 e1l = lane < P1 ? ff_split(a.e1[lane]) : make_float2(0.f, 0.f);
    const float2 hl = ff_mul_f(ff_split(a.h), (float)lane);    // h * lane
    const float2 da = ff_split(2.0 * a.a);
    const int64_t nw = (int64_t)gridDim.x * kAdjFFWarps;
    for (int64_t base = ((int64_t)blockIdx.x * kAdjFFWarps + wid) * 32; base < a.ns;
         base += nw * 32) {
        // per-source factors of this lane's source, in FP64, then float-float
        const int64_t sl = base + lane;
        int mx = 0, my = 0, ec = 0;
        float2 x0 = make_float2(0.f, 0.f), e3x = x0, e3y = x0, qx = x0, qy = x0;
        float2 c[5];
#pragma unroll
        for (int k = 0; k < 5; k++) c[k] = x0;
        if (sl < a.ns) {
            const double2 S = a.sp[sl];
            double px, py;
            closest_node(S.x, S.y, a.Lhx, a.Lhy, a.h, P, mx, my, px, py);
            x0 = ff_split(exp(a.a * (px * px + py * py + 2.0 * a.w * px)) *
                          exp(2.0 * a.a * a.w * py));
            e3x = ff_split(exp(-2.0 * a.a * a.h * px));
            e3y = ff_split(exp(-2.0 * a.a * a.h * py));
            qx = ff_split(px + a.w);
            qy = ff_split(py + a.w);
            double cm = 0.0, cv[5];
#pragma unroll
            for (int k = 0; k < 5; k++) {
                cv[k] = a.coef[5 * sl + k];
                cm = fmax(cm, fabs(cv[k]));
            }
            if (cm > 0.0 && cm <= 1.7976931348623157e308) frexp(cm, &ec);   // cm < 2^ec
#pragma unroll
            for (int k = 0; k < 5; k++) c[k] = ff_split(ldexp(cv[k], -ec));
        }
        const int cnt = (int)min((int64_t)32, a.ns - base);
        for (int j = 0; j < cnt; j++) {
            const int smx = __shfl_sync(~0u, mx, j), smy = __shfl_sync(~0u, my, j);
            const int sec = __shfl_sync(~0u, ec, j);
            const float2 sx0 = shfl_ff(x0, j);
            const float2 b3x = shfl_ff(e3x, j), b3y = shfl_ff(e3y, j);
            const float2 sqx = shfl_ff(qx, j), sqy = shfl_ff(qy, j);
            float2 sc[5];
#pragma unroll
            for (int k = 0; k < 5; k++) sc[k] = shfl_ff(c[k], j);
            // e3^lane by a product scan across lanes
            float2 px_ = lane >= 1 ? b3x : make_float2(1.f, 0.f);
            float2 py_ = lane >= 1 ? b3y : make_float2(1.f, 0.f);
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float2 tx = shfl_up_ff(px_, o), ty = shfl_up_ff(py_, o);
                if (lane >= o) {
                    px_ = ff_mul(px_, tx);
                    py_ = ff_mul(py_, ty);
                }
            }
            // lane as column i: wx_i, wx'_i; lane as row j: wy_j, wy'_j
            // (the derivative factor 2a (p + w - h i) of the weight exponent)
            const float2 wx = ff_mul(ff_mul(sx0, e1l), px_);
            const float2 wxd = ff_mul(wx, ff_mul(da, ff_sub(sqx, hl)));
            const float2 wy = ff_mul(e1l, py_);
            const float2 wyd = ff_mul(wy, ff_mul(da, ff_sub(sqy, hl)));
            // column sums as Dot2 accumulators (float sum + float error term),
            // normalised once after the last column
            float As[5], Ac[5], Bs[5], Bc[5];
#pragma unroll
            for (int k = 0; k < 5; k++) As[k] = Ac[k] = Bs[k] = Bc[k] = 0.f;
            const int row = lane < P1 ? wrap_index(smy + lane, a.My) : 0;
            int col = wrap_index(smx, a.Mx);
            for (int i = 0; i <= P; i++) {
                const float2 wxi = shfl_ff(wx, i), wxdi = shfl_ff(wxd, i);
                if (lane < P1) {
                    const float2 *g = a.gff + (size_t)col * a.My + row;
                    float2 v[5];
#pragma unroll
                    for (int k = 0; k < 5; k++) v[k] = __ldg(g + k * G);
#pragma unroll
                    for (int k = 0; k < 5; k++) {
                        ff_dot_acc(wxi, v[k], As[k], Ac[k]);
                        ff_dot_acc(wxdi, v[k], Bs[k], Bc[k]);
                    }
                }
                if (++col == a.Mx) col = 0;
            }
            float2 A[5], B[5];
#pragma unroll
            for (int k = 0; k < 5; k++) {
                A[k] = ff_norm(As[k], Ac[k]);
                B[k] = ff_norm(Bs[k], Bc[k]);
            }
            // rows: values, and the gradients through the coefficients
            float2 r[7], ca = make_float2(0.f, 0.f), cb = ca;
#pragma unroll
            for (int k = 0; k < 5; k++) {
                r[k] = ff_mul(wy, A[k]);
                ca = ff_fma(sc[k], A[k], ca);
                cb = ff_fma(sc[k], B[k], cb);
            }
            r[5] = ff_mul(wy, cb);
            r[6] = ff_mul(wyd, ca);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
                for (int k = 0; k < 7; k++) r[k] = ff_add(r[k], shfl_xor_ff(r[k], o));
            }
            if (lane == 0) {
                double *out = a.out + 7 * (base + j);
                const double sv = ldexp(a.scale, -sg), sgr = ldexp(a.scale, sec - sg);
#pragma unroll
                for (int k = 0; k < 5; k++) out[k] = ff_to_double(r[k]) * sv;
                out[5] = ff_to_double(r[5]) * sgr;
                out[6] = ff_to_double(r[6]) * sgr;
            }
        }
    }
}

template __global__ void k_gather_adj_ff<24>(GatherAdjArgs);
template __global__ void k_gather_adj_ff<0>(GatherAdjArgs);

// Float range for the float-float adjoint gather: every weight factor's
// exponent (x0, e3^i up to i = 31, e1) within 80 of 0.
bool adj_gather_ff_ok(double a, double h, double w, int P)
{
    const double ah2 = std::fabs(a) * h * h;
    const double c = P / 2 + 1;
    const double m = std::max(std::max(2.0 + 2.0 * std::fabs(w) / h, 62.0), c * c);
    return ah2 * m <= 80.0;
}


// sum_t w_dlp(t) (the zero-mode term's weight), partial sums per block.
__global__ void __launch_bounds__(256) k_wsum_part(int64_t n, const double *__restrict__ w,
                                                   int stride, int off, double2 *__restrict__ part)
{
    __shared__ double2 red[8];
    double sx = 0.0, sy = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        sx += w[stride * i + off];
        sy += w[stride * i + off + 1];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(~0u, sx, o);
        sy += __shfl_xor_sync(~0u, sy, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_double2(sx, sy);
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 t = red[0];
        for (int k = 1; k < 8; k++) {
            t.x += red[k].x;
            t.y += red[k].y;
        }
        part[blockIdx.x] = t;
    }
}

// part[nparts] = the sum of part[0 .. nparts-1], added in index order.
__global__ void k_wsum_final(int nparts, double2 *__restrict__ part)
{
    if (threadIdx.x != 0) return;
    double2 t = make_double2(0.0, 0.0);
    for (int b = 0; b < nparts; b++) {
        t.x += part[b].x;
        t.y += part[b].y;
    }
    part[nparts] = t;
}

// Combine the real-space (gr, 7 per sorted source, unscaled) and k-space (gk,
// 7 per sorted source, scaled) adjoint parts with the DLP zero-mode term and
// the chain rule S = f (x) n; write gradients in the caller's source order.
__global__ void k_adj_assemble(int64_t n, const int *__restrict__ perm,
                               const double *__restrict__ gr, const double *__restrict__ gk,
                               const double2 *__restrict__ wsum,
                               const double2 *__restrict__ praw, const double2 *__restrict__ fd,
                               const double2 *__restrict__ nrm, double inv_area, int slp, int dlp,
                               double2 *__restrict__ g_pos, double2 *__restrict__ g_fs,
                               double2 *__restrict__ g_fd, double2 *__restrict__ g_n)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int i = perm[j];
    const double *r = gr + 7 * j, *k = gk + 7 * j;
    const double q = 1.0 / (4.0 * kPi);
    double gp1 = r[5] * q + k[5], gp2 = r[6] * q + k[6];
    if (slp && g_fs) g_fs[i] = make_double2(r[0] * q + k[0], r[1] * q + k[1]);
    if (dlp) {
        const double Wx = wsum->x, Wy = wsum->y;
        const double2 x = praw[i], f = fd[i], m = nrm[i];
        const double zw = (Wx * x.x + Wy * x.y) * inv_area;        // d J / d (f.n)
        const double gS11 = -r[2] * q + k[2] + zw, gS12 = -r[3] * q + k[3];
        const double gS22 = -r[4] * q + k[4] + zw;
        const double fn = f.x * m.x + f.y * m.y;
        gp1 += fn * Wx * inv_area;
        gp2 += fn * Wy * inv_area;
        if (g_fd) g_fd[i] = make_double2(m.x * gS11 + m.y * gS12, m.x * gS12 + m.y * gS22);
        if (g_n) g_n[i] = make_double2(f.x * gS11 + f.y * gS12, f.x * gS12 + f.y * gS22);
    }
    if (g_pos) g_pos[i] = make_double2(gp1, gp2);
}

// ===========================================================================
// Small helpers
// ===========================================================================

// x -> mod(x + L/2, L) - L/2 as numpy.mod computes it (exact fmod, then +L
// when the sign differs from L): the MATLAB drivers' wrap
// (StokesSLP_ewald_2p.m:75-78).
__device__ __forceinline__ double wrap_coord(double x, double L)
{
    const double a = xadd(x, 0.5 * L);
    double r = fmod(a, L);
    if (r != 0.0) {
        if ((r < 0.0) != (L < 0.0)) r = xadd(r, L);
    } else {
        r = copysign(0.0, L);
    }
    return xsub(r, 0.5 * L);
}

__global__ void k_wrap(int64_t n, const double2 *__restrict__ p, double Lx, double Ly,
                       double2 *__restrict__ out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 q = p[i];
    out[i] = make_double2(wrap_coord(q.x, Lx), wrap_coord(q.y, Ly));
}

// Partial sums of (f.n) x_src over blocks (DLP k=0 term,
// StokesDLP_ewald_2p.m:150-151); finished by k_zero_mode_final.
__global__ void __launch_bounds__(256) k_zero_mode_part(int64_t n, const double2 *__restrict__ p,
                                                        const double2 *__restrict__ f,
                                                        const double2 *__restrict__ nrm,
                                                        double2 *__restrict__ part)
{
    __shared__ double2 red[8];
    double sx = 0.0, sy = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double2 q = p[i], ff = f[i], m = nrm[i];
        const double fn = ff.x * m.x + ff.y * m.y;
        sx += fn * q.x;
        sy += fn * q.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(~0u, sx, o);
        sy += __shfl_xor_sync(~0u, sy, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_double2(sx, sy);
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 s = red[0];
        for (int w = 1; w < 8; w++) {
            s.x += red[w].x;
            s.y += red[w].y;
        }
        part[blockIdx.x] = s;
    }
}

__global__ void k_zero_mode_final(int nparts, const double2 *__restrict__ part, double inv_area,
                                  double2 *__restrict__ zm)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double2 s = make_double2(0.0, 0.0);
    for (int i = 0; i < nparts; i++) {
        s.x += part[i].x;
        s.y += part[i].y;
    }
    *zm = make_double2(s.x * inv_area, s.y * inv_area);
}

// Final assembly in original target order.
//   mode 0: SLP real only     u = ur / (4 pi)
//   mode 1: DLP real only     u = ur / 4 / pi
//   mode 2: k-space only      u = uk
//   mode 3: SLP driver        u = ur/(4 pi) + uk
//   mode 4: DLP driver        u = -(ur/4/pi + uk - zm)
// ur (sorted order, raw sums) and uk (sorted order, scaled) may be NULL when
// unused; ur_out / uk_out (original order) receive the parts when non-NULL.
__global__ void k_assemble(int64_t n, int mode, const int *__restrict__ perm,
                           const double2 *__restrict__ ur, const double2 *__restrict__ uk,
                           const double2 *__restrict__ zm, double2 *__restrict__ u,
                           double2 *__restrict__ ur_out, double2 *__restrict__ uk_out)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int i = perm[j];
    double2 r = make_double2(0.0, 0.0), k = make_double2(0.0, 0.0);
    if (ur) {
        r = ur[j];
        if (mode == 1 || mode == 4) {
            r.x = r.x / 4.0 / kPi;
            r.y = r.y / 4.0 / kPi;
        } else {
            r.x = r.x / (4.0 * kPi);
            r.y = r.y / (4.0 * kPi);
        }
    }
    if (uk) {
        k = uk[j];
        if (mode == 4) {
            const double2 z = *zm;
            k.x -= z.x;
            k.y -= z.y;
        }
    }
    double2 v;
    switch (mode) {
    case 0: case 1: v = r; break;
    case 2: v = k; break;
    case 3: v = make_double2(r.x + k.x, r.y + k.y); break;
    default: v = make_double2(-(r.x + k.x), -(r.y + k.y)); break;
    }
    u[i] = v;
    if (ur_out) ur_out[i] = r;
    if (uk_out) uk_out[i] = k;
}

// ===========================================================================
// Host launchers
// ===========================================================================
static inline unsigned grid_for(int64_t n, int block)
{
    int64_t g = (n + block - 1) / block;
    return (unsigned)(g < 1 ? 1 : g);
}

// Number of SMs of the current device (cached per process for device 0..63).
int sm_count()
{
    static int cache[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 152;
    if (!cache[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = v > 0 ? v : 152;
    }
    return cache[dev];
}

cudaError_t launch_bin(const BinArgs &a, int *start, int nbox, int *perm, int *sorted_box,
                       double2 *sorted_pos, float2 *sorted_pos_f, cudaStream_t st,
                       int64_t &launches, float2 *sorted_pos_lo)
{
    cudaError_t e = cudaMemsetAsync(a.count, 0, sizeof(int) * (size_t)nbox, st);
    if (e != cudaSuccess) return e;
    if (a.n > 0) {
        k_bin_count<<<grid_for(a.n, 256), 256, 0, st>>>(a);
        launches++;
    }
    k_scan<<<1, 1024, 0, st>>>(a.count, nbox, start);
    launches++;
    if (a.n > 0) {
        k_bin_place<<<grid_for(a.n, 256), 256, 0, st>>>(a.n, a.box, a.rank, start, perm,
                                                         sorted_box, a.p, sorted_pos,
                                                         sorted_pos_f, sorted_pos_lo);
        launches++;
    }
    return cudaGetLastError();
}

cudaError_t launch_src_coef(int64_t n, const int *perm, const double2 *f_slp,
                            const double2 *f_dlp, const double2 *nrm, double *coef, int nc,
                            cudaStream_t st, int64_t &launches)
{
    if (n <= 0) return cudaSuccess;
    k_src_coef<<<grid_for(n, 256), 256, 0, st>>>(n, perm, f_slp, f_dlp, nrm, coef, nc);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_src_coef_ff(int64_t n, const double *coef, int nc, bool slp, bool dlp,
                               float2 *out, int ncf, cudaStream_t st, int64_t &launches,
                               int64_t ostride, bool tails)
{
    if (n <= 0) return cudaSuccess;
    k_src_coef_ff<<<grid_for(n, 256), 256, 0, st>>>(n, coef, nc, slp, dlp, out,
                                                     ostride > 0 ? ostride : ncf, tails ? 1 : 0);
    launches++;
    return cudaGetLastError();
}

template <int FORM>
static void launch_real_form(const RealArgs &a, bool slp, bool dlp, unsigned g, cudaStream_t st)
{
    if (slp && dlp) k_real<true, true, FORM><<<g, kRealWarps * 32, 0, st>>>(a);
    else if (slp) k_real<true, false, FORM><<<g, kRealWarps * 32, 0, st>>>(a);
    else k_real<false, true, FORM><<<g, kRealWarps * 32, 0, st>>>(a);
}

cudaError_t launch_real(const RealArgs &a, bool slp, bool dlp, cudaStream_t st,
                        int64_t &launches, int form)
{
    if (a.ntar <= 0) return cudaSuccess;
    const int64_t want = (a.ntar + kRealWarps - 1) / kRealWarps;
    // Six 4-warp blocks per SM (the launch bound holds 80 registers: 24 warps
    // resident), persistent over the sorted targets.  The k-space chain
    // (high-priority stream) takes what is left.  With 8-warp blocks at 94
    // registers only 16 warps fitted: 19.9 ms per evaluation at 2^20 points,
    // against 18.6 with 20 warps and 18.45 with 24.
    const int64_t cap = (int64_t)sm_count() * SE2P_REAL_MINB;
    const unsigned g = (unsigned)(want < cap ? want : cap);
    if (form == kFormF32) launch_real_form<kFormF32>(a, slp, dlp, g, st);
    else if (form == kFormFF) launch_real_form<kFormFF>(a, slp, dlp, g, st);
    else launch_real_form<kFormFP64>(a, slp, dlp, g, st);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_spread(const SpreadArgs &a, int nc, cudaStream_t st, int64_t &launches)
{
    if (a.ns <= 0) return cudaSuccess;
    const int64_t warps = (a.ns + 31) / 32;
    const int64_t want = (warps + kSpreadWarps - 1) / kSpreadWarps;
    const int64_t cap = (int64_t)sm_count() * 8;
    const unsigned g = (unsigned)(want < cap ? want : cap);
    switch (nc) {
    case 2: k_spread<2><<<g, kSpreadWarps * 32, 0, st>>>(a); break;
    case 3: k_spread<3><<<g, kSpreadWarps * 32, 0, st>>>(a); break;
    case 4: k_spread<4><<<g, kSpreadWarps * 32, 0, st>>>(a); break;
    default: k_spread<5><<<g, kSpreadWarps * 32, 0, st>>>(a); break;
    }
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_filter_matrix_table(const FilterArgs &a, double *mtab, cudaStream_t st,
                                       int64_t &launches)
{
    const int64_t n = (int64_t)a.Mx * (a.My / 2 + 1);
    k_filter_matrix_table<<<grid_for(n, 256), 256, 0, st>>>(a, mtab);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_filter(const FilterArgs &a, cudaStream_t st, int64_t &launches)
{
    const int64_t n = (int64_t)a.Mx * (a.My / 2 + 1);
    k_filter<<<grid_for(n, 256), 256, 0, st>>>(a);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_gather(const GatherArgs &a, int nc, cudaStream_t st, int64_t &launches)
{
    if (a.nt <= 0) return cudaSuccess;
    // one resident block per SM, grid-stride over the sorted targets
    unsigned g = grid_for(a.nt, 256);
    if (g > (unsigned)sm_count()) g = (unsigned)sm_count();
    if (a.gmax) {
        // two resident blocks per SM (128 registers): the integer sums wait on
        // loads, so they want more warps than the FP64-bound gather
        const unsigned gf =
            std::min(grid_for(a.nt, kGatherThreads), (unsigned)(sm_count() * (512 / kGatherThreads)));
        constexpr int B = kGatherThreads;
        if (nc == 2) {
            if (a.P == 24) k_gather_fix<2, 24><<<gf, B, 0, st>>>(a);
            else if (a.P == 12) k_gather_fix<2, 12><<<gf, B, 0, st>>>(a);
            else k_gather_fix<2, 0><<<gf, B, 0, st>>>(a);
        } else {
            if (a.P == 24) k_gather_fix<4, 24><<<gf, B, 0, st>>>(a);
            else if (a.P == 12) k_gather_fix<4, 12><<<gf, B, 0, st>>>(a);
            else k_gather_fix<4, 0><<<gf, B, 0, st>>>(a);
        }
        launches++;
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (nc == 2) {
        if (a.P == 24) k_gather<2, 24><<<g, 256, 0, st>>>(a);
        else if (a.P == 12) k_gather<2, 12><<<g, 256, 0, st>>>(a);
        else k_gather<2, 0><<<g, 256, 0, st>>>(a);
    } else {
        if (a.P == 24) k_gather<4, 24><<<g, 256, 0, st>>>(a);
        else if (a.P == 12) k_gather<4, 12><<<g, 256, 0, st>>>(a);
        else k_gather<4, 0><<<g, 256, 0, st>>>(a);
    }
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_wrap(int64_t n, const double2 *p, double Lx, double Ly, double2 *out,
                        cudaStream_t st, int64_t &launches)
{
    if (n <= 0) return cudaSuccess;
    k_wrap<<<grid_for(n, 256), 256, 0, st>>>(n, p, Lx, Ly, out);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_zero_mode(int64_t n, const double2 *p, const double2 *f, const double2 *nrm,
                             double inv_area, double2 *part, double2 *zm, cudaStream_t st,
                             int64_t &launches)
{
    k_zero_mode_part<<<kZeroModeParts, 256, 0, st>>>(n, p, f, nrm, part);
    k_zero_mode_final<<<1, 32, 0, st>>>(kZeroModeParts, part, inv_area, zm);
    launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_assemble(int64_t n, int mode, const int *perm, const double2 *ur,
                            const double2 *uk, const double2 *zm, double2 *u, double2 *ur_out,
                            double2 *uk_out, cudaStream_t st, int64_t &launches)
{
    if (n <= 0) return cudaSuccess;
    k_assemble<<<grid_for(n, 256), 256, 0, st>>>(n, mode, perm, ur, uk, zm, u, ur_out, uk_out);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_sorted_pair(int64_t n, const int *perm, const double2 *a, const double2 *b,
                               double *out, cudaStream_t st, int64_t &launches)
{
    if (n <= 0) return cudaSuccess;
    k_sorted_pair<<<grid_for(n, 256), 256, 0, st>>>(n, perm, a, b, out);
    launches++;
    return cudaGetLastError();
}

template <int FORM>
static void launch_real_adj_form(const RealArgs &a, bool slp, bool dlp, unsigned g,
                                 cudaStream_t st)
{
    if (slp && dlp) k_real_adj<true, true, FORM><<<g, kAdjWarps * 32, 0, st>>>(a);
    else if (slp) k_real_adj<true, false, FORM><<<g, kAdjWarps * 32, 0, st>>>(a);
    else k_real_adj<false, true, FORM><<<g, kAdjWarps * 32, 0, st>>>(a);
}

cudaError_t launch_real_adj(const RealArgs &a, bool slp, bool dlp, cudaStream_t st,
                            int64_t &launches, int form)
{
    if (a.nouter <= 0) return cudaSuccess;
    const int64_t want = (a.nouter + kAdjWarps - 1) / kAdjWarps;
    // as many 4-warp blocks as fit at once (5 per SM at the launch bound), so
    // that no second wave of persistent blocks trails the first
    const int64_t cap = (int64_t)sm_count() * 5;
    const unsigned g = (unsigned)(want < cap ? want : cap);
    if (form == kFormFF) launch_real_adj_form<kFormFF>(a, slp, dlp, g, st);
    else launch_real_adj_form<kFormFP64>(a, slp, dlp, g, st);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_filter_adj(const FilterArgs &a, cudaStream_t st, int64_t &launches)
{
    const int64_t n = (int64_t)a.Mx * (a.My / 2 + 1);
    k_filter_adj<<<grid_for(n, 256), 256, 0, st>>>(a);
    launches++;
    return cudaGetLastError();
}

// Rate probe of the L2 atomic units: every thread adds 1 to `iters` words of
// an n-word array small enough to stay in L2, lane l of a warp on word w + l
// (the spread's stencil rows issue their 64-bit atomics the same way).
__global__ void k_probe_red64(unsigned long long *__restrict__ a, int64_t n, int iters)
{
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) % n;
    for (int k = 0; k < iters; k++) {
        atomicAdd(a + w, 1ull);
        w += nth;
        if (w >= n) w -= n;
    }
}

cudaError_t launch_probe_red64(unsigned long long *a, int64_t n, int iters, int64_t *count,
                               cudaStream_t st)
{
    const unsigned g = (unsigned)sm_count() * 8;
    if ((int64_t)g * 256 > n) return cudaErrorInvalidValue;   // one wrap per step at most
    k_probe_red64<<<g, 256, 0, st>>>(a, n, iters);
    *count = (int64_t)g * 256 * iters;
    return cudaGetLastError();
}

cudaError_t launch_gather_adj(const GatherAdjArgs &a, cudaStream_t st, int64_t &launches)
{
    if (a.ns <= 0) return cudaSuccess;
    if (a.gff) {
        const int64_t n = 5 * (int64_t)a.Mx * a.My;
        k_grid_to_ff<<<grid_for(n, 256), 256, 0, st>>>(a.grid, n, a.gmax, a.gff);
        const int64_t warps = (a.ns + 31) / 32;
        const int64_t want = (warps + kAdjFFWarps - 1) / kAdjFFWarps;
        const int64_t cap = (int64_t)sm_count() * 2;
        const unsigned gf = (unsigned)(want < cap ? want : cap);
        if (a.P == 24) k_gather_adj_ff<24><<<gf, kAdjFFWarps * 32, 0, st>>>(a);
        else k_gather_adj_ff<0><<<gf, kAdjFFWarps * 32, 0, st>>>(a);
        launches += 2;
    }
    const unsigned g = grid_for(a.ns, 256);
    if (a.P == 24) k_gather_adj<24><<<g, 256, 0, st>>>(a);
    else k_gather_adj<0><<<g, 256, 0, st>>>(a);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_adj_assemble(int64_t n, const int *perm, const double *gr, const double *gk,
                                const double *w, int64_t nt, double2 *part,
                                const double2 *praw, const double2 *fd, const double2 *nrm,
                                double inv_area, int slp, int dlp, double2 *g_pos,
                                double2 *g_fs, double2 *g_fd, double2 *g_n, cudaStream_t st,
                                int64_t &launches)
{
    if (dlp) {
        k_wsum_part<<<kZeroModeParts, 256, 0, st>>>(nt, w, 4, 2, part);
        k_wsum_final<<<1, 32, 0, st>>>(kZeroModeParts, part);
        launches += 2;
    }
    if (n > 0) {
        k_adj_assemble<<<grid_for(n, 256), 256, 0, st>>>(n, perm, gr, gk, part + kZeroModeParts,
                                                         praw, fd, nrm, inv_area, slp, dlp,
                                                         g_pos, g_fs, g_fd, g_n);
        launches++;
    }
    return cudaGetLastError();
}

}  // namespace se2p

namespace se2p {

static unsigned stream_grid(int64_t n)
{
    const int64_t want = (n + 255) / 256, cap = (int64_t)sm_count() * 16;
    return (unsigned)(want < cap ? (want < 1 ? 1 : want) : cap);
}

cudaError_t launch_pack_fixed_pairs(const long long *grid, int nc, int64_t G,
                                    const unsigned long long *bound, double2 *z, cudaStream_t st,
                                    int64_t &launches)
{
    k_pack_fixed_pairs<<<stream_grid((int64_t)((nc + 1) / 2) * G), 256, 0, st>>>(grid, nc, G,
                                                                                 bound, z);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_spread_bound(const SpreadArgs &a, int nc, double kfac, int mult, double *ws,
                                cudaStream_t st, int64_t &launches)
{
    const BoundAxis ax = bound_axis(a.Mx, a.P, a.a, a.h), ay = bound_axis(a.My, a.P, a.a, a.h);
    const int64_t nb = (int64_t)ax.nb * ay.nb;
    cudaError_t e = cudaMemsetAsync(ws, 0, sizeof(double) * (size_t)spread_bound_words(a.Mx, a.My, a.P), st);
    if (e != cudaSuccess) return e;
    double *bins = ws, *t = ws + nb;
    unsigned long long *bound = reinterpret_cast<unsigned long long *>(ws + 2 * nb);
    int *cnt = reinterpret_cast<int *>(ws + 2 * nb + 1), *tc = cnt + nb;
    if (a.ns > 0) {
        k_spread_bin_sum<<<stream_grid(a.ns), 256, 0, st>>>(a, nc, ax.nb, ay.nb, bins, cnt, bound);
        launches++;
    }
    k_bound_x<<<stream_grid(nb), 256, 0, st>>>(bins, cnt, ax, ay.nb, t, tc);
    k_bound_y_max<<<stream_grid(nb), 256, 0, st>>>(t, tc, ay, ax.nb, kfac, mult, bound);
    launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_gather_fix_multi(const GatherArgs &a, int nc, int nr, int64_t gstride,
                                    int64_t ostride, cudaStream_t st, int64_t &launches)
{
    if (a.nt <= 0 || nr <= 0) return cudaSuccess;
    const unsigned gf = std::min(grid_for(a.nt, 256), (unsigned)sm_count() * 2);
    if (nc == 2) {
        if (a.P == 24) k_gather_fix_multi<2, 24><<<gf, 256, 0, st>>>(a, nr, gstride, ostride);
        else k_gather_fix_multi<2, 0><<<gf, 256, 0, st>>>(a, nr, gstride, ostride);
    } else {
        if (a.P == 24) k_gather_fix_multi<4, 24><<<gf, 256, 0, st>>>(a, nr, gstride, ostride);
        else k_gather_fix_multi<4, 0><<<gf, 256, 0, st>>>(a, nr, gstride, ostride);
    }
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_gather_fp64_fallback(const GatherArgs &a, int nc, cudaStream_t st,
                                        int64_t &launches)
{
    if (a.nt <= 0) return cudaSuccess;
    unsigned g = grid_for(a.nt, 256);
    if (g > (unsigned)sm_count()) g = (unsigned)sm_count();
    if (nc == 2) {
        if (a.P == 24) k_gather<2, 24><<<g, 256, 0, st>>>(a);
        else if (a.P == 12) k_gather<2, 12><<<g, 256, 0, st>>>(a);
        else k_gather<2, 0><<<g, 256, 0, st>>>(a);
    } else {
        if (a.P == 24) k_gather<4, 24><<<g, 256, 0, st>>>(a);
        else if (a.P == 12) k_gather<4, 12><<<g, 256, 0, st>>>(a);
        else k_gather<4, 0><<<g, 256, 0, st>>>(a);
    }
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_spread_fix_multi(const SpreadArgs &a, int nc, int kY, int nr, int64_t cstride,
                                    int64_t gstride, int bstride, cudaStream_t st,
                                    int64_t &launches)
{
    if (a.ns <= 0 || nr <= 0) return cudaSuccess;
    const int64_t warps = (a.ns + 31) / 32;
    const int64_t want = (warps + kSpreadWarps - 1) / kSpreadWarps;
    const int64_t cap = (int64_t)sm_count() * 8;
    const unsigned g = (unsigned)(want < cap ? want : cap);
    switch (nc) {
    case 2: k_spread_fix_multi<2><<<g, kSpreadWarps * 32, 0, st>>>(a, kY, nr, cstride, gstride, bstride); break;
    case 3: k_spread_fix_multi<3><<<g, kSpreadWarps * 32, 0, st>>>(a, kY, nr, cstride, gstride, bstride); break;
    case 5: k_spread_fix_multi<5><<<g, kSpreadWarps * 32, 0, st>>>(a, kY, nr, cstride, gstride, bstride); break;
    default: return cudaErrorInvalidValue;
    }
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_spread_fix(const SpreadArgs &a, int nc, int kY, cudaStream_t st,
                              int64_t &launches)
{
    if (a.ns <= 0) return cudaSuccess;
    const int64_t warps = (a.ns + 31) / 32;
    const int64_t want = (warps + kSpreadWarps - 1) / kSpreadWarps;
    const int64_t cap = (int64_t)sm_count() * 8;
    const unsigned g = (unsigned)(want < cap ? want : cap);
    switch (nc) {
    case 2: k_spread_fix<2><<<g, kSpreadWarps * 32, 0, st>>>(a, kY); break;
    case 3: k_spread_fix<3><<<g, kSpreadWarps * 32, 0, st>>>(a, kY); break;
    case 4: k_spread_fix<4><<<g, kSpreadWarps * 32, 0, st>>>(a, kY); break;
    default: k_spread_fix<5><<<g, kSpreadWarps * 32, 0, st>>>(a, kY); break;
    }
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_pack_real_pairs(const double *grid, int nc, int64_t G, double2 *z,
                                   cudaStream_t st, int64_t &launches)
{
    k_pack_real_pairs<<<stream_grid((int64_t)((nc + 1) / 2) * G), 256, 0, st>>>(grid, nc, G, z);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_unpack_real_pairs(const double2 *z, int nout, int64_t G, double *grid,
                                     cudaStream_t st, int64_t &launches, unsigned long long *gmax)
{
    k_unpack_real_pairs<<<stream_grid((int64_t)((nout + 1) / 2) * G), 256, 0, st>>>(z, nout, G,
                                                                                    grid, gmax);
    launches++;
    return cudaGetLastError();
}

// Position of box (bx, by) in patch-major order (patches of pw x ph boxes,
// the last patch column and row narrower).
__device__ __forceinline__ int patch_rank(int bx, int by, int nx, int ny, int pw, int ph)
{
    const int ppx = bx / pw, ppy = by / ph;
    const int hrow = min(ph, ny - ppy * ph), wpat = min(pw, nx - ppx * pw);
    return ppy * ph * nx + ppx * pw * hrow + (by - ppy * ph) * wpat + (bx - ppx * pw);
}

__global__ void k_patch_counts(const int *__restrict__ tstart, int nx, int ny, int pw, int ph,
                               int *__restrict__ pcount)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nx * ny) return;
    const int bx = b % nx, by = b / nx;
    pcount[patch_rank(bx, by, nx, ny, pw, ph)] = tstart[b + 1] - tstart[b];
}

__global__ void k_patch_fill(const int *__restrict__ tstart, const int *__restrict__ tbox,
                             int64_t nt, int nx, int ny, int pw, int ph,
                             const int *__restrict__ pstart, int *__restrict__ order)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int b = tbox[t];
    const int q = patch_rank(b % nx, b / nx, nx, ny, pw, ph);
    order[pstart[q] + (t - tstart[b])] = (int)t;
}

cudaError_t launch_patch_order(const int *tstart, const int *tbox, int64_t nt, int nx, int ny,
                               int pw, int ph, int *pcount, int *pstart, int *order,
                               cudaStream_t st, int64_t &launches)
{
    if (nt <= 0) return cudaSuccess;
    const int nbox = nx * ny;
    k_patch_counts<<<grid_for(nbox, 256), 256, 0, st>>>(tstart, nx, ny, pw, ph, pcount);
    cudaError_t e = launch_scan(pcount, nbox, pstart, st, launches);
    if (e != cudaSuccess) return e;
    k_patch_fill<<<grid_for(nt, 256), 256, 0, st>>>(tstart, tbox, nt, nx, ny, pw, ph, pstart,
                                                     order);
    launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_grid_to_fixed(double *grid, int nout, int64_t G, const unsigned long long *gmax,
                                 int Bg, cudaStream_t st, int64_t &launches)
{
    if (nout <= 0) return cudaSuccess;
    const dim3 grd(stream_grid(G), (unsigned)nout);
    k_grid_to_fixed<<<grd, 256, 0, st>>>(grid, G, gmax, Bg);
    launches++;
    return cudaGetLastError();
}

}  // namespace se2p

namespace se2p {

// Exclusive scan of n counts into start[0..n] (one block).
cudaError_t launch_scan(const int *count, int n, int *start, cudaStream_t st, int64_t &launches)
{
    k_scan<<<1, 1024, 0, st>>>(count, n, start);
    launches++;
    return cudaGetLastError();
}

}  // namespace se2p

namespace se2p {

cudaError_t launch_split_half_spectra_t(const double2 *z, int nc, int Mx, int My, double2 *specT,
                                        cudaStream_t st, int64_t &launches, bool fold)
{
    const int H1 = My / 2 + 1;
    const dim3 g((H1 + kTT - 1) / kTT, (Mx + kTT - 1) / kTT, (nc + 1) / 2);
    k_split_half_spectra_t<<<g, 256, 0, st>>>(z, nc, Mx, My, specT, fold && (nc & 1) ? 1 : 0);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_join_half_spectra_t(const double2 *specT, int nout, int Mx, int My, double2 *z,
                                       cudaStream_t st, int64_t &launches)
{
    const dim3 g((My + kTT - 1) / kTT, (Mx + kTT - 1) / kTT, (nout + 1) / 2);
    k_join_half_spectra_t<<<g, 256, 0, st>>>(specT, nout, Mx, My, z);
    launches++;
    return cudaGetLastError();
}

}  // namespace se2p
