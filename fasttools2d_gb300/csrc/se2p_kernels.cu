// se2p_kernels.cu -- sm_103a kernels of the doubly-periodic spectral Ewald
// (SE) summation of the 2D Stokeslet (SLP) and stresslet (DLP).
//
// The reference (FastTools2D, PeriodicEwald/src/mex) runs these loops on the
// CPU with OpenMP; here each is a GB300 kernel.  All arithmetic is FP64.
// GB300 issues about 2 FP64 FMA per clock per SM (1/58 of its FP32 rate), so
// the kernels are organised to keep every FP64 warp instruction fully
// populated: accepted real-space pairs are compacted before the Pade/exp
// work, the spread walks a flattened (P+1)^2 stencil, and the gather gives
// each lane its own target.  Index, compare and shuffle work is nearly free
// next to the FP64 pipe.
#include "se2p_internal.cuh"

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
                            double2 *__restrict__ sp)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = box[i];
    const int j = start[b] + rank[i];
    perm[j] = (int)i;
    if (sorted_box) sorted_box[j] = b;
    sp[j] = p[i];
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

// ===========================================================================
// Real-space pair sums (PE/src/mex/StokesSLP/mex_stokes_slp_real.cpp:131-333,
// PE/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:103-187), fused.
//
// One warp per target.  The warp walks the target's own box (every pair, no
// cutoff) and its 8 periodic neighbour boxes (pairs with r2 < cut2), 32
// candidate sources at a time.  Candidates are tested with the reference's
// exact arithmetic and the accepted ones are compacted into a per-warp queue;
// whenever 32 are queued, each lane evaluates one pair.  The SLP and DLP
// tests are separate because the reference forms the offsets in different
// orders (SLP s-(t-z), DLP (s-t)+z); flag bit 0 = SLP pair, bit 1 = DLP pair.
// ===========================================================================
constexpr int kRealWarps = 8;
__constant__ int c_nb_dx[9] = {0, -1, -1, -1, 0, 0, 1, 1, 1};
__constant__ int c_nb_dy[9] = {0, -1, 0, 1, -1, 1, -1, 0, 1};

template <bool SLP, bool DLP>
__device__ __forceinline__ void real_pair(const RealArgs &a, int s, int k, int fl, double2 T,
                                          double2 z, double &s1, double &s2, double &d1,
                                          double &d2)
{
    const double2 S = a.sp[s];
    if (SLP && (fl & 1)) {
        double dx, dy;
        if (k == 0) {
            dx = xsub(T.x, S.x);
            dy = xsub(T.y, S.y);
        } else {
            dx = xsub(S.x, xsub(T.x, z.x));
            dy = xsub(S.y, xsub(T.y, z.y));
        }
        const double r2 = xadd(xmul(dx, dx), xmul(dy, dy));
        const double x = xmul(xmul(r2, a.xi), a.xi);
        const double e = exp(-x);
        const double E = e1_pade(x, e);
        const double f1 = a.coef[(int64_t)a.nc * s], f2 = a.coef[(int64_t)a.nc * s + 1];
        const double g = e / r2;
        const double q = dx * f2 - dy * f1;
        s1 += 0.5 * E * f1 + g * dy * q;
        s2 += 0.5 * E * f2 - g * dx * q;
    }
    if (DLP && (fl & 2)) {
        double x1, x2;
        if (k == 0) {
            x1 = xsub(S.x, T.x);
            x2 = xsub(S.y, T.y);
        } else {
            x1 = xadd(xsub(S.x, T.x), z.x);
            x2 = xadd(xsub(S.y, T.y), z.y);
        }
        const double r2 = xadd(xmul(x1, x1), xmul(x2, x2));
        const double e2 = exp(-a.xi2 * r2);
        const double pf = 2.0 * a.xi2;
        const double fb = -4.0 * (1.0 + a.xi2 * r2) / r2 / r2;
        const double *Sc = a.coef + (int64_t)a.nc * s + a.doff;
        const double S11 = Sc[0], S1221 = Sc[1], S22 = Sc[2];
        const double T111 = x1 * x1 * x1 * fb + pf * 3.0 * x1;
        const double T112 = x1 * x1 * x2 * fb + pf * x2;
        const double T122 = x1 * x2 * x2 * fb + pf * x1;
        const double T222 = x2 * x2 * x2 * fb + pf * 3.0 * x2;
        d1 += e2 * (T111 * S11 + T112 * S1221 + T122 * S22);
        d2 += e2 * (T112 * S11 + T122 * S1221 + T222 * S22);
    }
}

template <bool SLP, bool DLP>
__global__ void __launch_bounds__(kRealWarps * 32) k_real(RealArgs a)
{
    __shared__ int2 q[kRealWarps][64];
    __shared__ int nbb[kRealWarps][9];
    __shared__ double2 nbz[kRealWarps][9];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t nw = (int64_t)gridDim.x * kRealWarps;
    for (int64_t t = (int64_t)blockIdx.x * kRealWarps + wid; t < a.ntar; t += nw) {
        const int tb = a.tbox[t];
        const int bx = tb % a.nx, by = tb / a.nx;
        if (lane < 9) {
            const int ux = bx + c_nb_dx[lane], uy = by + c_nb_dy[lane];
            const int wx = (ux + a.nx) % a.nx, wy = (uy + a.ny) % a.ny;
            nbb[wid][lane] = wy * a.nx + wx;
            nbz[wid][lane] = make_double2(xdiv(xmul(a.Lx, (double)(ux - wx)), (double)a.nx),
                                          xdiv(xmul(a.Ly, (double)(uy - wy)), (double)a.ny));
        }
        __syncwarp();
        const double2 T = a.tp[t];
        double s1 = 0.0, s2 = 0.0, d1 = 0.0, d2 = 0.0;
        int qn = 0;
        for (int k = 0; k < 9; k++) {
            const int sb = nbb[wid][k];
            const int b0 = a.sstart[sb], b1 = a.sstart[sb + 1];
            const double2 z = nbz[wid][k];
            for (int base = b0; base < b1; base += 32) {
                const int s = base + lane;
                int fl = 0;
                if (s < b1) {
                    const double2 S = a.sp[s];
                    if (k == 0) {
                        const double dx = xsub(T.x, S.x), dy = xsub(T.y, S.y);
                        const double r2 = xadd(xmul(dx, dx), xmul(dy, dy));
                        if (r2 == 0.0) {
                            // SLP self term (mex_stokes_slp_real.cpp:161-163); DLP skips r2 == 0.
                            if (SLP) {
                                const double *f = a.coef + (int64_t)a.nc * s;
                                s1 += a.self_c * f[0];
                                s2 += a.self_c * f[1];
                            }
                        } else {
                            fl = 3;
                        }
                    } else {
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
                const unsigned m = __ballot_sync(~0u, fl != 0);
                if (fl) q[wid][qn + __popc(m & ((1u << lane) - 1u))] = make_int2(s, (k << 2) | fl);
                qn += __popc(m);
                __syncwarp();
                if (qn >= 32) {
                    const int2 e = q[wid][lane];
                    __syncwarp();
                    if (lane < qn - 32) q[wid][lane] = q[wid][lane + 32];
                    qn -= 32;
                    const int kk = e.y >> 2;
                    real_pair<SLP, DLP>(a, e.x, kk, e.y & 3, T, nbz[wid][kk], s1, s2, d1, d2);
                    __syncwarp();
                }
            }
        }
        if (lane < qn) {
            const int2 e = q[wid][lane];
            const int kk = e.y >> 2;
            real_pair<SLP, DLP>(a, e.x, kk, e.y & 3, T, nbz[wid][kk], s1, s2, d1, d2);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            if (SLP) {
                s1 += __shfl_xor_sync(~0u, s1, o);
                s2 += __shfl_xor_sync(~0u, s2, o);
            }
            if (DLP) {
                d1 += __shfl_xor_sync(~0u, d1, o);
                d2 += __shfl_xor_sync(~0u, d2, o);
            }
        }
        if (lane == 0) {
            if (SLP) a.u_slp[t] = make_double2(s1, s2);
            if (DLP) a.u_dlp[t] = make_double2(d1, d2);
        }
        __syncwarp();
    }
}

template __global__ void k_real<true, false>(RealArgs);
template __global__ void k_real<false, true>(RealArgs);
template __global__ void k_real<true, true>(RealArgs);

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

__device__ __forceinline__ int wrap_index(int i, int M)
{
    i %= M;
    return i < 0 ? i + M : i;
}

template <int NC>
__global__ void __launch_bounds__(kSpreadWarps * 32) k_spread(SpreadArgs a)
{
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
template __global__ void k_spread<3>(SpreadArgs);
template __global__ void k_spread<5>(SpreadArgs);

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

// SLP filter (mex_stokes_slp_kspace.cpp:197-208) applied to (h1, h2).
__device__ __forceinline__ void slp_mode(double k1, double k2, double xi, double eta,
                                         double2 h1, double2 h2, double2 &o1, double2 &o2)
{
    const double K2 = k1 * k1 + k2 * k2;
    const double e = (1.0 / (K2 * K2) + 0.25 / (K2 * xi * xi)) * exp(-0.25 * (1 - eta) / (xi * xi) * K2);
    o1.x = k2 * (k2 * h1.x - k1 * h2.x) * e;
    o1.y = k2 * (k2 * h1.y - k1 * h2.y) * e;
    o2.x = k1 * (k1 * h2.x - k2 * h1.x) * e;
    o2.y = k1 * (k1 * h2.y - k2 * h1.y) * e;
}

// DLP filter (mex_stokes_dlp_kspace.cpp:228-251) applied to (h1, h2+h3, h4).
__device__ __forceinline__ void dlp_mode(double k1, double k2, double xi, double eta,
                                         double2 h1, double2 h23, double2 h4, double2 &o1,
                                         double2 &o2)
{
    const double K2 = k1 * k1 + k2 * k2;
    const double e = exp(-0.25 * (1 - eta) / (xi * xi) * K2) / K2 / K2;
    const double t = 1 + 0.25 * K2 / xi / xi;
    const double B111 = 3.0 * k1 * K2 - 2.0 * k1 * k1 * k1;
    const double B112 = k2 * K2 - 2.0 * k1 * k1 * k2;
    const double B122 = k1 * K2 - 2.0 * k1 * k2 * k2;
    const double B211 = k2 * K2 - 2.0 * k2 * k1 * k1;
    const double B212 = k1 * K2 - 2.0 * k2 * k1 * k2;
    const double B222 = 3.0 * k2 * K2 - 2.0 * k2 * k2 * k2;
    const double et = e * t;
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
    const int jx = (int)(idx / H), jy = (int)(idx - (int64_t)jx * H);
    double2 *sp = reinterpret_cast<double2 *>(a.spec);
    const bool zero = (jx == 0 && jy == 0);
    const bool nyq = (jx == a.Mx / 2) || (jy == a.My / 2);
    const double k1 = kfreq(jx, a.Mx, a.Lx), k2 = kfreq(jy, a.My, a.Ly);
    // Index partner -j mod M: frequency negated except on the Nyquist index.
    const double k1p = (jx == a.Mx / 2) ? k1 : -k1;
    const double k2p = (jy == a.My / 2) ? k2 : -k2;
    const double sc = a.scale;
    double2 so1, so2, do1, do2;
    if (a.slp_in >= 0) {
        const double2 h1 = sp[a.slp_in * G + idx], h2 = sp[(a.slp_in + 1) * G + idx];
        slp_mode(k1, k2, a.xi, a.eta, h1, h2, so1, so2);
        if (nyq) {
            double2 p1, p2;
            slp_mode(k1p, k2p, a.xi, a.eta, h1, h2, p1, p2);
            so1.x = 0.5 * (so1.x + p1.x); so1.y = 0.5 * (so1.y + p1.y);
            so2.x = 0.5 * (so2.x + p2.x); so2.y = 0.5 * (so2.y + p2.y);
        }
        so1.x *= sc; so1.y *= sc; so2.x *= sc; so2.y *= sc;
        if (zero) so1 = so2 = make_double2(0.0, 0.0);
    }
    if (a.dlp_in >= 0) {
        const double2 h1 = sp[a.dlp_in * G + idx], h23 = sp[(a.dlp_in + 1) * G + idx];
        const double2 h4 = sp[(a.dlp_in + 2) * G + idx];
        dlp_mode(k1, k2, a.xi, a.eta, h1, h23, h4, do1, do2);
        if (nyq) {
            double2 p1, p2;
            dlp_mode(k1p, k2p, a.xi, a.eta, h1, h23, h4, p1, p2);
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

// ===========================================================================
// Gather (PE/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:264-329 and
// PE/src/mex/StokesDLP/mex_stokes_dlp_kspace.cpp:334-400): one lane per
// target; per stencil column the NC grid values are reduced against Wy, then
// weighted by Wx.  Output k of target t holds grids 2k, 2k+1, times scale.
// ===========================================================================
template <int NC, int PT>
__global__ void __launch_bounds__(256) k_gather(GatherArgs a)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.nt) return;
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

template __global__ void k_gather<2, 24>(GatherArgs);
template __global__ void k_gather<4, 24>(GatherArgs);
template __global__ void k_gather<2, 12>(GatherArgs);
template __global__ void k_gather<4, 12>(GatherArgs);
template __global__ void k_gather<2, 0>(GatherArgs);
template __global__ void k_gather<4, 0>(GatherArgs);

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
static int sm_count()
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
                       double2 *sorted_pos, cudaStream_t st, int64_t &launches)
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
                                                         sorted_box, a.p, sorted_pos);
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

cudaError_t launch_real(const RealArgs &a, bool slp, bool dlp, cudaStream_t st,
                        int64_t &launches)
{
    if (a.ntar <= 0) return cudaSuccess;
    const int64_t want = (a.ntar + kRealWarps - 1) / kRealWarps;
    const int64_t cap = (int64_t)sm_count() * 8;
    const unsigned g = (unsigned)(want < cap ? want : cap);
    if (slp && dlp) k_real<true, true><<<g, kRealWarps * 32, 0, st>>>(a);
    else if (slp) k_real<true, false><<<g, kRealWarps * 32, 0, st>>>(a);
    else k_real<false, true><<<g, kRealWarps * 32, 0, st>>>(a);
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
    default: k_spread<5><<<g, kSpreadWarps * 32, 0, st>>>(a); break;
    }
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
    const unsigned g = grid_for(a.nt, 256);
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

}  // namespace se2p
