// se2p_geom.cu -- the real-space operator of a fixed point set, for batched
// (multi-RHS) evaluation.
//
// For one geometry (sources, targets, normals, Ewald parameters) the real
// space is a sparse linear map from the per-source coefficients to the target
// velocities.  Each accepted pair (t, s) contributes
//   SLP  u += A f,  A = [[h - g x2^2, g x1 x2], [g x1 x2, h - g x1^2]],
//        h = E1(xi^2 r^2)/2, g = exp(-xi^2 r^2)/r^2
//        (the contraction of PE/src/mex/StokesSLP/mex_stokes_slp_real.cpp:206-214)
//   DLP  u += B S,  S = (S11, S12+S21, S22),
//        B = [[b0, b1, b2], [b1, b2, b3]] with, for e = exp(-xi^2 r^2),
//        fb = -4 (1 + xi^2 r^2)/r^4, pf = 2 xi^2:
//        b0 = e x1 (fb x1^2 + 3 pf), b1 = e x2 (fb x1^2 + pf),
//        b2 = e x1 (fb x2^2 + pf),   b3 = e x2 (fb x2^2 + 3 pf)
//        (PE/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:125-138, :165-181),
// with x = s - t (+ image shift).  The SLP self term at r^2 == 0 is the pair
// A = self_c I.  The operator is built once -- same candidate boxes, FP32
// pre-test with its rounding band, the reference's exact FP64 cutoff test --
// and stored as rows by sorted target: the source index and seven
// coefficients per pair in 8-byte slots -- float-float for far pairs
// (computed in float-float, as in k_real), FP64 for near pairs and the self
// term.  Applying it to R right-hand sides is then a sparse product, one
// lane per target row, float-float sums for the far entries and FP64 sums
// for the near ones.  The rows are stored sliced: 32 consecutive sorted
// targets form a slice, padded to its longest row, and entry k of the
// slice's row l sits at slice[w] + 32 k + l, so the 32 lanes of a warp read
// 32 consecutive slots per coefficient (a row-after-row layout spread each
// load over 32 sectors, and the apply ran at 0.9 TB/s).
#include "se2p_internal.cuh"

namespace se2p {

namespace {

__constant__ int g_nb_dx[9] = {0, -1, -1, -1, 0, 0, 1, 1, 1};
__constant__ int g_nb_dy[9] = {0, -1, 0, 1, -1, 1, -1, 0, 1};
__constant__ double g_exp_tab[64] = SE2P_EXP2_TAB64;

constexpr int kGeomWarps = 8;

// Accept flags of candidate s for target t (bit 0 SLP, bit 1 DLP); self is
// set for an own-box source at r^2 == 0 (SLP self term, DLP skip).  Same
// decisions as k_real.
__device__ __forceinline__ int cand_flags(const RealArgs &a, double2 T, float2 Tf, int k, int s,
                                          double2 z, float2 zf, bool &self)
{
    self = false;
    if (k == 0) {
        const float2 Sf = a.spf[s];
        const float dxf = Tf.x - Sf.x, dyf = Tf.y - Sf.y;
        if (dxf * dxf + dyf * dyf > 0.0f) return 3;
        const double2 S = a.sp[s];
        const double dx = xsub(T.x, S.x), dy = xsub(T.y, S.y);
        if (xadd(xmul(dx, dx), xmul(dy, dy)) == 0.0) {
            self = true;
            return 0;
        }
        return 3;
    }
    const float2 Sf = a.spf[s];
    const float dxf = Sf.x - (Tf.x - zf.x), dyf = Sf.y - (Tf.y - zf.y);
    const float r2f = dxf * dxf + dyf * dyf;
    const float ex = 0x1p-22f * (fabsf(Sf.x) + fabsf(Tf.x) + fabsf(zf.x));
    const float ey = 0x1p-22f * (fabsf(Sf.y) + fabsf(Tf.y) + fabsf(zf.y));
    const float band = 2.0f * (ex * (2.0f * fabsf(dxf) + ex) + ey * (2.0f * fabsf(dyf) + ey) +
                               0x1p-22f * r2f);
    if (r2f + band < a.cut2f) return 3;
    if (r2f - band >= a.cut2f) return 0;
    const double2 S = a.sp[s];
    int fl = 0;
    const double dx = xsub(S.x, xsub(T.x, z.x)), dy = xsub(S.y, xsub(T.y, z.y));
    if (xadd(xmul(dx, dx), xmul(dy, dy)) < a.cut2) fl |= 1;
    const double x1 = xadd(xsub(S.x, T.x), z.x), x2 = xadd(xsub(S.y, T.y), z.y);
    if (xadd(xmul(x1, x1), xmul(x2, x2)) < a.cut2) fl |= 2;
    return fl;
}

}  // namespace

// Pass 1 (FILL = false): entries per target row.  Pass 2 (FILL = true): the
// entries themselves, entry k of row t at slice[t / 32] + 32 k + t % 32:
// source, target and meta = k | fl << 4 | self << 6.  One warp per sorted
// target; lanes over the virtual concatenation of the nine neighbour boxes'
// sources.
template <bool SLP, bool DLP, bool FILL>
__global__ void __launch_bounds__(kGeomWarps * 32) k_geom_rows(RealArgs a, int *rowcnt,
                                                              const int *slice, int *src,
                                                              int *tgt, unsigned char *meta)
{
    __shared__ int s_nbs[kGeomWarps][9], s_nbp[kGeomWarps][10];
    __shared__ double2 s_nbz[kGeomWarps][9];
    __shared__ float2 s_nbzf[kGeomWarps][9];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t nw = (int64_t)gridDim.x * kGeomWarps;
    for (int64_t t = (int64_t)blockIdx.x * kGeomWarps + wid; t < a.ntar; t += nw) {
        const int tb = a.tbox[t];
        const double2 T = a.tp[t];
        const float2 Tf = a.tpf[t];
        int cntk = 0;
        if (lane < 9) {
            const int ux = tb % a.nx + g_nb_dx[lane], uy = tb / a.nx + g_nb_dy[lane];
            const int wx = (ux + a.nx) % a.nx, wy = (uy + a.ny) % a.ny;
            const int sb = wy * a.nx + wx;
            const int b0 = a.sstart[sb];
            cntk = a.sstart[sb + 1] - b0;
            s_nbs[wid][lane] = b0;
            const double zx = ux < 0 ? a.zxm : (ux >= a.nx ? a.zxp : 0.0);
            const double zy = uy < 0 ? a.zym : (uy >= a.ny ? a.zyp : 0.0);
            s_nbz[wid][lane] = make_double2(zx, zy);
            s_nbzf[wid][lane] = make_float2((float)zx, (float)zy);
        }
        int incl = cntk;
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) {
            const int v = __shfl_up_sync(~0u, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane < 9) s_nbp[wid][lane + 1] = incl;
        if (lane == 0) s_nbp[wid][0] = 0;
        __syncwarp();
        const int total = s_nbp[wid][9];
        int base = 0;                                // entries of row t so far
        const int64_t sb = FILL ? (int64_t)slice[t >> 5] + (t & 31) : 0;
        for (int v0 = 0; v0 < total; v0 += 32) {
            const int v = v0 + lane;
            int fl = 0, s = 0, k = 0;
            bool self = false;
            if (v < total) {
                while (v >= s_nbp[wid][k + 1]) k++;
                s = s_nbs[wid][k] + (v - s_nbp[wid][k]);
                fl = cand_flags(a, T, Tf, k, s, s_nbz[wid][k], s_nbzf[wid][k], self);
                if (!SLP) fl &= 2;
                if (!DLP) fl &= 1;
            }
            const bool take = fl != 0 || (SLP && self);
            const unsigned m = __ballot_sync(~0u, take);
            if (FILL && take) {
                const int64_t e = sb + ((int64_t)(base + __popc(m & ((1u << lane) - 1u))) << 5);
                src[e] = s;
                tgt[e] = (int)t;
                meta[e] = (unsigned char)(k | (fl << 4) | (self ? 64 : 0));
            }
            base += __popc(m);
        }
        if (!FILL && lane == 0) rowcnt[t] = base;
        __syncwarp();
    }
}

// Slots of each slice of 32 rows: 32 times its longest row.
__global__ void k_geom_slices(const int *__restrict__ rowptr, int64_t nt, int *__restrict__ slen)
{
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= (nt + 31) / 32) return;
    int m = 0;
    for (int64_t t = 32 * w; t < min(nt, 32 * w + 32); t++) m = max(m, rowptr[t + 1] - rowptr[t]);
    slen[w] = 32 * m;
}

// The seven coefficients of every entry (thread per entry), stored SoA in
// 8-byte slots cf[c * nnz + e], c = 0..2 SLP (a11, a12, a22), 3..6 DLP
// (b0..b3).  Far pairs (1.0001 < xi^2 r^2 < 63.9 by the FP32 estimate) are
// computed and stored in float-float.  Near pairs and the self term --
// where the entries are large and a density's contraction can cancel -- are
// computed in FP64 with each kernel's own offset form and stored as doubles;
// the sign bit of src[e] marks them.
template <bool SLP, bool DLP>
__global__ void __launch_bounds__(256) k_geom_coef(RealArgs a, int64_t nnz, int *src,
                                                   const int *tgt, const unsigned char *meta,
                                                   float2 *cf)
{
    __shared__ float2 tabff[64];
    for (int i = threadIdx.x; i < 64; i += blockDim.x) tabff[i] = ff_split(g_exp_tab[i]);
    __syncthreads();
    const float2 xi2ff = ff_split(a.xi2), pfff = ff_split(a.pf);
    const float2 zero = make_float2(0.f, 0.f);
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int t = tgt[e];
        if (t < 0) continue;                         // a slice's padding slot
        const int s = src[e], mt = meta[e];
        const int k = mt & 15, fl = (mt >> 4) & 3;
        const bool self = (mt & 64) != 0;
        float2 c[7] = {zero, zero, zero, zero, zero, zero, zero};
        double cd[7] = {0, 0, 0, 0, 0, 0, 0};
        bool near = true;   // FP64 coefficients (self term and near pairs)
        if (self) {
            cd[0] = cd[2] = a.self_c;
        } else {
            const double2 S = a.sp[s], T = a.tp[t];
            const int tb = a.tbox[t];
            const int ux = tb % a.nx + g_nb_dx[k], uy = tb / a.nx + g_nb_dy[k];
            const double zx = ux < 0 ? a.zxm : (ux >= a.nx ? a.zxp : 0.0);
            const double zy = uy < 0 ? a.zym : (uy >= a.ny ? a.zyp : 0.0);
            const double x1d = (S.x - T.x) + zx, x2d = (S.y - T.y) + zy;   // DLP form
            const float r2e = (float)x1d * (float)x1d + (float)x2d * (float)x2d;
            const float xe = r2e * a.xi2f;
            if (xe > 1.0001f && xe < 63.9f) {
                near = false;
                const float2 x1 = ff_split(x1d), x2 = ff_split(x2d);
                const float2 r2 = ff_add(ff_sqr(x1), ff_sqr(x2));
                const float2 x = ff_mul(r2, xi2ff);
                const float2 ex = ff_exp_neg(x, tabff);
                const float2 ir2 = ff_rcp(r2);
                const float2 x11 = ff_sqr(x1), x22 = ff_sqr(x2);
                if (SLP && (fl & 1)) {
                    const float2 h = ff_scale(ff_mul(ex, ff_g_e1(x, a.gtab)), 0.5f);
                    const float2 g = ff_mul(ex, ir2);
                    c[0] = ff_sub(h, ff_mul(g, x22));
                    c[1] = ff_mul(g, ff_mul(x1, x2));
                    c[2] = ff_sub(h, ff_mul(g, x11));
                }
                if (DLP && (fl & 2)) {
                    const float2 fb = ff_scale(ff_mul(ff_add_f(x, 1.0f), ff_sqr(ir2)), -4.0f);
                    const float2 p3 = ff_mul_f(pfff, 3.0f);
                    const float2 f1 = ff_mul(fb, x11), f2 = ff_mul(fb, x22);
                    const float2 ex1 = ff_mul(ex, x1), ex2 = ff_mul(ex, x2);
                    c[3] = ff_mul(ex1, ff_add(f1, p3));
                    c[4] = ff_mul(ex2, ff_add(f1, pfff));
                    c[5] = ff_mul(ex1, ff_add(f2, pfff));
                    c[6] = ff_mul(ex2, ff_add(f2, p3));
                }
            } else {
                if (SLP && (fl & 1)) {
                    const double d1 = S.x - (T.x - zx), d2 = S.y - (T.y - zy);   // SLP form
                    const double r2 = fma(d1, d1, d2 * d2);
                    const double x = r2 * a.xi2;
                    const double ex = exp(-x);
                    const double h = 0.5 * e1_pade(x, ex), g = ex / r2;
                    cd[0] = h - g * d2 * d2;
                    cd[1] = g * d1 * d2;
                    cd[2] = h - g * d1 * d1;
                }
                if (DLP && (fl & 2)) {
                    const double r2 = fma(x1d, x1d, x2d * x2d);
                    const double x = r2 * a.xi2;
                    const double ex = exp(-x);
                    const double ir2 = 1.0 / r2;
                    const double fb = -4.0 * (1.0 + x) * ir2 * ir2, pf = a.pf;
                    const double f1 = fb * x1d * x1d, f2 = fb * x2d * x2d;
                    cd[3] = ex * x1d * (f1 + 3.0 * pf);
                    cd[4] = ex * x2d * (f1 + pf);
                    cd[5] = ex * x1d * (f2 + pf);
                    cd[6] = ex * x2d * (f2 + 3.0 * pf);
                }
            }
        }
        if (near) {
            double *cfd = reinterpret_cast<double *>(cf);
#pragma unroll
            for (int i = 0; i < 7; i++) cfd[(int64_t)i * nnz + e] = cd[i];
            src[e] = s | (int)0x80000000u;
        } else {
#pragma unroll
            for (int i = 0; i < 7; i++) cf[(int64_t)i * nnz + e] = c[i];
        }
    }
}

// y = A x for R right-hand sides at once; one lane per sorted target row.
// cff: per RHS, ncf float-float coefficients per sorted source (SLP f1, f2 at
// 0, 1; DLP S11, S12+S21, S22 at doff), RHS r at cff + r * rstride.  Output
// ur[r * nt + t] (raw sums, sorted order) per kind.
template <bool SLP, bool DLP, int R>
__global__ void __launch_bounds__(256) k_geom_apply(int64_t nt, int64_t nnz, const int *rowptr,
                                                    const int *slice, const int *src,
                                                    const float2 *cf,
                                                    const float2 *cff, int ncf, int doff,
                                                    int64_t rstride, const double *cfd_rhs,
                                                    int nc, int doffd, int64_t rstrided, int nr,
                                                    double2 *ur_slp, double2 *ur_dlp)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    float su[R][4], sc[R][4];   // Dot2 accumulators: SLP u1, u2, DLP u1, u2
    double ud[R][4];            // FP64 sums of the near entries
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
            su[r][i] = sc[r][i] = 0.f;
            ud[r][i] = 0.0;
        }
    const double *cfd = reinterpret_cast<const double *>(cf);
    const int n = rowptr[t + 1] - rowptr[t];
    const int64_t e0 = (int64_t)slice[t >> 5] + (t & 31);
    for (int k = 0; k < n; k++) {
        const int64_t e = e0 + ((int64_t)k << 5);
        const int sraw = src[e];
        const int s = sraw & 0x7fffffff;
        if (sraw < 0) {
            double A0 = 0, A1 = 0, A2 = 0, B0 = 0, B1 = 0, B2 = 0, B3 = 0;
            if (SLP) {
                A0 = cfd[e];
                A1 = cfd[nnz + e];
                A2 = cfd[2 * nnz + e];
            }
            if (DLP) {
                B0 = cfd[3 * nnz + e];
                B1 = cfd[4 * nnz + e];
                B2 = cfd[5 * nnz + e];
                B3 = cfd[6 * nnz + e];
            }
#pragma unroll
            for (int r = 0; r < R; r++) {
                if (r >= nr) break;
                const double *q = cfd_rhs + r * rstrided + (int64_t)nc * s;
                if (SLP) {
                    const double f1 = q[0], f2 = q[1];
                    ud[r][0] = fma(A0, f1, fma(A1, f2, ud[r][0]));
                    ud[r][1] = fma(A1, f1, fma(A2, f2, ud[r][1]));
                }
                if (DLP) {
                    const double S11 = q[doffd], S12 = q[doffd + 1], S22 = q[doffd + 2];
                    ud[r][2] = fma(B0, S11, fma(B1, S12, fma(B2, S22, ud[r][2])));
                    ud[r][3] = fma(B1, S11, fma(B2, S12, fma(B3, S22, ud[r][3])));
                }
            }
            continue;
        }
        float2 A0, A1, A2, B0, B1, B2, B3;
        if (SLP) {
            A0 = cf[e];
            A1 = cf[nnz + e];
            A2 = cf[2 * nnz + e];
        }
        if (DLP) {
            B0 = cf[3 * nnz + e];
            B1 = cf[4 * nnz + e];
            B2 = cf[5 * nnz + e];
            B3 = cf[6 * nnz + e];
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            if (r >= nr) break;
            const float2 *q = cff + r * rstride + (int64_t)ncf * s;
            if (SLP) {
                const float2 f1 = q[0], f2 = q[1];
                ff_dot_acc(A0, f1, su[r][0], sc[r][0]);
                ff_dot_acc(A1, f2, su[r][0], sc[r][0]);
                ff_dot_acc(A1, f1, su[r][1], sc[r][1]);
                ff_dot_acc(A2, f2, su[r][1], sc[r][1]);
            }
            if (DLP) {
                const float2 S11 = q[doff], S12 = q[doff + 1], S22 = q[doff + 2];
                ff_dot_acc(B0, S11, su[r][2], sc[r][2]);
                ff_dot_acc(B1, S12, su[r][2], sc[r][2]);
                ff_dot_acc(B2, S22, su[r][2], sc[r][2]);
                ff_dot_acc(B1, S11, su[r][3], sc[r][3]);
                ff_dot_acc(B2, S12, su[r][3], sc[r][3]);
                ff_dot_acc(B3, S22, su[r][3], sc[r][3]);
            }
        }
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
        if (r >= nr) break;
        if (SLP)
            ur_slp[r * nt + t] =
                make_double2(ud[r][0] + ff_to_double(ff_norm(su[r][0], sc[r][0])),
                             ud[r][1] + ff_to_double(ff_norm(su[r][1], sc[r][1])));
        if (DLP)
            ur_dlp[r * nt + t] =
                make_double2(ud[r][2] + ff_to_double(ff_norm(su[r][2], sc[r][2])),
                             ud[r][3] + ff_to_double(ff_norm(su[r][3], sc[r][3])));
    }
}

// u[perm[j]] += the real-space part of the drivers' assembly: SLP ur/(4 pi),
// DLP -(ur/4/pi) (the k-space part with its sign and zero mode is already in u).
__global__ void k_geom_add(int64_t n, const int *__restrict__ perm, const double2 *__restrict__ ur,
                           int dlp, double2 *__restrict__ u)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int i = perm[j];
    double2 r = ur[j], v = u[i];
    if (dlp) {
        v.x -= r.x / 4.0 / kPi;
        v.y -= r.y / 4.0 / kPi;
    } else {
        v.x += r.x / (4.0 * kPi);
        v.y += r.y / (4.0 * kPi);
    }
    u[i] = v;
}

static unsigned geom_grid(int64_t n, int block)
{
    const int64_t g = (n + block - 1) / block;
    return (unsigned)(g < 1 ? 1 : g);
}

cudaError_t launch_geom_rows(const RealArgs &a, bool slp, bool dlp, bool fill, int *rowcnt,
                             const int *slice, int *src, int *tgt, unsigned char *meta,
                             cudaStream_t st, int64_t &launches)
{
    if (a.ntar <= 0) return cudaSuccess;
    const int64_t want = (a.ntar + kGeomWarps - 1) / kGeomWarps;
    const int64_t cap = (int64_t)sm_count() * 8;
    const unsigned g = (unsigned)(want < cap ? want : cap);
#define SE2P_ROWS(S, D, F) \
    k_geom_rows<S, D, F><<<g, kGeomWarps * 32, 0, st>>>(a, rowcnt, slice, src, tgt, meta)
    if (fill) {
        if (slp && dlp) SE2P_ROWS(true, true, true);
        else if (slp) SE2P_ROWS(true, false, true);
        else SE2P_ROWS(false, true, true);
    } else {
        if (slp && dlp) SE2P_ROWS(true, true, false);
        else if (slp) SE2P_ROWS(true, false, false);
        else SE2P_ROWS(false, true, false);
    }
#undef SE2P_ROWS
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_geom_coef(const RealArgs &a, bool slp, bool dlp, int64_t nnz, int *src,
                             const int *tgt, const unsigned char *meta, float2 *cf,
                             cudaStream_t st, int64_t &launches)
{
    if (nnz <= 0) return cudaSuccess;
    const int64_t want = (nnz + 255) / 256, cap = (int64_t)sm_count() * 16;
    const unsigned g = (unsigned)(want < cap ? want : cap);
    if (slp && dlp) k_geom_coef<true, true><<<g, 256, 0, st>>>(a, nnz, src, tgt, meta, cf);
    else if (slp) k_geom_coef<true, false><<<g, 256, 0, st>>>(a, nnz, src, tgt, meta, cf);
    else k_geom_coef<false, true><<<g, 256, 0, st>>>(a, nnz, src, tgt, meta, cf);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_geom_slices(const int *rowptr, int64_t nt, int *slen, cudaStream_t st,
                               int64_t &launches)
{
    if (nt <= 0) return cudaSuccess;
    k_geom_slices<<<geom_grid((nt + 31) / 32, 256), 256, 0, st>>>(rowptr, nt, slen);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_geom_apply(bool slp, bool dlp, int64_t nt, int64_t nnz, const int *rowptr,
                              const int *slice, const int *src, const float2 *cf,
                              const float2 *cff, int ncf,
                              int doff, int64_t rstride, const double *cfd_rhs, int nc,
                              int doffd, int64_t rstrided, int nr, double2 *ur_slp,
                              double2 *ur_dlp, cudaStream_t st, int64_t &launches)
{
    if (nt <= 0 || nr <= 0) return cudaSuccess;
    const unsigned g = geom_grid(nt, 256);
#define SE2P_APPLY(S, D, R)                                                                  \
    k_geom_apply<S, D, R><<<g, 256, 0, st>>>(nt, nnz, rowptr, slice, src, cf, cff, ncf, doff,   \
                                             rstride,                                          \
                                             cfd_rhs, nc, doffd, rstrided, nr, ur_slp, ur_dlp)
    if (nr > 2) {
        if (slp && dlp) SE2P_APPLY(true, true, 4);
        else if (slp) SE2P_APPLY(true, false, 4);
        else SE2P_APPLY(false, true, 4);
    } else if (nr == 2) {
        if (slp && dlp) SE2P_APPLY(true, true, 2);
        else if (slp) SE2P_APPLY(true, false, 2);
        else SE2P_APPLY(false, true, 2);
    } else {
        if (slp && dlp) SE2P_APPLY(true, true, 1);
        else if (slp) SE2P_APPLY(true, false, 1);
        else SE2P_APPLY(false, true, 1);
    }
#undef SE2P_APPLY
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_geom_add(int64_t n, const int *perm, const double2 *ur, bool dlp, double2 *u,
                            cudaStream_t st, int64_t &launches)
{
    if (n <= 0) return cudaSuccess;
    k_geom_add<<<geom_grid(n, 256), 256, 0, st>>>(n, perm, ur, dlp ? 1 : 0, u);
    launches++;
    return cudaGetLastError();
}

}  // namespace se2p
