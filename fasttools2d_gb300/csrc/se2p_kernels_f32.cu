// se2p_kernels_f32.cu -- the FP32-grid k-space kernels (spread, filter,
// gather) of the mixed-precision form.
//
// For tolerances >= 1e-6 the grid work runs in FP32: GB300 issues FP32 at
// ~58x its FP64 rate, so these kernels become bound by atomics and memory
// instead of the FP64 pipe.  Discrete decisions stay exactly the reference's:
// the stencil origin (FindClosestNode) and the in-cell offset p are computed
// in FP64.  The exponent of the fast-Gaussian-gridding weights
// (PE/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:64-67, :95-99),
//   a (p^2 + 2 w p) + a h^2 (i - P/2)^2 - 2 a h p i      (a = -2 xi^2 / eta),
// is regrouped as a (p - h (i - P/2))^2 + 2 a p (w - h P/2): the second term
// is a per-point factor (1 when w = h P/2), taken once in FP64, and the
// first is formed in FP32.  Its rounding moves a weight e^-x by about
// x e^-x 2^-22 <= 1e-7 of the largest weight, well inside the form's 1e-6.
#include "se2p_internal.cuh"

namespace se2p {

// The per-point factor exp(2 a p (w - h P/2)) of one axis (FP64; 1 when w = h P/2).
__device__ __forceinline__ double axis_factor(double p, double a, double w, double h, int P)
{
    const double dw = w - h * (double)(P / 2);
    return dw == 0.0 ? 1.0 : exp(2.0 * a * p * dw);
}

// exp(a (p - h (i - P/2))^2) in FP32 (af = a, hf = h, pf = p as floats).
__device__ __forceinline__ float axis_weight(float af, float hf, float pf, int P, int i)
{
    const float d = fmaf(-hf, (float)(i - P / 2), pf);
    return __expf(af * d * d);
}

__device__ __forceinline__ int wrapi(int i, int M)
{
    i %= M;
    return i < 0 ? i + M : i;
}

// ---------------------------------------------------------------------------
// FP32 spread: one warp per source, lanes over the flattened (P+1)^2 stencil.
// The grids are interleaved per node ([node][W], W = 2 for the SLP pair, 4
// otherwise, the DLP-only form's fourth lane zero) so that a node takes one
// vector atomic (red.global.add.v2/v4.f32) instead of one per component; the
// fifth component of SLP+DLP follows as a plain grid at grid + 4 G.
// ---------------------------------------------------------------------------
constexpr int kSpreadWarpsF = 8;

template <int NC>
__global__ void __launch_bounds__(kSpreadWarpsF * 32, 4) k_spread_f32(SpreadArgsF a)
{
    __shared__ float wsh[kSpreadWarpsF][NC + 1][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P1 = a.P + 1, NN = P1 * P1;
    const size_t G = (size_t)a.Mx * a.My;
    // (i, jj) of flattened stencil entry q = lane + 32 k, stepped without division
    const int di = 32 / P1, dj = 32 - di * P1, i0 = lane / P1, j0 = lane - i0 * P1;
    const bool once = a.Mx > a.P && a.My > a.P;      // a stencil wraps at most once
    const int64_t nw = (int64_t)gridDim.x * kSpreadWarpsF;
    for (int64_t base = ((int64_t)blockIdx.x * kSpreadWarpsF + wid) * 32; base < a.ns;
         base += nw * 32) {
        const int64_t sl = base + lane;
        int mx = 0, my = 0;
        float pxf = 0.f, pyf = 0.f;
        float cf[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) cf[c] = 0.f;
        if (sl < a.ns) {
            const double2 S = a.sp[sl];
            double px, py;
            closest_node(S.x, S.y, a.Lhx, a.Lhy, a.h, a.P, mx, my, px, py);
            pxf = (float)px;
            pyf = (float)py;
            const double E = axis_factor(px, a.a, a.w, a.h, a.P) * axis_factor(py, a.a, a.w, a.h, a.P);
#pragma unroll
            for (int c = 0; c < NC; c++) cf[c] = (float)(a.coef[NC * sl + c] * E);
        }
        const float af = (float)a.a, hf = (float)a.h;
        const int cnt = (int)min((int64_t)32, a.ns - base);
        for (int j = 0; j < cnt; j++) {
            const int smx = __shfl_sync(~0u, mx, j), smy = __shfl_sync(~0u, my, j);
            const float spx = __shfl_sync(~0u, pxf, j), spy = __shfl_sync(~0u, pyf, j);
            float sc[NC];
#pragma unroll
            for (int c = 0; c < NC; c++) sc[c] = __shfl_sync(~0u, cf[c], j);
            if (lane < P1) {
                const float wx = axis_weight(af, hf, spx, a.P, lane);
#pragma unroll
                for (int c = 0; c < NC; c++) wsh[wid][c][lane] = sc[c] * wx;
                wsh[wid][NC][lane] = axis_weight(af, hf, spy, a.P, lane);
            }
            __syncwarp();
            const int c0 = wrapi(smx, a.Mx), r0 = wrapi(smy, a.My);
            int i = i0, jj = j0;
            for (int qd = lane; qd < NN; qd += 32, i += di, jj += dj) {
                if (jj >= P1) {
                    jj -= P1;
                    i++;
                }
                int col = c0 + i, row = r0 + jj;
                if (once) {
                    col = col >= a.Mx ? col - a.Mx : col;
                    row = row >= a.My ? row - a.My : row;
                } else {
                    col %= a.Mx;
                    row %= a.My;
                }
                const float wy = wsh[wid][NC][jj];
                const size_t node = (size_t)col * a.My + row;
                if (NC == 2) {
                    atomicAdd(reinterpret_cast<float2 *>(a.grid) + node,
                              make_float2(wsh[wid][0][i] * wy, wsh[wid][1][i] * wy));
                } else {
                    atomicAdd(reinterpret_cast<float4 *>(a.grid) + node,
                              make_float4(wsh[wid][0][i] * wy, wsh[wid][1][i] * wy,
                                          wsh[wid][2][i] * wy, NC > 3 ? wsh[wid][3 % NC][i] * wy : 0.f));
                    if (NC == 5) atomicAdd(a.grid + 4 * G + node, wsh[wid][4 % NC][i] * wy);
                }
            }
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------------------
// FP32 filter on the half spectrum; same modes, Nyquist projection, -i and
// 1/(Mx My) as k_filter (se2p_kernels.cu).
// ---------------------------------------------------------------------------
// dk = 2 pi / L, formed on the host
__device__ __forceinline__ float kfreq_f(int j, int M, double dk)
{
    return (float)(dk * (double)(j <= M / 2 ? j : j - M));
}

__device__ __forceinline__ void slp_mode_f(float k1, float k2, float c1, float c2, float2 h1,
                                           float2 h2, float2 &o1, float2 &o2)
{
    // c1 = 1/(4 xi^2), c2 = (1-eta)/(4 xi^2)
    const float K2 = k1 * k1 + k2 * k2;
    const float e = (1.f / (K2 * K2) + c1 / K2) * __expf(-c2 * K2);
    o1.x = k2 * (k2 * h1.x - k1 * h2.x) * e;
    o1.y = k2 * (k2 * h1.y - k1 * h2.y) * e;
    o2.x = k1 * (k1 * h2.x - k2 * h1.x) * e;
    o2.y = k1 * (k1 * h2.y - k2 * h1.y) * e;
}

__device__ __forceinline__ void dlp_mode_f(float k1, float k2, float c1, float c2, float2 h1,
                                           float2 h23, float2 h4, float2 &o1, float2 &o2)
{
    const float K2 = k1 * k1 + k2 * k2;
    const float et = __expf(-c2 * K2) / (K2 * K2) * (1.f + c1 * K2);
    const float B111 = 3.f * k1 * K2 - 2.f * k1 * k1 * k1;
    const float B112 = k2 * K2 - 2.f * k1 * k1 * k2;
    const float B122 = k1 * K2 - 2.f * k1 * k2 * k2;
    const float B222 = 3.f * k2 * K2 - 2.f * k2 * k2 * k2;
    o1.x = et * (B111 * h1.x + B112 * h23.x + B122 * h4.x);
    o1.y = et * (B111 * h1.y + B112 * h23.y + B122 * h4.y);
    o2.x = et * (B112 * h1.x + B122 * h23.x + B222 * h4.x);
    o2.y = et * (B112 * h1.y + B122 * h23.y + B222 * h4.y);
}

__global__ void k_filter_f32(FilterArgsF a)
{
    const int H = a.My / 2 + 1;
    const int64_t G = (int64_t)a.Mx * H;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= G) return;
    const int jx = (int)((unsigned long long)idx / (unsigned)H);
    const int jy = (int)(idx - (int64_t)jx * H);
    float2 *sp = a.spec;
    const bool zero = (jx == 0 && jy == 0);
    const bool nyq = (jx == a.Mx / 2) || (jy == a.My / 2);
    const float k1 = kfreq_f(jx, a.Mx, a.dkx), k2 = kfreq_f(jy, a.My, a.dky);
    const float k1p = (jx == a.Mx / 2) ? k1 : -k1;
    const float k2p = (jy == a.My / 2) ? k2 : -k2;
    const float c1 = a.c1, c2 = a.c2;
    const float sc = a.scale;
    float2 so1, so2, do1, do2;
    if (a.slp_in >= 0) {
        const float2 h1 = sp[a.slp_in * G + idx], h2 = sp[(a.slp_in + 1) * G + idx];
        slp_mode_f(k1, k2, c1, c2, h1, h2, so1, so2);
        if (nyq) {
            float2 p1, p2;
            slp_mode_f(k1p, k2p, c1, c2, h1, h2, p1, p2);
            so1.x = 0.5f * (so1.x + p1.x); so1.y = 0.5f * (so1.y + p1.y);
            so2.x = 0.5f * (so2.x + p2.x); so2.y = 0.5f * (so2.y + p2.y);
        }
        so1.x *= sc; so1.y *= sc; so2.x *= sc; so2.y *= sc;
        if (zero) so1 = so2 = make_float2(0.f, 0.f);
    }
    if (a.dlp_in >= 0) {
        const float2 h1 = sp[a.dlp_in * G + idx], h23 = sp[(a.dlp_in + 1) * G + idx];
        const float2 h4 = sp[(a.dlp_in + 2) * G + idx];
        dlp_mode_f(k1, k2, c1, c2, h1, h23, h4, do1, do2);
        if (nyq) {
            float2 p1, p2;
            dlp_mode_f(k1p, k2p, c1, c2, h1, h23, h4, p1, p2);
            do1.x = 0.5f * (do1.x - p1.x); do1.y = 0.5f * (do1.y - p1.y);
            do2.x = 0.5f * (do2.x - p2.x); do2.y = 0.5f * (do2.y - p2.y);
        }
        do1 = make_float2(do1.y * sc, -do1.x * sc);
        do2 = make_float2(do2.y * sc, -do2.x * sc);
        if (zero) do1 = do2 = make_float2(0.f, 0.f);
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

// ---------------------------------------------------------------------------
// FP32 gather: one lane per target; FP32 weights and sums (the per-point factor in FP64).
// The NC grids are interleaved per node ([node][NC], the C2R's strided
// output), one vector load per node.
// ---------------------------------------------------------------------------
// PT > 0: the stencil width as a template constant (PT = P), so the row
// weights take PT + 1 registers and four blocks fit per SM.
template <int NC, int PT>
__global__ void __launch_bounds__(256, 4) k_gather_f32(GatherArgsF a)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.nt) return;
    constexpr int PM = PT > 0 ? PT : kMaxP;
    const int P = PT > 0 ? PT : a.P;
    const double2 T = a.tp[t];
    int mx, my;
    double px, py;
    closest_node(T.x, T.y, a.Lhx, a.Lhy, a.h, P, mx, my, px, py);
    const double E = axis_factor(px, a.a, a.w, a.h, P) * axis_factor(py, a.a, a.w, a.h, P);
    const float af = (float)a.a, hf = (float)a.h, pxf = (float)px, pyf = (float)py;
    float wy[PM + 1];
#pragma unroll
    for (int j = 0; j <= PM; j++)
        if (j <= P) wy[j] = axis_weight(af, hf, pyf, P, j);
    float acc[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) acc[c] = 0.f;
    const bool rows_inside = my >= 0 && my + P < a.My;
    for (int i = 0; i <= P; i++) {
        const size_t col = (size_t)wrapi(mx + i, a.Mx) * a.My;
        float tc[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) tc[c] = 0.f;
#pragma unroll
        for (int j = 0; j <= PM; j++) {
            if (j <= P) {
                const int row = rows_inside ? my + j : wrapi(my + j, a.My);
                float v[NC];
                if (NC == 2) {
                    const float2 q = __ldg(reinterpret_cast<const float2 *>(a.grid) + col + row);
                    v[0] = q.x;
                    v[1] = q.y;
                } else {
                    const float4 q = __ldg(reinterpret_cast<const float4 *>(a.grid) + col + row);
                    v[0] = q.x;
                    v[1 % NC] = q.y;
                    v[2 % NC] = q.z;
                    v[3 % NC] = q.w;
                }
#pragma unroll
                for (int c = 0; c < NC; c++) tc[c] = fmaf(wy[j], v[c], tc[c]);
            }
        }
        const float wx = axis_weight(af, hf, pxf, P, i);
#pragma unroll
        for (int c = 0; c < NC; c++) acc[c] = fmaf(wx, tc[c], acc[c]);
    }
    const double sE = a.scale * E;
#pragma unroll
    for (int k = 0; k < NC / 2; k++)
        a.out[k * a.nt + t] = make_double2((double)acc[2 * k] * sE, (double)acc[2 * k + 1] * sE);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline unsigned grid_for_f(int64_t n, int block)
{
    int64_t g = (n + block - 1) / block;
    return (unsigned)(g < 1 ? 1 : g);
}

cudaError_t launch_spread_f32(const SpreadArgsF &a, int nc, int sms, cudaStream_t st,
                              int64_t &launches)
{
    if (a.ns <= 0) return cudaSuccess;
    const int64_t warps = (a.ns + 31) / 32;
    const int64_t want = (warps + kSpreadWarpsF - 1) / kSpreadWarpsF;
    const int64_t cap = (int64_t)sms * 8;
    const unsigned g = (unsigned)(want < cap ? want : cap);
    switch (nc) {
    case 2: k_spread_f32<2><<<g, kSpreadWarpsF * 32, 0, st>>>(a); break;
    case 3: k_spread_f32<3><<<g, kSpreadWarpsF * 32, 0, st>>>(a); break;
    default: k_spread_f32<5><<<g, kSpreadWarpsF * 32, 0, st>>>(a); break;
    }
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_filter_f32(const FilterArgsF &a, cudaStream_t st, int64_t &launches)
{
    const int64_t n = (int64_t)a.Mx * (a.My / 2 + 1);
    k_filter_f32<<<grid_for_f(n, 256), 256, 0, st>>>(a);
    launches++;
    return cudaGetLastError();
}

cudaError_t launch_gather_f32(const GatherArgsF &a, int nc, cudaStream_t st, int64_t &launches)
{
    if (a.nt <= 0) return cudaSuccess;
    const unsigned g = grid_for_f(a.nt, 256);
    if (a.P == 12) {
        if (nc == 2) k_gather_f32<2, 12><<<g, 256, 0, st>>>(a);
        else k_gather_f32<4, 12><<<g, 256, 0, st>>>(a);
    } else {
        if (nc == 2) k_gather_f32<2, 0><<<g, 256, 0, st>>>(a);
        else k_gather_f32<4, 0><<<g, 256, 0, st>>>(a);
    }
    launches++;
    return cudaGetLastError();
}

}  // namespace se2p
