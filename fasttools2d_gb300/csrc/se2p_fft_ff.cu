// se2p_fft_ff.cu -- batched 1D complex FFTs of contiguous rows in
// float-float arithmetic (the FP64 form's k-space transforms).
//
// cuFFT's double-precision C2C of the grid lengths the spectral Ewald method
// uses (2688 = 2^7 3 7 at tolerance 1e-10 and a million points) runs on the
// FP64 pipe, which GB300 provides at 1/73 of its FP32 rate: the four 1D
// passes of one evaluation took 7 ms, more than any other stage.  Here each
// row is transformed in shared memory with float-float arithmetic (about 48
// significant bits) on the FP32 pipe.  The FFT's rounding errors are spread
// over all modes, and the k-space sums average them: errors of 2^-46 relative
// to the spectra's mean magnitude, injected into the oracle's transforms,
// change its SLP and DLP k-space results by 1e-15 to 7e-15, far inside the
// 1e-12 parity bound (the systematic errors of float-float Gaussian weights
// do not average out, which is why the spread and gather stay exact).
//
// One CTA per row: the row is read once as doubles (staged in shared memory
// for the exponent scan), scaled by a power of two that
// puts its largest entry near 2^64 (exact; the FFT of a row of L <= 2^13
// values grows it by at most L), split into float-float pairs with integer
// operations, transformed by mixed-radix Stockham stages (radices 8, 4, 6, 2,
// 7, 5, 3, ping-pong between two shared buffers), and written back as doubles
// rebuilt with integer operations (float <-> double conversions run at the
// FP64 rate on GB300).  Twiddles exp(-2 pi i m / L) come from a per-length
// table built in long double on the host; the odd radices take their
// constants cos, sin(2 pi m / R) from the same table (entry m L / R).
//
// The transform is unnormalised with cuFFT's sign convention (forward
// exp(-2 pi i j k / L)), so it replaces cufftExecZ2Z on the same layout.
#include "se2p_internal.cuh"
#include <math_constants.h>

namespace se2p {

namespace {

struct fc {
    float2 r, i;   // real and imaginary parts, each (hi, lo)
};

__device__ __forceinline__ fc fc_add(const fc &a, const fc &b) { return {ff_add(a.r, b.r), ff_add(a.i, b.i)}; }
__device__ __forceinline__ fc fc_sub(const fc &a, const fc &b) { return {ff_sub(a.r, b.r), ff_sub(a.i, b.i)}; }
// a * (s i), s = +-1
__device__ __forceinline__ fc fc_mul_si(const fc &a, float s)
{
    return s > 0.f ? fc{ff_neg(a.i), a.r} : fc{a.i, ff_neg(a.r)};
}
__device__ __forceinline__ fc fc_mulr(const fc &a, float2 c) { return {ff_mul(a.r, c), ff_mul(a.i, c)}; }

// x1 y1 - x2 y2 in float-float (products exact to the float-float level).
__device__ __forceinline__ float2 ff_dd(float2 x1, float2 y1, float2 x2, float2 y2)
{
    const float p1 = x1.x * y1.x;
    float e1 = fmaf(x1.x, y1.x, -p1);
    e1 = fmaf(x1.x, y1.y, e1);
    e1 = fmaf(x1.y, y1.x, e1);
    const float p2 = x2.x * y2.x;
    float e2 = fmaf(x2.x, y2.x, -p2);
    e2 = fmaf(x2.x, y2.y, e2);
    e2 = fmaf(x2.y, y2.x, e2);
    float s, t;
    two_sum(p1, -p2, s, t);
    t += e1 - e2;
    float h, l;
    fast_two_sum(s, t, h, l);
    return make_float2(h, l);
}

// a * w, w a twiddle (already conjugated for the inverse)
__device__ __forceinline__ fc fc_mul(const fc &a, const fc &w)
{
    return {ff_dd(a.r, w.r, a.i, w.i), ff_dd(a.r, w.i, ff_neg(a.i), w.r)};
}

__device__ __forceinline__ fc tw_load(const float4 *tw, int m, float s)
{
    const float4 t = __ldg(tw + m);
    // table holds exp(-2 pi i m / L); the inverse (s = +1) takes its conjugate
    return s < 0.f ? fc{make_float2(t.x, t.y), make_float2(t.z, t.w)}
                   : fc{make_float2(t.x, t.y), make_float2(-t.z, -t.w)};
}

// Shared buffer: four float arrays (re hi, re lo, im hi, im lo) of Lp =
// sh_len(L) words each, element k at k + k/32: the padding word per 32 turns
// the stride-R stores of the early stages (R = 2, 4, 8) into at most 2-way
// bank conflicts.
__host__ __device__ __forceinline__ int sh_len(int L) { return L + (L >> 5) + 1; }
__device__ __forceinline__ fc sh_get(const float *b, int Lp, int k)
{
    k += k >> 5;
    return {make_float2(b[k], b[Lp + k]), make_float2(b[2 * Lp + k], b[3 * Lp + k])};
}
__device__ __forceinline__ void sh_put(float *b, int Lp, int k, const fc &v)
{
    k += k >> 5;
    b[k] = v.r.x;
    b[Lp + k] = v.r.y;
    b[2 * Lp + k] = v.i.x;
    b[3 * Lp + k] = v.i.y;
}

// Radix-R butterflies of one Stockham stage.  Input element r of butterfly j
// is A[j + r L/R]; it is multiplied by w^(k r L/(Ns R)), k = j mod Ns, the
// R-point DFT is taken, and output r goes to B[(j / Ns) Ns R + k + r Ns].
template <int R>
__device__ __forceinline__ void dft(fc *v, float s, const fc *cst);

template <>
__device__ __forceinline__ void dft<2>(fc *v, float, const fc *)
{
    const fc a = v[0], b = v[1];
    v[0] = fc_add(a, b);
    v[1] = fc_sub(a, b);
}

template <>
__device__ __forceinline__ void dft<4>(fc *v, float s, const fc *)
{
    const fc t0 = fc_add(v[0], v[2]), t1 = fc_sub(v[0], v[2]);
    const fc t2 = fc_add(v[1], v[3]), t3 = fc_mul_si(fc_sub(v[1], v[3]), s);   // W4 = s i
    v[0] = fc_add(t0, t2);
    v[2] = fc_sub(t0, t2);
    v[1] = fc_add(t1, t3);
    v[3] = fc_sub(t1, t3);
}

// cst[0].r = sqrt(1/2)
template <>
__device__ __forceinline__ void dft<8>(fc *v, float s, const fc *cst)
{
    fc e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft<4>(e, s, nullptr);
    dft<4>(o, s, nullptr);
    const float2 h = cst[0].r;
    // W8 = (1 + s i) sqrt(1/2), W8^2 = s i, W8^3 = (-1 + s i) sqrt(1/2)
    const fc o1 = fc_mulr(fc_add(o[1], fc_mul_si(o[1], s)), h);
    const fc o2 = fc_mul_si(o[2], s);
    const fc o3 = fc_mulr(fc_sub(fc_mul_si(o[3], s), o[3]), h);
    v[0] = fc_add(e[0], o[0]);
    v[4] = fc_sub(e[0], o[0]);
    v[1] = fc_add(e[1], o1);
    v[5] = fc_sub(e[1], o1);
    v[2] = fc_add(e[2], o2);
    v[6] = fc_sub(e[2], o2);
    v[3] = fc_add(e[3], o3);
    v[7] = fc_sub(e[3], o3);
}

// Float-float dot-product accumulator: the heads are summed by TwoSum, and
// each product's FMA-formed error, its cross terms and the TwoSum errors go
// into an unnormalised tail; one normalisation at the end.  A term costs 12
// FP32 operations against 18 for a product and an add normalised separately.
struct ffacc {
    float s, t;
};
__device__ __forceinline__ ffacc acc_from(float2 x) { return {x.x, x.y}; }
__device__ __forceinline__ ffacc acc_prod(float2 c, float2 x)
{
    const float p = c.x * x.x;
    float e = fmaf(c.x, x.x, -p);
    e = fmaf(c.x, x.y, e);
    e = fmaf(c.y, x.x, e);
    return {p, e};
}
__device__ __forceinline__ void acc_add(ffacc &a, float2 x)
{
    float s, q;
    two_sum(a.s, x.x, s, q);
    a.s = s;
    a.t += q + x.y;
}
__device__ __forceinline__ void acc_fma(ffacc &a, float2 c, float2 x)
{
    const ffacc p = acc_prod(c, x);
    float s, q;
    two_sum(a.s, p.s, s, q);
    a.s = s;
    a.t += q + p.t;
}
__device__ __forceinline__ float2 acc_get(const ffacc &a) { return ff_norm(a.s, a.t); }

// Odd R: with s_n = a_n + a_(R-n), d_n = a_n - a_(R-n),
// A_k = a_0 + sum_n cos(2 pi n k / R) s_n, B_k = sum_n sin(2 pi n k / R) d_n,
// X_k = A_k + s i B_k, X_(R-k) = A_k - s i B_k.  cst[m] = (cos, sin)(2 pi m / R),
// m = 1 .. (R-1)/2, as the .r and .i fields.  The sums X_0, A_k and B_k are
// float-float dot products (ffacc).
template <int R>
__device__ __forceinline__ void dft_odd(fc *v, float s, const fc *cst)
{
    constexpr int h = (R - 1) / 2;
    fc sm[h], df[h];
#pragma unroll
    for (int n = 1; n <= h; n++) {
        sm[n - 1] = fc_add(v[n], v[R - n]);
        df[n - 1] = fc_sub(v[n], v[R - n]);
    }
    const fc a0 = v[0];
    ffacc x0r = acc_from(a0.r), x0i = acc_from(a0.i);
#pragma unroll
    for (int n = 0; n < h; n++) {
        acc_add(x0r, sm[n].r);
        acc_add(x0i, sm[n].i);
    }
#pragma unroll
    for (int k = 1; k <= h; k++) {
        ffacc Ar = acc_from(a0.r), Ai = acc_from(a0.i), Br = {0.f, 0.f}, Bi = {0.f, 0.f};
#pragma unroll
        for (int n = 1; n <= h; n++) {
            int m = (n * k) % R;
            const bool neg = m > h;                  // sin(2 pi (R-m)/R) = -sin(2 pi m/R)
            if (neg) m = R - m;
            const float2 c = cst[m - 1].r;
            const float2 sn = neg ? ff_neg(cst[m - 1].i) : cst[m - 1].i;
            acc_fma(Ar, c, sm[n - 1].r);
            acc_fma(Ai, c, sm[n - 1].i);
            if (n == 1) {
                Br = acc_prod(sn, df[0].r);
                Bi = acc_prod(sn, df[0].i);
            } else {
                acc_fma(Br, sn, df[n - 1].r);
                acc_fma(Bi, sn, df[n - 1].i);
            }
        }
        const fc A = {acc_get(Ar), acc_get(Ai)};
        const fc iB = fc_mul_si(fc{acc_get(Br), acc_get(Bi)}, s);
        v[k] = fc_add(A, iB);
        v[R - k] = fc_sub(A, iB);
    }
    v[0] = {acc_get(x0r), acc_get(x0i)};
}

template <>
__device__ __forceinline__ void dft<3>(fc *v, float s, const fc *cst) { dft_odd<3>(v, s, cst); }
template <>
__device__ __forceinline__ void dft<5>(fc *v, float s, const fc *cst) { dft_odd<5>(v, s, cst); }
template <>
__device__ __forceinline__ void dft<7>(fc *v, float s, const fc *cst) { dft_odd<7>(v, s, cst); }

// R = 6 = 2 x 3 by the prime-factor (Good-Thomas) split, with no inner
// twiddles: 3-point DFTs of inputs (0, 2, 4) and (3, 5, 1), then 2-point
// DFTs of their outputs, which land at (3 k1 + 4 k2) mod 6.  cst as for R = 3.
template <>
__device__ __forceinline__ void dft<6>(fc *v, float s, const fc *cst)
{
    fc a[3] = {v[0], v[2], v[4]}, b[3] = {v[3], v[5], v[1]};
    dft_odd<3>(a, s, cst);
    dft_odd<3>(b, s, cst);
    v[0] = fc_add(a[0], b[0]);
    v[3] = fc_sub(a[0], b[0]);
    v[4] = fc_add(a[1], b[1]);
    v[1] = fc_sub(a[1], b[1]);
    v[2] = fc_add(a[2], b[2]);
    v[5] = fc_sub(a[2], b[2]);
}

template <int R>
__device__ void stage(const float *A, float *B, int L, int Ns, unsigned magic, float s,
                      const float4 *tw)
{
    // the constants of the R-point DFT from the twiddle table
    fc cst[R / 2 > 0 ? R / 2 : 1];
    if (R == 8) {
        const fc w = tw_load(tw, L / 8, -1.f);       // exp(-i pi/4): re = sqrt(1/2)
        cst[0] = w;
    } else if (R & 1) {
#pragma unroll
        for (int m = 1; m <= R / 2; m++) {
            const fc w = tw_load(tw, m * (L / R), -1.f);   // cos - i sin
            cst[m - 1] = {w.r, ff_neg(w.i)};
        }
    } else if (R == 6) {
        const fc w = tw_load(tw, L / 3, -1.f);       // the 3-point constants
        cst[0] = {w.r, ff_neg(w.i)};
    }
    const int nb = L / R, stride = L / (Ns * R), Lp = sh_len(L);
    for (int j = threadIdx.x; j < nb; j += blockDim.x) {
        const int k = Ns == 1 ? 0 : j - (int)__umulhi((unsigned)j, magic) * Ns;   // j mod Ns
        fc v[R];
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = sh_get(A, Lp, j + r * nb);
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; r++) v[r] = fc_mul(v[r], tw_load(tw, k * r * stride, s));
        }
        dft<R>(v, s, cst);
        const int o = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; r++) sh_put(B, Lp, o + r * Ns, v[r]);
    }
}

// exact: hi + lo rebuilt as a double with integer operations (truncated to
// 53 bits), times 2^e.  hi, lo normalised float-float (|lo| <= ulp(hi)/2),
// finite, and the result in the normal range.
__device__ __forceinline__ double ff_to_double_scaled(float hi, float lo, int e)
{
    const unsigned hb = __float_as_uint(hi), lb = __float_as_uint(lo);
    const int eh = (int)((hb >> 23) & 0xff);
    if (eh == 0) return 0.0;
    if (eh == 0xff) return (double)hi;               // inf, NaN (rare: the slow conversion)
    long long m = (long long)((hb & 0x7fffffu) | 0x800000u) << 29;   // units 2^(eh-179)
    const int el = (int)((lb >> 23) & 0xff);
    if (el != 0) {
        const long long ml = (long long)((lb & 0x7fffffu) | 0x800000u);
        const int sh = el - eh + 29;
        long long d = sh >= 0 ? (ml << sh) : (sh > -40 ? (ml >> (-sh)) : 0);
        m += ((lb ^ hb) >> 31) ? -d : d;
    }
    int be = eh + 896 + e;                           // biased double exponent of 2^52 m ... units
    if (m >= (1ll << 53)) {
        m >>= 1;
        be++;
    } else if (m < (1ll << 52)) {
        m <<= 1;
        be--;
    }
    if (be <= 0) return 0.0;
    if (be >= 0x7ff) return hi > 0.f ? CUDART_INF : -CUDART_INF;
    const unsigned long long bits = ((unsigned long long)(hb >> 31) << 63) |
                                    ((unsigned long long)be << 52) |
                                    ((unsigned long long)m & ((1ull << 52) - 1));
    return __longlong_as_double((long long)bits);
}

// a > 0 rounded to 24 bits (to nearest, ties up): the float's bit pattern,
// and in *rem the remainder a - rounded (|rem| <= 2^(bits-25)).  a < 2^62.
__device__ __forceinline__ unsigned u64_round_float(unsigned long long a, long long *rem)
{
    const int nb = 64 - __clzll(a);
    const int sh = nb - 24;
    unsigned long long mh;
    if (sh <= 0) {
        mh = a << (-sh);
        if (rem) *rem = 0;
    } else {
        mh = (a + (1ull << (sh - 1))) >> sh;
        if (rem) *rem = (long long)a - (long long)(mh << sh);
    }
    int ex = nb - 1;
    if (mh >> 24) {                                  // rounding carried into bit 24
        mh >>= 1;
        ex++;
    }
    return ((unsigned)(ex + 127) << 23) | ((unsigned)mh & 0x7fffffu);
}

// An int64 (|v| < 2^62) as float-float with integer operations.
__device__ __forceinline__ float2 ll_to_ff(long long v)
{
    if (v == 0) return make_float2(0.f, 0.f);
    const unsigned sv = v < 0 ? 0x80000000u : 0u;
    const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    long long r;
    const float hi = __uint_as_float(sv | u64_round_float(a, &r));
    if (r == 0) return make_float2(hi, 0.f);
    const unsigned sr = ((r < 0) != (v < 0)) ? 0x80000000u : 0u;
    const unsigned long long ar = r < 0 ? 0ull - (unsigned long long)r : (unsigned long long)r;
    return make_float2(hi, __uint_as_float(sr | u64_round_float(ar, nullptr)));
}

// d 2^-e as float-float (ff_split of the scaled value, the scaling done on
// the exponent field)
__device__ __forceinline__ float2 ff_split_scaled(double d, int e)
{
    const int ex = (__double2hiint(d) >> 20) & 0x7ff;
    if (ex == 0) return make_float2(0.f, 0.f);
    if (ex == 0x7ff) return ff_split(d);             // inf, NaN stay so
    const int ne = ex - e;
    if (ne <= 0) return make_float2(0.f, 0.f);
    const long long b = __double_as_longlong(d);
    const long long nb = (b & ~(0x7ffll << 52)) | ((long long)ne << 52);
    return ff_split(__longlong_as_double(nb));
}

__global__ void __launch_bounds__(256) k_fft_rows_ff(double2 *__restrict__ data, int64_t rows,
                                                     FftRowsFF p, const float4 *__restrict__ tw)
{
    extern __shared__ float fsh[];
    __shared__ int emax_w[8];
    const int L = p.L, Lp = sh_len(L);
    const float s = (float)p.sign;
    float *A = fsh, *B = fsh + 4 * Lp;
    // fused pack from int64 planes: the values need no row scaling (|v| <
    // 2^60 stays far inside the float range after the transform's growth by
    // at most L); the 2^-S of the fixed-point grid is applied on the way out
    const unsigned long long bnd = p.bound ? *p.bound : kFixedOff;
    const bool fixed_in = p.pack_in && bnd != kFixedOff;
    const int S = fixed_in ? fix_shift(bnd) : 0;
    for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
        double2 *d = data + row * L;
        const int64_t q = p.Mx ? row / p.Mx : 0, xr = row - q * p.Mx;
        int64_t off_re = (2 * q) * p.G + xr * L, off_im = (2 * q + 1) * p.G + xr * L;
        bool has_im = 2 * q + 1 < p.npl_in;
        if (p.fold && 2 * q + 1 == p.npl_in) {        // the folded plane: rows xr, xr + Mx/2
            off_im = (2 * q) * p.G + (xr + p.Mx / 2) * L;
            has_im = true;
        }
        int e;
        if (fixed_in) {
            const long long *g = static_cast<const long long *>(p.pack_in);
            for (int k = threadIdx.x; k < L; k += blockDim.x) {
                const long long vr = g[off_re + k], vi = has_im ? g[off_im + k] : 0;
                sh_put(A, Lp, k, fc{ll_to_ff(vr), ll_to_ff(vi)});
            }
            e = -S;
        } else {
            // the row as doubles into B (4 Lp floats >= L double2), and its
            // largest exponent
            double2 *raw = reinterpret_cast<double2 *>(B);
            int em = 0;
            for (int k = threadIdx.x; k < L; k += blockDim.x) {
                double2 v;
                if (p.pack_in) {
                    const double *g = static_cast<const double *>(p.pack_in);
                    v = make_double2(g[off_re + k], has_im ? g[off_im + k] : 0.0);
                } else {
                    v = d[k];
                }
                raw[k] = v;
                em = max(em, max((__double2hiint(v.x) >> 20) & 0x7ff, (__double2hiint(v.y) >> 20) & 0x7ff));
            }
            for (int o = 16; o > 0; o >>= 1) em = max(em, __shfl_xor_sync(~0u, em, o));
            if ((threadIdx.x & 31) == 0) emax_w[threadIdx.x >> 5] = em;
            __syncthreads();
            em = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) em = max(em, emax_w[w]);
            // scale 2^-e brings the largest finite entry to [2^63, 2^64) (no
            // scaling of a zero row or of one with an inf or NaN, which then
            // spreads through the row as in an FP64 transform)
            e = (em == 0 || em == 0x7ff) ? 0 : em - 1023 - 63;
            for (int k = threadIdx.x; k < L; k += blockDim.x) {
                const double2 v = raw[k];
                sh_put(A, Lp, k, fc{ff_split_scaled(v.x, e), ff_split_scaled(v.y, e)});
            }
        }
        __syncthreads();
        int Ns = 1;
        for (int st = 0; st < p.nst; st++) {
            const int R = p.radix[st];
            const unsigned mg = p.magic[st];
            switch (R) {
            case 8: stage<8>(A, B, L, Ns, mg, s, tw); break;
            case 4: stage<4>(A, B, L, Ns, mg, s, tw); break;
            case 6: stage<6>(A, B, L, Ns, mg, s, tw); break;
            case 2: stage<2>(A, B, L, Ns, mg, s, tw); break;
            case 7: stage<7>(A, B, L, Ns, mg, s, tw); break;
            case 5: stage<5>(A, B, L, Ns, mg, s, tw); break;
            default: stage<3>(A, B, L, Ns, mg, s, tw); break;
            }
            Ns *= R;
            float *t = A;
            A = B;
            B = t;
            __syncthreads();
        }
        if (p.unpack_out) {
            // fused unpack: real and imaginary parts to their planes, with the
            // largest |value| for the fixed-point gather
            const bool has_im = 2 * q + 1 < p.npl_out;
            unsigned long long m = 0;
            for (int k = threadIdx.x; k < L; k += blockDim.x) {
                const fc v = sh_get(A, Lp, k);
                const double re = ff_to_double_scaled(v.r.x, v.r.y, e);
                p.unpack_out[off_re + k] = re;
                m = max(m, (unsigned long long)__double_as_longlong(fabs(re)));
                if (has_im) {
                    const double im = ff_to_double_scaled(v.i.x, v.i.y, e);
                    p.unpack_out[off_im + k] = im;
                    m = max(m, (unsigned long long)__double_as_longlong(fabs(im)));
                }
            }
            if (p.gmax) {
                for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(~0u, m, o));
                if ((threadIdx.x & 31) == 0 && m) atomicMax(p.gmax + q, m);
            }
        } else {
            for (int k = threadIdx.x; k < L; k += blockDim.x) {
                const fc v = sh_get(A, Lp, k);
                d[k] = make_double2(ff_to_double_scaled(v.r.x, v.r.y, e),
                                    ff_to_double_scaled(v.i.x, v.i.y, e));
            }
        }
        // the next row reuses both buffers and emax_w
        A = fsh;
        B = fsh + 4 * Lp;
        __syncthreads();
    }
}

}  // namespace

bool fft_rows_ff_plan(int L, FftRowsFF &p)
{
    p.L = L;
    p.nst = 0;
    if (L < 2 || L > kFftFFMaxLen) return false;
    int n = L;
    while (n % 8 == 0 && p.nst < kFftFFMaxStages) { p.radix[p.nst++] = 8; n /= 8; }
    while (n % 4 == 0 && p.nst < kFftFFMaxStages) { p.radix[p.nst++] = 4; n /= 4; }
    while (n % 6 == 0 && p.nst < kFftFFMaxStages) { p.radix[p.nst++] = 6; n /= 6; }
    while (n % 2 == 0 && p.nst < kFftFFMaxStages) { p.radix[p.nst++] = 2; n /= 2; }
    for (int r : {7, 5, 3})
        while (n % r == 0 && p.nst < kFftFFMaxStages) { p.radix[p.nst++] = r; n /= r; }
    unsigned long long Ns = 1;
    for (int st = 0; st < p.nst; st++) {
        // (the first stage, Ns = 1, takes k = 0 without it)
        p.magic[st] = Ns == 1 ? 0u : (unsigned)(((1ull << 32) + Ns - 1) / Ns);
        Ns *= (unsigned long long)p.radix[st];
    }
    return n == 1;
}

void fft_rows_ff_twiddles(int L, float4 *host)
{
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int m = 0; m < L; m++) {
        const long double a = -2.0L * pi * (long double)m / (long double)L;
        const long double c = cosl(a), sn = sinl(a);
        const float ch = (float)c, sh = (float)sn;
        host[m] = make_float4(ch, (float)(c - (long double)ch), sh, (float)(sn - (long double)sh));
    }
}

cudaError_t launch_fft_rows_ff(double2 *data, int64_t rows, const FftRowsFF &p, const float4 *tw,
                               cudaStream_t st, int64_t &launches)
{
    if (rows <= 0) return cudaSuccess;
    const size_t smem = sizeof(float) * 8 * (size_t)sh_len(p.L);
    cudaError_t e = cudaFuncSetAttribute(k_fft_rows_ff, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const int per_sm = (int)std::max<size_t>(1, (size_t)(200 * 1024) / (smem + 1024));
    const int64_t cap = (int64_t)sm_count() * per_sm;
    const unsigned g = (unsigned)(rows < cap ? rows : cap);
    k_fft_rows_ff<<<g, 256, smem, st>>>(data, rows, p, tw);
    launches++;
    return cudaGetLastError();
}

}  // namespace se2p
