/*
 * se2p_oracle.c -- CPU ORACLE (test infrastructure only).
 *
 * A plain-C restatement of the doubly-periodic spectral Ewald (SE) path of
 * FastTools2D for the 2D Stokeslet (SLP) and stresslet (DLP).  It exists so
 * that tests, the smoke check and the CPU baseline of the benchmark have a
 * reference to compare the CUDA library against.  Nothing in the product
 * (the fasttools2d_gb300 package or libse2p) links, loads or calls it.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the FastTools2D project root, PE = PeriodicEwald).  The arithmetic follows
 * the reference operation by operation where the order decides a discrete
 * outcome (box index, cutoff test, grid-node snap), so that the pair sets and
 * stencils are identical; elsewhere it follows the same formulas.
 *
 * Build with -ffp-contract=off: the reference is compiled for x86 SSE, which
 * never fuses a*b+c; a fused multiply-add would move pairs across the cutoff.
 *
 * The FFT step is not here: the reference calls MATLAB's fft2/ifft2 through
 * mexCallMATLAB (PE/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:148-149,
 * :236-237); the Python side of the oracle (oracle/oracle.py) does the same
 * with numpy/scipy FFTs on the grids produced by or_*_spread.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_PI 3.1415926535897932385

/* ------------------------------------------------------------------------ */
/* Cell binning: PE/src/mex/common/ewald_tools.cpp:7-80 (Assign).           */
/* box = clamp(floor(nside*(x/L + 0.5))), row-major box id by*nside_x+bx,   */
/* then a stable counting sort.  perm[k] = input index of the k-th sorted   */
/* point; start[b]..start[b+1] is box b's range.                            */
/* ------------------------------------------------------------------------ */
static int or_box1(double x, double L, int nside)
{
    int b = (int)floor(nside * (x / L + 0.5));
    if (b < 0) b = 0;
    if (b >= nside) b = nside - 1;
    return b;
}

void or_assign(const double *p, int64_t n, double Lx, double Ly, int nside_x,
               int nside_y, int32_t *perm, int32_t *start)
{
    int64_t nbox = (int64_t)nside_x * nside_y;
    int32_t *box = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int64_t *fill = (int64_t *)calloc((size_t)nbox + 1, sizeof(int64_t));
    for (int64_t j = 0; j < n; j++) {
        int bx = or_box1(p[2 * j], Lx, nside_x);
        int by = or_box1(p[2 * j + 1], Ly, nside_y);
        box[j] = by * nside_x + bx;
        fill[box[j] + 1]++;
    }
    for (int64_t b = 0; b < nbox; b++) fill[b + 1] += fill[b];
    for (int64_t b = 0; b <= nbox; b++) start[b] = (int32_t)fill[b];
    for (int64_t j = 0; j < n; j++) perm[fill[box[j]]++] = (int32_t)j;
    free(box);
    free(fill);
}

/* ------------------------------------------------------------------------ */
/* Grid snap: PE/src/mex/common/ewald_tools.cpp:86-114 (FindClosestNode).   */
/* ------------------------------------------------------------------------ */
void or_find_closest_node(double x, double y, double Lx, double Ly, double h,
                          int P, int *mx, int *my, double *px, double *py)
{
    const double snap = 1e-13;
    double ox = x - h * floor(x / h);
    double oy = y - h * floor(y / h);
    double hx = Lx / 2.0, hy = Ly / 2.0;
    int ix = (int)(floor((x + hx) / h) - P / 2);
    int iy = (int)(floor((y + hy) / h) - P / 2);
    if (fabs(ox) < snap || fabs(ox - h) < snap) ox = 0;
    if (fabs(oy) < snap || fabs(oy - h) < snap) oy = 0;
    if (ox == 0 && remainder((x + hx) / h - P / 2, 1) < 0) ix++;
    if (oy == 0 && remainder((y + hy) / h - P / 2, 1) < 0) iy++;
    *mx = ix; *my = iy; *px = ox; *py = oy;
}

/* ------------------------------------------------------------------------ */
/* E1 by the reference's three-regime Pade split:                           */
/* PE/src/mex/StokesSLP/mex_stokes_slp_real.cpp:19-47 (coefficients, listed */
/* as interleaved numerator/denominator pairs, highest power first) and     */
/* :166-205 (evaluation).                                                   */
/* ------------------------------------------------------------------------ */
static const double E1_FAR[8] = {
    -17.70313744792479226930481672752649, -2.03222164752550948918496942496859,
    -9.56230625623594754358691716333851, 24.24775264986217493401454703416675,
    -0.99999982131078080094255255971802, 34.82867640350680460414878325536847,
    -0.00000000083503088648841284312372, 11.56228921223568129050818242831156};
static const double E1_MID[22] = {
    -1185.45720315201027667, -0.776491285282330997549,
    -14751.4895786128450662, 1229.20784182403048905,
    -54844.4587226402067411, 18455.4124737722049515,
    -86273.1567711649528784, 86722.3403467334749201,
    -66598.2652345418633509, 180329.498380501819718,
    -27182.6254466733970467, 192104.047790227984431,
    -6046.8250112711035463, 113057.05869159631492,
    -724.581482791462469795, 38129.5594484818471461,
    -43.3058660811817946037, 7417.37624454689546708,
    -0.999999999999998811143, 809.193214954550328455,
    -0.121013190657725568138e-18, 45.3058660811801465927};
static const double E1_NEAR_Y = 0.66373538970947265625;
static const double E1_NEAR[12] = {
    -0.000111507792921197858394, -0.528611029520217142048e-6,
    -0.00399167106081113256961, 0.000131049900798434683324,
    -0.0368031736257943745142, 0.00427347600017103698101,
    -0.245088216639761496153, 0.056770677104207528384,
    0.0320913665303559189999, 0.37091387659397013215,
    0.0865197248079397976498, 1.0};

/* Horner on interleaved pairs: a = num(z), b = den(z). */
static void or_pair_horner(const double *c, int len, double z, double *a, double *b)
{
    double n = c[0], d = c[1];
    for (int k = 2; k < len; k += 2) {
        n = z * n + c[k];
        d = z * d + c[k + 1];
    }
    *a = n; *b = d;
}

/* Returns E1(x) and sets *ex = exp(-x). */
double or_e1(double x, double *ex)
{
    double e = exp(-x), a, b;
    *ex = e;
    if (x >= 16) {
        double r = 1 / x;
        or_pair_horner(E1_FAR, 8, r, &a, &b);
        return e * (r + a / (b + x));
    } else if (x > 1) {
        double r = 1 / x;
        or_pair_horner(E1_MID, 22, r, &a, &b);
        return e * (r + a / (b + x));
    }
    or_pair_horner(E1_NEAR, 12, x, &a, &b);
    return a / b + x - log(x) - E1_NEAR_Y;
}

/* ------------------------------------------------------------------------ */
/* Shared neighbour-box walk of both real-space sums.                        */
/* PE/src/mex/StokesSLP/mex_stokes_slp_real.cpp:131-333 and                  */
/* PE/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:103-187: for every target   */
/* box, all pairs of the box itself (no cutoff), then the 8 neighbour boxes  */
/* (periodic, with an image shift) under r2 < Lx*Ly/nside_x/nside_y.         */
/* ------------------------------------------------------------------------ */
static const int NB_DX[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
static const int NB_DY[8] = {-1, 0, 1, -1, 1, -1, 0, 1};

typedef struct {
    double *sp, *tp;           /* sorted positions, interleaved */
    int32_t *sperm, *tperm, *sstart, *tstart;
} or_cells;

static void or_cells_build(or_cells *c, const double *psrc, int64_t ns,
                           const double *ptar, int64_t nt, double Lx, double Ly,
                           int nx, int ny)
{
    int64_t nbox = (int64_t)nx * ny;
    c->sperm = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ns > 0 ? ns : 1));
    c->tperm = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nt > 0 ? nt : 1));
    c->sstart = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nbox + 1));
    c->tstart = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nbox + 1));
    or_assign(psrc, ns, Lx, Ly, nx, ny, c->sperm, c->sstart);
    or_assign(ptar, nt, Lx, Ly, nx, ny, c->tperm, c->tstart);
    c->sp = (double *)malloc(sizeof(double) * 2 * (size_t)(ns > 0 ? ns : 1));
    c->tp = (double *)malloc(sizeof(double) * 2 * (size_t)(nt > 0 ? nt : 1));
    for (int64_t j = 0; j < ns; j++) {
        c->sp[2 * j] = psrc[2 * (int64_t)c->sperm[j]];
        c->sp[2 * j + 1] = psrc[2 * (int64_t)c->sperm[j] + 1];
    }
    for (int64_t j = 0; j < nt; j++) {
        c->tp[2 * j] = ptar[2 * (int64_t)c->tperm[j]];
        c->tp[2 * j + 1] = ptar[2 * (int64_t)c->tperm[j] + 1];
    }
}

static void or_cells_free(or_cells *c)
{
    free(c->sp); free(c->tp); free(c->sperm); free(c->tperm);
    free(c->sstart); free(c->tstart);
}

/* ------------------------------------------------------------------------ */
/* SLP real space: PE/src/mex/StokesSLP/mex_stokes_slp_real.cpp:58-357.     */
/* u(t) = 1/(4pi) sum_s [ E1(xi^2 r^2)/2 f + e^{-xi^2 r^2}((r.f)r/r^2 - f) ] */
/* with (-gamma/2 - 1 - log xi) f at r2 == 0 (:124, :161-163).              */
/* Written with the cross product q = dx f2 - dy f1:                        */
/*   u1 += E1/2 f1 + (e/r2) dy q,  u2 += E1/2 f2 - (e/r2) dx q.             */
/* ------------------------------------------------------------------------ */
void or_slp_real(const double *psrc, int64_t ns, const double *ptar, int64_t nt,
                 const double *f, double xi, int nx, int ny, double Lx, double Ly,
                 double *u)
{
    or_cells c;
    or_cells_build(&c, psrc, ns, ptar, nt, Lx, Ly, nx, ny);
    int64_t nbox = (int64_t)nx * ny;
    double *fs = (double *)malloc(sizeof(double) * 2 * (size_t)(ns > 0 ? ns : 1));
    for (int64_t j = 0; j < ns; j++) {
        fs[2 * j] = f[2 * (int64_t)c.sperm[j]];
        fs[2 * j + 1] = f[2 * (int64_t)c.sperm[j] + 1];
    }
    double *us = (double *)calloc(2 * (size_t)(nt > 0 ? nt : 1), sizeof(double));
    const double self = -1.288607832450766155 - log(xi);
    const double cut2 = Lx * Ly / nx / ny;

#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t b = 0; b < nbox; b++) {
        int32_t t0 = c.tstart[b], t1 = c.tstart[b + 1];
        if (t0 == t1) continue;
        int bx = (int)(b % nx), by = (int)(b / nx);
        for (int32_t t = t0; t < t1; t++) {
            double tx = c.tp[2 * t], ty = c.tp[2 * t + 1];
            double a1 = 0, a2 = 0;
            /* own box: every pair, no cutoff */
            for (int32_t s = c.sstart[b]; s < c.sstart[b + 1]; s++) {
                double dx = tx - c.sp[2 * s], dy = ty - c.sp[2 * s + 1];
                double r2 = dx * dx + dy * dy;
                double f1 = fs[2 * s], f2 = fs[2 * s + 1];
                if (r2 == 0) {
                    a1 += self * f1;
                    a2 += self * f2;
                    continue;
                }
                double e, E1 = or_e1(r2 * xi * xi, &e);
                double g = e / r2, q = dx * f2 - dy * f1;
                a1 += 0.5 * E1 * f1 + g * dy * q;
                a2 += 0.5 * E1 * f2 - g * dx * q;
            }
            for (int k = 0; k < 8; k++) {
                int ux = bx + NB_DX[k], uy = by + NB_DY[k];
                int wx = (ux + nx) % nx, wy = (uy + ny) % ny;
                int64_t sb = (int64_t)wy * nx + wx;
                if (c.sstart[sb] == c.sstart[sb + 1]) continue;
                double zx = (Lx * (ux - wx)) / nx, zy = (Ly * (uy - wy)) / ny;
                double qx = tx - zx, qy = ty - zy;
                for (int32_t s = c.sstart[sb]; s < c.sstart[sb + 1]; s++) {
                    double dx = c.sp[2 * s] - qx, dy = c.sp[2 * s + 1] - qy;
                    double r2 = dx * dx + dy * dy;
                    if (!(r2 < cut2)) continue;
                    double f1 = fs[2 * s], f2 = fs[2 * s + 1];
                    double e, E1 = or_e1(r2 * xi * xi, &e);
                    double g = e / r2, q = dx * f2 - dy * f1;
                    a1 += 0.5 * E1 * f1 + g * dy * q;
                    a2 += 0.5 * E1 * f2 - g * dx * q;
                }
            }
            us[2 * t] = a1;
            us[2 * t + 1] = a2;
        }
    }
    for (int64_t j = 0; j < nt; j++) {
        u[2 * (int64_t)c.tperm[j]] = us[2 * j] / (4 * OR_PI);
        u[2 * (int64_t)c.tperm[j] + 1] = us[2 * j + 1] / (4 * OR_PI);
    }
    free(us); free(fs);
    or_cells_free(&c);
}

/* ------------------------------------------------------------------------ */
/* DLP real space: PE/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:15-211.     */
/* S = f (x) n per source (:81-91); per pair (r = s - t, r2 != 0):          */
/*   T_ijk = e^{-xi^2 r2} [ -4(1+xi^2 r2)/r2^2 r_i r_j r_k                   */
/*                          + 2 xi^2 (delta_jk r_i + delta_ij r_k + ...) ]   */
/* contracted as u_i += T_i11 S11 + T_i12 (S12+S21) + T_i22 S22 (:125-138).  */
/* ------------------------------------------------------------------------ */
static inline void or_dlp_pair(double x1, double x2, double r2, double xi2,
                               const double *S, double *a1, double *a2)
{
    double e2 = exp(-xi2 * r2);
    double pf = 2 * xi2;
    double fb = -4 * (1 + xi2 * r2) / r2 / r2;
    double T111 = x1 * x1 * x1 * fb + pf * 3 * x1;
    double T112 = x1 * x1 * x2 * fb + pf * x2;
    double T122 = x1 * x2 * x2 * fb + pf * x1;
    double T211 = x2 * x1 * x1 * fb + pf * x2;
    double T212 = x2 * x1 * x2 * fb + pf * x1;
    double T222 = x2 * x2 * x2 * fb + pf * 3 * x2;
    *a1 += e2 * (T111 * S[0] + T112 * (S[1] + S[2]) + T122 * S[3]);
    *a2 += e2 * (T211 * S[0] + T212 * (S[1] + S[2]) + T222 * S[3]);
}

void or_dlp_real(const double *psrc, int64_t ns, const double *ptar, int64_t nt,
                 const double *f, const double *nrm, double xi, int nx, int ny,
                 double Lx, double Ly, double *u)
{
    or_cells c;
    or_cells_build(&c, psrc, ns, ptar, nt, Lx, Ly, nx, ny);
    int64_t nbox = (int64_t)nx * ny;
    double *S = (double *)malloc(sizeof(double) * 4 * (size_t)(ns > 0 ? ns : 1));
    for (int64_t j = 0; j < ns; j++) {
        int64_t o = c.sperm[j];
        S[4 * j] = f[2 * o] * nrm[2 * o];
        S[4 * j + 1] = f[2 * o] * nrm[2 * o + 1];
        S[4 * j + 2] = f[2 * o + 1] * nrm[2 * o];
        S[4 * j + 3] = f[2 * o + 1] * nrm[2 * o + 1];
    }
    double *us = (double *)calloc(2 * (size_t)(nt > 0 ? nt : 1), sizeof(double));
    const double cut2 = Lx * Ly / nx / ny;
    const double xi2 = xi * xi;

#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t b = 0; b < nbox; b++) {
        int32_t t0 = c.tstart[b], t1 = c.tstart[b + 1];
        if (t0 == t1) continue;
        int bx = (int)(b % nx), by = (int)(b / nx);
        for (int32_t t = t0; t < t1; t++) {
            double tx = c.tp[2 * t], ty = c.tp[2 * t + 1];
            double a1 = 0, a2 = 0;
            for (int32_t s = c.sstart[b]; s < c.sstart[b + 1]; s++) {
                double x1 = c.sp[2 * s] - tx, x2 = c.sp[2 * s + 1] - ty;
                double r2 = x1 * x1 + x2 * x2;
                if (r2 == 0) continue;
                or_dlp_pair(x1, x2, r2, xi2, S + 4 * s, &a1, &a2);
            }
            for (int k = 0; k < 8; k++) {
                int ux = bx + NB_DX[k], uy = by + NB_DY[k];
                int wx = (ux + nx) % nx, wy = (uy + ny) % ny;
                int64_t sb = (int64_t)wy * nx + wx;
                if (c.sstart[sb] == c.sstart[sb + 1]) continue;
                double zx = (Lx * (ux - wx)) / nx, zy = (Ly * (uy - wy)) / ny;
                for (int32_t s = c.sstart[sb]; s < c.sstart[sb + 1]; s++) {
                    double x1 = c.sp[2 * s] - tx + zx, x2 = c.sp[2 * s + 1] - ty + zy;
                    double r2 = x1 * x1 + x2 * x2;
                    if (!(r2 < cut2)) continue;
                    or_dlp_pair(x1, x2, r2, xi2, S + 4 * s, &a1, &a2);
                }
            }
            us[2 * t] = a1;
            us[2 * t + 1] = a2;
        }
    }
    for (int64_t j = 0; j < nt; j++) {
        u[2 * (int64_t)c.tperm[j]] = us[2 * j] / 4 / OR_PI;
        u[2 * (int64_t)c.tperm[j] + 1] = us[2 * j + 1] / 4 / OR_PI;
    }
    free(us); free(S);
    or_cells_free(&c);
}

/* ------------------------------------------------------------------------ */
/* Fast Gaussian gridding weights, shared by spread and gather:             */
/* PE/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:64-67 (e1 table) and      */
/* :86-99 (per-point factors), :104-129 (column/row recurrences).           */
/* Node (mx+i, my+j) of point (x,y) gets wx[i]*wy[j] with                    */
/*   wx[i] = ex*e4y*e1[i]*e3x^i   (ex includes py^2: the reference folds    */
/*   wy[j] = e1[j]*e3y^j           the y factor into the column product).   */
/* ------------------------------------------------------------------------ */
typedef struct {
    int mx, my;
    double wx[64], wy[64];
} or_stencil;

static void or_e1_table(double xi, double eta, double h, int P, double *e1)
{
    double a = -2 * xi * xi / eta * h * h;
    for (int j = -P / 2; j <= P / 2; j++) e1[j + P / 2] = exp(a * j * j);
}

static void or_weights(double x, double y, double xi, double eta, double Lx,
                       double Ly, double h, double w, int P, const double *e1,
                       or_stencil *st)
{
    double px, py;
    or_find_closest_node(x, y, Lx, Ly, h, P, &st->mx, &st->my, &px, &py);
    double a = -2 * xi * xi / eta;
    double ex = exp(a * (px * px + py * py + 2 * w * px));
    double e4y = exp(2 * a * w * py);
    double e3x = exp(-2 * a * h * px);
    double e3y = exp(-2 * a * h * py);
    for (int i = 0; i <= P; i++) {
        st->wx[i] = ex * e4y * e1[i];
        ex *= e3x;
    }
    double ey = 1.0;
    for (int j = 0; j <= P; j++) {
        st->wy[j] = ey * e1[j];
        ey *= e3y;
    }
}

/* ------------------------------------------------------------------------ */
/* Spread: SLP PE/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:64-130 with   */
/* H1 += W f1, H2 += W f2; DLP PE/src/mex/StokesDLP/mex_stokes_dlp_kspace.  */
/* cpp:79-150 with H1 += W n1 f1, H2 += W n2 f1, H3 += W n1 f2,             */
/* H4 += W n2 f2.  Grids are My x Mx column-major (y fastest).  ncomp = 2   */
/* (SLP, nrm == NULL) or 4 (DLP).  Column locks as in the reference         */
/* (:73-75, :107, :127).                                                    */
/* ------------------------------------------------------------------------ */
void or_spread(const double *psrc, int64_t ns, const double *f, const double *nrm,
               double xi, double eta, int Mx, int My, double Lx, double Ly,
               double w, int P, double *H)
{
    const double h = Lx / Mx;
    const int nc = nrm ? 4 : 2;
    const size_t G = (size_t)Mx * My;
    double e1[64];
    or_e1_table(xi, eta, h, P, e1);
    memset(H, 0, sizeof(double) * G * nc);
#ifdef _OPENMP
    omp_lock_t *locks = (omp_lock_t *)malloc(sizeof(omp_lock_t) * Mx);
    for (int j = 0; j < Mx; j++) omp_init_lock(&locks[j]);
#endif
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < ns; k++) {
        or_stencil st;
        or_weights(psrc[2 * k], psrc[2 * k + 1], xi, eta, Lx, Ly, h, w, P, e1, &st);
        double c[4];
        if (nc == 2) {
            c[0] = f[2 * k]; c[1] = f[2 * k + 1];
        }
        for (int i = 0; i <= P; i++) {
            int col = (i + st.mx + Mx) % Mx;
            double *Hc = H + (size_t)col * My;
#ifdef _OPENMP
            omp_set_lock(&locks[col]);
#endif
            for (int j = 0; j <= P; j++) {
                int row = (j + st.my + My) % My;
                double W = st.wx[i] * st.wy[j];
                if (nc == 2) {
                    Hc[row] += W * c[0];
                    Hc[G + row] += W * c[1];
                } else {
                    double n1 = nrm[2 * k], n2 = nrm[2 * k + 1];
                    double f1 = f[2 * k], f2 = f[2 * k + 1];
                    Hc[row] += W * n1 * f1;
                    Hc[G + row] += W * n2 * f1;
                    Hc[2 * G + row] += W * n1 * f2;
                    Hc[3 * G + row] += W * n2 * f2;
                }
            }
#ifdef _OPENMP
            omp_unset_lock(&locks[col]);
#endif
        }
    }
#ifdef _OPENMP
    for (int j = 0; j < Mx; j++) omp_destroy_lock(&locks[j]);
    free(locks);
#endif
}

/* ------------------------------------------------------------------------ */
/* k-space filters on full complex spectra (split re/im, My x Mx col-major).*/
/* Frequency of column j: 2pi/Lx * (j <= Mx/2 ? j : j - Mx); of row k:      */
/* 2pi/Ly * (k <= My/2 ? k : k - My) (the reference's split loops).  The    */
/* zero mode is set to 0.                                                   */
/* SLP: PE/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:189-229.             */
/* DLP: PE/src/mex/StokesDLP/mex_stokes_dlp_kspace.cpp:219-285 (H2 and H3   */
/* enter only as H2+H3).                                                    */
/* ------------------------------------------------------------------------ */
static inline double or_kfreq(int j, int M, double L)
{
    return 2.0 * OR_PI / L * (j <= M / 2 ? j : j - M);
}

void or_slp_filter(double *re, double *im, int Mx, int My, double Lx, double Ly,
                   double xi, double eta)
{
    const size_t G = (size_t)Mx * My;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Mx; j++) {
        double k1 = or_kfreq(j, Mx, Lx);
        for (int k = 0; k < My; k++) {
            size_t o = (size_t)j * My + k;
            double k2 = or_kfreq(k, My, Ly);
            double K2 = k1 * k1 + k2 * k2;
            double e = (1.0 / (K2 * K2) + 0.25 / (K2 * xi * xi)) *
                       exp(-0.25 * (1 - eta) / (xi * xi) * K2);
            double *A[2] = {re, im};
            for (int p = 0; p < 2; p++) {
                double h1 = A[p][o], h2 = A[p][G + o];
                A[p][o] = k2 * (k2 * h1 - k1 * h2) * e;
                A[p][G + o] = k1 * (k1 * h2 - k2 * h1) * e;
            }
        }
    }
    re[0] = re[G] = im[0] = im[G] = 0;
}

void or_dlp_filter(double *re, double *im, int Mx, int My, double Lx, double Ly,
                   double xi, double eta)
{
    const size_t G = (size_t)Mx * My;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Mx; j++) {
        double k1 = or_kfreq(j, Mx, Lx);
        for (int k = 0; k < My; k++) {
            size_t o = (size_t)j * My + k;
            double k2 = or_kfreq(k, My, Ly);
            double K2 = k1 * k1 + k2 * k2;
            double e = exp(-0.25 * (1 - eta) / (xi * xi) * K2) / K2 / K2;
            double t = 1 + 0.25 * K2 / xi / xi;
            double B111 = 3.0 * k1 * K2 - 2.0 * k1 * k1 * k1;
            double B112 = k2 * K2 - 2.0 * k1 * k1 * k2;
            double B122 = k1 * K2 - 2.0 * k1 * k2 * k2;
            double B211 = k2 * K2 - 2.0 * k2 * k1 * k1;
            double B212 = k1 * K2 - 2.0 * k2 * k1 * k2;
            double B222 = 3.0 * k2 * K2 - 2.0 * k2 * k2 * k2;
            double *A[2] = {re, im};
            for (int p = 0; p < 2; p++) {
                double h1 = A[p][o], h23 = A[p][G + o] + A[p][2 * G + o],
                       h4 = A[p][3 * G + o];
                A[p][o] = e * t * (B111 * h1 + B112 * h23 + B122 * h4);
                A[p][G + o] = e * t * (B211 * h1 + B212 * h23 + B222 * h4);
            }
        }
    }
    re[0] = re[G] = im[0] = im[G] = 0;
}

/* ------------------------------------------------------------------------ */
/* Gather: PE/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:264-329 (same in  */
/* PE/src/mex/StokesDLP/mex_stokes_dlp_kspace.cpp:334-400):                 */
/* u_c(t) = s * sum_nodes W * Ht_c, s = (4 xi^2/eta)^2 h^2/pi/(4 pi).       */
/* ------------------------------------------------------------------------ */
void or_gather(const double *ptar, int64_t nt, const double *Ht, double xi,
               double eta, int Mx, int My, double Lx, double Ly, double w, int P,
               double *u)
{
    const double h = Lx / Mx;
    const size_t G = (size_t)Mx * My;
    double e1[64];
    or_e1_table(xi, eta, h, P, e1);
    double s = 4 * xi * xi / eta;
    s = s * s * h * h / OR_PI;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < nt; k++) {
        or_stencil st;
        or_weights(ptar[2 * k], ptar[2 * k + 1], xi, eta, Lx, Ly, h, w, P, e1, &st);
        double a1 = 0, a2 = 0;
        for (int i = 0; i <= P; i++) {
            const double *Hc = Ht + (size_t)((i + st.mx + Mx) % Mx) * My;
            for (int j = 0; j <= P; j++) {
                int row = (j + st.my + My) % My;
                double W = st.wx[i] * st.wy[j];
                a1 += W * Hc[row];
                a2 += W * Hc[G + row];
            }
        }
        u[2 * k] = a1 * (s / (4 * OR_PI));
        u[2 * k + 1] = a2 * (s / (4 * OR_PI));
    }
}

/* Thread count used by the OpenMP loops (for reporting). */
int or_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
