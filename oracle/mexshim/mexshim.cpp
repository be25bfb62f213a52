// mexshim.cpp -- implementation of the mex.h stand-in (test infrastructure).
#include "mex.h"
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>

struct mxArray_tag {
    size_t m, n;
    double *pr, *pi;
};

// fft callback: inverse=0 -> fft2, 1 -> ifft2 (with 1/(m n)).  im may be NULL.
typedef int (*shim_fft_cb)(int inverse, size_t m, size_t n, const double *re,
                           const double *im, double *out_re, double *out_im);
static shim_fft_cb g_fft = nullptr;

// Functions registered with mexAtExit; shim_run_atexit plays MATLAB's
// "clear mex" and runs them once.
static void (*g_atexit[16])(void);
static int g_natexit = 0;

namespace {
struct MexError : std::runtime_error {
    explicit MexError(const char *m) : std::runtime_error(m) {}
};
}

extern "C" {
double *mxGetPr(const mxArray *a) { return a->pr; }
double *mxGetPi(const mxArray *a) { return a->pi; }
void mxSetPi(mxArray *a, double *pi) { a->pi = pi; }
size_t mxGetM(const mxArray *a) { return a->m; }
size_t mxGetN(const mxArray *a) { return a->n; }
double mxGetScalar(const mxArray *a) { return a->pr[0]; }
mxArray *mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity c)
{
    mxArray *a = new mxArray_tag;
    a->m = m; a->n = n;
    a->pr = static_cast<double *>(calloc(m * n + 1, sizeof(double)));
    a->pi = c == mxCOMPLEX ? static_cast<double *>(calloc(m * n + 1, sizeof(double))) : nullptr;
    return a;
}
void mxDestroyArray(mxArray *a)
{
    if (!a) return;
    free(a->pr);
    free(a->pi);
    delete a;
}
void *mxMalloc(size_t n) { return malloc(n ? n : 1); }
void *mxCalloc(size_t n, size_t size) { return calloc(n ? n : 1, size ? size : 1); }
void mxFree(void *p) { free(p); }
void mexErrMsgTxt(const char *msg) { throw MexError(msg); }
int mexPrintf(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    int r = vprintf(fmt, ap);
    va_end(ap);
    return r;
}
int mexCallMATLAB(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *name)
{
    if (nlhs != 1 || nrhs != 1) throw MexError("mexshim: only 1-in/1-out calls");
    int inv;
    if (!strcmp(name, "fft2")) inv = 0;
    else if (!strcmp(name, "ifft2")) inv = 1;
    else throw MexError("mexshim: unsupported mexCallMATLAB target");
    if (!g_fft) throw MexError("mexshim: no fft callback registered");
    const mxArray *x = prhs[0];
    mxArray *y = mxCreateDoubleMatrix(x->m, x->n, mxCOMPLEX);
    if (g_fft(inv, x->m, x->n, x->pr, x->pi, y->pr, y->pi) != 0) {
        mxDestroyArray(y);
        throw MexError("mexshim: fft callback failed");
    }
    plhs[0] = y;
    return 0;
}

int mexAtExit(void (*fn)(void))
{
    for (int i = 0; i < g_natexit; ++i)
        if (g_atexit[i] == fn) return 0;
    if (g_natexit == 16) return 1;
    g_atexit[g_natexit++] = fn;
    return 0;
}

// ---- loader-facing helpers ----------------------------------------------
void shim_set_fft(shim_fft_cb cb) { g_fft = cb; }

void shim_run_atexit(void)
{
    while (g_natexit > 0) g_atexit[--g_natexit]();
}

typedef void (*mexfn_t)(int, mxArray **, int, const mxArray **);

// Calls a MEX gateway; returns 0 or 1 with the error text in err.
int shim_call(void *fn, int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs,
              char *err, size_t errlen)
{
    try {
        reinterpret_cast<mexfn_t>(fn)(nlhs, plhs, nrhs, prhs);
    } catch (const std::exception &e) {
        snprintf(err, errlen, "%s", e.what());
        return 1;
    }
    return 0;
}
}
