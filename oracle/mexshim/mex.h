/*
 * mex.h -- minimal stand-in for MATLAB's MEX/MX API (test infrastructure).
 *
 * Lets the FastTools2D spectral-Ewald MEX sources compile unchanged into
 * shared objects under oracle/_ref/, so the reference itself can pin the
 * oracle.  Arrays are column-major doubles with separate real/imaginary
 * buffers (the R2017b "separate complex" layout the sources use).  fft2 and
 * ifft2 reached through mexCallMATLAB are served by a callback that the
 * Python loader registers (oracle/ref_mex.py).  mexErrMsgTxt throws; the
 * loader's entry point catches it and returns the message.
 */
#ifndef SE2P_MEXSHIM_MEX_H
#define SE2P_MEXSHIM_MEX_H
#include <stddef.h>

typedef size_t mwSize;
typedef struct mxArray_tag mxArray;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

#ifdef __cplusplus
extern "C" {
#endif
double *mxGetPr(const mxArray *a);
double *mxGetPi(const mxArray *a);
void mxSetPi(mxArray *a, double *pi);
size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
double mxGetScalar(const mxArray *a);
mxArray *mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity c);
void mxDestroyArray(mxArray *a);
void *mxMalloc(size_t n);
void *mxCalloc(size_t n, size_t size);
void mxFree(void *p);
void mexErrMsgTxt(const char *msg);
int mexPrintf(const char *fmt, ...);
int mexCallMATLAB(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *name);
int mexAtExit(void (*fn)(void));
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
#ifdef __cplusplus
}
#endif
#endif
