// mex_stokes_dlp_kspace(psrc, ptar, xi, eta, f, n, Mx, My, Lx, Ly, w, P) on the GPU
// (replaces PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_kspace.cpp).
#include "se2p_mexgw.hpp"
using namespace se2p_mexgw;

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if (nrhs != 12) mexErrMsgTxt("Incorrect number of input parameters");
    need_2xn(prhs[0], "psrc must be a 2xn matrix.");
    need_2xn(prhs[1], "ptar must be a 2xn matrix.");
    need_2xn(prhs[4], "f must be a 2xn matrix.");
    need_2xn(prhs[5], "n must be a 2xn matrix.");
    if (mxGetN(prhs[4]) != mxGetN(prhs[0])) mexErrMsgTxt("psrc and f must be the same size.");
    if (mxGetN(prhs[5]) != mxGetN(prhs[0])) mexErrMsgTxt("psrc and n must be the same size.");
    const mwSize ns = mxGetN(prhs[0]), nt = mxGetN(prhs[1]);
    plhs[0] = mxCreateDoubleMatrix(2, nt, mxREAL);
    check(se2p_dlp_kspace(plan(), mxGetPr(prhs[0]), (int64_t)ns, mxGetPr(prhs[1]), (int64_t)nt,
                          mxGetScalar(prhs[2]), mxGetScalar(prhs[3]), mxGetPr(prhs[4]),
                          mxGetPr(prhs[5]), as_int(prhs[6]), as_int(prhs[7]),
                          mxGetScalar(prhs[8]), mxGetScalar(prhs[9]), mxGetScalar(prhs[10]),
                          as_int(prhs[11]), mxGetPr(plhs[0])));
}
