// mex_stokes_dlp_real(psrc, ptar, f, n, xi, nside_x, nside_y, Lx, Ly) on the GPU
// (replaces PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_real.cpp).
#include "se2p_mexgw.hpp"
using namespace se2p_mexgw;

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if (nrhs != 9) mexErrMsgTxt("Incorrect number of input parameters");
    need_2xn(prhs[0], "psrc must be a 2xn matrix.");
    need_2xn(prhs[1], "ptar must be a 2xn matrix.");
    need_2xn(prhs[2], "f must be a 2xn matrix.");
    need_2xn(prhs[3], "n must be a 2xn matrix.");
    if (mxGetN(prhs[2]) != mxGetN(prhs[0])) mexErrMsgTxt("psrc and f must be the same size.");
    if (mxGetN(prhs[3]) != mxGetN(prhs[0])) mexErrMsgTxt("psrc and n must be the same size.");
    const mwSize ns = mxGetN(prhs[0]), nt = mxGetN(prhs[1]);
    plhs[0] = mxCreateDoubleMatrix(2, nt, mxREAL);
    check(se2p_dlp_real(plan(), mxGetPr(prhs[0]), (int64_t)ns, mxGetPr(prhs[1]), (int64_t)nt,
                        mxGetPr(prhs[2]), mxGetPr(prhs[3]), mxGetScalar(prhs[4]), as_int(prhs[5]),
                        as_int(prhs[6]), mxGetScalar(prhs[7]), mxGetScalar(prhs[8]),
                        mxGetPr(plhs[0])));
}
