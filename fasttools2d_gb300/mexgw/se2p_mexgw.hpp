// se2p_mexgw.hpp -- shared part of the four MATLAB MEX gateways that route
// FastTools2D's spectral-Ewald calls to libse2p (the GPU).
//
// Built against MATLAB's mex.h they replace the CPU gateways of
// PeriodicEwald/src/mex/Stokes{SLP,DLP}/ one for one: same names, same
// argument order, plhs[0] a new 2 x Ntar double matrix.  All four make the
// argument-count and 2xN checks of the DLP gateways, with their messages
// (mex_stokes_dlp_real.cpp:20-34); the reference's SLP gateways check less
// (slp_kspace only the shapes, slp_real nothing).  Arrays are ordinary host
// mxArrays; libse2p stages them to the GPU and back.
#pragma once
#include <cstdio>

#include "mex.h"
#include "se2p.h"

namespace se2p_mexgw {

// One plan per MATLAB session (stream, workspace, cuFFT plans), released at exit.
inline se2p_plan &plan_ref()
{
    static se2p_plan p = nullptr;
    return p;
}

inline void release_plan() { se2p_plan_destroy(plan_ref()); plan_ref() = nullptr; }

inline se2p_plan plan()
{
    se2p_plan &p = plan_ref();
    if (!p) {
        if (se2p_plan_create(&p, 0) != SE2P_OK) mexErrMsgTxt("se2p: no CUDA device");
        mexAtExit(release_plan);
    }
    return p;
}

inline void need_2xn(const mxArray *a, const char *msg)
{
    if (mxGetM(a) != 2) mexErrMsgTxt(msg);
}

inline void check(int rc)
{
    if (rc != SE2P_OK) mexErrMsgTxt(se2p_plan_last_error(plan()));
}

inline int as_int(const mxArray *a) { return static_cast<int>(mxGetScalar(a)); }

}  // namespace se2p_mexgw
