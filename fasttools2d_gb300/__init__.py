"""fasttools2d_gb300 -- doubly-periodic spectral Ewald summation of the 2D
Stokeslet (SLP) and stresslet (DLP) on NVIDIA GB300 (sm_103a).

A drop-in for the spectral-Ewald path of FastTools2D (PeriodicEwald): the
four MEX gateways (``mex``), the two MATLAB drivers (``ewald``), and the C
ABI underneath (``include/se2p.h``, ``libse2p.so``).
"""
from ._lib import Plan, Se2pError, default_plan, load  # noqa: F401
from .ewald import (EwaldParams, Geometry, StokesDLP_ewald_2p, StokesSLP_ewald_2p,  # noqa: F401
                    dlp_ewald, select_params, slp_ewald, stokes_ewald, stokes_ewald_adjoint)
from .mex import (mex_stokes_dlp_kspace, mex_stokes_dlp_real,  # noqa: F401
                  mex_stokes_slp_kspace, mex_stokes_slp_real)

__version__ = "0.1.0"
