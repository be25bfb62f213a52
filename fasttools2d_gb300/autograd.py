"""torch.autograd binding of the SLP+DLP spectral-Ewald evaluation.

A thin ``torch.autograd.Function`` over se2p_stokes_ewald (forward) and
se2p_stokes_ewald_adjoint (backward), used to check the hand-written adjoint
kernels against finite differences.  Tensors are (N, 2) float64 on the GPU;
gradients flow to the source positions, SLP forces, DLP densities and normals.
The target positions take no gradient: a ptar that requires one (for
instance the source positions passed again as targets, the usual
boundary-integral self-evaluation) raises, since its part of the gradient
would otherwise be missing without notice.
"""
from __future__ import annotations

import torch

from .ewald import EwaldParams, stokes_ewald, stokes_ewald_adjoint


class StokesEwald(torch.autograd.Function):
    @staticmethod
    def forward(ctx, psrc, ptar, f_slp, f_dlp, n, prm: EwaldParams, plan):
        if ctx.needs_input_grad[1]:
            raise NotImplementedError(
                "stokes_ewald_torch: gradients with respect to the target positions are not "
                "implemented; pass ptar.detach() (when ptar is psrc, the gradient would lack "
                "the target-position part)")
        u_slp, u_dlp = stokes_ewald(psrc, ptar, f_slp, f_dlp, n, prm, plan=plan)
        ctx.save_for_backward(psrc, ptar, f_slp, f_dlp, n)
        ctx.prm, ctx.plan = prm, plan
        return u_slp, u_dlp

    @staticmethod
    def backward(ctx, gu_slp, gu_dlp):
        psrc, ptar, f_slp, f_dlp, n = ctx.saved_tensors
        if gu_slp is None:
            gu_slp = torch.zeros_like(ptar)
        if gu_dlp is None:
            gu_dlp = torch.zeros_like(ptar)
        gp, gfs, gfd, gn = stokes_ewald_adjoint(psrc, ptar, f_slp, f_dlp, n,
                                                gu_slp.contiguous(), gu_dlp.contiguous(),
                                                ctx.prm, plan=ctx.plan)
        return gp, None, gfs, gfd, gn, None, None


def stokes_ewald_torch(psrc, ptar, f_slp, f_dlp, n, prm: EwaldParams, plan=None):
    """(u_slp, u_dlp) = SE Stokeslet and stresslet sums, differentiable in
    psrc, f_slp, f_dlp and n."""
    return StokesEwald.apply(psrc, ptar, f_slp, f_dlp, n, prm, plan)
