"""Derivatives of ln|psi| with respect to the variational parameters, on the GPU.

``dlnpsi_dparams(walkers)`` returns, per walker, the blocks the reference collects
from ``grad(evaluate_ln_wavefunction)`` for stochastic reconfiguration
(jqmc/jqmc_mcmc.py:856-876; names and shapes of wavefunction.py:515-676,
jastrow_factor.py:2110-2124, determinant.py:389-399):

  "j1_param" (W,), "j2_param" (W,), "j3_matrix" (W, A3, A3+1), "lambda_matrix" (W, *lambda.shape)

computed by the adjoint kernel ``jqmc_dlnpsi_dparam`` (FP64, AO tables recomputed
from the positions).  A geminal written in an MO basis gets its lambda block
mapped from the AO basis of the walker tables: d/d lambda_MO = C_up D_AO C_dn^T.

``LnPsi`` wraps ln|psi| = ln|det G| + J as a ``torch.autograd.Function`` whose
backward is that kernel: ``ln_psi(walkers, params)`` returns a (W,) tensor whose
``.backward()`` fills ``params[k].grad`` with sum_w g_w d ln psi_w / d theta_k.
The parameter values are those the ``GpuSystem`` was built with; the tensors in
``params`` only carry the gradients.
"""

from __future__ import annotations

import numpy as np
import torch

BLOCKS = ("j1_param", "j2_param", "j3_matrix", "lambda_matrix")


def _mo_maps(walkers):
    g = walkers.sys.ham.wavefunction_data.geminal_data
    up, dn = g.orb_data_up_spin, g.orb_data_dn_spin
    if hasattr(up, "mo_coefficients"):
        dev = walkers.sys.device
        return (torch.as_tensor(np.asarray(up.mo_coefficients), dtype=torch.float64, device=dev),
                torch.as_tensor(np.asarray(dn.mo_coefficients), dtype=torch.float64, device=dev))
    return None


def dlnpsi_dparams(walkers, lam: bool = True) -> dict:
    """Per-walker derivative blocks of ln|psi| (FP64 walkers, current positions)."""
    if walkers.precision != "fp64":
        raise ValueError("parameter derivatives are computed on FP64 walkers")
    ham = walkers.sys.ham
    jd = ham.wavefunction_data.jastrow_data
    j1, j2, j3, dl = walkers.dlnpsi_dparam(lam=lam)
    out = {}
    if jd.jastrow_one_body_data is not None:
        out["j1_param"] = j1
    if jd.jastrow_two_body_data is not None:
        out["j2_param"] = j2
    if j3 is not None:
        out["j3_matrix"] = j3
    if dl is not None:
        maps = _mo_maps(walkers)
        if maps is not None:
            cu, cd = maps
            dl = torch.einsum("pa,wab,qb->wpq", cu, dl, cd)
        out["lambda_matrix"] = dl
    return out


class LnPsi(torch.autograd.Function):
    """ln|psi| per walker with the adjoint kernel as its backward."""

    @staticmethod
    def forward(ctx, walkers, *params):
        ld, _, jj = walkers.log_psi()
        ctx.walkers = walkers
        ctx.names = walkers._grad_names
        return ld + jj

    @staticmethod
    def backward(ctx, g):
        blocks = dlnpsi_dparams(ctx.walkers, lam="lambda_matrix" in ctx.names)
        grads = []
        for name in ctx.names:
            d = blocks[name]
            grads.append(torch.einsum("w,w...->...", g, d))
        return (None, *grads)


def ln_psi(walkers, params: dict) -> torch.Tensor:
    """ln|psi| (W,) differentiable with respect to the tensors in ``params``
    (keys among BLOCKS, shapes of one walker's block)."""
    names = [k for k in BLOCKS if k in params]
    walkers._grad_names = names
    return LnPsi.apply(walkers, *[params[k] for k in names])
