"""Variational parameter blocks and the stochastic-reconfiguration (SR) step.

* ``VariationalParameterBlock``, ``get_variational_blocks`` and
  ``apply_block_updates`` follow jqmc/wavefunction.py:112-245 (blocks and their
  symmetry callbacks), :292-342 (block updates) and :515-676 (block list), with
  the parameter rules of jastrow_factor.py:1965-2060 and determinant.py:260-380:
  a J3 matrix whose square part (all columns but the last) is symmetric keeps it
  symmetric, and so does a symmetric lambda (its paired block when rectangular).
* ``sr_direction`` is the SR solve of jqmc_mcmc.py:2960-3345 (one process): the
  weighted, centred derivative samples X and the energy column F, the diagonal
  of S for normalisation and freezing, then (S + eps diag S)^-1 f through the
  primal K x K system when there are fewer parameters K than samples, else the
  dual samples x samples system, each either by a direct solve or by conjugate
  gradients (jqmc_mcmc.py:2564-2610).  The reductions (X^T X, X X^T, X^T F, the
  CG matrix-vector products) run where the samples are, the GPU in the driver.
"""

from __future__ import annotations

import dataclasses
from dataclasses import dataclass
from typing import Callable

import numpy as np
import torch

# jqmc/_setting.py:74-75, :149
ATOL_CONSISTENCY = 1.0e-8
RTOL_CONSISTENCY = 1.0e-6
MIN_S_DIAG_ABS = 1.0e-10


@dataclass(frozen=True)
class VariationalParameterBlock:
    """One contiguous slice of the parameter vector (wavefunction.py:112-170)."""

    name: str
    values: np.ndarray
    shape: tuple
    size: int
    symmetrize_metric: Callable | None = None

    def apply_update(self, delta_flat: np.ndarray, learning_rate: float) -> "VariationalParameterBlock":
        """values + learning_rate * delta, reshaped to the block's shape."""
        new = np.asarray(self.values, dtype=np.float64).reshape(-1) + learning_rate * np.asarray(delta_flat, np.float64)
        return dataclasses.replace(self, values=new.reshape(self.shape))


def _j3_is_symmetric(j_matrix: np.ndarray) -> bool:
    sq = np.asarray(j_matrix)[:, :-1]
    return sq.ndim == 2 and sq.shape[0] == sq.shape[1] and sq.shape[1] >= 1 and np.allclose(sq, sq.T, atol=ATOL_CONSISTENCY)


def _lambda_paired_columns(lam: np.ndarray) -> int:
    """Columns of the symmetric paired block of lambda, 0 when it is not symmetric."""
    lam = np.asarray(lam)
    if lam.ndim != 2:
        return 0
    n = lam.shape[0]
    paired = lam[:, :n]
    if paired.shape[1] == n and np.allclose(paired, paired.T, atol=ATOL_CONSISTENCY, rtol=RTOL_CONSISTENCY):
        return n
    return 0


def _symmetrize_leading_square(shape: tuple, ncols: int) -> Callable:
    """flat (size,) or (batch, size) -> the same with its leading ncols x ncols
    block replaced by (B + B^T)/2; the identity when ncols is 0."""

    def sym(arr):
        if ncols == 0:
            return arr
        a = np.array(arr, dtype=np.float64)
        batch = a.reshape((-1,) + tuple(shape))
        sq = batch[:, :, :ncols]
        batch[:, :, :ncols] = 0.5 * (sq + np.swapaxes(sq, -1, -2))
        return batch.reshape(a.shape)

    return sym


def get_variational_blocks(wavefunction_data, opt_J1_param: bool = True, opt_J2_param: bool = True,
                           opt_J3_param: bool = True, opt_JNN_param: bool = True, opt_lambda_param: bool = False,
                           opt_J3_basis_exp: bool = False, opt_J3_basis_coeff: bool = False,
                           opt_lambda_basis_exp: bool = False, opt_lambda_basis_coeff: bool = False) -> list:
    """Blocks j1_param, j2_param, j3_matrix, lambda_matrix in the reference's order
    (wavefunction.py:515-676).  AO-basis exponents and coefficients are not
    variational on the walker path; asking for them raises."""
    if opt_J3_basis_exp or opt_J3_basis_coeff or opt_lambda_basis_exp or opt_lambda_basis_coeff:
        raise NotImplementedError("AO-basis exponents and coefficients are not variational on the walker path")
    blocks = []
    jd = wavefunction_data.jastrow_data
    if jd is not None:
        if opt_J1_param and jd.jastrow_one_body_data is not None:
            v = np.asarray(jd.jastrow_one_body_data.jastrow_1b_param, dtype=np.float64)
            blocks.append(VariationalParameterBlock("j1_param", v, (), 1))
        if opt_J2_param and jd.jastrow_two_body_data is not None:
            v = np.asarray(jd.jastrow_two_body_data.jastrow_2b_param, dtype=np.float64)
            blocks.append(VariationalParameterBlock("j2_param", v, (), 1))
        if opt_J3_param and jd.jastrow_three_body_data is not None:
            v = np.asarray(jd.jastrow_three_body_data.j_matrix, dtype=np.float64)
            ncols = v.shape[1] - 1 if _j3_is_symmetric(v) else 0
            blocks.append(VariationalParameterBlock("j3_matrix", v, v.shape, v.size, _symmetrize_leading_square(v.shape, ncols)))
    if opt_lambda_param:
        v = np.asarray(wavefunction_data.geminal_data.lambda_matrix, dtype=np.float64)
        blocks.append(VariationalParameterBlock("lambda_matrix", v, v.shape, v.size,
                                                _symmetrize_leading_square(v.shape, _lambda_paired_columns(v))))
    return blocks


def apply_block_updates(wavefunction_data, blocks: list, thetas: np.ndarray, learning_rate: float):
    """A new Wavefunction_data with each block moved by learning_rate * its slice of
    thetas; blocks whose slice is all zero are left alone (wavefunction.py:292-342)."""
    jd, gd = wavefunction_data.jastrow_data, wavefunction_data.geminal_data
    thetas = np.asarray(thetas, dtype=np.float64)
    if thetas.shape != (sum(b.size for b in blocks),):
        raise ValueError(f"thetas has shape {thetas.shape}; the blocks hold {sum(b.size for b in blocks)} parameters")
    pos = 0
    for b in blocks:
        delta = thetas[pos:pos + b.size]
        pos += b.size
        if not np.any(delta):
            continue
        new = b.apply_update(delta, learning_rate).values
        if b.name == "j1_param":
            jd = dataclasses.replace(jd, jastrow_one_body_data=dataclasses.replace(jd.jastrow_one_body_data,
                                                                                   jastrow_1b_param=float(new)))
        elif b.name == "j2_param":
            jd = dataclasses.replace(jd, jastrow_two_body_data=dataclasses.replace(jd.jastrow_two_body_data,
                                                                                   jastrow_2b_param=float(new)))
        elif b.name == "j3_matrix":
            j3 = jd.jastrow_three_body_data
            ncols = j3.j_matrix.shape[1] - 1 if _j3_is_symmetric(j3.j_matrix) else 0
            new = _symmetrize_leading_square(new.shape, ncols)(new)
            jd = dataclasses.replace(jd, jastrow_three_body_data=dataclasses.replace(j3, j_matrix=new))
        elif b.name == "lambda_matrix":
            new = _symmetrize_leading_square(new.shape, _lambda_paired_columns(gd.lambda_matrix))(new)
            gd = dataclasses.replace(gd, lambda_matrix=new)
        else:
            raise ValueError(f"unknown variational block {b.name!r}")
    return dataclasses.replace(wavefunction_data, jastrow_data=jd, geminal_data=gd)


# ---------------------------------------------------------------- SR
def conjugate_gradient(b: torch.Tensor, apply_A: Callable, x0: torch.Tensor, max_iter: int, tol: float):
    """(x, |r|, iterations) of plain CG on A x = b, stopping when |r| <= tol or on
    a vanishing p^T A p (jqmc_mcmc.py:2564-2610)."""
    x = x0.clone()
    r = b - apply_A(x)
    p = r.clone()
    rs_old = float(r @ r)
    if not np.isfinite(rs_old):
        raise FloatingPointError("non-finite initial residual in SR-CG")
    if np.sqrt(rs_old) <= tol:
        return x, np.sqrt(rs_old), 0
    tiny = np.finfo(np.float64).tiny
    it = 0
    for i in range(int(max_iter)):
        Ap = apply_A(p)
        denom = float(p @ Ap)
        if not np.isfinite(denom) or abs(denom) <= tiny:
            break
        alpha = rs_old / denom
        x = x + alpha * p
        r = r - alpha * Ap
        rs_new = float(r @ r)
        it = i + 1
        if not np.isfinite(rs_new):
            raise FloatingPointError("non-finite residual in SR-CG")
        if np.sqrt(rs_new) <= tol:
            rs_old = rs_new
            break
        p = r + (rs_new / rs_old) * p
        rs_old = rs_new
    return x, np.sqrt(rs_old), it


@dataclass
class SRResult:
    theta: np.ndarray          # (K,) update direction, frozen entries 0
    f: np.ndarray              # (K,) generalized force -2 cov_w(O, e_L)
    diag_S: np.ndarray         # (K,) diagonal of S after the floor
    frozen: np.ndarray         # (K,) bool, diag S <= MIN_S_DIAG_ABS or non-finite
    e_L_bar: float
    cg_iterations: int
    cg_residual: float
    warm_start: torch.Tensor | None   # CG solution to start the next step from


def sr_direction(O, e_L, w_L, epsilon: float, cg_flag: bool = True, cg_max_iter: int = 10**6, cg_tol: float = 1.0e-8,
                 warm_start: torch.Tensor | None = None, device=None) -> SRResult:
    """theta = (S + epsilon diag S)^-1 f from samples O (..., K), e_L (...), w_L (...)
    (jqmc_mcmc.py:2960-3345 on one process)."""
    dev = torch.device(device) if device is not None else (O.device if isinstance(O, torch.Tensor) else torch.device("cpu"))
    O = torch.as_tensor(O, dtype=torch.float64, device=dev)
    K = O.shape[-1]
    O = O.reshape(-1, K)
    e = torch.as_tensor(e_L, dtype=torch.float64, device=dev).reshape(-1)
    w = torch.as_tensor(w_L, dtype=torch.float64, device=dev).reshape(-1)
    if e.shape[0] != O.shape[0] or w.shape[0] != O.shape[0]:
        raise ValueError(f"{O.shape[0]} derivative samples but {e.shape[0]} energies and {w.shape[0]} weights")
    Wt = w.sum()
    O_bar = (w @ O) / Wt
    e_bar = (w @ e) / Wt
    sw = torch.sqrt(w / Wt)
    X = (O - O_bar) * sw[:, None]                 # (samples, K): the reference's X_local^T
    F = -2.0 * sw * (e - e_bar)                   # (samples,)
    f = X.T @ F
    diag_S = (X * X).sum(dim=0)
    frozen = ~(torch.isfinite(diag_S) & (diag_S > MIN_S_DIAG_ABS))
    diag_S = torch.where(frozen, torch.full_like(diag_S, MIN_S_DIAG_ABS), diag_S)
    Xn = X / torch.sqrt(diag_S)
    S_count = Xn.shape[0]
    iters, res, ws = 0, 0.0, None
    if K < S_count:
        b = Xn.T @ F
        if not cg_flag:
            A = Xn.T @ Xn
            A.diagonal().add_(epsilon)
            th = torch.linalg.solve(A, b)
        else:
            x0 = warm_start if warm_start is not None and warm_start.shape == b.shape else torch.zeros_like(b)
            th, res, iters = conjugate_gradient(b, lambda v: Xn.T @ (Xn @ v) + epsilon * v, x0.to(dev), cg_max_iter, cg_tol)
            ws = th.clone()
    else:
        if not cg_flag:
            A = Xn @ Xn.T
            A.diagonal().add_(epsilon)
            th = Xn.T @ torch.linalg.solve(A, F)
        else:
            x0 = warm_start if warm_start is not None and warm_start.shape == F.shape else torch.zeros_like(F)
            y, res, iters = conjugate_gradient(F, lambda v: Xn @ (Xn.T @ v) + epsilon * v, x0.to(dev), cg_max_iter, cg_tol)
            th = Xn.T @ y
            ws = y.clone()
    theta = th / torch.sqrt(diag_S)
    theta = torch.where(frozen, torch.zeros_like(theta), theta)
    theta = torch.where(torch.isfinite(theta), theta, torch.zeros_like(theta))
    return SRResult(theta=theta.cpu().numpy(), f=f.cpu().numpy(), diag_S=diag_S.cpu().numpy(), frozen=frozen.cpu().numpy(),
                    e_L_bar=float(e_bar), cg_iterations=int(iters), cg_residual=float(res), warm_start=ws)
