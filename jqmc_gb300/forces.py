"""Nuclear forces: the per-walker terms of the Hellmann-Feynman + Pulay estimator.

The reference stores, per walker and measurement (jqmc_mcmc.py:760-852, without
space warp): force_HF = dE_L/dR, force_PP = d ln psi/dR and E_L force_PP, and
assembles F = -<force_HF> - 2 (<E_L force_PP> - <E_L><force_PP>) with a
jackknife (``get_aF``, :1191-1380; here ``statistics.jackknife_force``).

* d ln psi / dR: the adjoint kernel ``jqmc_dlnpsi_dR`` (FP64, analytic: minus
  each electron's grad ln psi restricted to the AOs centred on a nucleus, plus
  the J1 pair terms), from the walkers' cached tables.
* dE_L / dR: five-point central differences (error O(h^4)) of the GPU FP64
  local energy with each nucleus displaced by +-h, +-2h along x, y, z (the same
  electron configurations and the same quadrature rotation), on systems built
  once per displacement.  E_L depends on
  R through the AO centres, J1, the Coulomb and ECP terms and the ECP quadrature
  points (R_I + |r - R_I| R Omega); the differences follow all of them, as the
  reference's automatic differentiation of E_L does.
* Space warp (use_swct, jqmc_mcmc.py:795-845, swct.py): with the weights
  omega_{I i} = |r_i - R_I|^-4 / sum_J |r_i - R_J|^-4 the reference adds
  sum_i omega_{I i} dE_L/dr_i to force_HF and sum_i omega_{I i} d ln psi/dr_i
  + 1/2 sum_i grad_{r_i} omega_{I i} to force_PP.  The first sums are
  directional derivatives: moving nucleus I by delta together with every
  electron i by omega_{I i} delta gives dE_L/dR_I + sum_i omega_{I i} dE_L/dr_i,
  so the same five-point differences give force_HF with the electrons warped
  along; moving only the electrons gives the ln psi sum.
* LRDMC forces (jqmc_gfmc.py:1900-2000, :5980-6040, without space warp): the
  same terms with the LRDMC local energy (``LRDMCEnergyGradientFD``), averaged
  over the walkers with the projection weights before the branching.
"""

from __future__ import annotations

import copy
import ctypes as C

import numpy as np
import torch

from . import _lib
from .engine import GpuSystem, WalkerSet


def dlnpsi_dR(walkers: WalkerSet) -> torch.Tensor:
    """(W, natom, 3) d ln|psi| / dR at the walkers' positions (FP64 walkers)."""
    if walkers.precision != "fp64":
        raise ValueError("nuclear derivatives are computed on FP64 walkers")
    M = len(walkers.sys._keep["pos"])
    out = torch.empty((walkers.nwalk, M, 3), dtype=torch.float64, device=walkers.sys.device)
    d = walkers.desc()
    _lib.check(_lib.lib().jqmc_dlnpsi_dR(walkers.sys.handle, C.byref(d), C.c_void_p(out.data_ptr()), walkers.sys.stream),
               "jqmc_dlnpsi_dR")
    return out


def displaced(hamiltonian, atom: int, axis: int, delta: float):
    """A copy of the Hamiltonian with one nucleus moved (every component that
    holds the nuclear positions shares the one Structure_data of the copy)."""
    h = copy.deepcopy(hamiltonian)
    h.structure_data.positions[atom, axis] += delta
    return h


STENCIL = ((2.0, -1.0 / 12.0), (1.0, 8.0 / 12.0), (-1.0, -8.0 / 12.0), (-2.0, 1.0 / 12.0))   # (offset / h, weight)


def swct_omega(R: torch.Tensor, r: torch.Tensor) -> torch.Tensor:
    """(W, M, Ne) space-warp weights omega_{I i} for nuclei R (M, 3) and
    electrons r (W, Ne, 3) (jqmc/swct.py:20-60)."""
    d = r[:, None, :, :] - R[None, :, None, :]
    k = (d * d).sum(dim=-1) ** -2
    return k / k.sum(dim=1, keepdim=True)


def swct_domega(R: torch.Tensor, r: torch.Tensor) -> torch.Tensor:
    """(W, M, 3) sum_i grad_{r_i} omega_{I i} (jqmc/swct.py:90-110), in closed form:
    grad omega_I = omega_I (g_I - sum_J omega_J g_J), g_J = -4 (r - R_J) / |r - R_J|^2."""
    d = r[:, None, :, :] - R[None, :, None, :]
    d2 = (d * d).sum(dim=-1)
    k = d2 ** -2
    w = k / k.sum(dim=1, keepdim=True)
    g = -4.0 * d / d2[..., None]
    gbar = (w[..., None] * g).sum(dim=1, keepdim=True)
    return (w[..., None] * (g - gbar)).sum(dim=2)


def _warped(r: np.ndarray, omega_I: np.ndarray, axis: int, delta: float) -> np.ndarray:
    """r (W, Ne, 3) with every electron moved by omega_I (W, Ne) delta along axis."""
    out = r.copy()
    out[:, :, axis] += delta * omega_I
    return out


def warped_dlnpsi(system: GpuSystem, r_up, r_dn, h: float = 5e-4) -> torch.Tensor:
    """(W, natom, 3) sum_i omega_{I i} d ln|psi| / dr_i by five-point differences of
    the GPU ln|psi| with the electrons moved by omega_{I i} delta (nuclei fixed)."""
    r_up = np.asarray(r_up, dtype=np.float64)
    r_dn = np.asarray(r_dn, dtype=np.float64)
    n = r_up.shape[1]
    r = np.concatenate([r_up, r_dn], axis=1)
    R = np.asarray(system._keep["pos"], dtype=np.float64)
    om = swct_omega(torch.as_tensor(R), torch.as_tensor(r)).numpy()
    W, M = r.shape[0], R.shape[0]
    out = torch.empty((W, M, 3), dtype=torch.float64, device=system.device)
    for I in range(M):
        for k in range(3):
            acc = torch.zeros(W, dtype=torch.float64, device=system.device)
            for o, wgt in STENCIL:
                rw = _warped(r, om[:, I], k, o * h)
                ld, _, jj = WalkerSet(system, rw[:, :n], rw[:, n:]).log_psi()
                acc += wgt * (ld + jj)
            out[:, I, k] = acc / h
    return out


class ELGradientFD:
    """dE_L/dR by five-point central differences of the GPU FP64 local energy;
    the 12 natom displaced systems are built once and reused.  With ``warp`` the
    electrons move with each displaced nucleus by omega_{I i} delta, which gives
    dE_L/dR_I + sum_i omega_{I i} dE_L/dr_i (the space-warp force_HF)."""

    def __init__(self, hamiltonian, h: float = 5e-4, Nv: int = 6, warp: bool = False, non_local_move: str = "tmove"):
        self.h = h
        self.warp = warp
        self.R = np.asarray(hamiltonian.structure_data.positions, dtype=np.float64).copy()
        self.M = hamiltonian.structure_data.natom
        self.systems = [[[GpuSystem(displaced(hamiltonian, I, k, o * h), Nv=Nv, non_local_move=non_local_move)
                          for o, _ in STENCIL] for k in range(3)] for I in range(self.M)]

    def _energy(self, ws: WalkerSet, *args) -> torch.Tensor:
        """args: the rotations (W, 3) and, optionally, the AS cutoff (default 0)."""
        angles = args[0]
        eps_AS = args[1] if len(args) > 1 else 0.0
        return ws.vmc_measure(angles, eps_AS)[0]

    def __call__(self, r_up, r_dn, *args) -> torch.Tensor:
        """(W, natom, 3) at the configurations (W, n, 3); args: the rotations (W, 3)
        and the AS cutoff (the LRDMC form: the energy's draws)."""
        r_up = np.asarray(r_up, dtype=np.float64)
        r_dn = np.asarray(r_dn, dtype=np.float64)
        W, n = r_up.shape[0], r_up.shape[1]
        r = np.concatenate([r_up, r_dn], axis=1)
        om = swct_omega(torch.as_tensor(self.R), torch.as_tensor(r)).numpy() if self.warp else None
        out = torch.empty((W, self.M, 3), dtype=torch.float64, device=self.systems[0][0][0].device)
        for I in range(self.M):
            for k in range(3):
                acc = torch.zeros(W, dtype=torch.float64, device=out.device)
                for gs, (o, wgt) in zip(self.systems[I][k], STENCIL):
                    if self.warp:
                        rw = _warped(r, om[:, I], k, o * self.h)
                        ws = WalkerSet(gs, rw[:, :n], rw[:, n:])
                    else:
                        ws = WalkerSet(gs, r_up, r_dn)
                    acc += wgt * self._energy(ws, *args)
                    del ws
                out[:, I, k] = acc / self.h
        return out


class LRDMCEnergyGradientFD(ELGradientFD):
    """d e_L/dR of the LRDMC local energy V_diag + V_nondiag of the lattice-
    regularised Hamiltonian (jqmc_gfmc.py:5630-5650, the function whose gradient
    the reference's LRDMC force takes, :5842-5870) by the same five-point
    differences; call with the configurations and the energy's draws (W, 4)."""

    def __init__(self, hamiltonian, alat: float, h: float = 5e-4, Nv: int = 6, non_local_move: str = "tmove"):
        super().__init__(hamiltonian, h=h, Nv=Nv, non_local_move=non_local_move)
        self.alat = alat

    def _energy(self, ws: WalkerSet, *args) -> torch.Tensor:
        (last_draw,) = args
        return ws.lrdmc_energy(last_draw, self.alat)[0]
