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


class ELGradientFD:
    """dE_L/dR by five-point central differences of the GPU FP64 local energy;
    the 12 natom displaced systems are built once and reused."""

    def __init__(self, hamiltonian, h: float = 5e-4, Nv: int = 6):
        self.h = h
        self.M = hamiltonian.structure_data.natom
        self.systems = [[[GpuSystem(displaced(hamiltonian, I, k, o * h), Nv=Nv) for o, _ in STENCIL] for k in range(3)]
                        for I in range(self.M)]

    def _energy(self, ws: WalkerSet, *args) -> torch.Tensor:
        angles, eps_AS = args
        return ws.vmc_measure(angles, eps_AS)[0]

    def __call__(self, r_up, r_dn, *args) -> torch.Tensor:
        """(W, natom, 3) at the configurations (W, n, 3); args: the rotations (W, 3)
        and the AS cutoff."""
        r_up = np.asarray(r_up)
        r_dn = np.asarray(r_dn)
        W = r_up.shape[0]
        out = torch.empty((W, self.M, 3), dtype=torch.float64, device=self.systems[0][0][0].device)
        for I in range(self.M):
            for k in range(3):
                acc = torch.zeros(W, dtype=torch.float64, device=out.device)
                for gs, (_, wgt) in zip(self.systems[I][k], STENCIL):
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

    def __init__(self, hamiltonian, alat: float, h: float = 5e-4, Nv: int = 6):
        super().__init__(hamiltonian, h=h, Nv=Nv)
        self.alat = alat

    def _energy(self, ws: WalkerSet, *args) -> torch.Tensor:
        (last_draw,) = args
        return ws.lrdmc_energy(last_draw, self.alat)[0]
