"""VMC (Metropolis) driver on one GPU.

Mirrors ``MCMC`` of jqmc/jqmc_mcmc.py:129-1189: constructor arguments
(``mcmc_seed, num_walkers, num_mcmc_per_measurement, Dt, epsilon_AS``),
``run(num_mcmc_steps)``, the per-measurement ``e_L``/``w_L`` arrays, the
acceptance counters and the jackknife ``get_E``.  One MCMC step is
``num_mcmc_per_measurement`` single-electron proposals per walker (one fused
``jqmc_vmc_sweep`` launch) followed by the local energy with a freshly rotated
ECP quadrature (``jqmc_vmc_measure``).

Draws per proposal (jqmc_mcmc.py:4321-4500): electron selector in [0, N),
up index, dn index, Cartesian axis, a standard normal and the acceptance
uniform; per measurement three Euler angles U(-2pi, 2pi).  They come from a
seeded torch generator on the device, or are passed to ``run_block``.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from .engine import GpuSystem, WalkerSet
from .hamiltonians import Hamiltonian_data
from .statistics import jackknife_energy
from ._init_config import initial_electrons


class MCMC:
    def __init__(self, hamiltonian_data: Hamiltonian_data = None, mcmc_seed: int = 34467, num_walkers: int = 40,
                 num_mcmc_per_measurement: int = 16, Dt: float = 2.0, epsilon_AS: float = 1e-1, Nv: int = 6,
                 init_r_up=None, init_r_dn=None):
        hamiltonian_data.sanity_check()
        self.hamiltonian_data = hamiltonian_data
        self.num_walkers = num_walkers
        self.num_mcmc_per_measurement = num_mcmc_per_measurement
        self.Dt = Dt
        self.epsilon_AS = epsilon_AS
        self.sys = GpuSystem(hamiltonian_data, Nv=Nv)
        if init_r_up is None:
            st = hamiltonian_data.structure_data
            coul = hamiltonian_data.coulomb_potential_data
            init_r_up, init_r_dn = initial_electrons(st.positions, coul.effective_charges, self.sys.n_up, self.sys.n_dn,
                                                     num_walkers, mcmc_seed)
        self.walkers = WalkerSet(self.sys, init_r_up, init_r_dn)
        dev = self.sys.device
        self.gen = torch.Generator(device=dev)
        self.gen.manual_seed(mcmc_seed)
        self._accept = torch.zeros(num_walkers, dtype=torch.int32, device=dev)
        self._e_L, self._w_L = [], []
        self.mcmc_counter = 0
        self._proposals = 0

    def draws(self, K: int | None = None):
        K = self.num_mcmc_per_measurement if K is None else K
        W, n_up, n_dn = self.num_walkers, self.sys.n_up, self.sys.n_dn
        dev, g = self.sys.device, self.gen
        idraw = torch.stack([
            torch.randint(0, n_up + n_dn, (W, K), generator=g, device=dev),
            torch.randint(0, n_up, (W, K), generator=g, device=dev),
            torch.randint(0, max(n_dn, 1), (W, K), generator=g, device=dev),
            torch.randint(0, 3, (W, K), generator=g, device=dev)], dim=-1).to(torch.int32).contiguous()
        fdraw = torch.stack([torch.randn((W, K), generator=g, dtype=torch.float64, device=dev),
                             torch.rand((W, K), generator=g, dtype=torch.float64, device=dev)], dim=-1).contiguous()
        angles = (torch.rand((W, 3), generator=g, dtype=torch.float64, device=dev) * (4.0 * math.pi) - 2.0 * math.pi)
        return idraw, fdraw, angles

    def run_block(self, idraw, fdraw, angles):
        """One measurement: sweep + (e_L, w_L) device tensors."""
        self.walkers.vmc_sweep(idraw, fdraw, self.Dt, self.epsilon_AS, self._accept)
        self._proposals += idraw.shape[1]
        return self.walkers.vmc_measure(angles, self.epsilon_AS)

    def run(self, num_mcmc_steps: int = 0, max_time: int = 86400) -> None:
        for _ in range(num_mcmc_steps):
            eL, wL = self.run_block(*self.draws())
            self._e_L.append(eL.cpu().numpy())
            self._w_L.append(wL.cpu().numpy())
            self.mcmc_counter += 1

    @property
    def e_L(self) -> np.ndarray:
        return np.asarray(self._e_L)

    @property
    def e_L2(self) -> np.ndarray:
        return np.asarray(self._e_L) ** 2

    @property
    def w_L(self) -> np.ndarray:
        return np.asarray(self._w_L)

    @property
    def accepted_moves(self) -> int:
        return int(self._accept.sum())

    @property
    def rejected_moves(self) -> int:
        return self._proposals * self.num_walkers - self.accepted_moves

    def get_E(self, num_mcmc_warmup_steps: int = 50, num_mcmc_bin_blocks: int = 10):
        return jackknife_energy(self.e_L[num_mcmc_warmup_steps:], self.e_L2[num_mcmc_warmup_steps:],
                                self.w_L[num_mcmc_warmup_steps:], num_mcmc_bin_blocks)
