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

from .adjoint import dlnpsi_dparams
from .engine import GpuSystem, WalkerSet
from .forces import ELGradientFD, dlnpsi_dR, swct_domega, warped_dlnpsi
from .hamiltonians import Hamiltonian_data
from .statistics import jackknife_energy, jackknife_force
from ._init_config import initial_electrons


class MCMC:
    def __init__(self, hamiltonian_data: Hamiltonian_data = None, mcmc_seed: int = 34467, num_walkers: int = 40,
                 num_mcmc_per_measurement: int = 16, Dt: float = 2.0, epsilon_AS: float = 1e-1,
                 comput_log_WF_param_deriv: bool = False, comput_e_L_param_deriv: bool = False,
                 comput_position_deriv: bool = False, random_discretized_mesh: bool = True, use_swct: bool = True,
                 Nv: int = 6, init_r_up=None, init_r_dn=None, force_fd_step: float = 5e-4):
        """The reference's MCMC driver (jqmc_mcmc.py:129-143) on the GPU path, with
        the same arguments in the same order and defaults, then Nv (quadrature
        points), initial electrons and the finite-difference step of the force
        terms.  comput_e_L_param_deriv=True is refused."""
        if comput_e_L_param_deriv:
            raise NotImplementedError("d e_L / d c (comput_e_L_param_deriv) is not on the GPU path")
        hamiltonian_data.sanity_check()
        self.hamiltonian_data = hamiltonian_data
        self.num_walkers = num_walkers
        self.num_mcmc_per_measurement = num_mcmc_per_measurement
        self.Dt = Dt
        self.epsilon_AS = epsilon_AS
        self.random_discretized_mesh = random_discretized_mesh
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
        # per-measurement derivative observables (jqmc_mcmc.py:756-876)
        self.comput_log_WF_param_deriv = comput_log_WF_param_deriv
        self.comput_position_deriv = comput_position_deriv
        self._param_grads = {}
        self._force_HF, self._force_PP, self._E_L_force_PP = [], [], []
        self.use_swct = use_swct
        self._fd_step = force_fd_step
        self._el_grad = ELGradientFD(hamiltonian_data, h=force_fd_step, Nv=Nv, warp=use_swct) if comput_position_deriv else None

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
        if not self.random_discretized_mesh:   # identity rotations (jqmc_mcmc.py:724-727)
            angles.zero_()
        return idraw, fdraw, angles

    def run_block(self, idraw, fdraw, angles):
        """One measurement: sweep + (e_L, w_L) device tensors."""
        self.walkers.vmc_sweep(idraw, fdraw, self.Dt, self.epsilon_AS, self._accept)
        self._proposals += idraw.shape[1]
        return self.walkers.vmc_measure(angles, self.epsilon_AS)

    def run(self, num_mcmc_steps: int = 0, max_time: int = 86400) -> None:
        for _ in range(num_mcmc_steps):
            idraw, fdraw, angles = self.draws()
            eL, wL = self.run_block(idraw, fdraw, angles)
            self._e_L.append(eL.cpu().numpy())
            self._w_L.append(wL.cpu().numpy())
            if self.comput_log_WF_param_deriv:
                for name, g in dlnpsi_dparams(self.walkers).items():
                    self._param_grads.setdefault(name, []).append(g.cpu().numpy())
            if self.comput_position_deriv:
                fpp = dlnpsi_dR(self.walkers)
                r = self.walkers.r.cpu().numpy()
                n = self.sys.n_up
                fhf = self._el_grad(r[:, :n], r[:, n:], angles, self.epsilon_AS)   # warped with use_swct
                if self.use_swct:   # jqmc_mcmc.py:836-842
                    R = torch.as_tensor(self.sys._keep["pos"], device=self.walkers.r.device)
                    fpp = (fpp + warped_dlnpsi(self.sys, r[:, :n], r[:, n:], self._fd_step)
                           + 0.5 * swct_domega(R, self.walkers.r))
                self._force_HF.append(fhf.cpu().numpy())
                self._force_PP.append(fpp.cpu().numpy())
                self._E_L_force_PP.append((eL[:, None, None] * fpp).cpu().numpy())
            self.mcmc_counter += 1

    @property
    def dln_Psi_dc(self) -> dict:
        """Per-measurement, per-walker d ln psi / d theta blocks (collect_param_grads names)."""
        return {k: np.asarray(v) for k, v in self._param_grads.items()}

    def get_aF(self, num_mcmc_warmup_steps: int = 50, num_mcmc_bin_blocks: int = 10):
        """(force_mean, force_std), (natom, 3) in Hartree/bohr (jqmc_mcmc.py:1191-1380)."""
        if not self.comput_position_deriv:
            raise ValueError("construct MCMC with comput_position_deriv=True to measure forces")
        k = num_mcmc_warmup_steps
        return jackknife_force(self.w_L[k:], self.e_L[k:], np.asarray(self._force_HF)[k:], np.asarray(self._force_PP)[k:],
                               np.asarray(self._E_L_force_PP)[k:], num_mcmc_bin_blocks)

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
