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

Wavefunction optimisation (jqmc_mcmc.py:1372-1700, :2368-3800): ``get_dln_WF``
assembles the stored per-walker derivative blocks, ``get_gF`` gives the
generalized forces with jackknife errors, and ``run_optimize`` alternates
sampling with the SR update of ``variational.sr_direction``.  Setting
``hamiltonian_data`` rebuilds the device tables, keeps the walkers' positions
and clears the stored samples (jqmc_mcmc.py:4129-4145).
"""

from __future__ import annotations

import math
import time

import numpy as np
import torch

from .adjoint import dlnpsi_dparams
from .engine import GpuSystem, WalkerSet
from .forces import ELGradientFD, dlnpsi_dR, swct_domega, warped_dlnpsi
from .hamiltonians import Hamiltonian_data
from .statistics import jackknife_energy, jackknife_force, jackknife_generalized_force
from .variational import apply_block_updates, get_variational_blocks, sr_direction
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
        self.num_walkers = num_walkers
        self.num_mcmc_per_measurement = num_mcmc_per_measurement
        self.Dt = Dt
        self.epsilon_AS = epsilon_AS
        self.random_discretized_mesh = random_discretized_mesh
        self.Nv = Nv
        self.force_fd_step = force_fd_step
        self.comput_log_WF_param_deriv = comput_log_WF_param_deriv
        self.comput_position_deriv = comput_position_deriv
        self.use_swct = use_swct
        self._opt_lambda = True
        self._build(hamiltonian_data, init_r_up, init_r_dn, mcmc_seed)
        self.gen = torch.Generator(device=self.sys.device)
        self.gen.manual_seed(mcmc_seed)

    def _build(self, hamiltonian_data: Hamiltonian_data, r_up, r_dn, seed: int = 0) -> None:
        """Device tables and walkers for hamiltonian_data, stored samples cleared."""
        hamiltonian_data.sanity_check()
        sys_new = GpuSystem(hamiltonian_data, Nv=self.Nv)
        if r_up is None:
            st = hamiltonian_data.structure_data
            coul = hamiltonian_data.coulomb_potential_data
            r_up, r_dn = initial_electrons(st.positions, coul.effective_charges, sys_new.n_up, sys_new.n_dn,
                                           self.num_walkers, seed)
        self._hamiltonian_data = hamiltonian_data
        self.sys = sys_new
        self.walkers = WalkerSet(self.sys, r_up, r_dn)
        self._accept = torch.zeros(self.num_walkers, dtype=torch.int32, device=self.sys.device)
        self._e_L, self._w_L = [], []
        self.mcmc_counter = 0
        self._proposals = 0
        # per-measurement derivative observables (jqmc_mcmc.py:756-876)
        self._param_grads = {}
        self._force_HF, self._force_PP, self._E_L_force_PP = [], [], []
        self._el_grad = (ELGradientFD(hamiltonian_data, h=self.force_fd_step, Nv=self.Nv, warp=self.use_swct)
                         if self.comput_position_deriv else None)

    @property
    def hamiltonian_data(self) -> Hamiltonian_data:
        return self._hamiltonian_data

    @hamiltonian_data.setter
    def hamiltonian_data(self, hamiltonian_data: Hamiltonian_data) -> None:
        """New parameters: device tables rebuilt, walkers kept where they are, stored
        samples and counters cleared (jqmc_mcmc.py:4129-4145, :260-290)."""
        r = self.walkers.r.cpu().numpy()
        n = self.sys.n_up
        self._build(hamiltonian_data, r[:, :n], r[:, n:])

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
        """num_mcmc_steps measurements, stopping early once max_time seconds have
        passed (jqmc_mcmc.py:448, :940-947)."""
        t0 = time.perf_counter()
        for _ in range(num_mcmc_steps):
            if time.perf_counter() - t0 > max_time:
                break
            idraw, fdraw, angles = self.draws()
            eL, wL = self.run_block(idraw, fdraw, angles)
            self._e_L.append(eL.cpu().numpy())
            self._w_L.append(wL.cpu().numpy())
            if self.comput_log_WF_param_deriv:
                for name, g in dlnpsi_dparams(self.walkers, lam=self._opt_lambda).items():
                    self._param_grads.setdefault(name, []).append(g.cpu().numpy())
            if self.comput_position_deriv:
                fpp = dlnpsi_dR(self.walkers)
                r = self.walkers.r.cpu().numpy()
                n = self.sys.n_up
                fhf = self._el_grad(r[:, :n], r[:, n:], angles, self.epsilon_AS)   # warped with use_swct
                if self.use_swct:   # jqmc_mcmc.py:836-842
                    R = torch.as_tensor(self.sys._keep["pos"], device=self.walkers.r.device)
                    fpp = (fpp + warped_dlnpsi(self.sys, r[:, :n], r[:, n:], self.force_fd_step)
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

    # ---------------------------------------------------------------- optimisation
    def get_dln_WF(self, blocks: list, num_mcmc_warmup_steps: int = 50, chosen_param_index: list | None = None,
                   lambda_projectors: tuple | None = None, num_orb_projection: int | None = None) -> np.ndarray:
        """O (M - warmup, num_walkers, K): the stored d ln psi / dc blocks in the order
        of ``blocks``, each passed through its symmetry callback
        (jqmc_mcmc.py:1372-1513)."""
        if lambda_projectors is not None or num_orb_projection is not None:
            raise NotImplementedError("the MO-projected lambda optimisation (opt_with_projected_MOs) is not built")
        grads = self.dln_Psi_dc
        M, nw = self.mcmc_counter, self.num_walkers
        parts = []
        for b in blocks:
            if b.name not in grads:
                raise ValueError(f"no stored derivatives for block {b.name!r}: construct MCMC with "
                                 "comput_log_WF_param_deriv=True and run it first")
            g = grads[b.name].reshape(M, nw, b.size)
            if b.symmetrize_metric is not None:
                g = b.symmetrize_metric(g.reshape(M * nw, b.size)).reshape(M, nw, b.size)
            parts.append(g)
        O = np.concatenate(parts, axis=2) if parts else np.zeros((M, nw, 0))
        O = O[num_mcmc_warmup_steps:]
        return O if chosen_param_index is None else O[:, :, chosen_param_index]

    def get_gF(self, num_mcmc_warmup_steps: int = 50, num_mcmc_bin_blocks: int = 10,
               chosen_param_index: list | None = None, blocks: list | None = None,
               lambda_projectors: tuple | None = None, num_orb_projection: int | None = None):
        """(generalized_force_mean, generalized_force_std) over the parameters of
        ``blocks`` (default: the wavefunction's blocks) (jqmc_mcmc.py:1515-1700)."""
        if blocks is None:
            blocks = get_variational_blocks(self.hamiltonian_data.wavefunction_data)
        O = self.get_dln_WF(blocks, num_mcmc_warmup_steps, chosen_param_index, lambda_projectors, num_orb_projection)
        k = num_mcmc_warmup_steps
        return jackknife_generalized_force(self.w_L[k:], self.e_L[k:], O, num_mcmc_bin_blocks)

    def run_optimize(self, num_mcmc_steps: int = 100, num_opt_steps: int = 1, wf_dump_freq: int = 10,
                     max_time: int = 86400, num_mcmc_warmup_steps: int = 0, num_mcmc_bin_blocks: int = 100,
                     opt_J1_param: bool = True, opt_J2_param: bool = True, opt_J3_param: bool = True,
                     opt_JNN_param: bool = True, opt_lambda_param: bool = False, opt_with_projected_MOs: bool = False,
                     opt_J3_basis_exp: bool = False, opt_J3_basis_coeff: bool = False,
                     opt_lambda_basis_exp: bool = False, opt_lambda_basis_coeff: bool = False,
                     optimizer_kwargs: dict | None = None) -> list:
        """SR optimisation (jqmc_mcmc.py:2368-3800): per step, ``num_mcmc_steps``
        measurements, E and f with jackknife errors, theta = (S + eps diag S)^-1 f
        from the samples, then every block moved by delta * theta and the sampler
        reset on the new wavefunction.  optimizer_kwargs: method "sr" with delta
        (1e-3), epsilon (1e-3), cg_flag (True), cg_max_iter (1e6), cg_tol (1e-8).
        Returns one record per step: E, E_std, max |f|, max |f|/f_std, the CG
        iterations.  wf_dump_freq is accepted for the reference's signature; no
        checkpoint files are written.  The linear method (use_lm), optax
        optimisers, projected-MO and AO-basis optimisation raise."""
        kw = dict(optimizer_kwargs or {})
        method = str(kw.pop("method", "sr")).lower()
        if method != "sr":
            raise NotImplementedError(f"optimizer {method!r}: only SR is built (optax is not available)")
        if kw.get("use_lm", False):
            raise RuntimeError("use_lm requires comput_e_L_param_deriv=True.")
        if opt_with_projected_MOs:
            raise NotImplementedError("opt_with_projected_MOs is not built")
        if not self.comput_log_WF_param_deriv:
            raise ValueError("construct MCMC with comput_log_WF_param_deriv=True to optimise the wavefunction")
        delta = float(kw.get("delta", 1.0e-3))
        epsilon = float(kw.get("epsilon", 1.0e-3))
        cg_flag = bool(kw.get("cg_flag", True))
        cg_max_iter = int(kw.get("cg_max_iter", int(1e6)))
        cg_tol = float(kw.get("cg_tol", 1.0e-8))
        flags = dict(opt_J1_param=opt_J1_param, opt_J2_param=opt_J2_param, opt_J3_param=opt_J3_param,
                     opt_JNN_param=opt_JNN_param, opt_lambda_param=opt_lambda_param, opt_J3_basis_exp=opt_J3_basis_exp,
                     opt_J3_basis_coeff=opt_J3_basis_coeff, opt_lambda_basis_exp=opt_lambda_basis_exp,
                     opt_lambda_basis_coeff=opt_lambda_basis_coeff)
        get_variational_blocks(self.hamiltonian_data.wavefunction_data, **flags)     # option check before sampling
        self._opt_lambda = opt_lambda_param
        history = []
        warm = {}
        t0 = time.perf_counter()
        try:
            for _ in range(num_opt_steps):
                self.run(num_mcmc_steps=num_mcmc_steps, max_time=max_time)
                E, E_std, _, _ = self.get_E(num_mcmc_warmup_steps, num_mcmc_bin_blocks)
                if not np.isfinite(E):
                    break
                wf = self.hamiltonian_data.wavefunction_data
                blocks = get_variational_blocks(wf, **flags)
                f, f_std = self.get_gF(num_mcmc_warmup_steps, num_mcmc_bin_blocks, blocks=blocks)
                O = self.get_dln_WF(blocks, num_mcmc_warmup_steps)
                k = num_mcmc_warmup_steps
                key = (O.shape[2], O.shape[0] * O.shape[1])
                sr = sr_direction(O, self.e_L[k:], self.w_L[k:], epsilon, cg_flag, cg_max_iter, cg_tol,
                                  warm_start=warm.get(key), device=self.sys.device)
                if sr.warm_start is not None:
                    warm[key] = sr.warm_start
                ok = np.isfinite(f_std) & (np.abs(f_std) > np.finfo(np.float64).eps)
                sn = np.zeros_like(f)
                sn[ok] = np.abs(f[ok]) / f_std[ok]
                history.append(dict(E=E, E_std=E_std, max_f=float(np.max(np.abs(f))) if f.size else 0.0,
                                    max_f_over_std=float(np.max(sn)) if sn.size else 0.0,
                                    cg_iterations=sr.cg_iterations, frozen=int(np.sum(sr.frozen))))
                new_wf = apply_block_updates(wf, blocks, sr.theta, delta)
                ham = self.hamiltonian_data
                self.hamiltonian_data = Hamiltonian_data(structure_data=ham.structure_data,
                                                         coulomb_potential_data=ham.coulomb_potential_data,
                                                         wavefunction_data=new_wf)
                if time.perf_counter() - t0 > max_time:
                    break
        finally:
            self._opt_lambda = True
        return history
