"""LRDMC driver with fixed projection count (GFMC_n), on one GPU.

Mirrors ``GFMC_n`` of jqmc/jqmc_gfmc.py:4191-6990: the constructor arguments,
``run(num_mcmc_steps)``, the stored per-branching observables and ``get_E``.
One "MCMC step" is one branching cycle: ``num_mcmc_per_measurement``
projections of every walker (one fused ``jqmc_lrdmc_project`` launch), the FP64
rebuild of G^-1 and the tables carried by rank-1 updates from the positions
(``jqmc_lu_rebuild_refine``), the local energy at the final positions
(``jqmc_lrdmc_energy``), the weighted averages, and the comb reconfiguration
(``jqmc_branch_comb`` + ``jqmc_walker_gather``).  The reference recomputes G^-1
from the positions after branching (jqmc_gfmc.py:6319); rebuilding just before
the energy instead gives the same state after the gather (which copies the
rebuilt tables) and lets the mixed-precision form measure E_L on fresh tables
rather than on tables that carry a block of float rank-1 updates.

Random numbers: per projection the three Euler angles U(-2pi, 2pi) and the move
uniform; per branching one comb offset zeta.  They are drawn on the device from
a seeded torch generator (or passed explicitly to ``run_block``).  The JAX
threefry stream of the reference is not reproduced.
"""

from __future__ import annotations

import math
import time

import numpy as np
import torch

from .engine import GpuSystem, WalkerSet, branch_comb
from .hamiltonians import Hamiltonian_data
from .forces import LRDMCEnergyGradientFD, dlnpsi_dR
from .statistics import gfmc_G_L, jackknife_energy, jackknife_force
from ._init_config import initial_electrons


def _check_lrdmc_options(non_local_move: str, comput_position_deriv: bool, use_swct: bool = False,
                         epsilon_PW: float = 0.0, precision: str = "fp64") -> None:
    if non_local_move not in ("tmove", "dltmove"):
        raise NotImplementedError(f"non_local_move={non_local_move!r}: 'tmove' or 'dltmove'")
    if comput_position_deriv:
        if use_swct:
            raise NotImplementedError("the space-warp transformation of the LRDMC forces is not on the GPU path")
        if epsilon_PW > 0.0:
            raise NotImplementedError("the nodal regularisation of the LRDMC forces (epsilon_PW > 0) is not on the GPU path")
        if precision != "fp64":
            raise ValueError("LRDMC forces are computed on FP64 walkers (precision='fp64')")


class _ForceTerms:
    """Per-step LRDMC force observables (jqmc_gfmc.py:1940-2000, :5980-6040): the
    walkers' d e_L/dR, d ln psi/dR and e_L d ln psi/dR averaged with weights f
    (w for GFMC_t, w / (V_diag - E_scf) for GFMC_n) before the branching."""

    def __init__(self, hamiltonian_data, alat: float, Nv: int, h: float):
        self.grad = LRDMCEnergyGradientFD(hamiltonian_data, alat, h=h, Nv=Nv)
        self.HF, self.PP, self.ELPP = [], [], []

    def add(self, ws: WalkerSet, f: torch.Tensor, eL: torch.Tensor, last_draw: torch.Tensor) -> None:
        fpp = dlnpsi_dR(ws)
        r = ws.r.cpu().numpy()
        n = ws.sys.n_up
        fhf = self.grad(r[:, :n], r[:, n:], last_draw)
        fs = f.sum()
        avg = lambda x: (torch.einsum("w,wij->ij", f, x) / fs).cpu().numpy()[None]   # noqa: E731
        self.HF.append(avg(fhf))
        self.PP.append(avg(fpp))
        self.ELPP.append(avg(eL[:, None, None] * fpp))

    def arrays(self, skip: int):
        return tuple(np.asarray(x)[skip:] for x in (self.HF, self.PP, self.ELPP))


class GFMC_n:
    def __init__(self, hamiltonian_data: Hamiltonian_data = None, num_walkers: int = 40, num_mcmc_per_measurement: int = 16,
                 num_gfmc_collect_steps: int = 5, mcmc_seed: int = 34467, E_scf: float = 0.0, alat: float = 0.1,
                 random_discretized_mesh: bool = True, non_local_move: str = "tmove", comput_position_deriv: bool = False,
                 epsilon_PW: float = 0.0, use_swct: bool = False, Nv: int = 6, init_r_up=None, init_r_dn=None,
                 rebuild_after_branching: bool = True, precision: str = "fp64", force_fd_step: float = 5e-4):
        """The reference's GFMC_n (jqmc_gfmc.py:4222-4236) on the GPU path, with the
        same arguments in the same order, then Nv, initial electrons, the rebuild
        switch, the precision form and the finite-difference step of d e_L/dR.
        LRDMC forces (comput_position_deriv) run on FP64 walkers without space warp
        (use_swct) and nodal regularisation (epsilon_PW > 0), which raise."""
        _check_lrdmc_options(non_local_move, comput_position_deriv, use_swct, epsilon_PW, precision)
        hamiltonian_data.sanity_check()
        self.hamiltonian_data = hamiltonian_data
        self.num_walkers = num_walkers
        self.num_mcmc_per_measurement = num_mcmc_per_measurement
        self.E_scf = E_scf
        self.alat = alat
        self.random_discretized_mesh = random_discretized_mesh
        self.num_gfmc_collect_steps = num_gfmc_collect_steps
        self.rebuild_after_branching = rebuild_after_branching
        self.sys = GpuSystem(hamiltonian_data, Nv=Nv, non_local_move=non_local_move)
        if init_r_up is None:
            st = hamiltonian_data.structure_data
            coul = hamiltonian_data.coulomb_potential_data
            init_r_up, init_r_dn = initial_electrons(st.positions, coul.effective_charges, self.sys.n_up, self.sys.n_dn,
                                                     num_walkers, mcmc_seed)
        self.precision = precision
        self.walkers = WalkerSet(self.sys, init_r_up, init_r_dn, precision=precision)
        self._spare = WalkerSet.empty_like(self.walkers)
        dev = self.sys.device
        self.gen = torch.Generator(device=dev)
        self.gen.manual_seed(mcmc_seed)
        self._np_rng = np.random.default_rng(mcmc_seed)
        self._chosen = torch.empty(num_walkers, dtype=torch.int32, device=dev)
        self._cum = torch.empty(num_walkers, dtype=torch.float64, device=dev)
        self._e_L, self._e_L2, self._w_L = [], [], []
        self.mcmc_counter = 0
        self.comput_position_deriv = comput_position_deriv
        self._forces = _ForceTerms(hamiltonian_data, alat, Nv, force_fd_step) if comput_position_deriv else None

    # ------------------------------------------------------------------ draws
    def draws(self, K: int | None = None) -> torch.Tensor:
        K = self.num_mcmc_per_measurement if K is None else K
        d = torch.rand((self.num_walkers, K, 4), generator=self.gen, dtype=torch.float64, device=self.sys.device)
        if self.random_discretized_mesh:
            d[..., :3].mul_(4.0 * math.pi).sub_(2.0 * math.pi)
        else:
            d[..., :3].zero_()
        return d

    # ------------------------------------------------------------------ one branching cycle
    def run_block(self, draws: torch.Tensor, zeta: float):
        """Projection block + energy + reconfiguration.  Returns device scalars
        (w_sum, sum w/(Vd-E), sum w e/(Vd-E), sum w e^2/(Vd-E)) before branching."""
        ws = self.walkers
        w = torch.ones(self.num_walkers, dtype=torch.float64, device=self.sys.device)
        ws.lrdmc_project(draws, self.alat, self.E_scf, w)
        if self.rebuild_after_branching:
            ws.rebuild()
        last = draws[:, -1].contiguous()
        eL, vd = ws.lrdmc_energy(last, self.alat)
        f = w / (vd - self.E_scf)
        if self._forces is not None:   # at the configurations before the branching (jqmc_gfmc.py:5842-6040)
            self._forces.add(ws, f, eL, last)
        sums = torch.stack([w.sum(), f.sum(), (f * eL).sum(), (f * eL * eL).sum()])
        branch_comb(w, zeta, self._chosen, self._cum)
        self._spare.gather_from(ws, self._chosen)
        self.walkers, self._spare = self._spare, self.walkers
        return sums

    def run(self, num_mcmc_steps: int = 50, max_time: int = 86400) -> None:
        """num_mcmc_steps branching cycles, stopping early once max_time seconds have passed."""
        t0 = time.perf_counter()
        for _ in range(num_mcmc_steps):
            if time.perf_counter() - t0 > max_time:
                break
            zeta = float(self._np_rng.random())
            sums = self.run_block(self.draws(), zeta).cpu().numpy()
            w_avg = sums[0] / self.num_walkers
            self._w_L.append(w_avg)
            self._e_L.append(sums[2] / sums[1])
            self._e_L2.append(sums[3] / sums[1])
            self.mcmc_counter += 1

    # ------------------------------------------------------------------ observables
    @property
    def w_L(self) -> np.ndarray:
        """G_L weight products over the collect window (jqmc_gfmc.py:136-152)."""
        return gfmc_G_L(np.asarray(self._w_L, dtype=np.float64).reshape(-1, 1), self.num_gfmc_collect_steps)

    @property
    def bare_w_L(self) -> np.ndarray:
        """The per-step mean walker weights before the G_L products (jqmc_gfmc.py:4599-4601)."""
        return np.asarray(self._w_L, dtype=np.float64).reshape(-1, 1)

    @property
    def e_L(self) -> np.ndarray:
        return np.asarray(self._e_L, dtype=np.float64).reshape(-1, 1)[self.num_gfmc_collect_steps:]

    @property
    def e_L2(self) -> np.ndarray:
        return np.asarray(self._e_L2, dtype=np.float64).reshape(-1, 1)[self.num_gfmc_collect_steps:]

    def get_E(self, num_mcmc_warmup_steps: int = 50, num_mcmc_bin_blocks: int = 10):
        e, e2, w = self.e_L[num_mcmc_warmup_steps:], self.e_L2[num_mcmc_warmup_steps:], self.w_L[num_mcmc_warmup_steps:]
        return jackknife_energy(e, e2, w, num_mcmc_bin_blocks)

    def get_aF(self, num_mcmc_warmup_steps: int = 50, num_mcmc_bin_blocks: int = 10):
        """(force_mean, force_std), (natom, 3) in Hartree/bohr: the jackknife of
        jqmc_gfmc.py:6694-6800 over the G_L-weighted steps."""
        return _gfmc_forces(self, num_mcmc_warmup_steps, num_mcmc_bin_blocks)


def _gfmc_forces(drv, warmup: int, bins: int):
    if drv._forces is None:
        raise ValueError("construct the driver with comput_position_deriv=True to measure forces")
    hf, pp, elpp = drv._forces.arrays(drv.num_gfmc_collect_steps)
    k = warmup
    return jackknife_force(drv.w_L[k:], drv.e_L[k:], hf[k:], pp[k:], elpp[k:], bins)


class GFMC_t:
    """LRDMC driver with fixed projection time (GFMC_t), on one GPU.

    Mirrors ``GFMC_t`` of jqmc/jqmc_gfmc.py:208-2390: the constructor arguments,
    ``run(num_mcmc_steps)``, the stored per-branching observables and ``get_E``.
    One "MCMC step" is one branching cycle: every walker projects for time ``tau``
    (``jqmc_lrdmc_project_t`` in chunks of ``draws_per_call`` steps until no
    walker has time left; per step ``tau_update = min(tau_left, ln(1-xi)/V_nondiag)``
    and ``w *= exp(-tau_update e_L)``, jqmc_gfmc.py:724-1107), the FP64 rebuild of
    the tables carried by rank-1 updates, e_L at the final configuration, the
    weighted averages (jqmc_gfmc.py:1940-1996: sum w e_L / sum w) and the comb
    reconfiguration.  The reference runs all walkers in one lock-step while loop
    and keeps the e_L of its last iteration, which for a walker whose time was
    already spent is e_L at its final configuration with a fresh rotation; here
    each walker stops on its own and e_L is evaluated at the final configuration
    with a fresh rotation.
    """

    def __init__(self, hamiltonian_data: Hamiltonian_data = None, num_walkers: int = 40, num_gfmc_collect_steps: int = 5,
                 mcmc_seed: int = 34467, tau: float = 0.1, alat: float = 0.1, random_discretized_mesh: bool = True,
                 non_local_move: str = "tmove", comput_position_deriv: bool = False, epsilon_PW: float = 0.0,
                 use_swct: bool = False, Nv: int = 6, init_r_up=None, init_r_dn=None, precision: str = "fp64",
                 draws_per_call: int = 64, max_calls: int = 10000, force_fd_step: float = 5e-4):
        """The reference's GFMC_t (jqmc_gfmc.py:208-221) on the GPU path, with the
        same arguments in the same order, then Nv, initial electrons, the
        precision form, the draw batching and the finite-difference step of
        d e_L/dR.  LRDMC forces as in GFMC_n."""
        _check_lrdmc_options(non_local_move, comput_position_deriv, use_swct, epsilon_PW, precision)
        if not tau > 0.0:
            raise ValueError("tau must be positive")
        hamiltonian_data.sanity_check()
        self.hamiltonian_data = hamiltonian_data
        self.num_walkers = num_walkers
        self.num_gfmc_collect_steps = num_gfmc_collect_steps
        self.tau = tau
        self.alat = alat
        self.random_discretized_mesh = random_discretized_mesh
        self.draws_per_call = draws_per_call
        self.max_calls = max_calls
        self.sys = GpuSystem(hamiltonian_data, Nv=Nv, non_local_move=non_local_move)
        if init_r_up is None:
            st = hamiltonian_data.structure_data
            coul = hamiltonian_data.coulomb_potential_data
            init_r_up, init_r_dn = initial_electrons(st.positions, coul.effective_charges, self.sys.n_up, self.sys.n_dn,
                                                     num_walkers, mcmc_seed)
        self.precision = precision
        self.walkers = WalkerSet(self.sys, init_r_up, init_r_dn, precision=precision)
        self._spare = WalkerSet.empty_like(self.walkers)
        dev = self.sys.device
        self.gen = torch.Generator(device=dev)
        self.gen.manual_seed(mcmc_seed)
        self._np_rng = np.random.default_rng(mcmc_seed)
        W = num_walkers
        self._w = torch.empty(W, dtype=torch.float64, device=dev)
        self._tau_left = torch.empty(W, dtype=torch.float64, device=dev)
        self._nsteps = torch.zeros(W, dtype=torch.int32, device=dev)
        self._eL_last = torch.zeros(W, dtype=torch.float64, device=dev)
        self._chosen = torch.empty(W, dtype=torch.int32, device=dev)
        self._cum = torch.empty(W, dtype=torch.float64, device=dev)
        self._e_L, self._e_L2, self._w_L, self._proj = [], [], [], []
        self.mcmc_counter = 0
        self.comput_position_deriv = comput_position_deriv
        self._forces = _ForceTerms(hamiltonian_data, alat, Nv, force_fd_step) if comput_position_deriv else None

    def draws(self, K: int) -> torch.Tensor:
        """(W, K, 5): three rotation angles U(-2pi, 2pi), xi, and the move uniform."""
        d = torch.rand((self.num_walkers, K, 5), generator=self.gen, dtype=torch.float64, device=self.sys.device)
        if self.random_discretized_mesh:
            d[..., :3].mul_(4.0 * math.pi).sub_(2.0 * math.pi)
        else:
            d[..., :3].zero_()
        return d

    def project(self, draw_source=None):
        """Project every walker for time tau; returns (w, total projections per walker)."""
        ws = self.walkers
        self._w.fill_(1.0)
        self._tau_left.fill_(self.tau)
        total = torch.zeros(self.num_walkers, dtype=torch.int64, device=self.sys.device)
        for _ in range(self.max_calls):
            d = draw_source(self.draws_per_call) if draw_source is not None else self.draws(self.draws_per_call)
            ws.lrdmc_project_t(d, self.alat, self._w, self._tau_left, self._nsteps, self._eL_last)
            total += self._nsteps
            if not bool((self._tau_left > 0.0).any()):
                return self._w, total
        raise RuntimeError(f"GFMC_t: walkers still had time left after {self.max_calls} calls")

    def run_block(self, zeta: float, draw_source=None):
        """Projection for time tau + energy + reconfiguration.  Returns device scalars
        (w_sum, sum w e_L, sum w e_L^2, mean projections per walker) before branching."""
        w, total = self.project(draw_source)
        ws = self.walkers
        ws.rebuild()
        ang = self.draws(1)[:, 0, :4].contiguous()   # the energy reads 4 doubles per walker
        eL, _ = ws.lrdmc_energy(ang, self.alat)
        if self._forces is not None:   # jqmc_gfmc.py:1810-2000, weights w
            self._forces.add(ws, w, eL, ang)
        sums = torch.stack([w.sum(), (w * eL).sum(), (w * eL * eL).sum(), total.double().mean()])
        branch_comb(w, zeta, self._chosen, self._cum)
        self._spare.gather_from(ws, self._chosen)
        self.walkers, self._spare = self._spare, self.walkers
        return sums

    def run(self, num_mcmc_steps: int = 50, max_time: int = 86400) -> None:
        """num_mcmc_steps branching cycles, stopping early once max_time seconds have passed."""
        t0 = time.perf_counter()
        for _ in range(num_mcmc_steps):
            if time.perf_counter() - t0 > max_time:
                break
            zeta = float(self._np_rng.random())
            sums = self.run_block(zeta).cpu().numpy()
            self._w_L.append(sums[0] / self.num_walkers)
            self._e_L.append(sums[1] / sums[0])
            self._e_L2.append(sums[2] / sums[0])
            self._proj.append(sums[3])
            self.mcmc_counter += 1

    @property
    def w_L(self) -> np.ndarray:
        return gfmc_G_L(np.asarray(self._w_L, dtype=np.float64).reshape(-1, 1), self.num_gfmc_collect_steps)

    @property
    def bare_w_L(self) -> np.ndarray:
        """The per-step mean walker weights before the G_L products (jqmc_gfmc.py:4599-4601)."""
        return np.asarray(self._w_L, dtype=np.float64).reshape(-1, 1)

    @property
    def e_L(self) -> np.ndarray:
        return np.asarray(self._e_L, dtype=np.float64).reshape(-1, 1)[self.num_gfmc_collect_steps:]

    @property
    def e_L2(self) -> np.ndarray:
        return np.asarray(self._e_L2, dtype=np.float64).reshape(-1, 1)[self.num_gfmc_collect_steps:]

    @property
    def average_projection_counter(self) -> np.ndarray:
        return np.asarray(self._proj, dtype=np.float64)

    def get_E(self, num_mcmc_warmup_steps: int = 50, num_mcmc_bin_blocks: int = 10):
        e, e2, w = self.e_L[num_mcmc_warmup_steps:], self.e_L2[num_mcmc_warmup_steps:], self.w_L[num_mcmc_warmup_steps:]
        return jackknife_energy(e, e2, w, num_mcmc_bin_blocks)

    def get_aF(self, num_mcmc_warmup_steps: int = 50, num_mcmc_bin_blocks: int = 10):
        """(force_mean, force_std), (natom, 3) in Hartree/bohr (jqmc_gfmc.py:2587-2700)."""
        return _gfmc_forces(self, num_mcmc_warmup_steps, num_mcmc_bin_blocks)
