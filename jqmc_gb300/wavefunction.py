"""Wavefunction = Jastrow x geminal; mirrors ``Wavefunction_data`` (jqmc/wavefunction.py:248)."""

from __future__ import annotations

from dataclasses import dataclass, field

from .determinant import Geminal_data
from .jastrow_factor import Jastrow_data


@dataclass(frozen=True)
class Wavefunction_data:
    jastrow_data: Jastrow_data = field(default_factory=Jastrow_data)
    geminal_data: Geminal_data = field(default_factory=Geminal_data)

    def sanity_check(self) -> None:
        self.jastrow_data.sanity_check()
        self.geminal_data.sanity_check()

    def get_variational_blocks(self, **flags) -> list:
        """Variational parameter blocks (jqmc/wavefunction.py:515); flags opt_J1_param,
        opt_J2_param, opt_J3_param, opt_JNN_param, opt_lambda_param and the AO-basis flags."""
        from .variational import get_variational_blocks
        return get_variational_blocks(self, **flags)

    def apply_block_updates(self, blocks: list, thetas, learning_rate: float) -> "Wavefunction_data":
        """The wavefunction with every block moved by learning_rate * its slice of thetas
        (jqmc/wavefunction.py:292)."""
        from .variational import apply_block_updates
        return apply_block_updates(self, blocks, thetas, learning_rate)


# ---------------------------------------------------------------- evaluation (GPU: walker initialisation + jqmc_log_psi / jqmc_vmc_measure)
def evaluate_ln_wavefunction(wavefunction_data: Wavefunction_data, r_up_carts, r_dn_carts):
    """ln|psi| = ln|det G| + J (jqmc/wavefunction.py:678)."""
    from . import surface
    ld, _, jj, single = surface.wavefunction_parts(wavefunction_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(ld + jj, single)


def evaluate_wavefunction(wavefunction_data: Wavefunction_data, r_up_carts, r_dn_carts):
    """psi = sign(det G) exp(ln|det G| + J) (jqmc/wavefunction.py:779)."""
    from . import surface
    ld, sg, jj, single = surface.wavefunction_parts(wavefunction_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(sg * (ld + jj).exp(), single)


def evaluate_jastrow(wavefunction_data: Wavefunction_data, r_up_carts, r_dn_carts):
    """exp(J) (jqmc/wavefunction.py:817)."""
    from . import surface
    _, _, jj, single = surface.wavefunction_parts(wavefunction_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(jj.exp(), single)


def evaluate_determinant(wavefunction_data: Wavefunction_data, r_up_carts, r_dn_carts):
    """det G (jqmc/wavefunction.py:846)."""
    from . import surface
    ld, sg, _, single = surface.wavefunction_parts(wavefunction_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(sg * ld.exp(), single)


def compute_kinetic_energy(wavefunction_data: Wavefunction_data, r_up_carts, r_dn_carts):
    """-1/2 sum_i lap_i psi / psi (jqmc/wavefunction.py:872)."""
    from . import surface
    t, single = surface.kinetic_energy(wavefunction_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(t, single)


def evaluate_ln_wavefunction_fast(wavefunction_data: Wavefunction_data, r_up_carts, r_dn_carts, geminal_inv):
    """ln|psi| with a precomputed geminal inverse (jqmc/wavefunction.py:723): the same value as
    ``evaluate_ln_wavefunction``; ``geminal_inv`` is accepted and not read."""
    return evaluate_ln_wavefunction(wavefunction_data, r_up_carts, r_dn_carts)


def compute_kinetic_energy_all_elements(wavefunction_data: Wavefunction_data, r_up_carts, r_dn_carts):
    """Per-electron kinetic energies (T up (n_up,), T down (n_dn,)) (jqmc/wavefunction.py:1081),
    from the walker kernels (jqmc_electron_terms)."""
    from . import surface
    a, n = surface.electron_tables(surface.wavefunction_system(wavefunction_data), r_up_carts, r_dn_carts)
    return a[..., :n, 8], a[..., n:, 8]


def compute_discretized_kinetic_energy(alat: float, wavefunction_data: Wavefunction_data, r_up_carts, r_dn_carts, RT):
    """(r_up configurations (6N, n_up, 3), r_dn configurations (6N, n_dn, 3), elements
    (6N,)) of the six moves +-alat along the rows of RT for every electron, up
    electrons first; elements -psi(r')/psi(r) / (2 alat^2) (jqmc/wavefunction.py:1620),
    from the walker kernels (jqmc_kinetic_mesh)."""
    from . import surface
    return surface.discretized_kinetic(alat, wavefunction_data, r_up_carts, r_dn_carts, RT)
