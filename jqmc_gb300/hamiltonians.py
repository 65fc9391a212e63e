"""Hamiltonian = structure + Coulomb/ECP + wavefunction; mirrors ``Hamiltonian_data`` (jqmc/hamiltonians.py:83)."""

from __future__ import annotations

from dataclasses import dataclass, field

from .coulomb_potential import Coulomb_potential_data
from .structure import Structure_data
from .wavefunction import Wavefunction_data


@dataclass(frozen=True)
class Hamiltonian_data:
    structure_data: Structure_data = field(default_factory=Structure_data)
    coulomb_potential_data: Coulomb_potential_data = field(default_factory=Coulomb_potential_data)
    wavefunction_data: Wavefunction_data = field(default_factory=Wavefunction_data)

    def sanity_check(self) -> None:
        self.structure_data.sanity_check()
        self.coulomb_potential_data.sanity_check()
        self.wavefunction_data.sanity_check()


# ---------------------------------------------------------------- evaluation (GPU: walker initialisation + jqmc_vmc_measure)
def compute_local_energy(hamiltonian_data: Hamiltonian_data, r_up_carts, r_dn_carts, RT):
    """E_L with the non-local ECP quadrature rotated by RT (jqmc/hamiltonians.py:179);
    RT (3, 3) or one per configuration (W, 3, 3)."""
    from . import surface
    eL, single = surface.local_energy(hamiltonian_data, r_up_carts, r_dn_carts, RT)
    return surface.scalar_or_array(eL, single)


def compute_local_energy_fast(hamiltonian_data: Hamiltonian_data, r_up_carts, r_dn_carts, RT, geminal_inverse):
    """E_L with a precomputed geminal inverse (jqmc/hamiltonians.py:225): the same value as
    ``compute_local_energy``; the walker kernels form the inverse themselves, so
    ``geminal_inverse`` is accepted and not read."""
    return compute_local_energy(hamiltonian_data, r_up_carts, r_dn_carts, RT)
