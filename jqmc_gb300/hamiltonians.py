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
