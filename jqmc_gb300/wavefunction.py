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
