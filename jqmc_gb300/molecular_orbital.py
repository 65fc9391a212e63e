"""Molecular orbitals as a linear map of AOs.

Mirrors ``jqmc/molecular_orbital.py``: ``MOs_data`` (molecular_orbital.py:86-140)
and ``compute_MOs`` (molecular_orbital.py:240-261), MO = C (n_mo x n_ao) @ AO.
On the walker path a geminal written over MOs is folded into an AO-basis
pairing matrix ``lambda_AO = C_up^T lambda_MO C_dn`` once at set-up, so the
kernels only ever see AO tables.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .atomic_orbital import AOs_sphe_data


@dataclass(frozen=True)
class MOs_data:
    """Field-for-field mirror of ``MOs_data`` (molecular_orbital.py:133-140)."""

    num_mo: int = 0
    aos_data: AOs_sphe_data = field(default_factory=AOs_sphe_data)
    mo_coefficients: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))

    def __post_init__(self):
        object.__setattr__(self, "mo_coefficients", np.asarray(self.mo_coefficients, dtype=np.float64))

    @property
    def orb_num(self) -> int:
        return self.num_mo

    def sanity_check(self) -> None:
        if self.mo_coefficients.shape != (self.num_mo, self.aos_data.num_ao):
            raise ValueError(f"mo_coefficients.shape={self.mo_coefficients.shape} != ({self.num_mo}, {self.aos_data.num_ao})")
        self.aos_data.sanity_check()
