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

    def to_spherical(self) -> "MOs_data":
        """The MOs over spherical AOs (molecular_orbital.py:214-236): a Cartesian
        basis becomes its spherical shells and C_sph = C_cart transform_pinv
        (atomic_orbital.aos_cart_to_sphe); a spherical set is returned as it is.
        This is how a Cartesian TREXIO wavefunction reaches the walker kernels."""
        from .atomic_orbital import aos_cart_to_sphe
        if isinstance(self.aos_data, AOs_sphe_data):
            return self
        sph, pinv = aos_cart_to_sphe(self.aos_data)
        return MOs_data(num_mo=self.num_mo, aos_data=sph, mo_coefficients=self.mo_coefficients @ pinv)


# ---------------------------------------------------------------- evaluation (GPU: AO tables, then C x AO)
def compute_MOs(mos_data: MOs_data, r_carts) -> np.ndarray:
    """MO values (num_mo, N) at r_carts (N, 3) (jqmc/molecular_orbital.py:240)."""
    from . import surface
    return surface.as_numpy(surface.mo_vgl(mos_data, r_carts)[0])


def compute_MOs_grad(mos_data: MOs_data, r_carts):
    """(d/dx, d/dy, d/dz) of the MOs, each (num_mo, N) (jqmc/molecular_orbital.py)."""
    from . import surface
    t = surface.as_numpy(surface.mo_vgl(mos_data, r_carts))
    return t[1], t[2], t[3]


def compute_MOs_laplacian(mos_data: MOs_data, r_carts) -> np.ndarray:
    """Laplacians of the MOs (num_mo, N) (jqmc/molecular_orbital.py)."""
    from . import surface
    return surface.as_numpy(surface.mo_vgl(mos_data, r_carts)[4])


def compute_MOs_value_grad_lap(mos_data: MOs_data, r_carts):
    """(val, gx, gy, gz, lap) of the MOs, each (num_mo, N) (jqmc/molecular_orbital.py)."""
    from . import surface
    t = surface.as_numpy(surface.mo_vgl(mos_data, r_carts))
    return t[0], t[1], t[2], t[3], t[4]
