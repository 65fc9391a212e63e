"""J1 / J2 / J3 Jastrow factor data.

Mirrors ``jqmc/jastrow_factor.py``:
  * J1 (jastrow_factor.py:561-645, value 649-726): per electron-nucleus pair
    exp form  -(2Z)^(3/4) (1 - exp(-a (2Z)^(1/4) r)) / (2a),
    pade form -(2Z)^(3/4) r / (2 (1 + a (2Z)^(1/4) r)), Z the effective charge;
  * J2 (jastrow_factor.py:1111-1251): pade r/(2(1+b r)) or exp (1-exp(-b r))/(2b),
    the same for parallel and antiparallel pairs;
  * J3 (jastrow_factor.py:1317-1476, value 1744-1801): j_matrix (n, n+1) over an
    AO set; last column j1 gives sum_i j1 . phi(r_i); the square block J gives
    sum_{i<j same spin} phi_i^T J phi_j + sum_{i up, j dn} phi_i^T J phi_j.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .atomic_orbital import AOs_cart_data, AOs_sphe_data
from .structure import Structure_data


@dataclass(frozen=True)
class Jastrow_one_body_data:
    jastrow_1b_param: float = 1.0
    jastrow_1b_type: str = "exp"
    structure_data: Structure_data = field(default_factory=Structure_data)
    core_electrons: tuple = ()

    def sanity_check(self) -> None:
        if self.jastrow_1b_param < 0.0:
            raise ValueError(f"jastrow_1b_param = {self.jastrow_1b_param} must be non-negative.")
        if self.jastrow_1b_type not in ("exp", "pade"):
            raise ValueError(f"jastrow_1b_type = '{self.jastrow_1b_type}' must be 'exp' or 'pade'.")
        if len(self.core_electrons) != self.structure_data.natom:
            raise ValueError("len(core_electrons) must equal the number of nuclei")

    @property
    def effective_charges(self) -> np.ndarray:
        return np.asarray(self.structure_data.atomic_numbers, dtype=np.float64) - np.asarray(self.core_electrons, dtype=np.float64)


@dataclass(frozen=True)
class Jastrow_two_body_data:
    jastrow_2b_param: float = 1.0
    jastrow_2b_type: str = "pade"

    def sanity_check(self) -> None:
        if self.jastrow_2b_param < 0.0:
            raise ValueError(f"jastrow_2b_param = {self.jastrow_2b_param} must be non-negative.")
        if self.jastrow_2b_type not in ("exp", "pade"):
            raise ValueError(f"jastrow_2b_type = '{self.jastrow_2b_type}' must be 'exp' or 'pade'.")


@dataclass(frozen=True)
class Jastrow_three_body_data:
    orb_data: AOs_sphe_data = field(default_factory=AOs_sphe_data)
    j_matrix: np.ndarray = field(default_factory=lambda: np.zeros((0, 1)))

    def __post_init__(self):
        object.__setattr__(self, "j_matrix", np.asarray(self.j_matrix, dtype=np.float64))

    @property
    def orb_num(self) -> int:
        return self.orb_data.orb_num

    def sanity_check(self) -> None:
        if self.j_matrix.shape != (self.orb_num, self.orb_num + 1):
            raise ValueError(f"dim. of j_matrix = {self.j_matrix.shape} is incompatible with ({self.orb_num}, {self.orb_num + 1})")
        if not isinstance(self.orb_data, (AOs_sphe_data, AOs_cart_data)):
            raise NotImplementedError("the J3 basis must be an AO set (spherical or Cartesian) on the walker path")


@dataclass(frozen=True)
class Jastrow_data:
    jastrow_one_body_data: Jastrow_one_body_data | None = None
    jastrow_two_body_data: Jastrow_two_body_data | None = None
    jastrow_three_body_data: Jastrow_three_body_data | None = None
    jastrow_nn_data: object | None = None

    def sanity_check(self) -> None:
        if self.jastrow_nn_data is not None:
            raise NotImplementedError("the neural-network Jastrow is not on the walker path")
        for part in (self.jastrow_one_body_data, self.jastrow_two_body_data, self.jastrow_three_body_data):
            if part is not None:
                part.sanity_check()


# ---------------------------------------------------------------- evaluation (GPU: jqmc_log_psi's Jastrow output)
def _compute_ratio_Jastrow_part_rank1_update(jastrow_data: Jastrow_data, old_r_up_carts, old_r_dn_carts,
                                             new_r_up_carts_arr, new_r_dn_carts_arr, j3_state=None) -> np.ndarray:
    """exp(J(r') - J(r)) for G configurations r' (G, n, 3) against r
    (jqmc/jastrow_factor.py:2230-2693): J of all G + 1 configurations in one GPU
    evaluation.  j3_state (the reference's streaming cache) is accepted and not
    needed."""
    import torch

    from . import surface
    ou, od = np.asarray(old_r_up_carts, dtype=np.float64), np.asarray(old_r_dn_carts, dtype=np.float64)
    nu, nd = np.asarray(new_r_up_carts_arr, dtype=np.float64), np.asarray(new_r_dn_carts_arr, dtype=np.float64)
    if nu.ndim != 3 or nd.ndim != 3 or nu.shape[0] != nd.shape[0] or nu.shape[1:] != ou.shape or nd.shape[1:] != od.shape:
        raise ValueError(f"new configurations {nu.shape}, {nd.shape} do not match the old ones {ou.shape}, {od.shape}")
    jj, _ = surface.jastrow_value(jastrow_data, np.concatenate([ou[None], nu]), np.concatenate([od[None], nd]))
    return surface.as_numpy(torch.exp(jj[1:] - jj[0]))


def compute_Jastrow_part(jastrow_data: Jastrow_data, r_up_carts, r_dn_carts):
    """J = J1 + J2 + J3, without exp (jqmc/jastrow_factor.py:2127)."""
    from . import surface
    jj, single = surface.jastrow_value(jastrow_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(jj, single)


def compute_Jastrow_one_body(jastrow_one_body_data: Jastrow_one_body_data, r_up_carts, r_dn_carts):
    """J1 without exp (jqmc/jastrow_factor.py:649)."""
    from . import surface
    jj, single = surface.jastrow_value(Jastrow_data(jastrow_one_body_data=jastrow_one_body_data), r_up_carts, r_dn_carts,
                                       key_obj=jastrow_one_body_data)
    return surface.scalar_or_array(jj, single)


def compute_Jastrow_two_body(jastrow_two_body_data: Jastrow_two_body_data, r_up_carts, r_dn_carts):
    """J2 without exp (jqmc/jastrow_factor.py:1181)."""
    from . import surface
    jj, single = surface.jastrow_value(Jastrow_data(jastrow_two_body_data=jastrow_two_body_data), r_up_carts, r_dn_carts,
                                       key_obj=jastrow_two_body_data)
    return surface.scalar_or_array(jj, single)


def compute_Jastrow_three_body(jastrow_three_body_data: Jastrow_three_body_data, r_up_carts, r_dn_carts):
    """J3 without exp (jqmc/jastrow_factor.py:1744)."""
    from . import surface
    jj, single = surface.jastrow_value(Jastrow_data(jastrow_three_body_data=jastrow_three_body_data), r_up_carts,
                                       r_dn_carts, key_obj=jastrow_three_body_data)
    return surface.scalar_or_array(jj, single)


def compute_grads_and_laplacian_Jastrow_part(jastrow_data: Jastrow_data, r_up_carts, r_dn_carts):
    """(grad J up (n_up, 3), down (n_dn, 3), lap J up (n_up,), down (n_dn,))
    (jqmc/jastrow_factor.py:2983), from the walker kernels (jqmc_electron_terms)."""
    from . import surface
    n_up, n_dn = np.shape(r_up_carts)[-2], np.shape(r_dn_carts)[-2]
    a, n = surface.electron_tables(surface.jastrow_system(jastrow_data, n_up, n_dn), r_up_carts, r_dn_carts)
    return a[..., :n, 4:7], a[..., n:, 4:7], a[..., :n, 7], a[..., n:, 7]
