"""Geminal (AGP / Slater) determinant part of the wavefunction.

Mirrors ``jqmc/determinant.py``: ``Geminal_data`` (determinant.py:94-141).  The
geminal matrix is G_ij = phi_up(r_i)^T lambda_paired phi_dn(r_j), with the
unpaired block phi_up(r_i)^T lambda_unpaired for N_up > N_dn
(_compute_geminal_all_elements, determinant.py:1380-1402).

The walker kernels hold, per walker, G^-1 and the two "ratio tables"
T_up = lambda phi_dn G^-1 and T_dn = G^-1 phi_up^T lambda.  With them the ratio
for moving up-electron i to r' is phi(r') . T_up[:, i] and the gradient of
ln det for electron i is grad phi(r_i) . T_up[:, i]; both are the same numbers
the reference obtains from the row/column rebuild of determinant.py:1430-1526
and the traces of determinant.py:2141-2250.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .atomic_orbital import AOs_sphe_data
from .molecular_orbital import MOs_data


@dataclass(frozen=True)
class Geminal_data:
    """Field-for-field mirror of ``Geminal_data`` (determinant.py:110-120)."""

    num_electron_up: int = 0
    num_electron_dn: int = 0
    orb_data_up_spin: AOs_sphe_data | MOs_data = field(default_factory=AOs_sphe_data)
    orb_data_dn_spin: AOs_sphe_data | MOs_data = field(default_factory=AOs_sphe_data)
    lambda_matrix: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))

    def __post_init__(self):
        object.__setattr__(self, "lambda_matrix", np.asarray(self.lambda_matrix, dtype=np.float64))

    @property
    def orb_num_up(self) -> int:
        return self.orb_data_up_spin.orb_num

    @property
    def orb_num_dn(self) -> int:
        return self.orb_data_dn_spin.orb_num

    def sanity_check(self) -> None:
        """Same checks and messages as determinant.py:122-141."""
        if self.orb_num_up != self.orb_num_dn:
            raise ValueError(f"The number of up and down orbitals ({self.orb_num_up}, {self.orb_num_dn}) should be the same.")
        exp_shape = (self.orb_num_up, self.orb_num_dn + (self.num_electron_up - self.num_electron_dn))
        if self.lambda_matrix.shape != exp_shape:
            raise ValueError(f"dim. of lambda_matrix = {self.lambda_matrix.shape} is incompatible with {exp_shape}.")
        if self.num_electron_up < self.num_electron_dn:
            raise ValueError("Number of up electrons must not be smaller than dn electrons.")

    def ao_basis_lambda(self):
        """(aos_data, lambda_paired_AO, lambda_unpaired_AO) with any MO layer folded
        into the pairing matrix: lambda_AO = C_up^T lambda C_dn."""
        lam = self.lambda_matrix
        lp, lu = lam[:, : self.orb_num_dn], lam[:, self.orb_num_dn:]
        up, dn = self.orb_data_up_spin, self.orb_data_dn_spin
        if isinstance(up, MOs_data):
            cu = up.mo_coefficients
            cd = dn.mo_coefficients
            return up.aos_data, cu.T @ lp @ cd, cu.T @ lu
        return up, lp, lu


# ---------------------------------------------------------------- evaluation (GPU: walker initialisation + jqmc_log_psi)
def compute_geminal_all_elements(geminal_data: Geminal_data, r_up_carts, r_dn_carts) -> np.ndarray:
    """The geminal matrix G (n_up, n_dn) (jqmc/determinant.py:1336); (W, n_up, n_dn) for (W, n, 3) inputs."""
    from . import surface
    _, _, G, single = surface.geminal_log_det(geminal_data, r_up_carts, r_dn_carts)
    g = surface.as_numpy(G)
    return g[0] if single else g


def compute_ln_det_geminal_all_elements(geminal_data: Geminal_data, r_up_carts, r_dn_carts):
    """ln|det G| (jqmc/determinant.py:1028)."""
    from . import surface
    ld, _, _, single = surface.geminal_log_det(geminal_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(ld, single)


def compute_det_geminal_all_elements(geminal_data: Geminal_data, r_up_carts, r_dn_carts):
    """det G (jqmc/determinant.py:1186)."""
    from . import surface
    ld, sg, _, single = surface.geminal_log_det(geminal_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(sg * ld.exp(), single)


def compute_AS_regularization_factor(geminal_data: Geminal_data, r_up_carts, r_dn_carts):
    """Attaccalite-Sorella regularization factor (jqmc/determinant.py:1291)."""
    from . import surface
    R, single = surface.geminal_as_factor(geminal_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(R, single)


def compute_AS_regularization_factor_fast_update(geminal, geminal_inv):
    """The same factor from a given G and G^-1, (n, n) or (W, n, n) (jqmc/determinant.py:1223),
    evaluated on the GPU."""
    import torch

    from . import surface
    if not torch.cuda.is_available():
        raise surface.JqmcError("no CUDA device: the walker path runs only on the GPU")
    G = torch.as_tensor(np.asarray(geminal, dtype=np.float64), device="cuda")
    Gi = torch.as_tensor(np.asarray(geminal_inv, dtype=np.float64), device="cuda")
    single = G.ndim == 2
    if single:
        G, Gi = G[None], Gi[None]
    return surface.scalar_or_array(surface.as_factor(G, Gi), single)


def compute_grads_and_laplacian_ln_Det(geminal_data: Geminal_data, r_up_carts, r_dn_carts):
    """(grad ln|det| up (n_up, 3), down (n_dn, 3), lap ln|det| up (n_up,), down (n_dn,))
    (jqmc/determinant.py:1809), from the walker kernels (jqmc_electron_terms)."""
    from . import surface
    a, n = surface.electron_tables(surface.geminal_system(geminal_data), r_up_carts, r_dn_carts)
    return a[..., :n, 0:3], a[..., n:, 0:3], a[..., :n, 3], a[..., n:, 3]
