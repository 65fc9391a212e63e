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

    @property
    def is_mo_representation(self) -> bool:
        return isinstance(self.orb_data_up_spin, MOs_data) and isinstance(self.orb_data_dn_spin, MOs_data)

    @property
    def is_ao_representation(self) -> bool:
        return not isinstance(self.orb_data_up_spin, MOs_data) and not isinstance(self.orb_data_dn_spin, MOs_data)

    def symmetrize_lambda(self, mat):
        """(A + A^T)/2 on the paired block when the current lambda's paired block is
        symmetric (atol 1e-8, rtol 1e-6), else mat unchanged (determinant.py:332-380)."""
        from .variational import _lambda_paired_columns, _symmetrize_leading_square
        mat = np.asarray(mat, dtype=np.float64)
        return _symmetrize_leading_square(mat.shape, _lambda_paired_columns(self.lambda_matrix))(mat)

    def to_spherical(self) -> "Geminal_data":
        """Spherical orbitals (determinant.py:587-626): MOs through
        MOs_data.to_spherical with lambda unchanged; Cartesian AOs through the
        basis conversion, lambda_paired -> P_up^T lambda P_dn and lambda_unpaired ->
        P_up^T lambda (P the pseudo-inverse maps of aos_cart_to_sphe)."""
        from .atomic_orbital import aos_cart_to_sphe
        up, dn = self.orb_data_up_spin, self.orb_data_dn_spin
        if isinstance(up, MOs_data) or isinstance(dn, MOs_data):
            if not self.is_mo_representation:
                raise ValueError("Spherical conversion requires both spin channels to use MOs or both to use AOs.")
            return Geminal_data(self.num_electron_up, self.num_electron_dn, up.to_spherical(), dn.to_spherical(),
                                self.lambda_matrix)
        if isinstance(up, AOs_sphe_data) and isinstance(dn, AOs_sphe_data):
            return self
        sph_up, p_up = aos_cart_to_sphe(up)
        sph_dn, p_dn = aos_cart_to_sphe(dn)
        lp, lu = self.lambda_matrix[:, : self.orb_num_dn], self.lambda_matrix[:, self.orb_num_dn:]
        lam = np.hstack([p_up.T @ lp @ p_dn, p_up.T @ lu])
        return Geminal_data(self.num_electron_up, self.num_electron_dn, sph_up, sph_dn, lam)

    @classmethod
    def convert_from_MOs_to_AOs(cls, geminal_data: "Geminal_data") -> "Geminal_data":
        """The same geminal over the AOs: lambda_AO = C_up^T lambda C_dn (paired) and
        C_up^T lambda (unpaired) (determinant.py:687-722); AO geminals are returned as they are."""
        if geminal_data.is_ao_representation:
            return geminal_data
        if not geminal_data.is_mo_representation:
            raise NotImplementedError("mixed MO/AO geminals")
        aos, lp, lu = geminal_data.ao_basis_lambda()
        return cls(geminal_data.num_electron_up, geminal_data.num_electron_dn, aos,
                   geminal_data.orb_data_dn_spin.aos_data, np.hstack([lp, lu]))

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


def _geminal_ao_parts(geminal_data: Geminal_data):
    """(up AOs, down AOs, lambda paired, lambda unpaired) with any MO layer folded into lambda."""
    aos_up, lp, lu = geminal_data.ao_basis_lambda()
    dn = geminal_data.orb_data_dn_spin
    return aos_up, (dn.aos_data if isinstance(dn, MOs_data) else dn), lp, lu


def compute_geminal_up_one_row_elements(geminal_data: Geminal_data, r_up_cart, r_dn_carts) -> np.ndarray:
    """Row of G for one up electron at r_up_cart (1, 3): phi_up(r)^T lambda_paired
    phi_dn(r_dn) followed by phi_up(r)^T lambda_unpaired, shape (N_dn + N_unpaired,)
    (jqmc/determinant.py:1430-1478); AO values from the GPU (jqmc_ao_vgl)."""
    import torch

    from . import surface
    aos_up, aos_dn, lp, lu = _geminal_ao_parts(geminal_data)
    pu = surface.ao_vgl(aos_up, np.asarray(r_up_cart, dtype=np.float64).reshape(1, 3))[0][:, 0]
    t = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device=pu.device)   # noqa: E731
    r_dn = np.asarray(r_dn_carts, dtype=np.float64).reshape(-1, 3)
    paired = pu @ t(lp) @ surface.ao_vgl(aos_dn, r_dn)[0] if len(r_dn) else pu.new_zeros(0)
    return surface.as_numpy(torch.cat([paired, pu @ t(lu)]))


def compute_geminal_dn_one_column_elements(geminal_data: Geminal_data, r_up_carts, r_dn_cart) -> np.ndarray:
    """Column of G for one down electron at r_dn_cart (1, 3): phi_up(r_up)^T
    lambda_paired phi_dn(r), shape (N_up,) (jqmc/determinant.py:1482-1526)."""
    import torch

    from . import surface
    aos_up, aos_dn, lp, _ = _geminal_ao_parts(geminal_data)
    pd = surface.ao_vgl(aos_dn, np.asarray(r_dn_cart, dtype=np.float64).reshape(1, 3))[0][:, 0]
    pu = surface.ao_vgl(aos_up, np.asarray(r_up_carts, dtype=np.float64).reshape(-1, 3))[0]
    return surface.as_numpy(pu.T @ torch.as_tensor(np.asarray(lp, dtype=np.float64), device=pd.device) @ pd)


def _compute_ratio_determinant_part_rank1_update(geminal_data: Geminal_data, A_old_inv, old_r_up_carts, old_r_dn_carts,
                                                 new_r_up_carts_arr, new_r_dn_carts_arr) -> np.ndarray:
    """det G(r')/det G(r) for G configurations r' (G, n, 3) that each move one
    electron (determinant.py:1530-1662): the new row (up move) or column (down
    move) times the matching column or row of A_old_inv = G(r)^-1.  The AO
    values of all moved electrons come from two GPU calls; a configuration that
    moves no electron has ratio 1."""
    import torch

    from . import surface
    aos_up, aos_dn, lp, lu = _geminal_ao_parts(geminal_data)
    ou, od = np.asarray(old_r_up_carts, dtype=np.float64), np.asarray(old_r_dn_carts, dtype=np.float64)
    nu, nd = np.asarray(new_r_up_carts_arr, dtype=np.float64), np.asarray(new_r_dn_carts_arr, dtype=np.float64)
    if nu.ndim != 3 or nd.ndim != 3 or nu.shape[0] != nd.shape[0] or nu.shape[1:] != ou.shape or nd.shape[1:] != od.shape:
        raise ValueError(f"new configurations {nu.shape}, {nd.shape} do not match the old ones {ou.shape}, {od.shape}")
    G = nu.shape[0]
    mu = np.any(nu != ou[None], axis=-1)             # (G, n_up) moved up electrons
    md = np.any(nd != od[None], axis=-1)
    if np.any(mu.sum(1) + md.sum(1) > 1):
        raise ValueError("each new configuration must move one electron")
    gu, iu = np.nonzero(mu)
    gd, jd = np.nonzero(md)
    out = np.ones(G)
    if len(gu) == 0 and len(gd) == 0:
        return out
    dev = None
    if len(gu):
        pu = surface.ao_vgl(aos_up, nu[gu, iu])[0]                      # (A, K_up)
        dev = pu.device
    if len(gd):
        pdn = surface.ao_vgl(aos_dn, nd[gd, jd])[0]                     # (A, K_dn)
        dev = pdn.device
    t = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device=dev)   # noqa: E731
    Ginv = t(A_old_inv)
    if len(gu):
        paired = pu.T @ t(lp) @ surface.ao_vgl(aos_dn, od)[0] if len(od) else pu.new_zeros((pu.shape[1], 0))
        rows = torch.cat([paired, pu.T @ t(lu)], dim=1)                 # (K_up, n_up)
        out[gu] = surface.as_numpy((rows * Ginv[:, torch.as_tensor(iu, device=dev)].T).sum(1))
    if len(gd):
        cols = surface.ao_vgl(aos_up, ou)[0].T @ t(lp) @ pdn            # (n_up, K_dn)
        out[gd] = surface.as_numpy((Ginv[torch.as_tensor(jd, device=dev), :] * cols.T).sum(1))
    return out


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
