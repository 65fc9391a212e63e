"""Host-side statistics of the drivers (small arrays; NumPy).

* ``jackknife_energy`` -- binned weighted jackknife of jqmc_mcmc.py:1064-1189
  (MCMC.get_E) and jqmc_gfmc.py:6500-6600 (GFMC_n.get_E, one process).
* ``gfmc_G_L`` -- products of the last ``num_gfmc_collect_steps`` averaged
  weights, jqmc_gfmc.py:136-152.
* ``jackknife_force`` -- forces, jqmc_mcmc.py:1191-1380.
* ``jackknife_generalized_force`` -- dE/dc of the variational parameters,
  jqmc_mcmc.py:1515-1700 (MCMC.get_gF, one process).
"""

from __future__ import annotations

import numpy as np


def jackknife_energy(e_L: np.ndarray, e_L2: np.ndarray, w_L: np.ndarray, num_bin_blocks: int):
    """(E_mean, E_std, Var_mean, Var_std) from (M, nw) arrays of samples."""
    M = e_L.shape[0]
    if M < num_bin_blocks:
        raise ValueError(f"{M} samples cannot form {num_bin_blocks} bins")
    wb = np.ravel([np.sum(a, axis=0) for a in np.array_split(w_L, num_bin_blocks, axis=0)])
    web = np.ravel([np.sum(a, axis=0) for a in np.array_split(w_L * e_L, num_bin_blocks, axis=0)])
    we2b = np.ravel([np.sum(a, axis=0) for a in np.array_split(w_L * e_L2, num_bin_blocks, axis=0)])
    ws, wes, we2s = np.sum(wb), np.sum(web), np.sum(we2b)
    Mt = wb.size
    Ej = (wes - web) / (ws - wb)
    E2j = (we2s - we2b) / (ws - wb)
    Vj = E2j - Ej**2
    E_mean = np.sum(Ej) / Mt
    E_std = np.sqrt((Mt - 1) * np.sum((Ej - E_mean) ** 2) / Mt)
    V_mean = np.sum(Vj) / Mt
    V_std = np.sqrt((Mt - 1) * np.sum((Vj - V_mean) ** 2) / Mt)
    return float(E_mean), float(E_std), float(V_mean), float(V_std)


def gfmc_G_L(w_L: np.ndarray, num_gfmc_collect_steps: int) -> np.ndarray:
    """G_L[k] = prod_{j=k}^{k+n-1} w_L[j] for k = 0 .. A-n-1 (rows n..A-1 of the reference)."""
    A = w_L.shape[0]
    n = num_gfmc_collect_steps
    return np.stack([np.prod(w_L[k - n:k], axis=0) for k in range(n, A)]) if A > n else np.zeros((0,) + w_L.shape[1:])


def jackknife_force(w_L: np.ndarray, e_L: np.ndarray, force_HF: np.ndarray, force_PP: np.ndarray,
                    E_L_force_PP: np.ndarray, num_bin_blocks: int):
    """(force_mean, force_std), each (natom, 3), from (M, nw) weights and energies
    and (M, nw, natom, 3) per-walker force terms: F = -<force_HF> - 2 (<E_L force_PP>
    - <E_L> <force_PP>), jackknife over (bin, walker) samples (jqmc_mcmc.py:1191-1380)."""
    M = e_L.shape[0]
    if M < num_bin_blocks:
        raise ValueError(f"{M} samples cannot form {num_bin_blocks} bins")

    def binned(x):
        return np.concatenate([np.sum(a, axis=0) for a in np.array_split(x, num_bin_blocks, axis=0)], axis=0)

    wb = binned(w_L)                                          # (bins * nw,)
    web = binned(w_L * e_L)
    fhb = binned(np.einsum("iw,iwjk->iwjk", w_L, force_HF))   # (bins * nw, natom, 3)
    fpb = binned(np.einsum("iw,iwjk->iwjk", w_L, force_PP))
    efb = binned(np.einsum("iw,iwjk->iwjk", w_L, E_L_force_PP))
    ws, wes = wb.sum(), web.sum()
    fhs, fps, efs = fhb.sum(axis=0), fpb.sum(axis=0), efb.sum(axis=0)
    den = (ws - wb)[:, None, None]
    f_hf = -(fhs[None] - fhb) / den
    f_pulay = -2.0 * ((efs[None] - efb) / den - ((wes - web)[:, None, None] / den) * ((fps[None] - fpb) / den))
    fj = f_hf + f_pulay
    Mt = fj.shape[0]
    mean = fj.mean(axis=0)
    std = np.sqrt((Mt - 1) / Mt * np.sum((fj - mean) ** 2, axis=0))
    return mean, std


def jackknife_generalized_force(w_L: np.ndarray, e_L: np.ndarray, O: np.ndarray, num_bin_blocks: int):
    """(f_mean, f_std), each (K,), from (M, nw) weights and energies and (M, nw, K)
    derivatives d ln psi / dc: f = -2 (<e_L O> - <e_L> <O>), jackknife over the
    (bin, walker) samples with a centred second pass for the spread."""
    M = e_L.shape[0]
    if M < num_bin_blocks:
        raise ValueError(f"{M} samples cannot form {num_bin_blocks} bins")
    if O.shape[:2] != e_L.shape or w_L.shape != e_L.shape:
        raise ValueError(f"shapes w_L {w_L.shape}, e_L {e_L.shape} and O {O.shape} disagree")

    def binned(x):
        return np.concatenate([np.sum(a, axis=0) for a in np.array_split(x, num_bin_blocks, axis=0)], axis=0)

    wb = binned(w_L)                                 # (bins * nw,)
    web = binned(w_L * e_L)
    wOb = binned(w_L[:, :, None] * O)                # (bins * nw, K)
    weOb = binned((w_L * e_L)[:, :, None] * O)
    den = wb.sum() - wb
    eO_j = (weOb.sum(axis=0)[None] - weOb) / den[:, None]
    e_j = (web.sum() - web) / den
    O_j = (wOb.sum(axis=0)[None] - wOb) / den[:, None]
    fj = -2.0 * (eO_j - e_j[:, None] * O_j)
    Mt = fj.shape[0]
    mean = fj.sum(axis=0) / Mt
    var = np.sum((fj - mean) ** 2, axis=0) / Mt
    return mean, np.sqrt((Mt - 1) * var)
