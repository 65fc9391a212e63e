"""Host-side statistics of the drivers (small arrays; NumPy).

* ``jackknife_energy`` -- binned weighted jackknife of jqmc_mcmc.py:1064-1189
  (MCMC.get_E) and jqmc_gfmc.py:6500-6600 (GFMC_n.get_E, one process).
* ``gfmc_G_L`` -- products of the last ``num_gfmc_collect_steps`` averaged
  weights, jqmc_gfmc.py:136-152.
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
