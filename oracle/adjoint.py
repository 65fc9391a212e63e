"""Oracle: derivatives of ln|psi| with respect to the variational parameters (FP64).

Test infrastructure only (the GPU path never imports it).  Restates, per walker,
the gradient blocks the reference collects from grad(evaluate_ln_wavefunction):
  * block names and shapes   wavefunction.py:515-676 (get_variational_blocks),
                             jastrow_factor.py:2110-2124, determinant.py:389-399
                             (collect_param_grads), gathered per walker in
                             jqmc_mcmc.py:856-876
  * ln|psi| = ln|det G| + J1 + J2 + J3   wavefunction.py:723 (evaluate_ln_wavefunction)
The reference obtains these by automatic differentiation; here they are the
closed-form derivatives of the same functions (J1 jastrow_factor.py:649-726, J2
:1181-1251, J3 :1744-1801, geminal determinant.py:1380-1402), pinned by central
finite differences of ln|psi| (``fd_dlnpsi_dparams``).
"""

from __future__ import annotations

import copy

import numpy as np

from .ao import ao_value


def ln_psi(o, r_up, r_dn) -> float:
    _, ld = o.ln_det(r_up, r_dn)
    return float(ld + o.jastrow_total(r_up, r_dn))


def dlnpsi_dparams(o, r_up, r_dn) -> dict:
    """{"j1_param": float, "j2_param": float, "j3_matrix": (A3, A3+1), "lambda_matrix": lambda's shape}."""
    out = {}
    r = np.vstack([r_up, r_dn])
    if o.j1 is not None:
        Z, a = o.j1_Z, o.j1_a
        c = (2.0 * Z) ** 0.25
        A = (2.0 * Z) ** 0.75
        d = np.linalg.norm(r[:, None, :] - o.R[None], axis=-1)          # (N, M)
        if o.j1.jastrow_1b_type == "exp":
            ex = np.exp(-a * c[None] * d)
            dfa = -A[None] * (c[None] * d * ex / (2.0 * a) - (1.0 - ex) / (2.0 * a * a))
        else:
            q = 1.0 + a * c[None] * d
            dfa = A[None] * c[None] * d * d / (2.0 * q * q)
        out["j1_param"] = float(np.sum(dfa))
    if o.j2 is not None:
        b = o.j2_b
        iu, ju = np.triu_indices(len(r), k=1)
        rij = np.linalg.norm(r[iu] - r[ju], axis=-1)
        if o.j2.jastrow_2b_type == "pade":
            dfb = -rij * rij / (2.0 * (1.0 + b * rij) ** 2)
        else:
            ex = np.exp(-b * rij)
            dfb = rij * ex / (2.0 * b) - (1.0 - ex) / (2.0 * b * b)
        out["j2_param"] = float(np.sum(dfb))
    if o.j3 is not None:
        au, ad = ao_value(o.tab_j3, r_up), ao_value(o.tab_j3, r_dn)     # (A3, n)
        A3 = au.shape[0]
        D = np.zeros((A3, A3 + 1))
        for x in (au, ad):
            pfx = np.cumsum(x, axis=1) - x                                # sum over p < q
            D[:, :A3] += pfx @ x.T
        su, sd = au.sum(1), ad.sum(1)
        D[:, :A3] += np.outer(su, sd)
        D[:, A3] = su + sd
        out["j3_matrix"] = D
    G = o.geminal(r_up, r_dn)
    Gi = np.linalg.inv(G)
    pu, pd = o.orb_up(r_up), o.orb_dn(r_dn)                               # (n_orb, n)
    dp = pu @ Gi.T @ pd.T                                                 # d ln det / d lam_p
    du = pu @ Gi.T[:, pd.shape[1]:] if o.lam_u.shape[1] else np.zeros((pu.shape[0], 0))
    out["lambda_matrix"] = np.hstack([dp, du])
    return out


def _with(o, **kw):
    p = copy.copy(o)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def fd_dlnpsi_dparams(o, r_up, r_dn, h: float = 1e-5, j3_entries=None, lam_entries=None) -> dict:
    """Central differences of ln|psi| for the same blocks (all entries unless an
    explicit list of (row, col) entries is given for the matrix blocks)."""
    f = lambda p: ln_psi(p, r_up, r_dn)  # noqa: E731
    out = {}
    if o.j1 is not None:
        out["j1_param"] = (f(_with(o, j1_a=o.j1_a + h)) - f(_with(o, j1_a=o.j1_a - h))) / (2 * h)
    if o.j2 is not None:
        out["j2_param"] = (f(_with(o, j2_b=o.j2_b + h)) - f(_with(o, j2_b=o.j2_b - h))) / (2 * h)
    if o.j3 is not None:
        A3 = o.j3_mat.shape[0]
        D = np.full((A3, A3 + 1), np.nan)
        ents = j3_entries if j3_entries is not None else [(i, j) for i in range(A3) for j in range(A3 + 1)]
        for (i, j) in ents:
            vals = []
            for s in (h, -h):
                if j < A3:
                    m = o.j3_mat.copy()
                    m[i, j] += s
                    vals.append(f(_with(o, j3_mat=m)))
                else:
                    v = o.j3_vec.copy()
                    v[i] += s
                    vals.append(f(_with(o, j3_vec=v)))
            D[i, j] = (vals[0] - vals[1]) / (2 * h)
        out["j3_matrix"] = D
    P, Q = o.lam_p.shape
    D = np.full((P, Q), np.nan)
    ents = lam_entries if lam_entries is not None else [(i, j) for i in range(P) for j in range(Q)]
    for (i, j) in ents:
        vals = []
        for s in (h, -h):
            m = o.lam_p.copy()
            m[i, j] += s
            vals.append(f(_with(o, lam_p=m)))
        D[i, j] = (vals[0] - vals[1]) / (2 * h)
    out["lambda_matrix"] = D
    return out
