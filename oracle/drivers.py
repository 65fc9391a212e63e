"""Oracle: VMC Metropolis proposals, LRDMC (GFMC_n) projection steps, branching.

All randomness enters as explicit draws, so the oracle and the CUDA kernels
follow the same trajectory given the same arrays:

VMC proposal  (jqmc_mcmc.py:4316-4523, one ``body_fun``):
    idraw = (sel, up_index, dn_index, axis), fdraw = (gauss, uniform)
    is_up = sel < n_up; the Gaussian g*sigma moves one Cartesian axis; f_l scales
    sigma by the nearest effective charge; acceptance min(1, (R_AS * J * D)^2 T).
LRDMC step    (jqmc_gfmc.py:4779-5166, ``_body_step_core`` with the fresh
    continuum kinetic energy of ``_body_fun_n``):
    draw = (alpha, beta, gamma, u_move); rotation R(alpha, beta, gamma);
    kinetic mesh 6 shifts x electrons, ECP T-move mesh (NN=1, Nv points) x electrons,
    fixed-node split, discretised diagonal, w *= -sum_nondiag / (sum_diag - E_scf),
    move chosen by a sequential cumsum over the normalised FN weights and a
    left searchsorted, Sherman-Morrison update of G^-1.
GFMC_t step   (jqmc_gfmc.py:724-1107, ``_projection_t_core``):
    draw = (alpha, beta, gamma, xi, u_move); the same elements; e_L = diag + nondiag,
    tau_update = min(tau_left, ln(1 - xi) / nondiag), w *= exp(-tau_update e_L),
    and the move is made only while tau_left > 0 after the update.
Branching     (jqmc_gfmc.py:2010-2090 with one process): comb z_k = (k + zeta)/W
    over the cumulative normalised weights (sequential cumsum), left searchsorted.
"""

from __future__ import annotations

import numpy as np

from .wf import OracleSystem, rotation_matrix


class WalkerState:
    def __init__(self, r_up, r_dn, G, Ginv):
        self.r_up = np.array(r_up, dtype=np.float64)
        self.r_dn = np.array(r_dn, dtype=np.float64)
        self.G = np.array(G, dtype=np.float64)
        self.Ginv = np.array(Ginv, dtype=np.float64)

    def copy(self):
        return WalkerState(self.r_up, self.r_dn, self.G, self.Ginv)


def init_state(o: OracleSystem, r_up, r_dn) -> WalkerState:
    G = o.geminal(r_up, r_dn)
    return WalkerState(r_up, r_dn, G, np.linalg.inv(G))


def step_scale(o: OracleSystem, r):
    """f(r) = (1 + Z^2 d) / (Z^2 (1 + d)), d the distance to the nearest nucleus
    and Z its effective charge: the proposal's Gaussian width is f(r) Dt
    (jqmc_mcmc.py:4355-4361)."""
    a = o.nearest(r)
    Z = o.Zeff[a]
    d = np.linalg.norm(r - o.R[a])
    return 1.0 / Z**2 * (1.0 + Z**2 * d) / (1.0 + d)


def transition_ratio(o: OracleSystem, old, new, Dt: float) -> float:
    """T(new -> old) / T(old -> new) of the position-dependent Gaussian proposal
    (jqmc_mcmc.py:4395-4401)."""
    f_l, f_p = step_scale(o, old), step_scale(o, new)
    return (f_l / f_p) * np.exp(-(np.linalg.norm(new - old) ** 2) * (1.0 / (2.0 * f_p**2 * Dt**2) - 1.0 / (2.0 * f_l**2 * Dt**2)))


def vmc_proposal(o: OracleSystem, st: WalkerState, idraw, fdraw, Dt: float, eps_AS: float) -> bool:
    """One Metropolis proposal in place; returns accepted."""
    sel, up_i, dn_i, axis = (int(x) for x in idraw)
    gauss, u = float(fdraw[0]), float(fdraw[1])
    is_up = sel < o.n_up
    idx = up_i if is_up else dn_i
    old = (st.r_up if is_up else st.r_dn)[idx].copy()
    g = gauss * (step_scale(o, old) * Dt)
    new = old.copy()
    new[axis] += g
    T_ratio = transition_ratio(o, old, new, Dt)
    ru, rd = st.r_up.copy(), st.r_dn.copy()
    (ru if is_up else rd)[idx] = new
    J_ratio = np.exp(o.jastrow_total(ru, rd) - o.jastrow_total(st.r_up, st.r_dn))
    n = o.n_up
    if is_up:
        v = o.geminal(ru, rd)[idx] - st.G[idx]
        u_vec = np.zeros(n)
        u_vec[idx] = 1.0
    else:
        u_vec = o.geminal(ru, rd)[:, idx] - st.G[:, idx]
        v = np.zeros(n)
        v[idx] = 1.0
    Ainv_u = st.Ginv @ u_vec
    vT_Ainv = v @ st.Ginv
    det_ratio = 1.0 + v @ Ainv_u
    Ginv_new = st.Ginv - np.outer(Ainv_u, vT_Ainv) / det_ratio
    G_new = st.G.copy()
    if is_up:
        G_new[idx, :] += v
    else:
        G_new[:, idx] += u_vec
    Rp = o.as_factor(G_new, Ginv_new)
    Ro = o.as_factor(st.G, st.Ginv)
    R_AS_ratio = (max(Rp, eps_AS) / Rp) / (max(Ro, eps_AS) / Ro)
    R_ratio = (R_AS_ratio * J_ratio * det_ratio) ** 2.0
    p = min(1.0, R_ratio * T_ratio)
    if u < p:
        st.r_up, st.r_dn, st.G, st.Ginv = ru, rd, G_new, Ginv_new
        return True
    return False


def vmc_block(o, st, idraws, fdraws, Dt, eps_AS):
    acc = 0
    for k in range(len(idraws)):
        acc += vmc_proposal(o, st, idraws[k], fdraws[k], Dt, eps_AS)
    return acc


def vmc_measure(o: OracleSystem, st: WalkerState, angles, eps_AS: float):
    """(e_L, w_L) after a block: E_L with RT = R(angles).T (jqmc_mcmc.py:725-747)."""
    RT = rotation_matrix(*angles).T
    e = o.local_energy(st.r_up, st.r_dn, RT, st.Ginv)
    R = o.as_factor(st.G, st.Ginv)
    w = (R / max(R, eps_AS)) ** 2
    return e, w


# --------------------------------------------------------------------- LRDMC
def _ecp_moves(o: OracleSystem, st: WalkerState, R: np.ndarray, Nv: int, non_local_move: str):
    """(V_FN per mesh point, SP sum) of the non-local ECP.  'tmove': V with the full
    psi ratio, FN = min(V, 0), SP = sum max(V, 0) (jqmc_gfmc.py:4941-4979).
    'dltmove' (determinant locality): V with the determinant ratio alone, SP =
    sum max(V, 0), FN = min(V, 0) times the Jastrow ratio of the same mesh point
    (jqmc_gfmc.py:4980-5017, :920-946, :5553-5600)."""
    if non_local_move == "tmove":
        V, _ = o.ecp_nonlocal(st.r_up, st.r_dn, R.T, st.Ginv, Nv=Nv)
        return np.minimum(V, 0.0), float(np.sum(np.maximum(V, 0.0)))
    if non_local_move == "dltmove":
        pts = []

        def det_only(spin, i, rn):
            pts.append((spin, i, rn.copy()))
            return o.det_ratio_move(st.Ginv, st.r_up, st.r_dn, spin, i, rn)

        V, _ = o.ecp_nonlocal(st.r_up, st.r_dn, R.T, st.Ginv, Nv=Nv, ratio_fn=det_only)
        jr = np.array([o.jastrow_ratio_move(st.r_up, st.r_dn, s, i, rn) for s, i, rn in pts])
        return np.minimum(V, 0.0) * jr, float(np.sum(np.maximum(V, 0.0)))
    raise NotImplementedError(f"non_local_move={non_local_move!r}")


def lrdmc_terms(o: OracleSystem, st: WalkerState, R: np.ndarray, alat: float, Nv: int = 6,
                non_local_move: str = "tmove"):
    """(diag, nondiag, p_list, kin_elements, V_nonlocal_FN) at the walker's configuration
    with rotation R (jqmc_gfmc.py:4806-5030 / 5361-5550)."""
    N = o.n_up + o.n_dn
    tu, td = o.kinetic_elements(st.r_up, st.r_dn, st.Ginv)
    ke = np.concatenate([tu, td])
    el = o.discretized_kinetic(alat, st.r_up, st.r_dn, R.T, st.Ginv)
    fn = np.minimum(el, 0.0)
    nondiag = np.sum(fn)
    sp_kin = np.sum(np.maximum(el, 0.0))
    el6 = el.reshape(-1, 6)
    flip = np.any(el6 >= 0, axis=1)
    nd_elem = np.sum(el6 + 1.0 / (4.0 * alat**2), axis=1)
    r = np.vstack([st.r_up, st.r_dn])
    ei = o.coulomb_el_ion(r)
    ei_disc = o.coulomb_el_ion(r, alat)
    zv = ei + ke - nd_elem
    ei_use = ei if o.ecp else ei_disc
    opt = np.where(flip, np.maximum(zv, ei_use), zv)
    disc = o.coulomb_el_el(st.r_up, st.r_dn) + o.coulomb_ion_ion() + np.sum(opt[: o.n_up]) + np.sum(opt[o.n_up:])
    diag_kin = 3.0 / (2.0 * alat**2) * N
    if o.ecp:
        loc = o.ecp_local(st.r_up, st.r_dn)
        vfn, sp_ecp = _ecp_moves(o, st, R, Nv, non_local_move)
        nondiag = nondiag + np.sum(vfn)
        diag = diag_kin + disc + loc + sp_kin + sp_ecp
        p = np.concatenate([fn.ravel(), vfn.ravel()])
    else:
        diag = diag_kin + disc + sp_kin
        vfn = np.zeros(0)
        p = fn.ravel()
    return diag, nondiag, p, el, vfn


def choose_move(p: np.ndarray, u: float) -> int:
    """k = searchsorted(cumsum(p / sum(p)), u) with sequential sums, clamped to the last index."""
    s = 0.0
    for x in p:
        s += x
    cdf = 0.0
    for k, x in enumerate(p):
        cdf += x / s
        if cdf >= u:
            return k
    return len(p) - 1


def move_target(o: OracleSystem, st: WalkerState, k: int, R: np.ndarray, alat: float, Nv: int = 6):
    """(spin, index, r_new) of candidate k: kinetic mesh (electron-major, 6 shifts), then ECP mesh."""
    N = o.n_up + o.n_dn
    if k < 6 * N:
        e, s = divmod(k, 6)
        shift = alat * np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], float)[s] @ R.T
        spin, i = (0, e) if e < o.n_up else (1, e - o.n_up)
        return spin, i, (st.r_up if spin == 0 else st.r_dn)[i] + shift
    k -= 6 * N
    e, q = divmod(k, Nv)
    from .wf import _meshes
    pts = _meshes()[Nv][1] @ R.T
    spin, i = (0, e) if e < o.n_up else (1, e - o.n_up)
    ri = (st.r_up if spin == 0 else st.r_dn)[i]
    atom = o.nearest(ri)
    rel = o.R[atom] - ri
    return spin, i, ri + rel + np.linalg.norm(rel) * pts[q]


def sm_update(o: OracleSystem, st: WalkerState, spin: int, i: int, r_new):
    """Move one electron and Sherman-Morrison-update G^-1 (jqmc_gfmc.py:5083-5141)."""
    ru, rd = st.r_up.copy(), st.r_dn.copy()
    (ru if spin == 0 else rd)[i] = r_new
    Gn = o.geminal(ru, rd)
    n = o.n_up
    if spin == 0:
        v = Gn[i] - st.G[i]
        u_vec = np.zeros(n)
        u_vec[i] = 1.0
    else:
        u_vec = Gn[:, i] - st.G[:, i]
        v = np.zeros(n)
        v[i] = 1.0
    Ainv_u = st.Ginv @ u_vec
    vT_Ainv = v @ st.Ginv
    ratio = 1.0 + v @ Ainv_u
    st.Ginv = st.Ginv - np.outer(Ainv_u, vT_Ainv) / ratio
    G_new = st.G.copy()
    if spin == 0:
        G_new[i, :] += v
    else:
        G_new[:, i] += u_vec
    st.G = G_new
    st.r_up, st.r_dn = ru, rd


def lrdmc_step(o: OracleSystem, st: WalkerState, w: float, draw, alat: float, E_scf: float, Nv: int = 6,
               non_local_move: str = "tmove"):
    """One GFMC_n projection; returns (w_new, diag, nondiag, k)."""
    R = rotation_matrix(draw[0], draw[1], draw[2])
    diag, nondiag, p, _, _ = lrdmc_terms(o, st, R, alat, Nv, non_local_move)
    b_x = 1.0 / (diag - E_scf) * (-1.0 * nondiag)
    w = w * b_x
    k = choose_move(p, float(draw[3]))
    spin, i, rn = move_target(o, st, k, R, alat, Nv)
    sm_update(o, st, spin, i, rn)
    return w, diag, nondiag, k


def lrdmc_step_t(o: OracleSystem, st: WalkerState, w: float, tau_left: float, draw, alat: float, Nv: int = 6,
                 non_local_move: str = "tmove"):
    """One GFMC_t projection (jqmc_gfmc.py:724-1107): draw = (alpha, beta, gamma, xi, u).
    tau_update = min(tau_left, ln(1 - xi) / V_nondiag); w *= exp(-tau_update e_L);
    the chosen move is made only while time is left.  Returns (w, tau_left, e_L, moved)."""
    R = rotation_matrix(draw[0], draw[1], draw[2])
    diag, nondiag, p, _, _ = lrdmc_terms(o, st, R, alat, Nv, non_local_move)
    e_L = diag + nondiag
    tau_update = min(tau_left, np.log(1.0 - float(draw[3])) / nondiag)
    w = w * np.exp(-tau_update * e_L)
    tau_left = tau_left - tau_update
    if tau_left <= 0.0:
        return w, tau_left, e_L, False
    k = choose_move(p, float(draw[4]))
    spin, i, rn = move_target(o, st, k, R, alat, Nv)
    sm_update(o, st, spin, i, rn)
    return w, tau_left, e_L, True


def lrdmc_energy(o: OracleSystem, st: WalkerState, last_draw, alat: float, Nv: int = 6,
                 non_local_move: str = "tmove"):
    """(e_L, V_diag) at the walker's configuration with the last step's rotation
    (jqmc_gfmc.py:5361-5640, e_L = V_diag + V_nondiag)."""
    R = rotation_matrix(last_draw[0], last_draw[1], last_draw[2])
    diag, nondiag, _, _, _ = lrdmc_terms(o, st, R, alat, Nv, non_local_move)
    return diag + nondiag, diag


def branch_comb(w: np.ndarray, zeta: float) -> np.ndarray:
    """Chosen walker indices for the stochastic reconfiguration with one process
    (jqmc_gfmc.py:2020-2090)."""
    W = len(w)
    tot = 0.0
    for x in w:
        tot += x
    cum = np.empty(W)
    c = 0.0
    for k in range(W):
        c += w[k] / tot
        cum[k] = c
    z = (np.arange(W) + zeta) / W
    return np.minimum(np.searchsorted(cum, z, side="left"), W - 1).astype(np.int32)
