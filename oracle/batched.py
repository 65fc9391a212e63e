"""Walker-batched NumPy restatement of the GFMC_n projection step.

Test and baseline infrastructure (the CPU side of the measurement), never the
product: the same step as ``oracle.drivers.lrdmc_step`` (jqmc_gfmc.py:4779-5166,
``_body_step_core`` with the fresh continuum kinetic energy of ``_body_fun_n``)
for a batch of walkers at once, with every mesh point of every walker in one
array.  Instead of carrying G^-1 by Sherman-Morrison updates it forms G and
G^-1 from the positions at every step (the updated and the fresh inverse agree
to about 1e-13), so a step needs only the positions:

  * det ratios psi_det(r')/psi_det(r) = phi(r') . T_i with T_up = [lam_p Phi_dn,
    lam_u] G^-1 columns and T_dn = rows of G^-1 Phi_up lam_p (determinant.py
    :1530-1662, as ``OracleSystem.det_ratio_move``);
  * Jastrow ratios exp(dJ1 + dJ2 + dJ3) from pair-function differences and the
    J3 field h_e (jastrow_factor.py:649-726, 1181-1251, 1744-1801), as
    ``OracleSystem.jastrow_ratio_move``;
  * the continuum kinetic energy per electron, as
    ``OracleSystem.kinetic_elements`` (wavefunction.py:1142-1207);
  * the lattice and non-local ECP elements, the fixed-node split, the weight
    update and the move choice, as ``oracle.drivers.lrdmc_terms`` /
    ``choose_move`` / ``move_target`` (jqmc_gfmc.py:4806-5030).

``tests/test_oracle_batched.py`` holds it to ``oracle.drivers`` on the same
draws: equal moves, weights to 1e-10."""

from __future__ import annotations

import numpy as np

from .ao import ao_value, ao_vgl
from .wf import OracleSystem, _meshes, legendre, rotation_matrix

_E6 = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], dtype=np.float64)


def _solid_values(l: int, d: np.ndarray) -> np.ndarray:
    """The real solid harmonics of oracle.ao.solid_harmonics (same closed form,
    same row order m + l), values only: (2l+1, ...)."""
    from math import sqrt

    from .ao import _pi_terms
    x, y, z = d[..., 0], d[..., 1], d[..., 2]
    r2 = x * x + y * y + z * z
    S = np.zeros((2 * l + 1,) + x.shape)
    w = x + 1j * y
    for m in range(0, l + 1):
        P = np.zeros_like(x)
        for c, k, zp in _pi_terms(l, m):
            P = P + c * r2**k * z**zp
        if m == 0:
            S[l] = P
            continue
        wm = w**m
        S[l + m] = sqrt(2.0) * P * wm.real
        S[l - m] = sqrt(2.0) * P * wm.imag
    return S


class ShellAO:
    """AO values of a spherical AOTable evaluated shell by shell: the AOs of one
    shell (same centre, l and primitives) share their radial part and one set
    of 2l+1 solid harmonics, which oracle.ao.ao_value evaluates once per AO.
    Same values (tests/test_oracle_batched.py holds them to ao_value)."""

    def __init__(self, tab):
        self.A = tab.num_ao
        groups = {}
        for a in range(tab.num_ao):
            key = (tuple(np.round(tab.centers[a], 14)), int(tab.l[a]), tuple(tab.Z[a]), tuple(tab.cN[a]))
            groups.setdefault(key, []).append(a)
        self.by_l = {}
        for (c, l, Z, cN), aos in groups.items():
            self.by_l.setdefault(l, []).append((c, Z, cN, aos))
        self.tables = {}
        for l, shells in self.by_l.items():
            C = np.array([sh[0] for sh in shells])
            Zs = np.array([sh[1] for sh in shells])
            cNs = np.array([sh[2] for sh in shells])
            idx = -np.ones((len(shells), 2 * l + 1), dtype=int)
            for j, sh in enumerate(shells):
                for a in sh[3]:
                    idx[j, tab.m[a] + l] = a
            self.tables[l] = (C, Zs, cNs, idx)

    def values(self, pts: np.ndarray) -> np.ndarray:
        """(P, A) AO values at points (P, 3)."""
        out = np.zeros((pts.shape[0], self.A))
        for l, (C, Zs, cNs, idx) in self.tables.items():
            d = pts[:, None, :] - C[None]                                     # (P, S, 3)
            r2 = np.sum(d * d, axis=-1)
            rad = np.einsum("psk,sk->ps", np.exp(-Zs[None] * r2[:, :, None]), cNs)
            Sv = _solid_values(l, d)                                           # (2l+1, P, S)
            for j in range(2 * l + 1):
                ok = idx[:, j] >= 0
                out[:, idx[ok, j]] = (Sv[j] * rad)[:, ok]
        return out


class BatchedGFMCn:
    """GFMC_n projection of a batch of walkers (positions (W, N, 3), up first)."""

    def __init__(self, o: OracleSystem, alat: float, Nv: int = 6):
        self.o = o
        self.alat = float(alat)
        self.Nv = Nv
        self.n, self.nd = o.n_up, o.n_dn
        self.N = o.n_up + o.n_dn
        self.mesh_w, self.mesh_pts = _meshes()[Nv]
        self._shell_ao = {}
        if o.ecp:
            # per (atom, l): arrays of the channel's (exponent, coefficient, power)
            self.chan = {}
            for (a, l, ex, co, pw) in o.ecp_terms:
                self.chan.setdefault((int(a), int(l)), []).append((float(ex), float(co), float(pw)))
            self.chan = {k: np.array(v) for k, v in self.chan.items()}

    # ------------------------------------------------------------------ pieces
    def _ao(self, tab, pts):
        """(P, A) AO values: shell by shell for spherical tables, else oracle.ao.ao_value."""
        if tab.cart:
            return ao_value(tab, pts).T
        ev = self._shell_ao.get(id(tab))
        if ev is None:
            ev = self._shell_ao[id(tab)] = ShellAO(tab)
        return ev.values(pts)

    def _orb(self, tab, mo, pts):
        """Orbital values at points (P, 3) -> (P, A)."""
        v = self._ao(tab, pts)
        return v if mo is None else v @ mo.T

    def _V_channel(self, atom: np.ndarray, l: int, dist: np.ndarray) -> np.ndarray:
        """r^-2 sum_k c_k r^n_k exp(-alpha_k r^2) of channel l at each atom (elementwise)."""
        out = np.zeros_like(dist)
        for a in np.unique(atom):
            t = self.chan.get((int(a), int(l)))
            if t is None:
                continue
            m = atom == a
            d = dist[m]
            v = np.zeros_like(d)
            for ex, co, pw in t:
                v = v + co * d**pw * np.exp(-ex * d**2)
            out[m] = d**-2.0 * v
        return out

    def _j1(self, pts):
        """sum over nuclei of the J1 pair function at points (..., 3)."""
        o = self.o
        d = np.linalg.norm(pts[..., None, :] - o.R, axis=-1)
        a = o.j1_a
        c = (2.0 * o.j1_Z) ** 0.25
        A = (2.0 * o.j1_Z) ** 0.75
        if o.j1.jastrow_1b_type == "exp":
            return np.sum(-A * (1.0 / (2.0 * a)) * (1.0 - np.exp(-a * c * d)), axis=-1)
        return np.sum(-A * d / (2.0 * (1.0 + a * c * d)), axis=-1)

    def _j2f(self, d):
        o = self.o
        b = o.j2_b
        if o.j2.jastrow_2b_type == "pade":
            return d / 2.0 * (1.0 + b * d) ** (-1.0)
        return 1.0 / (2.0 * b) * (1.0 - np.exp(-b * d))

    def _j3_fields(self, a3):
        """h (W, N, A3) from the J3 AO values at the electrons a3 (W, N, A3): for an up
        electron i, j + J^T sum_{up < i} + J sum_{up > i} + J sum_dn; for a down electron
        j + J^T sum_{dn < j} + J sum_{dn > j} + J^T sum_up (OracleSystem.j3_fields)."""
        o = self.o
        J = o.j3_mat
        n = self.n
        au, ad = a3[:, :n], a3[:, n:]
        h = np.empty_like(a3)
        for blk, other, lo, cross_T in ((au, ad, 0, False), (ad, au, n, True)):
            cs = np.cumsum(blk, axis=1)
            tot = cs[:, -1:, :]
            pre = cs - blk
            suf = tot - cs
            ot = other.sum(axis=1)[:, None, :]
            cross = ot @ J if cross_T else ot @ J.T
            h[:, lo:lo + blk.shape[1]] = o.j3_vec + pre @ J + suf @ J.T + cross
        return h

    def _jastrow_ratio(self, r, pts, e_of, h, a3):
        """exp(J(r') - J(r)) for electron e_of[k] moved to pts[..., k, :] (pts (W, E, K, 3)
        with E electrons listed in e_of)."""
        o = self.o
        W = r.shape[0]
        re = r[:, e_of]                                                   # (W, E, 3)
        dJ = np.zeros(pts.shape[:-1])
        if o.j1 is not None:
            dJ += self._j1(pts) - self._j1(re)[:, :, None]
        if o.j2 is not None:
            dn_ = np.linalg.norm(pts[:, :, :, None, :] - r[:, None, None, :, :], axis=-1)   # (W, E, K, N)
            do_ = np.linalg.norm(re[:, :, None, :] - r[:, None, :, :], axis=-1)            # (W, E, N)
            f_new = self._j2f(dn_)
            f_old = self._j2f(do_)
            mask = np.ones((len(e_of), self.N))
            mask[np.arange(len(e_of)), e_of] = 0.0
            dJ += np.einsum("wekn,en->wek", f_new, mask) - np.einsum("wen,en->we", f_old, mask)[:, :, None]
        if o.j3 is not None:
            p3 = self._ao(o.tab_j3, pts.reshape(-1, 3)).reshape(W, len(e_of), pts.shape[2], -1)
            he = h[:, e_of]
            dJ += np.einsum("weka,wea->wek", p3, he) - np.einsum("wea,wea->we", a3[:, e_of], he)[:, :, None]
        return np.exp(dJ)

    def _det_ratio(self, pts, Tu, Td):
        """psi_det(r')/psi_det(r) for every electron's points pts (W, N, K, 3)."""
        o = self.o
        W, N, K, _ = pts.shape
        n = self.n
        pu = self._orb(o.tab_up, o.mo_up, pts[:, :n].reshape(-1, 3)).reshape(W, n, K, -1)
        pd = self._orb(o.tab_dn, o.mo_dn, pts[:, n:].reshape(-1, 3)).reshape(W, N - n, K, -1)
        ru = np.einsum("wika,wai->wik", pu, Tu)
        rd = np.einsum("wjka,wja->wjk", pd, Td)
        return np.concatenate([ru, rd], axis=1)

    def _kinetic(self, r, Ginv, h):
        """T_i = -1/2 (lap ln psi_i + |grad ln psi_i|^2) per electron (W, N)."""
        o = self.o
        W, N, _ = r.shape
        n, nd = self.n, self.nd
        vu = [x.T.reshape(W, n, -1) for x in ao_vgl(o.tab_up, r[:, :n].reshape(-1, 3))]
        vd = [x.T.reshape(W, nd, -1) for x in ao_vgl(o.tab_dn, r[:, n:].reshape(-1, 3))]
        if o.mo_up is not None:
            vu = [x @ o.mo_up.T for x in vu]
        if o.mo_dn is not None:
            vd = [x @ o.mo_dn.T for x in vd]
        Pd = np.einsum("ab,wjb->waj", o.lam_p, vd[0])                          # (W, A, nd)
        nunp = n - nd

        def up_block(x):
            paired = np.einsum("wia,waj->wij", x, Pd)
            if nunp == 0:
                return paired
            return np.concatenate([paired, np.einsum("wia,ab->wib", x, o.lam_u)], axis=2)

        gup = np.stack([up_block(vu[k]) for k in (1, 2, 3)], axis=1)           # (W, 3, n, n)
        lup = up_block(vu[4])
        g_up = np.einsum("wgij,wji->wgi", gup, Ginv)
        lap_up = -np.sum(g_up**2, axis=1) + np.einsum("wij,wji->wi", lup, Ginv)
        Ul = np.einsum("wia,ab->wib", vu[0], o.lam_p)                          # (W, n, A_dn)

        def dn_block(x):
            b = np.einsum("wib,wjb->wij", Ul, x)                                # (W, n, nd)
            if nunp == 0:
                return b
            return np.concatenate([b, np.zeros((W, n, nunp))], axis=2)

        gdn = np.stack([dn_block(vd[k]) for k in (1, 2, 3)], axis=1)
        ldn = dn_block(vd[4])
        g_dn_all = np.einsum("wij,wgji->wgi", Ginv, gdn)
        lap_dn = (-np.sum(g_dn_all**2, axis=1) + np.einsum("wij,wji->wi", Ginv, ldn))[:, :nd]
        g_dn = g_dn_all[:, :, :nd]
        g = np.concatenate([g_up, g_dn], axis=2).transpose(0, 2, 1)             # (W, N, 3)
        lap = np.concatenate([lap_up, lap_dn], axis=1)
        # Jastrow gradients and Laplacians
        if o.j1 is not None:
            Z, a = o.j1_Z, o.j1_a
            c, A = (2.0 * Z) ** 0.25, (2.0 * Z) ** 0.75
            dv = r[:, :, None, :] - o.R                                        # (W, N, M, 3)
            d = np.linalg.norm(dv, axis=-1)
            if o.j1.jastrow_1b_type == "exp":
                e = np.exp(-a * c * d)
                f1 = -A * c * e / 2.0
                f2 = A * a * c * c * e / 2.0
            else:
                q = 1.0 + a * c * d
                f1 = -A / (2.0 * q * q)
                f2 = A * a * c / (q**3)
            g = g + np.sum((f1 / d)[..., None] * dv, axis=2)
            lap = lap + np.sum(f2 + 2.0 * f1 / d, axis=2)
        if o.j2 is not None:
            b = o.j2_b
            dv = r[:, :, None, :] - r[:, None, :, :]                           # (W, N, N, 3)
            d = np.linalg.norm(dv, axis=-1)
            np.einsum("wii->wi", d)[...] = 1.0
            if o.j2.jastrow_2b_type == "pade":
                f1 = 1.0 / (2.0 * (1.0 + b * d) ** 2)
                f2 = -b / ((1.0 + b * d) ** 3)
            else:
                f1 = 0.5 * np.exp(-b * d)
                f2 = -0.5 * b * np.exp(-b * d)
            off = 1.0 - np.eye(N)
            g = g + np.einsum("wij,wijx->wix", f1 / d * off, dv)
            lap = lap + np.sum((f2 + 2.0 * f1 / d) * off, axis=2)
        if o.j3 is not None:
            v3 = [x.T.reshape(W, N, -1) for x in ao_vgl(o.tab_j3, r.reshape(-1, 3))]
            g = g + np.stack([np.einsum("wea,wea->we", v3[k], h) for k in (1, 2, 3)], axis=-1)
            lap = lap + np.einsum("wea,wea->we", v3[4], h)
        return -0.5 * (lap + np.sum(g * g, axis=-1))

    def _ecp(self, r, Rm, dnuc, Tu, Td, h, a3):
        """(local ECP energy (W,), non-local elements V (W, N, Nv), quadrature points
        (W, N, Nv, 3)) with the rotations Rm (coulomb_potential.py:601-661, :1478-1712
        with NN = 1, as OracleSystem.ecp_local / ecp_nonlocal)."""
        o = self.o
        W, N, _ = r.shape
        Nv = self.Nv
        atom = np.argmin(dnuc, axis=2)                                        # (W, N), first nearest
        loc = np.zeros(W)
        for a in range(o.M):
            loc += np.sum(self._V_channel(np.full((W, N), a), int(o.maxl1[a]), dnuc[:, :, a]), axis=1)
        Ra = o.R[atom]                                                        # (W, N, 3)
        rel = Ra - r
        dist = np.linalg.norm(rel, axis=-1)
        gq = np.einsum("qx,wyx->wqy", self.mesh_pts, Rm)                      # (W, Nv, 3): mesh R^T
        pe = r[:, :, None, :] + rel[:, :, None, :] + dist[:, :, None, None] * gq[:, None]
        cos_t = np.einsum("wex,wqx->weq", -rel / dist[..., None], gq / np.linalg.norm(gq, axis=-1)[..., None])
        lmax = o.maxl1[atom]                                                  # (W, N)
        wv = np.zeros((W, N, Nv))
        for l in range(int(o.maxl1.max())):
            Vl = self._V_channel(atom, l, dist)                               # (W, N)
            act = (l < lmax)[..., None]
            wv = wv + np.where(act, Vl[..., None] * (2 * l + 1) * legendre(l, cos_t) * self.mesh_w, 0.0)
        ratio_e = self._det_ratio(pe, Tu, Td) * self._jastrow_ratio(r, pe, np.arange(N), h, a3)
        return loc, wv * ratio_e, pe

    def tables(self, r, Ginv=None):
        """(Pu, Pdn, B, G, Ginv, Tu, Td, a3, h) at positions r; G^-1 from the positions
        unless given."""
        o = self.o
        W, N, _ = r.shape
        n, nd = self.n, self.nd
        Pu = self._orb(o.tab_up, o.mo_up, r[:, :n].reshape(-1, 3)).reshape(W, n, -1)
        Pdn = self._orb(o.tab_dn, o.mo_dn, r[:, n:].reshape(-1, 3)).reshape(W, nd, -1)
        B = np.einsum("ab,wjb->waj", o.lam_p, Pdn)                             # (W, A, nd)
        if n > nd:
            B = np.concatenate([B, np.broadcast_to(o.lam_u, (W,) + o.lam_u.shape)], axis=2)
        G = np.einsum("wia,waj->wij", Pu, B)
        if Ginv is None:
            Ginv = np.linalg.inv(G)
        Tu = B @ Ginv                                                          # (W, A, n)
        Td = np.einsum("wjk,wkb->wjb", Ginv[:, :nd, :], np.einsum("wia,ab->wib", Pu, o.lam_p))
        a3 = self._ao(o.tab_j3, r.reshape(-1, 3)).reshape(W, N, -1) if o.j3 is not None else None
        h = self._j3_fields(a3) if o.j3 is not None else None
        return Pu, Pdn, B, G, Ginv, Tu, Td, a3, h

    # ------------------------------------------------------------------ the step
    def step(self, r: np.ndarray, w: np.ndarray, draws: np.ndarray, E_scf: float):
        """One projection of every walker: r (W, N, 3), w (W,), draws (W, 4) = (alpha,
        beta, gamma, u_move).  Returns (r_new, w_new, diag, nondiag, k)."""
        diag, nondiag, p, pl, pe = self._terms(r, draws)
        W, N, _ = r.shape
        Nv = self.Nv
        E_scf = float(E_scf)
        w_new = w * (1.0 / (diag - E_scf) * (-1.0 * nondiag))
        # move choice: sequential cumulative sums, first index with cdf >= u
        s = np.cumsum(p, axis=1)[:, -1:]
        cdf = np.cumsum(p / s, axis=1)
        hit = cdf >= draws[:, 3:4]
        k = np.where(hit.any(axis=1), np.argmax(hit, axis=1), p.shape[1] - 1)
        r_new = r.copy()
        for wi in range(W):
            kk = int(k[wi])
            if kk < 6 * N:
                e, sft = divmod(kk, 6)
                r_new[wi, e] = pl[wi, e, sft]
            else:
                e, q = divmod(kk - 6 * N, Nv)
                r_new[wi, e] = pe[wi, e, q]
        return r_new, w_new, diag, nondiag, k

    def energy(self, r: np.ndarray, draws: np.ndarray):
        """(e_L, V_diag) of every walker with the rotation of draws[:, :3]
        (oracle.drivers.lrdmc_energy, jqmc_gfmc.py:5361-5640)."""
        diag, nondiag, _, _, _ = self._terms(r, draws)
        return diag + nondiag, diag

    def _terms(self, r: np.ndarray, draws: np.ndarray):
        """(diag, nondiag, p, lattice points, ECP points) of every walker."""
        o = self.o
        W, N, _ = r.shape
        n, nd = self.n, self.nd
        alat = self.alat
        Rm = np.stack([rotation_matrix(*d[:3]) for d in draws])               # (W, 3, 3)
        # geminal, inverse and the ratio tables
        _, _, _, _, Ginv, Tu, Td, a3, h = self.tables(r)
        ke = self._kinetic(r, Ginv, h)                                        # (W, N)
        allE = np.arange(N)
        # lattice elements
        shifts = alat * np.einsum("kx,wyx->wky", _E6, Rm)                     # (W, 6, 3): alat E6 R^T
        pl = r[:, :, None, :] + shifts[:, None]                               # (W, N, 6, 3)
        ratio_l = self._det_ratio(pl, Tu, Td) * self._jastrow_ratio(r, pl, allE, h, a3)
        el = -1.0 / (2.0 * alat**2) * ratio_l                                 # (W, N, 6)
        fn = np.minimum(el, 0.0)
        nondiag = fn.sum(axis=(1, 2))
        sp_kin = np.maximum(el, 0.0).sum(axis=(1, 2))
        flip = np.any(el >= 0.0, axis=2)
        nd_elem = np.sum(el + 1.0 / (4.0 * alat**2), axis=2)
        dnuc = np.linalg.norm(r[:, :, None, :] - o.R, axis=-1)                # (W, N, M)
        ei = np.sum(-o.Zeff / dnuc, axis=2)
        ei_disc = np.sum(-o.Zeff / np.maximum(dnuc, alat), axis=2)
        zv = ei + ke - nd_elem
        ei_use = ei if o.ecp else ei_disc
        opt = np.where(flip, np.maximum(zv, ei_use), zv)
        iu, ju = np.triu_indices(N, k=1)
        ee = np.sum(1.0 / np.linalg.norm(r[:, iu] - r[:, ju], axis=-1), axis=1)
        disc = ee + o.coulomb_ion_ion() + opt[:, :n].sum(axis=1) + opt[:, n:].sum(axis=1)
        diag_kin = 3.0 / (2.0 * alat**2) * N
        Nv = self.Nv
        if o.ecp:
            loc, V, pe = self._ecp(r, Rm, dnuc, Tu, Td, h, a3)
            vfn = np.minimum(V, 0.0)
            sp_ecp = np.maximum(V, 0.0).sum(axis=(1, 2))
            nondiag = nondiag + vfn.sum(axis=(1, 2))
            diag = diag_kin + disc + loc + sp_kin + sp_ecp
            p = np.concatenate([fn.reshape(W, -1), vfn.reshape(W, -1)], axis=1)
        else:
            diag = diag_kin + disc + sp_kin
            p = fn.reshape(W, -1)
            pe = None
        return diag, nondiag, p, pl, pe


class BatchedVMC:
    """Metropolis proposals and VMC measurements of a batch of walkers, as
    ``oracle.drivers.vmc_proposal`` / ``vmc_measure`` (jqmc_mcmc.py:4278-4533,
    E_L and w_L of :725-747): one proposal of every walker at once, G and G^-1
    carried by the same Sherman-Morrison updates, the Jastrow ratio from
    pair-function differences and the J3 field."""

    def __init__(self, o: OracleSystem, Dt: float, eps_AS: float, Nv: int = 6):
        self.o = o
        self.Dt, self.eps_AS = float(Dt), float(eps_AS)
        self.g = BatchedGFMCn(o, 0.2, Nv)   # shared pieces (orbitals, Jastrow, ECP)

    def init(self, r):
        """(G, G^-1) from the positions (W, N, 3)."""
        _, _, _, G, Ginv, _, _, _, _ = self.g.tables(r)
        return G, Ginv

    def _step_scale(self, p):
        """f(r) of the proposal width at points p (W, 3) (jqmc_mcmc.py:4355-4361)."""
        o = self.o
        d = np.linalg.norm(p[:, None, :] - o.R, axis=-1)
        a = np.argmin(d, axis=1)
        Z = o.Zeff[a]
        dd = d[np.arange(len(a)), a]
        return 1.0 / Z**2 * (1.0 + Z**2 * dd) / (1.0 + dd)

    @staticmethod
    def _as_factor(G, Ginv):
        F = np.sum(Ginv**2, axis=(1, 2))
        S = np.minimum(np.min(np.sum(G**2, axis=2), axis=1), np.min(np.sum(G**2, axis=1), axis=1))
        SF = S * F
        with np.errstate(divide="ignore"):
            return np.where(SF > 0.0, SF ** (-3.0 / 8.0), 0.0)

    def proposal(self, r, G, Ginv, idraw, fdraw):
        """One proposal of every walker in place: idraw (W, 4) = (sel, up index, down
        index, axis), fdraw (W, 2) = (gauss, uniform).  Returns the accepted mask."""
        o, gf = self.o, self.g
        W, N, _ = r.shape
        n, nd = o.n_up, o.n_dn
        ws = np.arange(W)
        sel, up_i, dn_i, axis = (idraw[:, k].astype(int) for k in range(4))
        gauss, u = fdraw[:, 0], fdraw[:, 1]
        is_up = sel < n
        idx = np.where(is_up, up_i, dn_i)
        e = np.where(is_up, idx, n + idx)
        old = r[ws, e].copy()
        f_l = self._step_scale(old)
        new = old.copy()
        new[ws, axis] += gauss * (f_l * self.Dt)
        f_p = self._step_scale(new)
        dist2 = np.sum((new - old) ** 2, axis=1)
        T_ratio = (f_l / f_p) * np.exp(-dist2 * (1.0 / (2.0 * f_p**2 * self.Dt**2) - 1.0 / (2.0 * f_l**2 * self.Dt**2)))
        # Jastrow ratio of the move
        dJ = np.zeros(W)
        if o.j1 is not None:
            dJ += gf._j1(new) - gf._j1(old)
        if o.j2 is not None:
            mask = np.ones((W, N))
            mask[ws, e] = 0.0
            dJ += np.sum((gf._j2f(np.linalg.norm(new[:, None, :] - r, axis=-1))
                          - gf._j2f(np.linalg.norm(old[:, None, :] - r, axis=-1))) * mask, axis=1)
        if o.j3 is not None:
            a3 = gf._ao(o.tab_j3, r.reshape(-1, 3)).reshape(W, N, -1)
            h = gf._j3_fields(a3)
            p3 = gf._ao(o.tab_j3, new)
            dJ += np.einsum("wa,wa->w", p3 - a3[ws, e], h[ws, e])
        J_ratio = np.exp(dJ)
        # geminal row (up) or column (down) at the new position, Sherman-Morrison
        Pu = gf._orb(o.tab_up, o.mo_up, r[:, :n].reshape(-1, 3)).reshape(W, n, -1)
        Pdn = gf._orb(o.tab_dn, o.mo_dn, r[:, n:].reshape(-1, 3)).reshape(W, nd, -1)
        pu_new = gf._orb(o.tab_up, o.mo_up, new)                             # (W, A)
        pd_new = gf._orb(o.tab_dn, o.mo_dn, new)
        row = np.einsum("wa,ab,wjb->wj", pu_new, o.lam_p, Pdn)
        if n > nd:
            row = np.concatenate([row, pu_new @ o.lam_u], axis=1)
        col = np.einsum("wia,ab,wb->wi", Pu, o.lam_p, pd_new)
        G_new, Ginv_new = G.copy(), Ginv.copy()
        det_ratio = np.empty(W)
        for w in range(W):
            i = idx[w]
            if is_up[w]:
                v = row[w] - G[w, i]
                Ainv_u = Ginv[w][:, i]
                vT_Ainv = v @ Ginv[w]
                det_ratio[w] = 1.0 + v @ Ainv_u
                G_new[w, i, :] += v
            else:
                u_vec = col[w] - G[w][:, i]
                Ainv_u = Ginv[w] @ u_vec
                vT_Ainv = Ginv[w][i, :]
                det_ratio[w] = 1.0 + Ainv_u[i]
                G_new[w][:, i] += u_vec
            Ginv_new[w] = Ginv[w] - np.outer(Ainv_u, vT_Ainv) / det_ratio[w]
        Rp = self._as_factor(G_new, Ginv_new)
        Ro = self._as_factor(G, Ginv)
        eps = self.eps_AS
        R_AS_ratio = (np.maximum(Rp, eps) / Rp) / (np.maximum(Ro, eps) / Ro)
        R_ratio = (R_AS_ratio * J_ratio * det_ratio) ** 2.0
        p = np.minimum(1.0, R_ratio * T_ratio)
        acc = u < p
        r[ws[acc], e[acc]] = new[acc]
        G[acc] = G_new[acc]
        Ginv[acc] = Ginv_new[acc]
        return acc

    def measure(self, r, G, Ginv, angles):
        """(e_L, w_L) of every walker with RT = R(angles).T (jqmc_mcmc.py:725-747)."""
        o, gf = self.o, self.g
        W, N, _ = r.shape
        n = o.n_up
        Rm = np.stack([rotation_matrix(*a) for a in angles])
        _, _, _, _, _, Tu, Td, a3, h = gf.tables(r, Ginv)
        ke = gf._kinetic(r, Ginv, h)
        dnuc = np.linalg.norm(r[:, :, None, :] - o.R, axis=-1)
        iu, ju = np.triu_indices(N, k=1)
        V = (o.coulomb_ion_ion() + np.sum(-o.Zeff / dnuc, axis=(1, 2))
             + np.sum(1.0 / np.linalg.norm(r[:, iu] - r[:, ju], axis=-1), axis=1))
        if o.ecp:
            loc, Vnl, _ = gf._ecp(r, Rm, dnuc, Tu, Td, h, a3)
            V = V + loc + Vnl.sum(axis=(1, 2))
        e = ke[:, :n].sum(axis=1) + ke[:, n:].sum(axis=1) + V
        R = self._as_factor(G, Ginv)
        w = (R / np.maximum(R, self.eps_AS)) ** 2
        return e, w
