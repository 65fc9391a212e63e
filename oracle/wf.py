"""Oracle: geminal determinant, Jastrow, Coulomb/ECP and the local energy (FP64).

Single-walker functions, restating (file:line in the reference project):
  * geminal G               determinant.py:1380-1402
  * ln|det G|, sign         determinant.py:1026-1111 (via LU here)
  * det grads / laps        determinant.py:2141-2250 (compute_grads_and_laplacian_ln_Det_fast)
  * rank-1 det ratio        determinant.py:1530-1662
  * AS regularisation       determinant.py:1223-1260
  * J1 / J2 / J3 values     jastrow_factor.py:649-726, 1181-1251, 1744-1801
  * J ratio                 jastrow_factor.py:2230-2693 (as exp(J(r') - J(r)))
  * J grads / laps          jastrow_factor.py:961-1034 (J1), 3435-3558 (J2), 4077-4156 (J3)
  * kinetic per electron    wavefunction.py:1142-1207
  * bare Coulomb            coulomb_potential.py:2224-2328, 2465-2571; discretised 2332-2378
  * ECP local               coulomb_potential.py:601-661
  * ECP non-local (NN)      coulomb_potential.py:1478-1712, Legendre _function_collections.py:48-66
  * local energy (fast)     hamiltonians.py:225-290
  * discretised kinetic     wavefunction.py:1740-1860
"""

from __future__ import annotations

import numpy as np

from .ao import AOTable, ao_value, ao_vgl

ECP_MESHES = None


def _meshes():
    global ECP_MESHES
    if ECP_MESHES is None:
        q = 1.0 / np.sqrt(3.0)
        th = np.array([0.0, np.pi] + [np.arctan(2.0)] * 5 + [np.pi - np.arctan(2.0)] * 5)
        ph = np.array([0.0, 0.0] + [2.0 * k * np.pi / 5.0 for k in range(5)] + [(2.0 * k + 1.0) * np.pi / 5.0 for k in range(5)])
        ico = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], axis=1)
        p = 1.0 / np.sqrt(2.0)
        o18 = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                        [p, p, 0], [p, -p, 0], [-p, p, 0], [-p, -p, 0], [p, 0, p], [p, 0, -p],
                        [-p, 0, p], [-p, 0, -p], [0, p, p], [0, -p, p], [0, p, -p], [0, -p, -p]], dtype=float)
        ECP_MESHES = {
            4: (np.full(4, 0.25), np.array([[q, q, q], [q, -q, -q], [-q, q, -q], [-q, -q, q]])),
            6: (np.full(6, 1.0 / 6.0), np.array([[1.0, 0, 0], [-1.0, 0, 0], [0, 1.0, 0], [0, -1.0, 0], [0, 0, 1.0], [0, 0, -1.0]])),
            12: (np.full(12, 1.0 / 12.0), ico),
            18: (np.array([1.0 / 6.0] * 6 + [1.0 / 15.0] * 12), o18),
        }
    return ECP_MESHES


def legendre(l: int, x):
    """P_0..P_6 as tabulated in _function_collections.py:48-66."""
    x = np.asarray(x, dtype=np.float64)
    return [np.ones_like(x), x, 0.5 * (3.0 * x**2 - 1), 0.5 * (5.0 * x**3 - 3.0 * x),
            (35.0 * x**4 - 30.0 * x**2 + 3.0) / 8.0, (63.0 * x**5 - 70 * x**3 + 15 * x) / 8.0,
            (231.0 * x**6 - 315.0 * x**4 + 105.0 * x**2 - 5) / 16.0][l]


def rotation_matrix(alpha, beta, gamma):
    """R of jqmc_mcmc.py:4228-4245 / jqmc_gfmc.py:4721-4736 (MCMC returns R.T)."""
    ca, sa, cb, sb, cg, sg = np.cos(alpha), np.sin(alpha), np.cos(beta), np.sin(beta), np.cos(gamma), np.sin(gamma)
    return np.array([[cb * cg, cg * sa * sb - ca * sg, sa * sg + ca * cg * sb],
                     [cb * sg, ca * cg + sa * sb * sg, ca * sb * sg - cg * sa],
                     [-sb, cb * sa, ca * cb]])


class OracleSystem:
    """Flattened tables of a Hamiltonian_data-like object (the product dataclasses)."""

    def __init__(self, ham):
        self.ham = ham
        st = ham.structure_data
        self.R = np.asarray(st.positions, dtype=np.float64)
        self.M = self.R.shape[0]
        g = ham.wavefunction_data.geminal_data
        self.n_up, self.n_dn = g.num_electron_up, g.num_electron_dn
        up, dn = g.orb_data_up_spin, g.orb_data_dn_spin
        self.mo_up = getattr(up, "mo_coefficients", None)
        self.mo_dn = getattr(dn, "mo_coefficients", None)
        self.tab_up = AOTable(up.aos_data if self.mo_up is not None else up)
        self.tab_dn = AOTable(dn.aos_data if self.mo_dn is not None else dn)
        lam = np.asarray(g.lambda_matrix, dtype=np.float64)
        self.lam_p = lam[:, : dn.orb_num]
        self.lam_u = lam[:, dn.orb_num:]
        jd = ham.wavefunction_data.jastrow_data
        self.j1 = jd.jastrow_one_body_data
        self.j2 = jd.jastrow_two_body_data
        self.j3 = jd.jastrow_three_body_data
        if self.j1 is not None:
            self.j1_Z = np.asarray(st.atomic_numbers, float) - np.asarray(self.j1.core_electrons, float)
            self.j1_a = float(self.j1.jastrow_1b_param)
        if self.j2 is not None:
            self.j2_b = float(self.j2.jastrow_2b_param)
        if self.j3 is not None:
            self.tab_j3 = AOTable(self.j3.orb_data)
            self.j3_mat = np.asarray(self.j3.j_matrix)[:, :-1]
            self.j3_vec = np.asarray(self.j3.j_matrix)[:, -1]
        c = ham.coulomb_potential_data
        self.ecp = bool(c.ecp_flag)
        self.Zeff = np.asarray(st.atomic_numbers, float) - (np.asarray(c.z_cores, float) if self.ecp else 0.0)
        if self.ecp:
            self.ecp_terms = list(zip(c.nucleus_index, c.ang_moms, c.exponents, c.coefficients, c.powers))
            self.maxl1 = np.asarray(c.max_ang_mom_plus_1, dtype=int)

    # ---------------------------------------------------------------- orbitals
    def orb_up(self, r):
        v = ao_value(self.tab_up, r)
        return v if self.mo_up is None else self.mo_up @ v

    def orb_dn(self, r):
        v = ao_value(self.tab_dn, r)
        return v if self.mo_dn is None else self.mo_dn @ v

    def orb_vgl(self, tab, mo, r):
        out = ao_vgl(tab, r)
        return out if mo is None else tuple(mo @ x for x in out)

    # ---------------------------------------------------------------- geminal
    def geminal(self, r_up, r_dn):
        """G (n_up, n_up): determinant.py:1380-1402."""
        pu, pd = self.orb_up(r_up), self.orb_dn(r_dn)
        return np.hstack([pu.T @ (self.lam_p @ pd), pu.T @ self.lam_u])

    def ln_det(self, r_up, r_dn):
        sign, ld = np.linalg.slogdet(self.geminal(r_up, r_dn))
        return sign, ld

    def det_grad_lap(self, r_up, r_dn, Ginv):
        """(grad_up (n_up,3), grad_dn (n_dn,3), lap_up, lap_dn): determinant.py:2141-2250."""
        vu = self.orb_vgl(self.tab_up, self.mo_up, r_up)
        vd = self.orb_vgl(self.tab_dn, self.mo_dn, r_dn)
        pd = self.lam_p @ vd[0]
        gup = np.stack([np.hstack([vu[k].T @ pd, vu[k].T @ self.lam_u]) for k in (1, 2, 3)])
        lup = np.hstack([vu[4].T @ pd, vu[4].T @ self.lam_u])
        nunp = self.n_up - self.n_dn
        gdn = np.stack([np.hstack([vu[0].T @ (self.lam_p @ vd[k]), np.zeros((self.n_up, nunp))]) for k in (1, 2, 3)])
        ldn = np.hstack([vu[0].T @ (self.lam_p @ vd[4]), np.zeros((self.n_up, nunp))])
        g_up = np.einsum("gij,ji->gi", gup, Ginv)
        g_dn = np.einsum("ij,gji->gi", Ginv, gdn)
        lap_up = -np.sum(g_up**2, axis=0) + np.einsum("ij,ji->i", lup, Ginv)
        lap_dn = -np.sum(g_dn**2, axis=0) + np.einsum("ij,ji->i", Ginv, ldn)
        return g_up.T, g_dn.T[: self.n_dn], lap_up, lap_dn[: self.n_dn]

    def det_ratio_move(self, Ginv, r_up, r_dn, spin, idx, r_new):
        """det G(r')/det G(r) for one electron moved (determinant.py:1530-1662)."""
        if spin == 0:
            row_new = np.hstack([(self.orb_up(r_new[None]).T @ (self.lam_p @ self.orb_dn(r_dn)))[0],
                                 (self.orb_up(r_new[None]).T @ self.lam_u)[0]])
            return float(row_new @ Ginv[:, idx])
        col_new = (self.orb_up(r_up).T @ (self.lam_p @ self.orb_dn(r_new[None])))[:, 0]
        return float(Ginv[idx, :] @ col_new)

    @staticmethod
    def as_factor(G, Ginv):
        """R_AS = (min(min row |G|^2, min col |G|^2) |G^-1|_F^2)^(-3/8) (determinant.py:1223-1260)."""
        F = np.sum(Ginv**2)
        S = min(np.min(np.sum(G**2, axis=1)), np.min(np.sum(G**2, axis=0)))
        SF = S * F
        return SF ** (-3.0 / 8.0) if SF > 0.0 else 0.0

    # ---------------------------------------------------------------- Jastrow
    def _j1_f(self, r):
        """sum over nuclei of the J1 pair function at one electron position."""
        d = np.linalg.norm(r[None, :] - self.R, axis=1)
        Z = self.j1_Z
        a = self.j1_a
        c = (2.0 * Z) ** 0.25
        A = (2.0 * Z) ** 0.75
        if self.j1.jastrow_1b_type == "exp":
            return np.sum(-A * (1.0 / (2.0 * a)) * (1.0 - np.exp(-a * c * d)))
        return np.sum(-A * d / (2.0 * (1.0 + a * c * d)))

    def _j2_f(self, rij):
        b = self.j2_b
        if self.j2.jastrow_2b_type == "pade":
            return rij / 2.0 * (1.0 + b * rij) ** (-1.0)
        return 1.0 / (2.0 * b) * (1.0 - np.exp(-b * rij))

    def jastrow(self, r_up, r_dn):
        """(J1, J2, J3) values (jastrow_factor.py:649-726, 1181-1251, 1744-1801)."""
        J1 = J2 = J3 = 0.0
        if self.j1 is not None:
            J1 = sum(self._j1_f(r) for r in np.vstack([r_up, r_dn]))
        if self.j2 is not None:
            d_ud = np.linalg.norm(r_up[:, None] - r_dn[None], axis=-1)
            J2 = np.sum(self._j2_f(d_ud))
            for rs in (r_up, r_dn):
                iu, ju = np.triu_indices(len(rs), k=1)
                J2 += np.sum(self._j2_f(np.linalg.norm(rs[iu] - rs[ju], axis=-1)))
        if self.j3 is not None:
            au, ad = ao_value(self.tab_j3, r_up), ao_value(self.tab_j3, r_dn)
            Ku = np.tril(np.ones((len(r_up), len(r_up))), k=-1)
            Kd = np.tril(np.ones((len(r_dn), len(r_dn))), k=-1)
            J3 = (self.j3_vec @ au.sum(1) + self.j3_vec @ ad.sum(1) + np.trace(au.T @ self.j3_mat @ au @ Ku)
                  + np.trace(ad.T @ self.j3_mat @ ad @ Kd) + au.sum(1) @ self.j3_mat @ ad.sum(1))
        return J1, J2, J3

    def jastrow_total(self, r_up, r_dn):
        return float(sum(self.jastrow(r_up, r_dn)))

    def jastrow_grad_lap(self, r_up, r_dn):
        """Per-electron grad J (N,3) and lap J (N,) over [up; dn] (jastrow_factor.py:961-1034,
        3435-3558, 4077-4156).  Analytic derivatives of the same pair functions."""
        r = np.vstack([r_up, r_dn])
        N = len(r)
        g = np.zeros((N, 3))
        lap = np.zeros(N)
        if self.j1 is not None:
            Z, a = self.j1_Z, self.j1_a
            c, A = (2.0 * Z) ** 0.25, (2.0 * Z) ** 0.75
            for i in range(N):
                dv = r[i][None, :] - self.R
                d = np.linalg.norm(dv, axis=1)
                if self.j1.jastrow_1b_type == "exp":
                    e = np.exp(-a * c * d)
                    f1 = -A * c * e / 2.0
                    f2 = A * a * c * c * e / 2.0
                else:
                    q = 1.0 + a * c * d
                    f1 = -A / (2.0 * q * q)
                    f2 = A * a * c / (q**3)
                g[i] += np.sum(f1[:, None] * dv / d[:, None], axis=0)
                lap[i] += np.sum(f2 + 2.0 * f1 / d)
        if self.j2 is not None:
            b = self.j2_b
            for i in range(N):
                for j in range(N):
                    if i == j:
                        continue
                    dv = r[i] - r[j]
                    d = np.linalg.norm(dv)
                    if self.j2.jastrow_2b_type == "pade":
                        f1 = 1.0 / (2.0 * (1.0 + b * d) ** 2)
                        f2 = -b / ((1.0 + b * d) ** 3)
                    else:
                        f1 = 0.5 * np.exp(-b * d)
                        f2 = -0.5 * b * np.exp(-b * d)
                    g[i] += f1 * dv / d
                    lap[i] += f2 + 2.0 * f1 / d
        if self.j3 is not None:
            h = self.j3_fields(r_up, r_dn)
            v = ao_vgl(self.tab_j3, r)
            for i in range(N):
                g[i] += np.array([v[k][:, i] @ h[:, i] for k in (1, 2, 3)])
                lap[i] += v[4][:, i] @ h[:, i]
        return g, lap

    def j3_fields(self, r_up, r_dn):
        """h (A3, N): dJ3/dphi(r_i) with phi(r_i) held as the free variable; J3 is linear
        in each electron's AO vector, so grad_i J3 = grad phi(r_i) . h_i."""
        au, ad = ao_value(self.tab_j3, r_up), ao_value(self.tab_j3, r_dn)
        J = self.j3_mat
        nu, nd = au.shape[1], ad.shape[1]
        h = np.zeros((J.shape[0], nu + nd))
        for i in range(nu):
            h[:, i] = self.j3_vec + J.T @ au[:, :i].sum(1) + J @ au[:, i + 1:].sum(1) + J @ ad.sum(1)
        for j in range(nd):
            h[:, nu + j] = self.j3_vec + J.T @ ad[:, :j].sum(1) + J @ ad[:, j + 1:].sum(1) + J.T @ au.sum(1)
        return h

    def kinetic_elements(self, r_up, r_dn, Ginv):
        """T_i = -1/2 (lap ln psi_i + |grad ln psi_i|^2) (wavefunction.py:1142-1207)."""
        gJ, lJ = self.jastrow_grad_lap(r_up, r_dn)
        gu, gd, lu, ld = self.det_grad_lap(r_up, r_dn, Ginv)
        g = gJ + np.vstack([gu, gd])
        lap = lJ + np.concatenate([lu, ld])
        T = -0.5 * (lap + np.sum(g * g, axis=1))
        return T[: self.n_up], T[self.n_up:]

    # ---------------------------------------------------------------- Coulomb / ECP
    def coulomb_el_ion(self, r, alat=None):
        d = np.linalg.norm(r[:, None, :] - self.R[None], axis=-1)
        if alat is not None:
            d = np.maximum(d, alat)
        return np.sum(-self.Zeff[None, :] / d, axis=1)

    def coulomb_el_el(self, r_up, r_dn):
        r = np.vstack([r_up, r_dn])
        iu, ju = np.triu_indices(len(r), k=1)
        return float(np.sum(1.0 / np.linalg.norm(r[iu] - r[ju], axis=-1)))

    def coulomb_ion_ion(self):
        iu, ju = np.triu_indices(self.M, k=1)
        if len(iu) == 0:
            return 0.0
        return float(np.sum(self.Zeff[iu] * self.Zeff[ju] / np.linalg.norm(self.R[iu] - self.R[ju], axis=-1)))

    def bare_coulomb(self, r_up, r_dn):
        r = np.vstack([r_up, r_dn])
        return self.coulomb_ion_ion() + float(np.sum(self.coulomb_el_ion(r))) + self.coulomb_el_el(r_up, r_dn)

    def _V_channel(self, atom, l, dist):
        """r^-2 sum_k c_k r^n_k exp(-alpha_k r^2) over the terms of one channel."""
        v = 0.0
        for (a, ll, ex, co, pw) in self.ecp_terms:
            if a == atom and ll == l:
                v = v + co * dist**pw * np.exp(-ex * dist**2)
        return dist**-2.0 * v

    def ecp_local(self, r_up, r_dn):
        """coulomb_potential.py:601-661."""
        r = np.vstack([r_up, r_dn])
        tot = 0.0
        for atom in range(self.M):
            d = np.linalg.norm(r - self.R[atom], axis=1)
            tot += float(np.sum(self._V_channel(atom, int(self.maxl1[atom]), d)))
        return tot

    def nearest(self, r):
        d = np.sqrt(np.sum((self.R - r) ** 2, axis=1))
        return int(np.argsort(d, kind="stable")[0])

    def ecp_nonlocal(self, r_up, r_dn, RT, Ginv, Nv=6, ratio_fn=None):
        """Per-mesh-point V_nl (up electrons first, then dn; each electron Nv points) and
        their sum: coulomb_potential.py:1478-1712 with NN=1.  ``ratio_fn(spin, i, r')``
        returns psi(r')/psi(r); by default the det x Jastrow ratio."""
        w, pts = _meshes()[Nv]
        pts = pts @ RT
        out = []
        if ratio_fn is None:
            ratio_fn = lambda s, i, rn: self.wf_ratio(Ginv, r_up, r_dn, s, i, rn)  # noqa: E731
        for spin, rs in ((0, r_up), (1, r_dn)):
            for i, ri in enumerate(rs):
                atom = self.nearest(ri)
                rel = self.R[atom] - ri
                dist = np.linalg.norm(rel)
                lmax = int(self.maxl1[atom])
                for q in range(Nv):
                    rn = ri + rel + dist * pts[q]
                    cos_t = np.dot(-rel / dist, pts[q] / np.linalg.norm(pts[q]))
                    ratio = ratio_fn(spin, i, rn)
                    v = 0.0
                    for l in range(lmax):
                        v += self._V_channel(atom, l, dist) * (2 * l + 1) * legendre(l, cos_t) * w[q] * ratio
                    out.append(v)
        out = np.array(out)
        return out, float(np.sum(out))

    # ---------------------------------------------------------------- ratios
    def jastrow_ratio_move(self, r_up, r_dn, spin, idx, r_new):
        ru, rd = r_up.copy(), r_dn.copy()
        (ru if spin == 0 else rd)[idx] = r_new
        return float(np.exp(self.jastrow_total(ru, rd) - self.jastrow_total(r_up, r_dn)))

    def wf_ratio(self, Ginv, r_up, r_dn, spin, idx, r_new):
        return self.det_ratio_move(Ginv, r_up, r_dn, spin, idx, r_new) * self.jastrow_ratio_move(r_up, r_dn, spin, idx, r_new)

    # ---------------------------------------------------------------- energies
    def local_energy(self, r_up, r_dn, RT, Ginv):
        """E_L = sum T_i + V_bare + V_ecp_loc + V_ecp_nl (hamiltonians.py:225-290)."""
        tu, td = self.kinetic_elements(r_up, r_dn, Ginv)
        V = self.bare_coulomb(r_up, r_dn)
        if self.ecp:
            V += self.ecp_local(r_up, r_dn) + self.ecp_nonlocal(r_up, r_dn, RT, Ginv)[1]
        return float(np.sum(tu) + np.sum(td) + V)

    def discretized_kinetic(self, alat, r_up, r_dn, RT, Ginv):
        """Elements -ratio/(2 a^2) for the 6 rotated +-a shifts of every electron, up
        electrons first (wavefunction.py:1740-1860)."""
        shifts = alat * np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], float) @ RT
        el = []
        for spin, rs in ((0, r_up), (1, r_dn)):
            for i, ri in enumerate(rs):
                for k in range(6):
                    el.append(-1.0 / (2.0 * alat**2) * self.wf_ratio(Ginv, r_up, r_dn, spin, i, ri + shifts[k]))
        return np.array(el)
