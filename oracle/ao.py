"""Oracle: spherical GTO values, gradients and Laplacians (FP64, NumPy).

Restates jqmc/atomic_orbital.py:
  * AO value   -- _compute_AOs_sphe_debug (atomic_orbital.py:1931-1981) and
                  _compute_AOs_sphe (atomic_orbital.py:2294-2349);
  * S_lm table -- _compute_S_l_m (atomic_orbital.py:2353-2585): real regular solid
                  harmonics r^l Y_lm scaled by sqrt(4pi/(2l+1)), index l^2 + (m + l);
  * value/grad/lap -- _compute_AOs_value_grad_lap_sphe (atomic_orbital.py:3511-3591):
        grad = pref S (-2 Z d) + pref grad S
        lap  = pref lap S + pref S (4 Z^2 r^2 - 6 Z) - 4 Z pref (grad S . d)

The solid harmonics are evaluated here from the closed form
    Pi_l^m(z, r^2) = sqrt((l-m)!/(l+m)!) sum_k (-1)^k 2^-l C(l,k) C(2l-2k,l) (l-2k)!/(l-2k-m)! r^2k z^(l-2k-m)
    C_l^m = sqrt(2) Pi_l^m Re (x+iy)^m,   S_l^m = sqrt(2) Pi_l^m Im (x+iy)^m,   C_l^0 = Pi_l^0
(the Racah-normalised real solid harmonics), which equals the reference's
explicit table entry by entry (pinned by tests/golden).  lap S = 0 since solid
harmonics are harmonic.

Cartesian AOs (AOs_cart_data; _compute_AOs_cart_debug atomic_orbital.py:1984-2030,
_compute_AOs_cart :2198-2290, _compute_AOs_value_grad_lap_cart :3378-3510) take
the monomial P = x^nx y^ny z^nz in place of S, the primitive normalisation
sqrt((2Z/pi)^(3/2) (8Z)^l nx!ny!nz!/((2nx)!(2ny)!(2nz)!)), and lap P (not zero)
adds R lap P to the Laplacian.  Pinned by tests/golden/cart.npz.
"""

from __future__ import annotations

from math import comb, factorial, pi, sqrt

import numpy as np


def _pi_terms(l: int, m: int):
    """[(coef, k, zpow)] for Pi_l^m = sum coef * (r^2)^k * z^zpow."""
    pref = sqrt(factorial(l - m) / factorial(l + m))
    terms = []
    for k in range((l - m) // 2 + 1):
        c = ((-1) ** k) * (2.0 ** -l) * comb(l, k) * comb(2 * l - 2 * k, l) * factorial(l - 2 * k) / factorial(l - 2 * k - m)
        terms.append((pref * c, k, l - 2 * k - m))
    return terms


def solid_harmonics(l: int, d: np.ndarray):
    """S (2l+1, ...) and grad S (2l+1, ..., 3) at displacement d (..., 3); row
    j is m = j - l, matching the reference's (l, m) ordering."""
    x, y, z = d[..., 0], d[..., 1], d[..., 2]
    r2 = x * x + y * y + z * z
    S = np.zeros((2 * l + 1,) + x.shape)
    G = np.zeros((2 * l + 1,) + x.shape + (3,))
    w = x + 1j * y
    for m in range(0, l + 1):
        P = np.zeros_like(x)
        dP_dz = np.zeros_like(x)
        dP_dr2 = np.zeros_like(x)
        for c, k, zp in _pi_terms(l, m):
            P = P + c * r2**k * z**zp
            if zp > 0:
                dP_dz = dP_dz + c * zp * r2**k * z ** (zp - 1)
            if k > 0:
                dP_dr2 = dP_dr2 + c * k * r2 ** (k - 1) * z**zp
        # grad of P(z, r2): dP/dx = dP/dr2 * 2x ; dP/dz = dP/dz + dP/dr2 * 2z
        gP = np.stack([dP_dr2 * 2 * x, dP_dr2 * 2 * y, dP_dz + dP_dr2 * 2 * z], axis=-1)
        if m == 0:
            S[l] = P
            G[l] = gP
            continue
        wm = w**m
        dwm = m * w ** (m - 1)       # d/dx (x+iy)^m ; d/dy = i * dwm
        A, B = wm.real, wm.imag
        gA = np.stack([dwm.real, (1j * dwm).real, np.zeros_like(x)], axis=-1)
        gB = np.stack([dwm.imag, (1j * dwm).imag, np.zeros_like(x)], axis=-1)
        s2 = sqrt(2.0)
        S[l + m] = s2 * P * A
        S[l - m] = s2 * P * B
        G[l + m] = s2 * (gP * A[..., None] + P[..., None] * gA)
        G[l - m] = s2 * (gP * B[..., None] + P[..., None] * gB)
    return S, G


def primitive_norm(l: int, Z):
    """N_p of atomic_orbital.py:2316-2323 times sqrt((2l+1)/4pi)."""
    n2 = (2.0 ** (2 * l + 3)) * factorial(l + 1) * (2.0 * Z) ** (l + 1.5) / (factorial(2 * l + 2) * sqrt(pi))
    return np.sqrt(n2) * sqrt((2 * l + 1) / (4.0 * pi))


def cartesian_norm(l: int, Z, nx: int, ny: int, nz: int):
    """Primitive normalisation of a Cartesian Gaussian (atomic_orbital.py:2005-2016)."""
    ratio = factorial(nx) * factorial(ny) * factorial(nz) / (factorial(2 * nx) * factorial(2 * ny) * factorial(2 * nz))
    return np.sqrt((2.0 * Z / pi) ** 1.5 * (8.0 * Z) ** l * ratio)


class AOTable:
    """Per-AO primitive tables (padded to the deepest contraction) extracted once
    from an AOs_sphe_data- or AOs_cart_data-like object."""

    def __init__(self, aos):
        self.num_ao = aos.num_ao
        self.centers = np.asarray(aos.structure_data.positions)[np.asarray(aos.nucleus_index, dtype=int)]
        self.l = np.asarray(aos.angular_momentums, dtype=int)
        self.cart = hasattr(aos, "polynominal_order_x")
        if self.cart:
            self.pw = np.stack([np.asarray(aos.polynominal_order_x, dtype=int), np.asarray(aos.polynominal_order_y, dtype=int),
                                np.asarray(aos.polynominal_order_z, dtype=int)], axis=1)          # (A, 3)
            self.m = np.zeros(self.num_ao, dtype=int)
        else:
            self.m = np.asarray(aos.magnetic_quantum_numbers, dtype=int)
        oi = np.asarray(aos.orbital_indices, dtype=int)
        ex = np.asarray(aos.exponents, dtype=np.float64)
        co = np.asarray(aos.coefficients, dtype=np.float64)
        kmax = int(np.max(np.bincount(oi, minlength=self.num_ao)))
        self.Z = np.zeros((self.num_ao, kmax))
        self.cN = np.zeros((self.num_ao, kmax))
        for a in range(self.num_ao):
            z, c = ex[oi == a], co[oi == a]
            self.Z[a, : len(z)] = z
            if self.cart:
                self.cN[a, : len(z)] = c * cartesian_norm(int(self.l[a]), z, *(int(x) for x in self.pw[a]))
            else:
                self.cN[a, : len(z)] = c * primitive_norm(int(self.l[a]), z)
        self.by_l = {l: np.nonzero(self.l == l)[0] for l in np.unique(self.l)}


def _common(tab: AOTable, r, need_grad: bool):
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    d = r[:, None, :] - tab.centers[None, :, :]                     # (P, A, 3)
    r2 = np.sum(d * d, axis=-1)                                      # (P, A)
    e = np.exp(-tab.Z[None, :, :] * r2[:, :, None])                  # (P, A, K)
    pref = tab.cN[None] * e                                          # (P, A, K)
    if tab.cart:
        return (d, r2, pref) + _monomials(tab.pw, d, need_grad)
    S = np.zeros(r2.shape)
    gS = np.zeros(d.shape) if need_grad else None
    for l, idx in tab.by_l.items():
        Sl, Gl = solid_harmonics(int(l), d[:, idx])                  # (2l+1, P, n), (2l+1, P, n, 3)
        sel = tab.m[idx] + l
        cols = np.arange(len(idx))
        S[:, idx] = Sl[sel, :, cols].T
        if need_grad:
            gS[:, idx] = np.transpose(Gl[sel, :, cols], (1, 0, 2))
    return d, r2, pref, S, gS, None


def _ipow(x, n):
    """x^n elementwise for integer n >= 0 per column (0^0 = 1); n may be negative (-> 0)."""
    n = np.asarray(n)
    return np.where(n >= 0, np.power(x, np.maximum(n, 0)), 0.0)


def _monomials(pw, d, need_grad):
    """(P, grad P, lap P) of x^nx y^ny z^nz at displacements d (P, A, 3)."""
    x, y, z = d[..., 0], d[..., 1], d[..., 2]
    nx, ny, nz = pw[:, 0][None], pw[:, 1][None], pw[:, 2][None]
    px, py, pz = _ipow(x, nx), _ipow(y, ny), _ipow(z, nz)
    P = px * py * pz
    if not need_grad:
        return P, None, None
    dx = nx * _ipow(x, nx - 1) * py * pz
    dy = ny * px * _ipow(y, ny - 1) * pz
    dz = nz * px * py * _ipow(z, nz - 1)
    lap = (nx * (nx - 1) * _ipow(x, nx - 2) * py * pz + ny * (ny - 1) * px * _ipow(y, ny - 2) * pz
           + nz * (nz - 1) * px * py * _ipow(z, nz - 2))
    return P, np.stack([dx, dy, dz], axis=-1), lap


def ao_value(tab: AOTable, r: np.ndarray) -> np.ndarray:
    """AO values (num_ao, P) at points r (P, 3)."""
    d, r2, pref, S, _, _ = _common(tab, r, False)
    return (pref.sum(-1) * S).T


def ao_vgl(tab: AOTable, r: np.ndarray):
    """(val, gx, gy, gz, lap), each (num_ao, P), following atomic_orbital.py:3560-3591."""
    d, r2, pref, S, gS, lapS = _common(tab, r, True)
    Z = tab.Z[None]                                                  # (1, A, K)
    ao_p = pref * S[..., None]                                       # (P, A, K)
    g = (ao_p[..., None] * (-2.0 * Z[..., None] * d[:, :, None, :]) + pref[..., None] * gS[:, :, None, :]).sum(2)
    gSd = np.sum(gS * d, axis=-1)                                    # (P, A)
    lap = (ao_p * (4.0 * Z**2 * r2[..., None] - 6.0 * Z) - 4.0 * Z * pref * gSd[..., None]).sum(-1)
    if lapS is not None:                                             # Cartesian: R lap P
        lap = lap + pref.sum(-1) * lapS
    val = ao_p.sum(-1)
    return val.T, g[..., 0].T, g[..., 1].T, g[..., 2].T, lap.T
