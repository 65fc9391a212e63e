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


class AOTable:
    """Per-AO primitive lists extracted once from an AOs_sphe_data-like object."""

    def __init__(self, aos):
        self.num_ao = aos.num_ao
        self.centers = np.asarray(aos.structure_data.positions)[np.asarray(aos.nucleus_index, dtype=int)]
        self.l = np.asarray(aos.angular_momentums, dtype=int)
        self.m = np.asarray(aos.magnetic_quantum_numbers, dtype=int)
        oi = np.asarray(aos.orbital_indices, dtype=int)
        ex = np.asarray(aos.exponents, dtype=np.float64)
        co = np.asarray(aos.coefficients, dtype=np.float64)
        self.prims = [(ex[oi == a], co[oi == a]) for a in range(self.num_ao)]


def ao_value(tab: AOTable, r: np.ndarray) -> np.ndarray:
    """AO values (num_ao, P) at points r (P, 3)."""
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((tab.num_ao, r.shape[0]))
    cache = {}
    for a in range(tab.num_ao):
        d = r - tab.centers[a]
        r2 = np.sum(d * d, axis=-1)
        l, m = int(tab.l[a]), int(tab.m[a])
        key = (tuple(tab.centers[a]), l)
        if key not in cache:
            cache[key] = solid_harmonics(l, d)[0]
        Z, c = tab.prims[a]
        rad = np.sum((c * primitive_norm(l, Z))[:, None] * np.exp(-Z[:, None] * r2[None, :]), axis=0)
        out[a] = rad * cache[key][m + l]
    return out


def ao_vgl(tab: AOTable, r: np.ndarray):
    """(val, gx, gy, gz, lap), each (num_ao, P), following atomic_orbital.py:3560-3591."""
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    P = r.shape[0]
    val = np.zeros((tab.num_ao, P))
    grad = np.zeros((tab.num_ao, P, 3))
    lap = np.zeros((tab.num_ao, P))
    cache = {}
    for a in range(tab.num_ao):
        d = r - tab.centers[a]
        r2 = np.sum(d * d, axis=-1)
        l, m = int(tab.l[a]), int(tab.m[a])
        key = (tuple(tab.centers[a]), l)
        if key not in cache:
            cache[key] = solid_harmonics(l, d)
        S = cache[key][0][m + l]
        gS = cache[key][1][m + l]
        Z, c = tab.prims[a]
        pref = (c * primitive_norm(l, Z))[:, None] * np.exp(-Z[:, None] * r2[None, :])   # (np, P)
        ao_p = pref * S[None, :]
        g = ao_p[..., None] * (-2.0 * Z[:, None, None] * d[None]) + pref[..., None] * gS[None]
        gSd = np.sum(gS * d, axis=-1)
        lp = ao_p * (4.0 * Z[:, None] ** 2 * r2[None, :] - 6.0 * Z[:, None]) - 4.0 * Z[:, None] * pref * gSd[None, :]
        val[a] = ao_p.sum(0)
        grad[a] = g.sum(0)
        lap[a] = lp.sum(0)
    return val, grad[..., 0], grad[..., 1], grad[..., 2], lap
