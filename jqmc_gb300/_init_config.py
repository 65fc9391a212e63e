"""Initial electron positions, the role of _generate_init_electron_configurations
(jqmc/_jqmc_utility.py:54-220).

The assignment of electrons to nuclei is deterministic and shared by all walkers:
- the nuclei are visited in a farthest-next order starting from nucleus 0;
- down electrons go round that order, each nucleus taking at most Z//2
  (Z the rounded valence charge); when every nucleus is full, nuclei with
  Z//2 = 0 and room left come first, then any nucleus with room;
- up electrons then complete each nucleus to Z in the same order;
- up electrons beyond the total charge go to random nuclei, drawn per walker.

Each electron sits at its nucleus plus a spherical offset: distance U(0.1, 1)
bohr, polar angle U(0, pi), azimuth U(0, 2 pi), as the reference draws them.
The random numbers come from a seeded numpy Generator, not the reference's
global numpy state.
"""

from __future__ import annotations

import numpy as np

MIN_DIST, MAX_DIST = 0.1, 1.0


def nucleus_order(coords) -> np.ndarray:
    """Nucleus 0, then repeatedly the unvisited nucleus farthest from the last one
    (first index on ties)."""
    c = np.asarray(coords, dtype=np.float64)
    M = c.shape[0]
    seq = [0]
    free = np.ones(M, dtype=bool)
    free[0] = False
    for _ in range(1, M):
        d2 = np.where(free, np.sum((c[seq[-1]] - c) ** 2, axis=1), -1.0)
        nxt = int(np.argmax(d2))
        seq.append(nxt)
        free[nxt] = False
    return np.array(seq, dtype=int)


def electron_owners(charges, coords, n_up: int, n_dn: int):
    """(up_template (n_up,), dn_template (n_dn,), n_random_up, order): the nucleus of
    every electron; the last n_random_up up electrons are drawn per walker."""
    z = np.array([int(round(float(q))) for q in np.asarray(charges)], dtype=int)
    order = nucleus_order(coords)
    M = len(z)
    cap_dn = z // 2
    occ_dn = np.zeros(M, dtype=int)
    occ = np.zeros(M, dtype=int)
    dn = np.empty(n_dn, dtype=int)
    j = 0
    for i in range(n_dn):
        for _ in range(100 * (M + 1) * (n_dn + 1)):
            a = order[j % M]
            j += 1
            if np.any(occ_dn < cap_dn):
                ok = occ_dn[a] < cap_dn[a]
            elif np.any((cap_dn == 0) & (occ < z)):
                ok = cap_dn[a] == 0 and occ[a] < z[a]
            else:
                ok = occ[a] < z[a]
            if ok:
                dn[i] = a
                occ_dn[a] += 1
                occ[a] += 1
                break
        else:
            raise ValueError(f"{n_dn} down electrons do not fit the nuclear charges {z.tolist()}")
    need_up = z - occ_dn
    up = np.empty(n_up, dtype=int)
    n_random = 0
    if n_up <= int(need_up.sum()):
        occ_up = np.zeros(M, dtype=int)
        j = 0
        for i in range(n_up):
            while True:
                a = order[j % M]
                j += 1
                if occ_up[a] < need_up[a]:
                    up[i] = a
                    occ_up[a] += 1
                    break
    else:
        k = 0
        for a in order:
            for _ in range(int(need_up[a])):
                up[k] = a
                k += 1
        n_random = n_up - k
    return up, dn, n_random, order


def _offsets(rng, shape) -> np.ndarray:
    d = rng.uniform(MIN_DIST, MAX_DIST, size=shape)
    th = rng.uniform(0.0, np.pi, size=shape)
    ph = rng.uniform(0.0, 2.0 * np.pi, size=shape)
    s = np.sin(th)
    return np.stack([d * s * np.cos(ph), d * s * np.sin(ph), d * np.cos(th)], axis=-1)


def initial_electrons(positions, valence, n_up: int, n_dn: int, num_walkers: int, seed: int):
    """(r_up (W, n_up, 3), r_dn (W, n_dn, 3)) for num_walkers walkers."""
    rng = np.random.default_rng(seed)
    pos = np.asarray(positions, dtype=np.float64)
    up, dn, n_random, order = electron_owners(valence, pos, n_up, n_dn)
    up_owner = np.broadcast_to(up, (num_walkers, n_up)).copy()
    if n_random:
        pick = rng.integers(0, len(order), size=(num_walkers, n_random))
        up_owner[:, n_up - n_random:] = order[pick]
    dn_owner = np.broadcast_to(dn, (num_walkers, n_dn))
    r_up = pos[up_owner] + _offsets(rng, (num_walkers, n_up))
    r_dn = pos[dn_owner] + _offsets(rng, (num_walkers, n_dn))
    return r_up, r_dn
