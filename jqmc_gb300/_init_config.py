"""Initial electron positions around the nuclei by valence count (spin balanced),
the role of _generate_init_electron_configurations (jqmc/_jqmc_utility.py:54-220):
electron k of the valence sequence sits on its nucleus plus an N(0, 1 bohr)
displacement; spins alternate."""

from __future__ import annotations

import numpy as np


def initial_electrons(positions, valence, n_up: int, n_dn: int, num_walkers: int, seed: int):
    rng = np.random.default_rng(seed)
    pos = np.asarray(positions, dtype=np.float64)
    owners = []
    for atom, v in enumerate(np.asarray(valence)):
        owners += [atom] * int(round(float(v)))
    total = n_up + n_dn
    while len(owners) < total:
        owners.append(len(owners) % len(pos))
    up_owner, dn_owner = [], []
    for k, atom in enumerate(owners[:total]):
        want_up = (k % 2 == 0 and len(up_owner) < n_up) or len(dn_owner) >= n_dn
        (up_owner if want_up else dn_owner).append(atom)
    r_up = pos[np.array(up_owner, dtype=int)][None] + rng.normal(size=(num_walkers, n_up, 3))
    r_dn = pos[np.array(dn_owner, dtype=int)][None] + rng.normal(size=(num_walkers, n_dn, 3))
    return r_up, r_dn
