"""Seeded synthetic molecules for the walker-path workloads.

No public dataset is involved: every workload is a seeded synthetic system with
the shapes and value distributions below.

* ``water_like``   -- 3 nuclei: O-like (Z=8, 2 core electrons -> Z_eff=6, ECP)
  at the origin and two H (Z=1) at (+-1.43, 1.11, 0) bohr; 8 valence electrons
  (4 up / 4 dn); ~40 spherical GTOs (l <= 2, 1-4 primitives per shell);
  Jastrow-Slater (MO geminal, 4 occupied MOs per spin); J3 on 20 AOs.
* ``ring12``       -- 6 C-like nuclei (Z=6, 2 core -> Z_eff=4, ECP) on a ring of
  radius 2.64 bohr and 6 H on radius 4.69 bohr; 30 electrons (15/15); ~200 AOs;
  JAGP geminal lambda = C_occ C_occ^T + 0.01 * sym(N(0,1)); J3 on 60 AOs.
* ``chain32``      -- 32-nucleus zig-zag chain (16 Z_eff=4 with ECP, 16 H),
  bond 2.6 bohr; 96 electrons (48/48) as the workload states (the nuclear
  charge sums to 80, so the system carries charge -16); ~740 AOs; JAGP; J3 on 64 AOs.
* ``random_molecule`` -- 1-20 nuclei with Z_eff in {1, 4, 6}, minimum separation
  2.0 bohr, water-like recipes per atom (the 64-molecule batching workload).

Basis recipe: exponents log-uniform in [0.05, 40] bohr^-2, contraction
coefficients U(0.1, 1) normalised so that <phi|phi> = 1.  MO coefficients are
N(0,1) orthonormalised by QR.  ECP: a local channel (terms with powers 1 and 3)
plus l = 0, 1 non-local channels (power 2), two terms each, alpha ~ U(1, 15),
c ~ N(0, 5).  Initial electrons: assigned to nuclei by valence count (spin
balanced) and displaced by N(0, 1 bohr).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from ._init_config import initial_electrons
from .atomic_orbital import AOs_sphe_data
from .coulomb_potential import Coulomb_potential_data
from .determinant import Geminal_data
from .hamiltonians import Hamiltonian_data
from .jastrow_factor import Jastrow_data, Jastrow_one_body_data, Jastrow_three_body_data, Jastrow_two_body_data
from .molecular_orbital import MOs_data
from .structure import Structure_data
from .wavefunction import Wavefunction_data

# shells per atom kind: list of (l, count)
RECIPE_SMALL = {"heavy": [(0, 4), (1, 3), (2, 2)], "H": [(0, 3), (1, 2)]}            # 23 / 9 AOs
RECIPE_LARGE = {"heavy": [(0, 5), (1, 4), (2, 3)], "H": [(0, 3), (1, 2), (2, 1)]}    # 32 / 14 AOs
J3_RECIPE_WATER = {"heavy": [(0, 2), (1, 1), (2, 1)], "H": [(0, 2), (1, 1)]}         # 10 / 5
J3_RECIPE_RING = {"heavy": [(0, 2), (1, 1)], "H": [(0, 2), (1, 1)]}                 # 5 / 5
J3_RECIPE_CHAIN = {"heavy": [(0, 1), (1, 1)], "H": []}                               # 4 / 0


def _overlap_normalised(l, za, zb):
    """Overlap of two normalised same-centre primitives of angular momentum l."""
    return (2.0 * np.sqrt(za * zb) / (za + zb)) ** (l + 1.5)


def build_basis(structure: Structure_data, kinds, recipe, rng) -> AOs_sphe_data:
    nucleus_index, orbital_indices, exps, coefs, ls, ms = [], [], [], [], [], []
    ao = 0
    for atom, kind in enumerate(kinds):
        for l, count in recipe[kind]:
            for _ in range(count):
                nprim = int(rng.integers(1, 5))
                z = np.sort(np.exp(rng.uniform(np.log(0.05), np.log(40.0), size=nprim)))[::-1]
                c = rng.uniform(0.1, 1.0, size=nprim)
                s = _overlap_normalised(l, z[:, None], z[None, :])
                c = c / np.sqrt(c @ s @ c)
                for m in range(-l, l + 1):
                    nucleus_index.append(atom)
                    ls.append(l)
                    ms.append(m)
                    for p in range(nprim):
                        orbital_indices.append(ao)
                        exps.append(z[p])
                        coefs.append(c[p])
                    ao += 1
    return AOs_sphe_data(
        structure_data=structure, nucleus_index=tuple(nucleus_index), num_ao=ao, num_ao_prim=len(exps),
        orbital_indices=tuple(orbital_indices), exponents=np.array(exps), coefficients=np.array(coefs),
        angular_momentums=tuple(ls), magnetic_quantum_numbers=tuple(ms),
    )


def build_ecp(structure: Structure_data, kinds, z_cores, rng) -> Coulomb_potential_data:
    ang, nuc, ex, co, pw = [], [], [], [], []
    maxl1 = []
    for atom, kind in enumerate(kinds):
        if kind == "H":
            # no pseudopotential: one local term with zero coefficient, so that every
            # nucleus is listed in the ECP table (as TREXIO inputs list them)
            maxl1.append(0)
            ang.append(0)
            nuc.append(atom)
            ex.append(1.0)
            co.append(0.0)
            pw.append(2)
            continue
        maxl1.append(2)
        for l, powers in ((2, (1, 3)), (0, (2, 2)), (1, (2, 2))):
            for n in powers:
                ang.append(l)
                nuc.append(atom)
                ex.append(float(rng.uniform(1.0, 15.0)))
                co.append(float(rng.normal(0.0, 5.0)))
                pw.append(n)
    return Coulomb_potential_data(
        structure_data=structure, ecp_flag=True, z_cores=tuple(z_cores), max_ang_mom_plus_1=tuple(maxl1),
        num_ecps=len(ang), ang_moms=tuple(ang), nucleus_index=tuple(nuc), exponents=tuple(ex),
        coefficients=tuple(co), powers=tuple(pw),
    )


def _orthonormal(n, rng):
    q, r = np.linalg.qr(rng.normal(size=(n, n)))
    return q * np.sign(np.diag(r))[None, :]


@dataclass
class SyntheticSystem:
    name: str
    hamiltonian: Hamiltonian_data
    n_up: int
    n_dn: int
    valence: np.ndarray

    def initial_electrons(self, num_walkers: int, seed: int = 0):
        """(W, n_up, 3), (W, n_dn, 3): electrons assigned to nuclei by valence count,
        alternating spins, displaced by N(0, 1 bohr)."""
        return initial_electrons(self.hamiltonian.structure_data.positions, self.valence, self.n_up, self.n_dn,
                                 num_walkers, seed)


def _assemble(name, positions, atomic_numbers, z_cores, kinds, n_up, n_dn, det_recipe, j3_recipe, rng,
              jsd: bool, jastrow_1b=1.0, jastrow_2b=1.0) -> SyntheticSystem:
    structure = Structure_data(positions=np.asarray(positions, float), atomic_numbers=tuple(atomic_numbers),
                               element_symbols=tuple("X" for _ in kinds), atomic_labels=tuple(f"X{i}" for i in range(len(kinds))))
    aos = build_basis(structure, kinds, det_recipe, rng)
    aos_j3 = build_basis(structure, kinds, j3_recipe, rng)
    coul = build_ecp(structure, kinds, z_cores, rng)
    A = aos.num_ao
    C = _orthonormal(A, rng)                  # columns orthonormal
    if jsd:
        mo_up = MOs_data(num_mo=n_up, aos_data=aos, mo_coefficients=C[:, :n_up].T.copy())
        geminal = Geminal_data(num_electron_up=n_up, num_electron_dn=n_dn, orb_data_up_spin=mo_up,
                               orb_data_dn_spin=mo_up, lambda_matrix=np.eye(n_up))
    else:
        c_occ = C[:, :n_up]
        noise = rng.normal(size=(A, A))
        lam = c_occ @ c_occ.T + 0.01 * 0.5 * (noise + noise.T)
        geminal = Geminal_data(num_electron_up=n_up, num_electron_dn=n_dn, orb_data_up_spin=aos,
                               orb_data_dn_spin=aos, lambda_matrix=lam)
    A3 = aos_j3.num_ao
    jm = rng.normal(size=(A3, A3))
    jmat = np.zeros((A3, A3 + 1))
    jmat[:, :A3] = 0.01 * 0.5 * (jm + jm.T)
    jmat[:, A3] = 0.01 * rng.normal(size=A3)
    jas = Jastrow_data(
        jastrow_one_body_data=Jastrow_one_body_data(jastrow_1b_param=jastrow_1b, jastrow_1b_type="exp",
                                                    structure_data=structure, core_electrons=tuple(float(z) for z in z_cores)),
        jastrow_two_body_data=Jastrow_two_body_data(jastrow_2b_param=jastrow_2b, jastrow_2b_type="pade"),
        jastrow_three_body_data=Jastrow_three_body_data(orb_data=aos_j3, j_matrix=jmat),
    )
    ham = Hamiltonian_data(structure_data=structure, coulomb_potential_data=coul,
                           wavefunction_data=Wavefunction_data(jastrow_data=jas, geminal_data=geminal))
    ham.sanity_check()
    valence = np.asarray(atomic_numbers, float) - np.asarray(z_cores, float)
    return SyntheticSystem(name, ham, n_up, n_dn, valence)


def water_like(seed: int = 0) -> SyntheticSystem:
    rng = np.random.default_rng(seed)
    pos = [[0.0, 0.0, 0.0], [1.43, 1.11, 0.0], [-1.43, 1.11, 0.0]]
    return _assemble("water_like", pos, (8, 1, 1), (2, 0, 0), ["heavy", "H", "H"], 4, 4,
                     RECIPE_SMALL, J3_RECIPE_WATER, rng, jsd=True)


def ring12(seed: int = 0) -> SyntheticSystem:
    rng = np.random.default_rng(seed)
    ang = np.arange(6) * np.pi / 3.0
    pos = [[2.64 * np.cos(a), 2.64 * np.sin(a), 0.0] for a in ang] + [[4.69 * np.cos(a), 4.69 * np.sin(a), 0.0] for a in ang]
    return _assemble("ring12", pos, (6,) * 6 + (1,) * 6, (2,) * 6 + (0,) * 6, ["heavy"] * 6 + ["H"] * 6, 15, 15,
                     RECIPE_SMALL, J3_RECIPE_RING, rng, jsd=False)


def chain32(seed: int = 0) -> SyntheticSystem:
    rng = np.random.default_rng(seed)
    bond = 2.6
    pos = [[k * bond * np.cos(np.pi / 6.0), (0.5 if k % 2 else -0.5) * bond * np.sin(np.pi / 6.0), 0.0] for k in range(32)]
    kinds = ["heavy" if k % 2 == 0 else "H" for k in range(32)]
    zs = tuple(6 if k == "heavy" else 1 for k in kinds)
    zc = tuple(2 if k == "heavy" else 0 for k in kinds)
    return _assemble("chain32", pos, zs, zc, kinds, 48, 48, RECIPE_LARGE, J3_RECIPE_CHAIN, rng, jsd=False)


def random_molecule(seed: int) -> SyntheticSystem:
    rng = np.random.default_rng(1000 + seed)
    natom = int(rng.integers(1, 21))
    pos = []
    while len(pos) < natom:
        p = rng.uniform(-2.0, 2.0, size=3) * (1.0 + natom ** (1.0 / 3.0))
        if all(np.linalg.norm(p - q) >= 2.0 for q in pos):
            pos.append(p)
    zeff = rng.choice([1, 4, 6], size=natom)
    if natom == 1 and zeff[0] == 1:
        zeff[0] = 4
    kinds = ["H" if z == 1 else "heavy" for z in zeff]
    zs = tuple(int(z + 2) if z > 1 else 1 for z in zeff)
    zc = tuple(2 if z > 1 else 0 for z in zeff)
    ne = int(np.sum(zeff))
    n_up = (ne + 1) // 2
    n_dn = ne // 2
    if n_up != n_dn:   # keep closed shells on the batching workload
        n_dn = n_up
    return _assemble(f"mol{seed}", pos, zs, zc, kinds, n_up, n_dn, RECIPE_SMALL, J3_RECIPE_WATER, rng, jsd=True)


SYSTEMS = {"water_like": water_like, "ring12": ring12, "chain32": chain32}
