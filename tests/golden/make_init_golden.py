"""Golden fixture for the initial electron assignment, made by running the
reference's _generate_init_electron_configurations (jqmc/_jqmc_utility.py:54-220)
on the NumPy stand-in for JAX (tests/golden/jaxshim).

Cases: the three synthetic systems (water_like, ring12, chain32) with their
valence charges and electron counts, and small nuclear sets that exercise the
other branches (odd counts, a homonuclear dimer, a hydrogen atom, more up
electrons than the total charge, nuclei with Z//2 = 0).  For each case the
reference's up and down owners of 64 walkers are stored in
tests/golden/init_owners.npz (up electrons past the total charge go to random
nuclei, so only their range can be compared).
Run: python tests/golden/make_init_golden.py
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REFERENCE = "/root/reference"
sys.path.insert(0, os.path.join(HERE, "jaxshim"))
sys.path.insert(0, REFERENCE)
sys.path.insert(0, ROOT)

from jqmc._jqmc_utility import _generate_init_electron_configurations  # noqa: E402

from jqmc_gb300 import synthetic  # noqa: E402


def cases():
    out = {}
    for name in ("water_like", "ring12", "chain32"):
        syn = synthetic.SYSTEMS[name]()
        h = syn.hamiltonian
        out[name] = (np.asarray(h.coulomb_potential_data.effective_charges, dtype=float),
                     np.asarray(h.structure_data.positions, dtype=float), syn.n_up, syn.n_dn)
    line = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 2.1], [0.0, 0.0, 4.4]])
    out["odd_triatomic"] = (np.array([6.0, 1.0, 1.0]), line, 5, 3)
    out["dimer"] = (np.array([5.0, 5.0]), line[:2], 5, 5)
    out["dimer_triplet"] = (np.array([4.0, 4.0]), line[:2], 5, 3)
    out["hydrogen"] = (np.array([1.0]), line[:1], 1, 0)
    out["excess_up"] = (np.array([1.0, 1.0]), line[:2], 3, 0)
    out["light_nuclei"] = (np.array([1.0, 1.0, 3.0]), line, 3, 2)
    return out


def main():
    out = {}
    for name, (z, c, nu, nd) in cases().items():
        np.random.seed(7)
        _, _, uo, do = _generate_init_electron_configurations(nu, nd, 64, z, c)
        out[f"{name}.charges"] = z
        out[f"{name}.coords"] = c
        out[f"{name}.n"] = np.array([nu, nd])
        out[f"{name}.up_owner"] = np.asarray(uo)
        out[f"{name}.dn_owner"] = np.asarray(do)
    out["cases"] = np.array(list(cases()))
    np.savez_compressed(os.path.join(HERE, "init_owners.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
