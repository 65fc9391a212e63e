"""Generate golden fixtures by running the reference's own functions.

Run from the repository root in a container that has the reference checked out
at /root/reference:

    python tests/golden/make_golden.py

JAX is not installed, so the reference modules are imported on top of the NumPy
stand-in in ``tests/golden/jaxshim`` (``jit`` = identity, ``vmap`` = Python
loop, ``lax`` control flow run eagerly; jax.numpy = NumPy in float64).  The
per-walker functions listed in ``CALLS`` are then executed unmodified on seeded
synthetic systems and electron configurations, and their outputs are written to
``tests/golden/<system>.npz`` together with the inputs.  The fixtures are
small; tests read only the .npz files, never the reference.
"""

from __future__ import annotations

import os
import sys
import traceback

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REFERENCE = "/root/reference"
sys.path.insert(0, os.path.join(HERE, "jaxshim"))
sys.path.insert(0, REFERENCE)
sys.path.insert(0, ROOT)

import jqmc.atomic_orbital as r_ao  # noqa: E402
import jqmc.coulomb_potential as r_cp  # noqa: E402
import jqmc.determinant as r_det  # noqa: E402
import jqmc.hamiltonians as r_ham  # noqa: E402
import jqmc.jastrow_factor as r_jas  # noqa: E402
import jqmc.molecular_orbital as r_mo  # noqa: E402
import jqmc.structure as r_st  # noqa: E402
import jqmc.swct as r_swct  # noqa: E402
import jqmc.wavefunction as r_wf  # noqa: E402

from jqmc_gb300 import synthetic  # noqa: E402
from jqmc_gb300.molecular_orbital import MOs_data  # noqa: E402


def to_ref_structure(s):
    return r_st.Structure_data(positions=np.asarray(s.positions), pbc_flag=False, atomic_numbers=tuple(s.atomic_numbers),
                               element_symbols=tuple(s.element_symbols), atomic_labels=tuple(s.atomic_labels))


def to_ref_aos(a, st):
    return r_ao.AOs_sphe_data(structure_data=st, nucleus_index=tuple(a.nucleus_index), num_ao=a.num_ao,
                              num_ao_prim=a.num_ao_prim, orbital_indices=tuple(a.orbital_indices),
                              exponents=np.asarray(a.exponents), coefficients=np.asarray(a.coefficients),
                              angular_momentums=tuple(a.angular_momentums),
                              magnetic_quantum_numbers=tuple(a.magnetic_quantum_numbers))


def to_ref_hamiltonian(h):
    st = to_ref_structure(h.structure_data)
    g = h.wavefunction_data.geminal_data

    def orb(o):
        if isinstance(o, MOs_data):
            return r_mo.MOs_data(num_mo=o.num_mo, aos_data=to_ref_aos(o.aos_data, st), mo_coefficients=np.asarray(o.mo_coefficients))
        return to_ref_aos(o, st)

    up = orb(g.orb_data_up_spin)
    dn = up if g.orb_data_dn_spin is g.orb_data_up_spin else orb(g.orb_data_dn_spin)
    gem = r_det.Geminal_data(num_electron_up=g.num_electron_up, num_electron_dn=g.num_electron_dn,
                             orb_data_up_spin=up, orb_data_dn_spin=dn, lambda_matrix=np.asarray(g.lambda_matrix))
    jd = h.wavefunction_data.jastrow_data
    j1 = jd.jastrow_one_body_data
    j2 = jd.jastrow_two_body_data
    j3 = jd.jastrow_three_body_data
    jas = r_jas.Jastrow_data(
        jastrow_one_body_data=r_jas.Jastrow_one_body_data(jastrow_1b_param=np.asarray(j1.jastrow_1b_param), jastrow_1b_type=j1.jastrow_1b_type,
                                                          structure_data=st, core_electrons=tuple(j1.core_electrons)),
        jastrow_two_body_data=r_jas.Jastrow_two_body_data(jastrow_2b_param=np.asarray(j2.jastrow_2b_param), jastrow_2b_type=j2.jastrow_2b_type),
        jastrow_three_body_data=r_jas.Jastrow_three_body_data(orb_data=to_ref_aos(j3.orb_data, st), j_matrix=np.asarray(j3.j_matrix)),
        jastrow_nn_data=None,
    )
    c = h.coulomb_potential_data
    coul = r_cp.Coulomb_potential_data(structure_data=st, ecp_flag=c.ecp_flag, z_cores=tuple(c.z_cores),
                                       max_ang_mom_plus_1=tuple(c.max_ang_mom_plus_1), num_ecps=c.num_ecps,
                                       ang_moms=tuple(c.ang_moms), nucleus_index=tuple(c.nucleus_index),
                                       exponents=tuple(c.exponents), coefficients=tuple(c.coefficients), powers=tuple(c.powers))
    wf = r_wf.Wavefunction_data(jastrow_data=jas, geminal_data=gem)
    return r_ham.Hamiltonian_data(structure_data=st, coulomb_potential_data=coul, wavefunction_data=wf)


def rotation(a, b, g):
    """Euler rotation of jqmc_mcmc.py:4228-4245 (returned R, callers transpose)."""
    ca, sa, cb, sb, cg, sg = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(g), np.sin(g)
    return np.array([[cb * cg, cg * sa * sb - ca * sg, sa * sg + ca * cg * sb],
                     [cb * sg, ca * cg + sa * sb * sg, ca * sb * sg - cg * sa],
                     [-sb, cb * sa, ca * cb]])


def make(sysname: str, nwalk: int, seed: int):
    syn = synthetic.SYSTEMS[sysname]()
    H = to_ref_hamiltonian(syn.hamiltonian)
    wfd = H.wavefunction_data
    gem = wfd.geminal_data
    jas = wfd.jastrow_data
    coul = H.coulomb_potential_data
    rng = np.random.default_rng(seed)
    r_up, r_dn = syn.initial_electrons(nwalk, seed=seed)
    angles = rng.uniform(-2 * np.pi, 2 * np.pi, size=(nwalk, 3))
    # single-electron moves for the ratio tests: (spin, index, displacement)
    moves_spin = rng.integers(0, 2, size=(nwalk, 8))
    moves_idx = rng.integers(0, min(syn.n_up, syn.n_dn), size=(nwalk, 8))
    moves_d = rng.normal(scale=0.3, size=(nwalk, 8, 3))
    out = {"r_up": r_up, "r_dn": r_dn, "angles": angles, "moves_spin": moves_spin, "moves_idx": moves_idx, "moves_d": moves_d}
    aos_det = gem.orb_data_up_spin.aos_data if hasattr(gem.orb_data_up_spin, "aos_data") else gem.orb_data_up_spin
    failures = []

    def call(name, fn):
        try:
            vals = [fn(w) for w in range(nwalk)]
            if isinstance(vals[0], tuple):
                for k in range(len(vals[0])):
                    out[f"{name}.{k}"] = np.stack([np.asarray(v[k], dtype=np.float64) for v in vals])
            else:
                out[name] = np.stack([np.asarray(v, dtype=np.float64) for v in vals])
        except Exception:  # noqa: BLE001 -- report and continue: some paths need real JAX
            failures.append(name)
            traceback.print_exc(limit=3)

    rall = lambda w: np.vstack([r_up[w], r_dn[w]])  # noqa: E731
    call("ao_debug", lambda w: np.asarray(r_ao._compute_AOs_sphe_debug(aos_det, rall(w))))
    call("ao", lambda w: r_ao.compute_AOs(aos_det, rall(w)))
    call("ao_vgl", lambda w: tuple(r_ao.compute_AOs_value_grad_lap(aos_det, rall(w))))
    call("geminal", lambda w: r_det.compute_geminal_all_elements(gem, r_up[w], r_dn[w]))
    call("det_debug", lambda w: r_det._compute_det_geminal_all_elements_debug(gem, r_up[w], r_dn[w]))
    call("AS", lambda w: r_det.compute_AS_regularization_factor(gem, r_up[w], r_dn[w]))
    call("swct_omega", lambda w: r_swct._evaluate_swct_omega_debug(H.structure_data, rall(w)))
    call("swct_domega", lambda w: r_swct._evaluate_swct_domega_debug(H.structure_data, rall(w)))
    call("J1", lambda w: r_jas.compute_Jastrow_one_body(jas.jastrow_one_body_data, r_up[w], r_dn[w]))
    call("J2", lambda w: r_jas.compute_Jastrow_two_body(jas.jastrow_two_body_data, r_up[w], r_dn[w]))
    call("J3", lambda w: r_jas.compute_Jastrow_three_body(jas.jastrow_three_body_data, r_up[w], r_dn[w]))
    call("J3_debug", lambda w: r_jas._compute_Jastrow_three_body_debug(jas.jastrow_three_body_data, r_up[w], r_dn[w]))
    call("J", lambda w: r_jas.compute_Jastrow_part(jas, r_up[w], r_dn[w]))

    def moved(w):
        ups, dns = [], []
        for k in range(moves_spin.shape[1]):
            u, d = r_up[w].copy(), r_dn[w].copy()
            if moves_spin[w, k] == 0:
                u[moves_idx[w, k]] += moves_d[w, k]
            else:
                d[moves_idx[w, k]] += moves_d[w, k]
            ups.append(u)
            dns.append(d)
        return np.stack(ups), np.stack(dns)

    call("J_ratio", lambda w: r_jas._compute_ratio_Jastrow_part_rank1_update(jas, r_up[w], r_dn[w], *moved(w)))
    call("J_grad_lap", lambda w: tuple(r_jas.compute_grads_and_laplacian_Jastrow_part(jas, r_up[w], r_dn[w])))
    ginv = lambda w: np.linalg.inv(np.asarray(r_det.compute_geminal_all_elements(gem, r_up[w], r_dn[w])))  # noqa: E731
    call("det_ratio", lambda w: r_det._compute_ratio_determinant_part_rank1_update(gem, ginv(w), r_up[w], r_dn[w], *moved(w)))
    call("det_grad_lap", lambda w: tuple(r_det.compute_grads_and_laplacian_ln_Det_fast(gem, r_up[w], r_dn[w], ginv(w))))
    call("AS_fast", lambda w: r_det.compute_AS_regularization_factor_fast_update(
        np.asarray(r_det.compute_geminal_all_elements(gem, r_up[w], r_dn[w])), ginv(w)))
    call("kinetic", lambda w: tuple(r_wf.compute_kinetic_energy_all_elements_fast_update(wfd, r_up[w], r_dn[w], ginv(w))))
    call("bare_coulomb", lambda w: r_cp._compute_bare_coulomb_potential_debug(coul, r_up[w], r_dn[w]))
    call("ecp_local", lambda w: r_cp._compute_ecp_local_parts_all_pairs_debug(coul, r_up[w], r_dn[w]))
    RT = lambda w: rotation(*angles[w]).T  # noqa: E731
    call("ecp_nonlocal", lambda w: r_cp.compute_ecp_non_local_parts_nearest_neighbors_fast_update(
        coul, wfd, r_up[w], r_dn[w], RT(w), ginv(w))[2:])
    # determinant locality (non_local_move='dltmove', jqmc_gfmc.py:4980-5017): V with the
    # determinant ratio only, and the Jastrow ratio at each of its mesh points
    def dlt(w):
        mu, md, V, _ = r_cp.compute_ecp_non_local_parts_nearest_neighbors_fast_update(
            coul, wfd, r_up[w], r_dn[w], RT(w), ginv(w), flag_determinant_only=True)
        jr = r_jas._compute_ratio_Jastrow_part_rank1_update(jas, r_up[w], r_dn[w], np.asarray(mu), np.asarray(md))
        return np.asarray(V), np.asarray(jr)

    call("ecp_nonlocal_det", dlt)
    call("local_energy", lambda w: r_ham.compute_local_energy_fast(H, r_up[w], r_dn[w], RT(w), ginv(w)))
    call("disc_kinetic", lambda w: r_wf.compute_discretized_kinetic_energy_fast_update(0.2, wfd, ginv(w), r_up[w], r_dn[w], RT(w).T)[2])
    path = os.path.join(HERE, f"{sysname}.npz")
    np.savez_compressed(path, **out)
    print(f"{sysname}: wrote {len(out)} arrays to {path}; failed: {failures}")
    return failures


if __name__ == "__main__":
    make("water_like", 4, 11)
    make("ring12", 2, 12)
