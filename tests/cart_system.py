"""A Cartesian test system for the tests: water_like (three nuclei, ECP, J1, J2,
J3) with its geminal basis re-expanded into Cartesian shells (each shell's
exponents and contraction coefficients, every (nx, ny, nz) component of its l),
a seeded symmetric pairing matrix over those AOs, and the J3 basis made
Cartesian the same way."""

import dataclasses

import numpy as np


def cartesian_from_spherical(sph):
    from jqmc_gb300.atomic_orbital import AOs_cart_data, cartesian_orders
    nuc, ls, pws, oi, ex, co = [], [], [], [], [], []
    ao = 0
    for s in sph.shells():
        for pw in cartesian_orders(s["l"]):
            nuc.append(s["atom"])
            ls.append(s["l"])
            pws.append(pw)
            oi += [ao] * len(s["exps"])
            ex += list(s["exps"])
            co += list(s["coefs"])
            ao += 1
    pw = np.array(pws, dtype=int)
    return AOs_cart_data(structure_data=sph.structure_data, nucleus_index=tuple(nuc), num_ao=ao, num_ao_prim=len(ex),
                         orbital_indices=tuple(oi), exponents=np.array(ex), coefficients=np.array(co),
                         angular_momentums=tuple(ls), polynominal_order_x=tuple(int(x) for x in pw[:, 0]),
                         polynominal_order_y=tuple(int(x) for x in pw[:, 1]),
                         polynominal_order_z=tuple(int(x) for x in pw[:, 2]))


def water_like_cartesian(seed: int = 7):
    """(synthetic system object, Hamiltonian_data with Cartesian AOs)."""
    from jqmc_gb300 import synthetic
    from jqmc_gb300.determinant import Geminal_data
    syn = synthetic.water_like()
    ham = syn.hamiltonian
    gem = ham.wavefunction_data.geminal_data
    cart = cartesian_from_spherical(gem.ao_basis_lambda()[0])
    A = cart.num_ao
    B = np.random.default_rng(seed).normal(size=(A, A)) / np.sqrt(A)
    gem_c = Geminal_data(num_electron_up=gem.num_electron_up, num_electron_dn=gem.num_electron_dn, orb_data_up_spin=cart,
                         orb_data_dn_spin=cart, lambda_matrix=0.5 * (B + B.T))
    jd = ham.wavefunction_data.jastrow_data
    j3 = jd.jastrow_three_body_data
    j3c = cartesian_from_spherical(j3.orb_data)
    jm = np.random.default_rng(seed + 1).normal(scale=0.01, size=(j3c.num_ao, j3c.num_ao + 1))
    jm[:, :-1] = 0.5 * (jm[:, :-1] + jm[:, :-1].T)
    jd = dataclasses.replace(jd, jastrow_three_body_data=dataclasses.replace(j3, orb_data=j3c, j_matrix=jm))
    wf = dataclasses.replace(ham.wavefunction_data, geminal_data=gem_c, jastrow_data=jd)
    return syn, dataclasses.replace(ham, wavefunction_data=wf)
