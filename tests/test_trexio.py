"""TREXIO input and the TurboRVB known answers of the reference's tests.

tests/golden/{water_ccecp,h2_ae}.npz hold TREXIO files of the reference's tests
converted by jqmc_gb300.trexio_wrapper (the script beside them), with the fixed
configurations, Jastrows and TurboRVB values of
test_comparison_with_turborvb_ECP.py (water ccECP: no Jastrow; two-body;
two- and three-body; one-, two- and three-body) and
test_comparison_with_turborvb_AE.py (H2, all electrons: no Jastrow; one-, two-
and three-body): (psi'/psi)^2, the kinetic energy and the potential, to the decimals the
reference asserts.  The oracle reproduces them; the reader itself is checked
on the reference's files when they are present.
"""

import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
TREXIO_DIR = "/root/reference/tests/trexio_example_files"


def trexio_case(fixture: str, case: str):
    """(Hamiltonian_data, configurations and TurboRVB values) of one case of a
    tests/golden fixture made by make_trexio_golden.py."""
    from jqmc_gb300.atomic_orbital import AOs_sphe_data
    from jqmc_gb300.coulomb_potential import Coulomb_potential_data
    from jqmc_gb300.determinant import Geminal_data
    from jqmc_gb300.hamiltonians import Hamiltonian_data
    from jqmc_gb300.jastrow_factor import (Jastrow_data, Jastrow_one_body_data, Jastrow_three_body_data,
                                           Jastrow_two_body_data)
    from jqmc_gb300.molecular_orbital import MOs_data
    from jqmc_gb300.structure import Structure_data
    from jqmc_gb300.wavefunction import Wavefunction_data
    g = np.load(os.path.join(HERE, "golden", fixture))
    labels = tuple(str(x) for x in g["labels"])
    st = Structure_data(positions=g["positions"], atomic_numbers=tuple(int(x) for x in g["atomic_numbers"]),
                        element_symbols=labels, atomic_labels=labels)
    aos = AOs_sphe_data(structure_data=st, nucleus_index=tuple(int(x) for x in g["ao_nucleus_index"]),
                        num_ao=len(g["ao_l"]), num_ao_prim=len(g["ao_exponents"]),
                        orbital_indices=tuple(int(x) for x in g["ao_orbital_indices"]), exponents=g["ao_exponents"],
                        coefficients=g["ao_coefficients"], angular_momentums=tuple(int(x) for x in g["ao_l"]),
                        magnetic_quantum_numbers=tuple(int(x) for x in g["ao_m"]))
    mu = MOs_data(num_mo=g["mo_up"].shape[0], aos_data=aos, mo_coefficients=g["mo_up"])
    md = MOs_data(num_mo=g["mo_dn"].shape[0], aos_data=aos, mo_coefficients=g["mo_dn"])
    gem = Geminal_data(num_electron_up=int(g["n_up"]), num_electron_dn=int(g["n_dn"]), orb_data_up_spin=mu,
                       orb_data_dn_spin=md, lambda_matrix=g["lambda_matrix"])
    if bool(g["ecp_flag"]):
        coul = Coulomb_potential_data(structure_data=st, ecp_flag=True, z_cores=tuple(int(x) for x in g["ecp_z_cores"]),
                                      max_ang_mom_plus_1=tuple(int(x) for x in g["ecp_maxl1"]), num_ecps=len(g["ecp_l"]),
                                      ang_moms=tuple(int(x) for x in g["ecp_l"]),
                                      nucleus_index=tuple(int(x) for x in g["ecp_nucleus_index"]),
                                      exponents=tuple(float(x) for x in g["ecp_exponents"]),
                                      coefficients=tuple(float(x) for x in g["ecp_coefficients"]),
                                      powers=tuple(int(x) for x in g["ecp_powers"]))
    else:
        coul = Coulomb_potential_data(structure_data=st, ecp_flag=False)
    c = {k[len(case) + 1:]: g[k] for k in g.files if k.startswith(case + "_")}
    a, b = float(c["j1_param"]), float(c["j2_param"])
    j1 = None if np.isnan(a) else Jastrow_one_body_data(jastrow_1b_param=a, structure_data=st,
                                                         core_electrons=tuple(float(x) for x in c["j1_core"]))
    j2 = None if np.isnan(b) else Jastrow_two_body_data(jastrow_2b_param=b)
    j3 = None
    if c["j3_matrix"].size:
        j3_aos = AOs_sphe_data(structure_data=st, nucleus_index=tuple(int(x) for x in c["j3_nucleus_index"]),
                               num_ao=len(c["j3_l"]), num_ao_prim=len(c["j3_exponents"]),
                               orbital_indices=tuple(int(x) for x in c["j3_orbital_indices"]),
                               exponents=c["j3_exponents"], coefficients=c["j3_coefficients"],
                               angular_momentums=tuple(int(x) for x in c["j3_l"]),
                               magnetic_quantum_numbers=tuple(int(x) for x in c["j3_m"]))
        j3 = Jastrow_three_body_data(orb_data=j3_aos, j_matrix=c["j3_matrix"])
    jas = Jastrow_data(jastrow_one_body_data=j1, jastrow_two_body_data=j2, jastrow_three_body_data=j3)
    ham = Hamiltonian_data(structure_data=st, coulomb_potential_data=coul,
                           wavefunction_data=Wavefunction_data(jastrow_data=jas, geminal_data=gem))
    ham.sanity_check()
    return ham, c


CASES = [("water_ccecp.npz", "nojas"), ("water_ccecp.npz", "j2"), ("water_ccecp.npz", "j23"),
         ("water_ccecp.npz", "j213"), ("h2_ae.npz", "nojas"), ("h2_ae.npz", "j123")]


@pytest.mark.parametrize("fixture,case", CASES)
def test_oracle_reproduces_turborvb(fixture, case):
    from oracle.wf import OracleSystem
    ham, c = trexio_case(fixture, case)
    o = OracleSystem(ham)
    s0, l0 = o.ln_det(c["old_r_up"], c["old_r_dn"])
    s1, l1 = o.ln_det(c["new_r_up"], c["new_r_dn"])
    dJ = o.jastrow_total(c["new_r_up"], c["new_r_dn"]) - o.jastrow_total(c["old_r_up"], c["old_r_dn"])
    ratio_sq = (s0 * s1 * np.exp(l1 - l0 + dJ)) ** 2
    Ginv = np.linalg.inv(o.geminal(c["new_r_up"], c["new_r_dn"]))
    tu, td = o.kinetic_elements(c["new_r_up"], c["new_r_dn"], Ginv)
    v = o.bare_coulomb(c["new_r_up"], c["new_r_dn"])
    if o.ecp:
        v += o.ecp_local(c["new_r_up"], c["new_r_dn"]) + o.ecp_nonlocal(c["new_r_up"], c["new_r_dn"], np.eye(3), Ginv)[1]
    d = [int(x) for x in c["decimals"]]
    np.testing.assert_almost_equal(ratio_sq, float(c["wf_ratio_sq"]), decimal=d[0])
    np.testing.assert_almost_equal(np.sum(tu) + np.sum(td), float(c["kinetic"]), decimal=d[1])
    np.testing.assert_almost_equal(v, float(c["potential"]), decimal=d[2])


@pytest.mark.skipif(not os.path.isdir(TREXIO_DIR), reason="the reference's TREXIO files are not present")
def test_reader_on_reference_files():
    """Every spherical file converts (and matches the fixture for water);
    Cartesian bases are refused."""
    from jqmc_gb300.trexio_wrapper import read_trexio_file
    g = np.load(os.path.join(HERE, "golden", "water_ccecp.npz"))
    st, aos, mu, md, gem, coul = read_trexio_file(os.path.join(TREXIO_DIR, "water_ccecp_ccpvqz.h5"))
    assert np.array_equal(aos.coefficients, g["ao_coefficients"]) and np.array_equal(mu.mo_coefficients, g["mo_up"])
    assert tuple(st.atomic_labels) == ("O", "H", "H") and tuple(st.atomic_numbers) == (8, 1, 1)
    for name, nup, ndn in (("H2_ae_ccpvqz.h5", 1, 1), ("H2_ecp_ccpvtz.h5", 1, 1), ("H_ecp_ccpvqz.h5", 1, 0)):
        st, aos, mu, md, gem, coul = read_trexio_file(os.path.join(TREXIO_DIR, name))
        gem.sanity_check()
        assert (gem.num_electron_up, gem.num_electron_dn) == (nup, ndn)
    with pytest.raises(NotImplementedError):
        read_trexio_file(os.path.join(TREXIO_DIR, "N2_ecp_ccpvtz_cart.h5"))
