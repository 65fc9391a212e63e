"""TREXIO input and the TurboRVB known answers of the reference's tests.

tests/golden/{water_ccecp,h2_ae}.npz hold TREXIO files of the reference's tests
converted by jqmc_gb300.trexio_wrapper (the script beside them), with the fixed
configurations, Jastrows and TurboRVB values of
test_comparison_with_turborvb_ECP.py (water ccECP: no Jastrow; two-body;
two- and three-body; one-, two- and three-body) and
test_comparison_with_turborvb_AE.py (H2, all electrons: no Jastrow; one-, two-
and three-body): (psi'/psi)^2, the kinetic energy and the potential, to the decimals the
reference asserts.  One case (j213step) follows a whole Metropolis step of
TurboRVB: the proposal's step scales and transition ratio, the geminals, the
AS regularisation and the final acceptance ratio.  The oracle reproduces them; the reader itself is checked
on the reference's files when they are present.
"""

import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _reference_trexio_dir():
    """The reference's TREXIO example files where the fixture recipe
    (tests/golden/make_trexio_golden.py) reads them; absent elsewhere."""
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_trexio_golden import REFERENCE
    return os.path.join(REFERENCE, "tests", "trexio_example_files")


TREXIO_DIR = _reference_trexio_dir()


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
         ("water_ccecp.npz", "j213"), ("water_ccecp.npz", "j213step"), ("h2_ae.npz", "nojas"), ("h2_ae.npz", "j123")]


def as_ratio_sq(R_old: float, R_new: float, eps: float) -> float:
    """The AS factor's share of (psi'/psi)^2 with cutoff eps (jqmc_mcmc.py:4485-4491)."""
    return ((max(R_new, eps) / R_new) / (max(R_old, eps) / R_old)) ** 2


@pytest.mark.parametrize("fixture,case", CASES)
def test_oracle_reproduces_turborvb(fixture, case):
    from oracle.wf import OracleSystem
    ham, c = trexio_case(fixture, case)
    o = OracleSystem(ham)
    s0, l0 = o.ln_det(c["old_r_up"], c["old_r_dn"])
    s1, l1 = o.ln_det(c["new_r_up"], c["new_r_dn"])
    dJ = o.jastrow_total(c["new_r_up"], c["new_r_dn"]) - o.jastrow_total(c["old_r_up"], c["old_r_dn"])
    ratio_sq = (s0 * s1 * np.exp(l1 - l0 + dJ)) ** 2
    if "eps_as" in c:
        G0, G1 = o.geminal(c["old_r_up"], c["old_r_dn"]), o.geminal(c["new_r_up"], c["new_r_dn"])
        ratio_sq *= as_ratio_sq(o.as_factor(G0, np.linalg.inv(G0)), o.as_factor(G1, np.linalg.inv(G1)), float(c["eps_as"]))
    Ginv = np.linalg.inv(o.geminal(c["new_r_up"], c["new_r_dn"]))
    tu, td = o.kinetic_elements(c["new_r_up"], c["new_r_dn"], Ginv)
    v = o.bare_coulomb(c["new_r_up"], c["new_r_dn"])
    if o.ecp:
        v += o.ecp_local(c["new_r_up"], c["new_r_dn"]) + o.ecp_nonlocal(c["new_r_up"], c["new_r_dn"], np.eye(3), Ginv)[1]
    d = [int(x) for x in c["decimals"]]
    np.testing.assert_almost_equal(ratio_sq, float(c["wf_ratio_sq"]), decimal=d[0])
    np.testing.assert_almost_equal(np.sum(tu) + np.sum(td), float(c["kinetic"]), decimal=d[1])
    np.testing.assert_almost_equal(v, float(c["potential"]), decimal=d[2])


def test_oracle_reproduces_turborvb_metropolis_step():
    """The rest of TurboRVB's Metropolis step on water with the two-, one- and
    three-body Jastrow (test_comparison_with_turborvb_ECP.py:646-950): step
    scales, T_ratio, the geminals, S = min over columns of sum_i G_ij^2,
    F = |G^-1|_F^2, R_AS = (S F)^(-3/8), reweight (R_AS / max(R_AS, eps))^2 and
    the final ratio, to the reference's 6 decimals (F to 1e-10 relative).
    The oracle's R_AS takes the smaller of the row and column minima, as the
    library does; it equals TurboRVB's here."""
    from oracle.drivers import step_scale, transition_ratio
    from oracle.wf import OracleSystem
    ham, c = trexio_case("water_ccecp.npz", "j213step")
    o = OracleSystem(ham)
    spin, idx = (int(x) for x in c["moved"])
    key = "r_up" if spin == 0 else "r_dn"
    old, new = c["old_" + key][idx], c["new_" + key][idx]
    dt, eps = float(c["dt"]), float(c["eps_as"])
    np.testing.assert_almost_equal(step_scale(o, old), float(c["fa"]), decimal=6)
    np.testing.assert_almost_equal(step_scale(o, new), float(c["fb"]), decimal=6)
    T = transition_ratio(o, old, new, dt)
    np.testing.assert_almost_equal(T, float(c["t_ratio"]), decimal=6)
    R = {}
    for when in ("old", "new"):
        G = o.geminal(c[f"{when}_r_up"], c[f"{when}_r_dn"])
        Gi = np.linalg.inv(G)
        np.testing.assert_almost_equal(G, c[f"geminal_{when}"], decimal=6)
        S = np.min(np.sum(G**2, axis=0))
        F = np.sum(Gi**2)
        np.testing.assert_almost_equal(S, float(c[f"s_{when}"]), decimal=6)
        np.testing.assert_allclose(F, float(c[f"f_{when}"]), rtol=1e-10)
        R[when] = o.as_factor(G, Gi)
        np.testing.assert_almost_equal((S * F) ** -0.375, float(c[f"r_as_{when}"]), decimal=6)
        np.testing.assert_almost_equal(R[when], float(c[f"r_as_{when}"]), decimal=6)
    np.testing.assert_almost_equal((R["new"] / max(R["new"], eps)) ** 2, float(c["reweight"]), decimal=6)
    s0, l0 = o.ln_det(c["old_r_up"], c["old_r_dn"])
    s1, l1 = o.ln_det(c["new_r_up"], c["new_r_dn"])
    dJ = o.jastrow_total(c["new_r_up"], c["new_r_dn"]) - o.jastrow_total(c["old_r_up"], c["old_r_dn"])
    ratio_sq = (s0 * s1 * np.exp(l1 - l0 + dJ)) ** 2 * as_ratio_sq(R["old"], R["new"], eps)
    np.testing.assert_almost_equal(ratio_sq * T, float(c["final_ratio"]), decimal=6)


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


@pytest.mark.skipif(not os.path.isdir(TREXIO_DIR), reason="the reference's TREXIO files are not present")
def test_cartesian_trexio_files():
    """Cartesian files give AOs_cart_data with (l+1)(l+2)/2 components per shell.
    H2 cc-pVDZ (s and p shells) in its Cartesian and spherical files spans one
    space, so the occupied MO of the two files agrees up to sign at any point:
    a check of the Cartesian conversion and normalisation (oracle AO values).
    The walker kernels take a Cartesian basis as one shell per AO."""
    from jqmc_gb300.atomic_orbital import AOs_cart_data
    from jqmc_gb300.engine import pack_basis
    from jqmc_gb300.trexio_wrapper import read_trexio_file
    from oracle.ao import AOTable, ao_value
    for name in sorted(f for f in os.listdir(TREXIO_DIR) if f.endswith("_cart.h5")):
        st, aos, mu, md, gem, coul = read_trexio_file(os.path.join(TREXIO_DIR, name))
        assert isinstance(aos, AOs_cart_data), name
        aos.sanity_check()
        gem.sanity_check()
        assert all(nx + ny + nz == l for l, nx, ny, nz in zip(aos.angular_momentums, aos.polynominal_order_x,
                                                               aos.polynominal_order_y, aos.polynominal_order_z))
    r = np.random.default_rng(0).normal(scale=1.2, size=(40, 3))
    mo = {}
    for kind in ("cart", "sphe"):
        st, aos, mu, md, gem, coul = read_trexio_file(os.path.join(TREXIO_DIR, f"H2_ae_ccpvdz_{kind}.h5"))
        mo[kind] = mu.mo_coefficients[0] @ ao_value(AOTable(aos), r)
    np.testing.assert_allclose(np.abs(mo["cart"]), np.abs(mo["sphe"]), rtol=1e-12, atol=1e-14)
    # s and p shells: to_spherical is exact, and gives a basis the walker kernels take
    st, aos, mu, md, gem, coul = read_trexio_file(os.path.join(TREXIO_DIR, "H2_ae_ccpvdz_cart.h5"))
    ms = mu.to_spherical()
    np.testing.assert_allclose(ms.mo_coefficients[0] @ ao_value(AOTable(ms.aos_data), r), mo["cart"], rtol=1e-12, atol=1e-14)
    pack_basis(ms.aos_data)
    cart = read_trexio_file(os.path.join(TREXIO_DIR, "N_ae_ccpvdz_cart.h5"))[1]
    assert max(cart.angular_momentums) == 2 and cart.num_ao == 15
    sh, _ = pack_basis(cart)   # one Cartesian shell (kind 1) per AO for the walker kernels
    assert sh.shape == (15, 8) and np.all(sh[:, 7] == 1)
