"""The reference's module-level evaluation functions (compute_AOs, compute_MOs,
compute_*geminal_all_elements, compute_AS_regularization_factor, compute_Jastrow_*,
evaluate_*, compute_kinetic_energy, compute_local_energy(_fast)) on the GPU path
against the oracle, for single configurations (Python floats, as the reference
returns) and walker batches."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module", params=["water_like", "ring12"])
def setup(request):
    from jqmc_gb300 import synthetic
    from oracle.wf import OracleSystem
    syn = synthetic.SYSTEMS[request.param]()
    o = OracleSystem(syn.hamiltonian)
    r_up, r_dn = syn.initial_electrons(3, seed=9)
    return syn, o, np.asarray(r_up), np.asarray(r_dn)


def test_ao_and_mo_tables(setup):
    from jqmc_gb300 import atomic_orbital as AO
    from jqmc_gb300 import molecular_orbital as MO
    from jqmc_gb300.molecular_orbital import MOs_data
    from oracle.ao import ao_vgl
    syn, o, _, _ = setup
    g = syn.hamiltonian.wavefunction_data.geminal_data
    aos = g.ao_basis_lambda()[0]
    pts = np.random.default_rng(4).normal(scale=2.0, size=(65, 3))
    ref = ao_vgl(o.tab_up, pts)
    assert rel(AO.compute_AOs(aos, pts), ref[0]) < 1e-12
    gx, gy, gz = AO.compute_AOs_grad(aos, pts)
    for got, k in ((gx, 1), (gy, 2), (gz, 3)):
        assert rel(got, ref[k]) < 1e-12
    assert rel(AO.compute_AOs_laplacian(aos, pts), ref[4]) < 1e-12
    for got, want in zip(AO.compute_AOs_value_grad_lap(aos, pts), ref):
        assert rel(got, want) < 1e-12
    orb = g.orb_data_up_spin
    if isinstance(orb, MOs_data):
        mref = o.orb_vgl(o.tab_up, o.mo_up, pts)
        assert rel(MO.compute_MOs(orb, pts), mref[0]) < 1e-12
        for got, want in zip(MO.compute_MOs_value_grad_lap(orb, pts), mref):
            assert rel(got, want) < 1e-12


def test_geminal_and_wavefunction(setup):
    from jqmc_gb300 import determinant as D
    from jqmc_gb300 import wavefunction as WF
    syn, o, r_up, r_dn = setup
    wf = syn.hamiltonian.wavefunction_data
    g = wf.geminal_data
    for w in range(2):
        G = o.geminal(r_up[w], r_dn[w])
        assert rel(D.compute_geminal_all_elements(g, r_up[w], r_dn[w]), G) < 1e-12
        sign, ld = o.ln_det(r_up[w], r_dn[w])
        got = D.compute_ln_det_geminal_all_elements(g, r_up[w], r_dn[w])
        assert isinstance(got, float) and abs(got - ld) < RTOL * max(1.0, abs(ld))
        assert rel(D.compute_det_geminal_all_elements(g, r_up[w], r_dn[w]), sign * np.exp(ld)) < 1e-10
        Ginv = np.linalg.inv(G)
        R_ref = o.as_factor(G, Ginv)
        assert abs(D.compute_AS_regularization_factor(g, r_up[w], r_dn[w]) - R_ref) < RTOL * max(1e-300, abs(R_ref))
        assert abs(D.compute_AS_regularization_factor_fast_update(G, Ginv) - R_ref) < 1e-13 * abs(R_ref)
        J = o.jastrow_total(r_up[w], r_dn[w])
        lnpsi = WF.evaluate_ln_wavefunction(wf, r_up[w], r_dn[w])
        assert abs(lnpsi - (ld + J)) < RTOL * max(1.0, abs(ld + J))
        assert abs(WF.evaluate_ln_wavefunction_fast(wf, r_up[w], r_dn[w], Ginv) - lnpsi) <= 1e-12 * max(1.0, abs(lnpsi))
        assert rel(WF.evaluate_jastrow(wf, r_up[w], r_dn[w]), np.exp(J)) < 1e-10
        assert rel(WF.evaluate_wavefunction(wf, r_up[w], r_dn[w]), sign * np.exp(ld + J)) < 1e-10
        tu, td = o.kinetic_elements(r_up[w], r_dn[w], np.linalg.inv(G))
        T = float(np.sum(tu) + np.sum(td))
        assert abs(WF.compute_kinetic_energy(wf, r_up[w], r_dn[w]) - T) < RTOL * max(1.0, abs(T))
    # a batch of configurations gives one value per configuration
    lds = D.compute_ln_det_geminal_all_elements(g, r_up, r_dn)
    assert lds.shape == (3,)
    assert rel(lds, [o.ln_det(r_up[w], r_dn[w])[1] for w in range(3)]) < RTOL


def test_jastrow_parts(setup):
    from jqmc_gb300 import jastrow_factor as JF
    syn, o, r_up, r_dn = setup
    jd = syn.hamiltonian.wavefunction_data.jastrow_data
    for w in range(2):
        J1, J2, J3 = o.jastrow(r_up[w], r_dn[w])
        assert abs(JF.compute_Jastrow_part(jd, r_up[w], r_dn[w]) - (J1 + J2 + J3)) < RTOL * max(1.0, abs(J1 + J2 + J3))
        if jd.jastrow_one_body_data is not None:
            assert abs(JF.compute_Jastrow_one_body(jd.jastrow_one_body_data, r_up[w], r_dn[w]) - J1) < RTOL * max(1.0, abs(J1))
        if jd.jastrow_two_body_data is not None:
            assert abs(JF.compute_Jastrow_two_body(jd.jastrow_two_body_data, r_up[w], r_dn[w]) - J2) < RTOL * max(1.0, abs(J2))
        if jd.jastrow_three_body_data is not None:
            assert abs(JF.compute_Jastrow_three_body(jd.jastrow_three_body_data, r_up[w], r_dn[w]) - J3) < RTOL * max(1.0, abs(J3))


def test_local_energy(setup):
    from jqmc_gb300 import hamiltonians as H
    from oracle.wf import rotation_matrix
    syn, o, r_up, r_dn = setup
    ham = syn.hamiltonian
    ang = np.random.default_rng(8).uniform(-2 * np.pi, 2 * np.pi, size=(3, 3))
    RT = np.stack([rotation_matrix(*a).T for a in ang])
    ref = [o.local_energy(r_up[w], r_dn[w], RT[w], np.linalg.inv(o.geminal(r_up[w], r_dn[w]))) for w in range(3)]
    got = H.compute_local_energy(ham, r_up[0], r_dn[0], RT[0])
    assert isinstance(got, float) and abs(got - ref[0]) < RTOL * max(1.0, abs(ref[0]))
    G0 = o.geminal(r_up[0], r_dn[0])
    assert abs(H.compute_local_energy_fast(ham, r_up[0], r_dn[0], RT[0], np.linalg.inv(G0)) - got) <= 1e-12 * max(1.0, abs(got))
    batch = H.compute_local_energy(ham, r_up, r_dn, RT)
    assert batch.shape == (3,)
    assert rel(batch, ref) < RTOL


@pytest.mark.parametrize("name", ["water_like", "ring12"])
def test_geminal_rows_columns_and_jastrow_ratios_match_reference(name, golden_dir):
    """compute_geminal_up_one_row_elements / _dn_one_column_elements rebuild the
    reference's geminal matrix row by row and column by column, and
    _compute_ratio_Jastrow_part_rank1_update reproduces the reference's ratios for
    its single-electron moves (tests/golden/<system>.npz, made by the reference)."""
    import os

    from jqmc_gb300 import determinant as D
    from jqmc_gb300 import jastrow_factor as J
    from jqmc_gb300 import synthetic
    g = np.load(os.path.join(golden_dir, f"{name}.npz"))
    wf = synthetic.SYSTEMS[name]().hamiltonian.wavefunction_data
    gem, jd = wf.geminal_data, wf.jastrow_data
    for w in range(g["r_up"].shape[0]):
        ru, rd = g["r_up"][w], g["r_dn"][w]
        G = g["geminal"][w]
        rows = np.stack([D.compute_geminal_up_one_row_elements(gem, ru[i:i + 1], rd) for i in range(len(ru))])
        cols = np.stack([D.compute_geminal_dn_one_column_elements(gem, ru, rd[j:j + 1]) for j in range(len(rd))], axis=1)
        assert rel(rows, G) < RTOL and rel(cols, G) < RTOL
        nu, nd = [], []
        for k in range(g["moves_spin"].shape[1]):
            u, d = ru.copy(), rd.copy()
            (u if g["moves_spin"][w, k] == 0 else d)[g["moves_idx"][w, k]] += g["moves_d"][w, k]
            nu.append(u)
            nd.append(d)
        ratio = J._compute_ratio_Jastrow_part_rank1_update(jd, ru, rd, np.stack(nu), np.stack(nd))
        assert rel(ratio, g["J_ratio"][w]) < RTOL
        dr = D._compute_ratio_determinant_part_rank1_update(gem, np.linalg.inv(G), ru, rd, np.stack(nu), np.stack(nd))
        assert rel(dr, g["det_ratio"][w]) < RTOL


@pytest.mark.parametrize("name", ["water_like", "ring12"])
def test_coulomb_module_functions_match_reference(name, golden_dir):
    """compute_bare_coulomb_potential(_el_ion, _el_el, _ion_ion, _el_ion_element_wise)
    and compute_ecp_local_parts_all_pairs from the walker initialisation's energy
    cache, against the reference's bare Coulomb and local ECP values
    (tests/golden/<system>.npz), batched and single."""
    import os

    from jqmc_gb300 import coulomb_potential as CP
    from jqmc_gb300 import synthetic
    g = np.load(os.path.join(golden_dir, f"{name}.npz"))
    coul = synthetic.SYSTEMS[name]().hamiltonian.coulomb_potential_data
    ru, rd = g["r_up"], g["r_dn"]
    v = CP.compute_bare_coulomb_potential(coul, ru, rd)
    assert rel(v, g["bare_coulomb"]) < RTOL
    parts = (CP.compute_bare_coulomb_potential_el_ion(coul, ru, rd) + CP.compute_bare_coulomb_potential_el_el(ru, rd)
             + CP.compute_bare_coulomb_potential_ion_ion(coul))
    assert rel(parts, g["bare_coulomb"]) < RTOL
    up, dn = CP.compute_bare_coulomb_potential_el_ion_element_wise(coul, ru, rd)
    assert rel(up.sum(1) + dn.sum(1), CP.compute_bare_coulomb_potential_el_ion(coul, ru, rd)) < RTOL
    assert rel(CP.compute_ecp_local_parts_all_pairs(coul, ru, rd), g["ecp_local"]) < RTOL
    single = CP.compute_bare_coulomb_potential(coul, ru[0], rd[0])
    assert isinstance(single, float) and abs(single - g["bare_coulomb"][0]) < RTOL * abs(g["bare_coulomb"][0])


@pytest.mark.parametrize("name", ["water_like", "ring12"])
def test_total_and_ecp_potential_match_reference(name, golden_dir):
    """compute_coulomb_potential and compute_ecp_coulomb_potential (E_L - T of the
    walker kernels) against the reference's bare Coulomb + local + non-local ECP
    with the same quadrature rotations (tests/golden/<system>.npz)."""
    import os

    from jqmc_gb300 import coulomb_potential as CP
    from jqmc_gb300 import synthetic
    from oracle.wf import rotation_matrix
    g = np.load(os.path.join(golden_dir, f"{name}.npz"))
    ham = synthetic.SYSTEMS[name]().hamiltonian
    coul, wf = ham.coulomb_potential_data, ham.wavefunction_data
    RT = np.stack([rotation_matrix(*a).T for a in g["angles"]])
    ecp = g["ecp_local"] + g["ecp_nonlocal.1"]
    v = CP.compute_coulomb_potential(coul, g["r_up"], g["r_dn"], RT, wavefunction_data=wf)
    assert rel(v, g["bare_coulomb"] + ecp) < RTOL
    assert rel(CP.compute_ecp_coulomb_potential(coul, wf, g["r_up"], g["r_dn"], RT), ecp) < 1e-9


def test_per_electron_tables(setup):
    """grad / lap of ln|det| and of J per electron, and the kinetic elements."""
    from jqmc_gb300 import determinant as D
    from jqmc_gb300 import jastrow_factor as JF
    from jqmc_gb300 import wavefunction as WF
    syn, o, r_up, r_dn = setup
    wf = syn.hamiltonian.wavefunction_data
    n = r_up.shape[1]
    for w in range(2):
        Ginv = np.linalg.inv(o.geminal(r_up[w], r_dn[w]))
        gu, gd, lu, ld = o.det_grad_lap(r_up[w], r_dn[w], Ginv)
        got = D.compute_grads_and_laplacian_ln_Det(wf.geminal_data, r_up[w], r_dn[w])
        for a, b in zip(got, (gu, gd, lu, ld)):
            assert a.shape == np.shape(b) and rel(a, b) < RTOL
        gJ, lJ = o.jastrow_grad_lap(r_up[w], r_dn[w])
        got = JF.compute_grads_and_laplacian_Jastrow_part(wf.jastrow_data, r_up[w], r_dn[w])
        for a, b in zip(got, (gJ[:n], gJ[n:], lJ[:n], lJ[n:])):
            assert a.shape == np.shape(b) and rel(a, b) < RTOL
        tu, td = o.kinetic_elements(r_up[w], r_dn[w], Ginv)
        Tu, Td = WF.compute_kinetic_energy_all_elements(wf, r_up[w], r_dn[w])
        assert rel(Tu, tu) < RTOL and rel(Td, td) < RTOL


def test_discretized_kinetic(setup):
    """The six rotated lattice moves of every electron: configurations and elements."""
    from jqmc_gb300 import wavefunction as WF
    from oracle.wf import rotation_matrix
    syn, o, r_up, r_dn = setup
    wf = syn.hamiltonian.wavefunction_data
    n = r_up.shape[1]
    ang = np.random.default_rng(12).uniform(-2 * np.pi, 2 * np.pi, size=3)
    RT = rotation_matrix(*ang).T
    Ginv = np.linalg.inv(o.geminal(r_up[0], r_dn[0]))
    cu, cd, el = WF.compute_discretized_kinetic_energy(0.2, wf, r_up[0], r_dn[0], RT)
    ref = o.discretized_kinetic(0.2, r_up[0], r_dn[0], RT, Ginv)
    assert el.shape == ref.shape and rel(el, ref) < RTOL
    N = 2 * n
    assert cu.shape == (6 * N, n, 3) and cd.shape == (6 * N, n, 3)
    shifts = 0.2 * np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], float) @ RT
    e, k = n + 1, 4          # a down electron's +z move
    assert np.allclose(cd[6 * e + k, e - n], r_dn[0][e - n] + shifts[k]) and np.array_equal(cu[6 * e + k], r_up[0])
