"""Pin the CPU oracle against outputs of the reference's own functions.

The fixtures in tests/golden/*.npz were produced by tests/golden/make_golden.py,
which executes jqmc's per-walker functions (AO, geminal, AS regularization,
Jastrow, Coulomb/ECP, kinetic, local energy, discretised kinetic mesh) on seeded
synthetic systems.
Every oracle quantity must agree to 1e-10 relative (the FP64 parity bar).
"""

import os

import numpy as np
import pytest

from jqmc_gb300 import synthetic
from oracle.ao import ao_value, ao_vgl
from oracle import swct
from oracle.wf import OracleSystem, rotation_matrix

RTOL = 1e-10


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("name", ["water_like", "ring12"])
def test_oracle_matches_reference_functions(name, golden_dir):
    g = np.load(os.path.join(golden_dir, f"{name}.npz"))
    o = OracleSystem(synthetic.SYSTEMS[name]().hamiltonian)
    for w in range(g["r_up"].shape[0]):
        ru, rd = g["r_up"][w], g["r_dn"][w]
        r = np.vstack([ru, rd])
        assert rel(ao_value(o.tab_up, r), g["ao"][w]) < RTOL
        assert rel(ao_value(o.tab_up, r), g["ao_debug"][w]) < RTOL
        v = ao_vgl(o.tab_up, r)
        for k in range(5):
            assert rel(v[k], g[f"ao_vgl.{k}"][w]) < RTOL, f"ao_vgl[{k}]"
        G = o.geminal(ru, rd)
        assert rel(G, g["geminal"][w]) < RTOL
        assert rel(np.linalg.det(G), g["det_debug"][w]) < RTOL
        J1, J2, J3 = o.jastrow(ru, rd)
        assert rel(J1, g["J1"][w]) < RTOL and rel(J2, g["J2"][w]) < RTOL
        assert rel(J3, g["J3"][w]) < RTOL and rel(J3, g["J3_debug"][w]) < RTOL
        assert rel(J1 + J2 + J3, g["J"][w]) < RTOL
        Gi = np.linalg.inv(G)
        assert rel(o.as_factor(G, Gi), g["AS"][w]) < RTOL and rel(o.as_factor(G, Gi), g["AS_fast"][w]) < RTOL
        R = synthetic.SYSTEMS[name]().hamiltonian.structure_data.positions
        assert rel(swct.omega(R, r), g["swct_omega"][w]) < RTOL
        # the reference's debug form of sum_i grad omega is a central difference (h = 1e-5)
        assert rel(swct.domega(R, r), g["swct_domega"][w]) < 1e-8
        gu, gd, lu, ld = o.det_grad_lap(ru, rd, Gi)
        for k, x in enumerate((gu, gd, lu, ld)):
            assert rel(x, g[f"det_grad_lap.{k}"][w]) < RTOL
        gJ, lJ = o.jastrow_grad_lap(ru, rd)
        n = o.n_up
        for k, x in enumerate((gJ[:n], gJ[n:], lJ[:n], lJ[n:])):
            assert rel(x, g[f"J_grad_lap.{k}"][w]) < RTOL
        tu, td = o.kinetic_elements(ru, rd, Gi)
        assert rel(tu, g["kinetic.0"][w]) < RTOL and rel(td, g["kinetic.1"][w]) < RTOL
        assert rel(o.bare_coulomb(ru, rd), g["bare_coulomb"][w]) < RTOL
        assert rel(o.ecp_local(ru, rd), g["ecp_local"][w]) < RTOL
        RT = rotation_matrix(*g["angles"][w]).T
        nl, snl = o.ecp_nonlocal(ru, rd, RT, Gi)
        assert rel(nl, g["ecp_nonlocal.0"][w]) < RTOL and rel(snl, g["ecp_nonlocal.1"][w]) < RTOL
        assert rel(o.local_energy(ru, rd, RT, Gi), g["local_energy"][w]) < RTOL
        assert rel(o.discretized_kinetic(0.2, ru, rd, RT.T, Gi), g["disc_kinetic"][w]) < RTOL
        jr, dr = [], []
        for k in range(g["moves_spin"].shape[1]):
            s, i = int(g["moves_spin"][w, k]), int(g["moves_idx"][w, k])
            rn = (ru if s == 0 else rd)[i] + g["moves_d"][w, k]
            jr.append(o.jastrow_ratio_move(ru, rd, s, i, rn))
            dr.append(o.det_ratio_move(Gi, ru, rd, s, i, rn))
        assert rel(jr, g["J_ratio"][w]) < RTOL
        assert rel(dr, g["det_ratio"][w]) < RTOL


def test_solid_harmonics_known_forms():
    from oracle.ao import solid_harmonics
    d = np.random.default_rng(0).normal(size=(7, 3))
    x, y, z = d.T
    S1, _ = solid_harmonics(1, d)
    assert np.allclose(S1, np.stack([y, z, x]))
    S2, _ = solid_harmonics(2, d)
    assert np.allclose(S2[0], np.sqrt(3) * x * y) and np.allclose(S2[2], 0.5 * (3 * z * z - (x * x + y * y + z * z)))
    # gradients against central differences, l <= 6
    for l in range(7):
        S, G = solid_harmonics(l, d)
        h = 1e-6
        fd = np.stack([(solid_harmonics(l, d + h * e)[0] - solid_harmonics(l, d - h * e)[0]) / (2 * h) for e in np.eye(3)], -1)
        assert np.max(np.abs(fd - G)) < 1e-6 * max(1.0, np.max(np.abs(G)))


@pytest.mark.parametrize("name", ["water_like", "ring12"])
def test_as_factor_matches_reference(name, golden_dir):
    """The AS factor of the module-level functions (torch, evaluated here on CPU
    tensors) against the reference's compute_AS_regularization_factor."""
    import torch

    from jqmc_gb300.surface import as_factor
    g = np.load(os.path.join(golden_dir, f"{name}.npz"))
    o = OracleSystem(synthetic.SYSTEMS[name]().hamiltonian)
    G = np.stack([o.geminal(g["r_up"][w], g["r_dn"][w]) for w in range(g["r_up"].shape[0])])
    Gi = np.linalg.inv(G)
    got = as_factor(torch.as_tensor(G), torch.as_tensor(Gi)).numpy()
    assert rel(got, g["AS"]) < RTOL


@pytest.mark.parametrize("name", ["water_like", "ring12"])
def test_swct_weights_match_reference(name, golden_dir):
    """The space-warp weights and their electron gradients of the force estimator
    (torch, evaluated here on CPU tensors) against the reference's."""
    import torch

    from jqmc_gb300.forces import swct_domega, swct_omega
    g = np.load(os.path.join(golden_dir, f"{name}.npz"))
    R = torch.as_tensor(synthetic.SYSTEMS[name]().hamiltonian.structure_data.positions)
    r = torch.as_tensor(np.concatenate([g["r_up"], g["r_dn"]], axis=1))
    assert rel(swct_omega(R, r).numpy(), g["swct_omega"]) < RTOL
    assert rel(swct_domega(R, r).numpy(), g["swct_domega"]) < 1e-8


@pytest.mark.parametrize("name", ["water_like", "ring12"])
def test_oracle_determinant_locality_matches_reference(name, golden_dir):
    """non_local_move='dltmove' (jqmc_gfmc.py:4980-5017): the reference's non-local
    ECP with flag_determinant_only=True and the Jastrow ratios at its mesh
    points pin the oracle's V_FN = min(V_det, 0) * J_ratio and SP = sum max(V_det, 0)."""
    from oracle import drivers as D
    g = np.load(os.path.join(golden_dir, f"{name}.npz"))
    o = OracleSystem(synthetic.SYSTEMS[name]().hamiltonian)
    for w in range(g["r_up"].shape[0]):
        st = D.init_state(o, g["r_up"][w], g["r_dn"][w])
        R = rotation_matrix(*g["angles"][w])
        V_det, jr = g["ecp_nonlocal_det.0"][w], g["ecp_nonlocal_det.1"][w]
        fn, sp = D._ecp_moves(o, st, R, 6, "dltmove")
        assert rel(fn, np.minimum(V_det, 0.0) * jr) < RTOL
        assert rel(sp, np.sum(np.maximum(V_det, 0.0))) < RTOL
        # with the full ratio (tmove) the same points give the reference's V
        fn_t, sp_t = D._ecp_moves(o, st, R, 6, "tmove")
        V = g["ecp_nonlocal.0"][w]
        assert rel(fn_t, np.minimum(V, 0.0)) < RTOL and rel(sp_t, np.sum(np.maximum(V, 0.0))) < RTOL
        assert np.any(jr != 1.0)
    with pytest.raises(NotImplementedError):
        D._ecp_moves(o, st, R, 6, "dla")


def _cart_aos(g):
    from jqmc_gb300.atomic_orbital import AOs_cart_data
    from jqmc_gb300.structure import Structure_data
    st = Structure_data(positions=g["positions"], atomic_numbers=(0,) * len(g["positions"]))
    return AOs_cart_data(structure_data=st, nucleus_index=tuple(int(x) for x in g["nucleus_index"]),
                         num_ao=len(g["angular_momentums"]), num_ao_prim=len(g["exponents"]),
                         orbital_indices=tuple(int(x) for x in g["orbital_indices"]), exponents=g["exponents"],
                         coefficients=g["coefficients"], angular_momentums=tuple(int(x) for x in g["angular_momentums"]),
                         polynominal_order_x=tuple(int(x) for x in g["polynominal_order_x"]),
                         polynominal_order_y=tuple(int(x) for x in g["polynominal_order_y"]),
                         polynominal_order_z=tuple(int(x) for x in g["polynominal_order_z"]))


def test_oracle_cartesian_aos_match_reference(golden_dir):
    """Cartesian AOs (s to g shells): values against the reference's debug and
    production functions, gradients and Laplacians against its fused
    value/grad/lap (tests/golden/make_cart_golden.py)."""
    from oracle.ao import AOTable
    g = np.load(os.path.join(golden_dir, "cart.npz"))
    aos = _cart_aos(g)
    aos.sanity_check()
    tab = AOTable(aos)
    assert rel(ao_value(tab, g["r"]), g["ao_debug"]) < RTOL
    assert rel(ao_value(tab, g["r"]), g["ao"]) < RTOL
    v = ao_vgl(tab, g["r"])
    for k in range(5):
        assert rel(v[k], g[f"ao_vgl.{k}"]) < RTOL, k
    assert max(aos.angular_momentums) == 4


def test_cartesian_to_spherical_matches_reference(golden_dir):
    """MOs_data.to_spherical (molecular_orbital.py:214-236) and the basis
    conversion behind it (atomic_orbital.py:1574-1690) against the reference's
    on the s-g Cartesian basis of tests/golden/cart.npz; MOs that lie in the
    spherical span come back unchanged in value."""
    from jqmc_gb300.atomic_orbital import aos_cart_to_sphe, spherical_to_cartesian_matrix
    from jqmc_gb300.molecular_orbital import MOs_data
    from oracle.ao import AOTable
    g = np.load(os.path.join(golden_dir, "cart.npz"))
    aos = _cart_aos(g)
    sph, pinv = aos_cart_to_sphe(aos)
    assert rel(pinv, g["to_sphe_pinv"]) < RTOL
    assert tuple(sph.angular_momentums) == tuple(g["to_sphe_l"]) and tuple(sph.magnetic_quantum_numbers) == tuple(g["to_sphe_m"])
    assert tuple(sph.nucleus_index) == tuple(g["to_sphe_nucleus_index"])
    assert np.array_equal(sph.exponents, g["to_sphe_exponents"]) and np.array_equal(sph.coefficients, g["to_sphe_coefficients"])
    mo = MOs_data(num_mo=3, aos_data=aos, mo_coefficients=g["mo_cart_coefficients"]).to_spherical()
    assert rel(mo.mo_coefficients, g["mo_sphe_coefficients"]) < RTOL
    # spherical span: C_cart = C_sph T reproduces the MO values exactly after the conversion
    T = np.linalg.pinv(pinv)
    c_sph = np.random.default_rng(5).normal(size=(2, sph.num_ao))
    back = MOs_data(num_mo=2, aos_data=aos, mo_coefficients=c_sph @ T).to_spherical()
    assert rel(back.mo_coefficients, c_sph) < 1e-10
    assert rel(back.mo_coefficients @ ao_value(AOTable(sph), g["r"]), (c_sph @ T) @ ao_value(AOTable(aos), g["r"])) < 1e-10
    for l in range(5):
        assert spherical_to_cartesian_matrix(l).shape == (2 * l + 1, (l + 1) * (l + 2) // 2)


def test_geminal_conversions_keep_the_geminal():
    """Geminal_data.convert_from_MOs_to_AOs (determinant.py:687-722) and
    to_spherical (:587-626) give the same geminal matrix (oracle values): the
    MO geminal of water_like over its AOs, and a Cartesian-AO geminal whose
    lambda lies in the spherical span (lambda_cart = T^T lambda_sph T) over the
    spherical shells, where lambda comes back exactly."""
    import dataclasses

    from cart_system import cartesian_from_spherical
    from jqmc_gb300.atomic_orbital import aos_cart_to_sphe
    from jqmc_gb300.determinant import Geminal_data
    syn = synthetic.water_like()
    ham = syn.hamiltonian
    gem = ham.wavefunction_data.geminal_data
    assert gem.is_mo_representation and not gem.is_ao_representation
    r_up, r_dn = syn.initial_electrons(2, seed=9)

    def geminal(g):
        o = OracleSystem(dataclasses.replace(ham, wavefunction_data=dataclasses.replace(ham.wavefunction_data, geminal_data=g)))
        return [o.geminal(r_up[w], r_dn[w]) for w in range(2)]

    ao = Geminal_data.convert_from_MOs_to_AOs(gem)
    assert ao.is_ao_representation and Geminal_data.convert_from_MOs_to_AOs(ao) is ao
    for a, b in zip(geminal(ao), geminal(gem)):
        assert rel(a, b) < 1e-12
    sph = ao.orb_data_up_spin
    cart = cartesian_from_spherical(sph)
    _, pinv = aos_cart_to_sphe(cart)
    T = np.linalg.pinv(pinv)
    lam_sph = ao.lambda_matrix
    gc = Geminal_data(gem.num_electron_up, gem.num_electron_dn, cart, cart, T.T @ lam_sph @ T)
    gs = gc.to_spherical()
    assert rel(gs.lambda_matrix, lam_sph) < 1e-10
    for a, b in zip(geminal(gs), geminal(gc)):
        assert rel(a, b) < 1e-10
    assert gem.to_spherical().lambda_matrix is gem.lambda_matrix
    sym = gs.symmetrize_lambda(gs.lambda_matrix + np.triu(np.ones_like(gs.lambda_matrix), 1))
    assert np.array_equal(sym, sym.T)
