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
