"""The TurboRVB known answers of the reference's tests on the GPU path: the
water ccECP/cc-pVQZ wavefunction read from TREXIO (tests/golden/water_ccecp.npz),
(psi'/psi)^2, the kinetic energy and the potential through the module-level
functions, to the decimals the reference asserts (6, 6, 5)."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def test_gpu_reproduces_turborvb():
    from jqmc_gb300 import hamiltonians as H
    from jqmc_gb300 import wavefunction as WF
    from test_trexio import water_ccecp
    ham, g = water_ccecp()
    wf = ham.wavefunction_data
    ratio_sq = (WF.evaluate_wavefunction(wf, g["new_r_up"], g["new_r_dn"])
                / WF.evaluate_wavefunction(wf, g["old_r_up"], g["old_r_dn"])) ** 2
    kin = WF.compute_kinetic_energy(wf, g["new_r_up"], g["new_r_dn"])
    pot = H.compute_local_energy(ham, g["new_r_up"], g["new_r_dn"], np.eye(3)) - kin
    np.testing.assert_almost_equal(ratio_sq, float(g["wf_ratio_sq"]), decimal=6)
    np.testing.assert_almost_equal(kin, float(g["kinetic"]), decimal=6)
    np.testing.assert_almost_equal(pot, float(g["potential"]), decimal=5)
