"""The TurboRVB known answers of the reference's tests on the GPU path: TREXIO
wavefunctions with the reference's Jastrows (tests/golden/{water_ccecp,h2_ae}.npz,
every case of test_trexio.CASES), (psi'/psi)^2, the kinetic
energy and the potential through the module-level functions, to the decimals
the reference asserts."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


from test_trexio import CASES  # noqa: E402


@pytest.mark.parametrize("fixture,case", CASES)
def test_gpu_reproduces_turborvb(fixture, case):
    from jqmc_gb300 import hamiltonians as H
    from jqmc_gb300 import wavefunction as WF
    from test_trexio import trexio_case
    ham, c = trexio_case(fixture, case)
    wf = ham.wavefunction_data
    ratio_sq = (WF.evaluate_wavefunction(wf, c["new_r_up"], c["new_r_dn"])
                / WF.evaluate_wavefunction(wf, c["old_r_up"], c["old_r_dn"])) ** 2
    kin = WF.compute_kinetic_energy(wf, c["new_r_up"], c["new_r_dn"])
    pot = H.compute_local_energy(ham, c["new_r_up"], c["new_r_dn"], np.eye(3)) - kin
    d = [int(x) for x in c["decimals"]]
    np.testing.assert_almost_equal(ratio_sq, float(c["wf_ratio_sq"]), decimal=d[0])
    np.testing.assert_almost_equal(kin, float(c["kinetic"]), decimal=d[1])
    np.testing.assert_almost_equal(pot, float(c["potential"]), decimal=d[2])
