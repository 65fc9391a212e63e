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
    if "eps_as" in c:
        from jqmc_gb300 import determinant as D
        from test_trexio import as_ratio_sq
        gem = wf.geminal_data
        ratio_sq *= as_ratio_sq(float(D.compute_AS_regularization_factor(gem, c["old_r_up"], c["old_r_dn"])),
                                float(D.compute_AS_regularization_factor(gem, c["new_r_up"], c["new_r_dn"])),
                                float(c["eps_as"]))
    kin = WF.compute_kinetic_energy(wf, c["new_r_up"], c["new_r_dn"])
    pot = H.compute_local_energy(ham, c["new_r_up"], c["new_r_dn"], np.eye(3)) - kin
    d = [int(x) for x in c["decimals"]]
    np.testing.assert_almost_equal(ratio_sq, float(c["wf_ratio_sq"]), decimal=d[0])
    np.testing.assert_almost_equal(kin, float(c["kinetic"]), decimal=d[1])
    np.testing.assert_almost_equal(pot, float(c["potential"]), decimal=d[2])


def test_gpu_geminal_and_as_factor_of_turborvb_step():
    """TurboRVB's geminals and AS factors of one Metropolis step
    (test_comparison_with_turborvb_ECP.py:646-950) from the GPU module
    functions, to the reference's 6 decimals."""
    from jqmc_gb300 import determinant as D
    from test_trexio import trexio_case
    ham, c = trexio_case("water_ccecp.npz", "j213step")
    gem = ham.wavefunction_data.geminal_data
    for when in ("old", "new"):
        G = D.compute_geminal_all_elements(gem, c[f"{when}_r_up"], c[f"{when}_r_dn"])
        np.testing.assert_almost_equal(G, c[f"geminal_{when}"], decimal=6)
        R = float(D.compute_AS_regularization_factor(gem, c[f"{when}_r_up"], c[f"{when}_r_dn"]))
        np.testing.assert_almost_equal(R, float(c[f"r_as_{when}"]), decimal=6)
        R_fast = float(D.compute_AS_regularization_factor_fast_update(G, np.linalg.inv(G)))
        np.testing.assert_almost_equal(R_fast, float(c[f"r_as_{when}"]), decimal=6)
