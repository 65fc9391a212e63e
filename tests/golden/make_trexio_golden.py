"""Fixture for the TurboRVB known-answer test, made from the reference's TREXIO file.

Reads tests/trexio_example_files/water_ccecp_ccpvqz.h5 of the reference (at
/root/reference) with jqmc_gb300.trexio_wrapper.read_trexio_file and stores the
converted arrays, with the fixed configurations and the TurboRVB values of the
reference's test_comparison_with_turborvb_ECP.py:105-130, as
tests/golden/water_ccecp.npz.  Run: python tests/golden/make_trexio_golden.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REFERENCE = "/root/reference"

from jqmc_gb300.trexio_wrapper import read_trexio_file  # noqa: E402


def main():
    st, aos, mu, md, gem, coul = read_trexio_file(os.path.join(REFERENCE, "tests", "trexio_example_files", "water_ccecp_ccpvqz.h5"))
    old_up = np.array([[-1.1345038587576, -0.698914730480577, -0.006290951981744008],
                       [-2.07761893946839, 1.30902541938751, -0.05220902114745041],
                       [0.276215481293413, 0.422863618938476, 0.27986648725301],
                       [-1.60902246286275, 0.499927465264998, 0.70010581636993]])
    old_dn = np.array([[-1.48583455555933, -1.01189391902775, 1.83998639430367],
                       [0.635659512640246, 0.398999201990364, -0.745191606127732],
                       [-2.00590358216444, 1.90796788491204, -0.195294104680795],
                       [-1.12726250654165, -0.739542218156325, -0.04817447678670805]])
    new_up = old_up.copy()
    new_up[2] = [0.276215481293413, -0.270740090536313, 0.27986648725301]
    np.savez_compressed(
        os.path.join(HERE, "water_ccecp.npz"),
        positions=st.positions, atomic_numbers=np.array(st.atomic_numbers), labels=np.array(st.atomic_labels),
        ao_nucleus_index=np.array(aos.nucleus_index), ao_orbital_indices=np.array(aos.orbital_indices),
        ao_exponents=aos.exponents, ao_coefficients=aos.coefficients, ao_l=np.array(aos.angular_momentums),
        ao_m=np.array(aos.magnetic_quantum_numbers), mo_up=mu.mo_coefficients, mo_dn=md.mo_coefficients,
        lambda_matrix=gem.lambda_matrix, n_up=gem.num_electron_up, n_dn=gem.num_electron_dn,
        ecp_z_cores=np.array(coul.z_cores), ecp_maxl1=np.array(coul.max_ang_mom_plus_1), ecp_l=np.array(coul.ang_moms),
        ecp_nucleus_index=np.array(coul.nucleus_index), ecp_exponents=np.array(coul.exponents),
        ecp_coefficients=np.array(coul.coefficients), ecp_powers=np.array(coul.powers),
        old_r_up=old_up, old_r_dn=old_dn, new_r_up=new_up, new_r_dn=old_dn,
        # TurboRVB values (no Jastrow; potential with RT = identity, Nv = 6, one nearest nucleus)
        wf_ratio_sq=0.919592366177397, kinetic=14.6961809426982, potential=-17.0152290468758 + 0.328893830058865)
    print("wrote", os.path.join(HERE, "water_ccecp.npz"))


if __name__ == "__main__":
    main()
