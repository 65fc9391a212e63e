"""Fixtures for the TurboRVB known-answer tests, made from the reference's TREXIO files.

Reads tests/trexio_example_files/{water_ccecp_ccpvqz,H2_ae_ccpvqz}.h5 of the
reference (at /root/reference) with jqmc_gb300.trexio_wrapper.read_trexio_file
and stores the converted arrays, with the fixed configurations, Jastrow
parameters and TurboRVB values of the reference's tests, as
tests/golden/water_ccecp.npz and tests/golden/h2_ae.npz:
- water, no Jastrow: test_comparison_with_turborvb_ECP.py:75-130;
- water, two-body Jastrow: test_comparison_with_turborvb_ECP.py:217-270;
- H2 all-electron, no Jastrow: test_comparison_with_turborvb_AE.py:64-102.
Per case c: c_old_r_up, c_old_r_dn, c_new_r_up, c_new_r_dn, c_j2_param (NaN
for none), c_wf_ratio_sq, c_kinetic, c_potential (potential with RT =
identity, Nv = 6, one nearest nucleus) and c_decimals (the decimals the
reference asserts for the three).  Run: python tests/golden/make_trexio_golden.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REFERENCE = "/root/reference"

from jqmc_gb300.trexio_wrapper import read_trexio_file  # noqa: E402


def dump(h5name: str, outname: str, cases: dict) -> None:
    st, aos, mu, md, gem, coul = read_trexio_file(os.path.join(REFERENCE, "tests", "trexio_example_files", h5name))
    out = dict(
        positions=st.positions, atomic_numbers=np.array(st.atomic_numbers), labels=np.array(st.atomic_labels),
        ao_nucleus_index=np.array(aos.nucleus_index), ao_orbital_indices=np.array(aos.orbital_indices),
        ao_exponents=aos.exponents, ao_coefficients=aos.coefficients, ao_l=np.array(aos.angular_momentums),
        ao_m=np.array(aos.magnetic_quantum_numbers), mo_up=mu.mo_coefficients, mo_dn=md.mo_coefficients,
        lambda_matrix=gem.lambda_matrix, n_up=gem.num_electron_up, n_dn=gem.num_electron_dn, ecp_flag=coul.ecp_flag,
        cases=np.array(list(cases)))
    if coul.ecp_flag:
        out.update(ecp_z_cores=np.array(coul.z_cores), ecp_maxl1=np.array(coul.max_ang_mom_plus_1),
                   ecp_l=np.array(coul.ang_moms), ecp_nucleus_index=np.array(coul.nucleus_index),
                   ecp_exponents=np.array(coul.exponents), ecp_coefficients=np.array(coul.coefficients),
                   ecp_powers=np.array(coul.powers))
    for name, c in cases.items():
        for k, v in c.items():
            out[f"{name}_{k}"] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, outname), **out)
    print("wrote", os.path.join(HERE, outname))


def main():
    w_old_up = np.array([[-1.1345038587576, -0.698914730480577, -0.006290951981744008],
                         [-2.07761893946839, 1.30902541938751, -0.05220902114745041],
                         [0.276215481293413, 0.422863618938476, 0.27986648725301],
                         [-1.60902246286275, 0.499927465264998, 0.70010581636993]])
    w_old_dn = np.array([[-1.48583455555933, -1.01189391902775, 1.83998639430367],
                         [0.635659512640246, 0.398999201990364, -0.745191606127732],
                         [-2.00590358216444, 1.90796788491204, -0.195294104680795],
                         [-1.12726250654165, -0.739542218156325, -0.04817447678670805]])
    w_new_up = w_old_up.copy()
    w_new_up[2] = [0.276215481293413, -0.270740090536313, 0.27986648725301]
    j_old_up = np.array([[-1.1345038587576, -0.698914730480577, -0.006290951981744008],
                         [-2.30366220171161, 1.47326376760292, 0.126403765463162],
                         [0.276215481293413, 0.422863618938476, 0.27986648725301],
                         [-2.54518559687882, 0.822753144911055, 0.70010581636993]])
    j_old_dn = np.array([[-1.42343008909407, -1.13669461924113, 0.525171318204107],
                         [1.90701925586575, 0.398999201990364, -0.745191606127732],
                         [-2.00590358216444, 1.90796788491204, -0.195294104680795],
                         [-1.12726250654165, -0.678049640381367, -0.656537799033216]])
    j_new_up = j_old_up.copy()
    j_new_up[2] = [0.276215481293413, -0.270740090536313, 0.27986648725301]
    dump("water_ccecp_ccpvqz.h5", "water_ccecp.npz", {
        "nojas": dict(old_r_up=w_old_up, old_r_dn=w_old_dn, new_r_up=w_new_up, new_r_dn=w_old_dn, j2_param=np.nan,
                      wf_ratio_sq=0.919592366177397, kinetic=14.6961809426982,
                      potential=-17.0152290468758 + 0.328893830058865, decimals=(6, 6, 5)),
        "j2": dict(old_r_up=j_old_up, old_r_dn=j_old_dn, new_r_up=j_new_up, new_r_dn=j_old_dn, j2_param=0.676718854150191,
                   wf_ratio_sq=0.881124604511419, kinetic=11.1237599317225,
                   potential=-27.03387193107 + 0.243517439611676, decimals=(6, 6, 5)),
    })
    h_old_up = np.array([[1.24966813461677, 1.61428085239132, -0.164635126284132]])
    h_old_dn = np.array([[0.429108885274501, -0.007401675646959482, -0.528818841020972]])
    h_new_dn = h_old_dn.copy()
    h_new_dn[0] = [0.429108885274501, -0.007401675646959482, -1.65889610184907]
    dump("H2_ae_ccpvqz.h5", "h2_ae.npz", {
        "nojas": dict(old_r_up=h_old_up, old_r_dn=h_old_dn, new_r_up=h_old_up, new_r_dn=h_new_dn, j2_param=np.nan,
                      wf_ratio_sq=1.27268619372079, kinetic=1.00473369916001, potential=-2.32849688911382,
                      decimals=(6, 6, 3)),
    })


if __name__ == "__main__":
    main()
