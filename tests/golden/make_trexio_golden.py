"""Fixtures for the TurboRVB known-answer tests, made from the reference's TREXIO files.

Reads tests/trexio_example_files/{water_ccecp_ccpvqz,H2_ae_ccpvqz}.h5 of the
reference (at /root/reference) with jqmc_gb300.trexio_wrapper.read_trexio_file
and stores the converted arrays, with the fixed configurations, Jastrow
parameters and TurboRVB values of the reference's tests, as
tests/golden/water_ccecp.npz and tests/golden/h2_ae.npz:
- water, no Jastrow: test_comparison_with_turborvb_ECP.py:75-130;
- water, two-body Jastrow: test_comparison_with_turborvb_ECP.py:217-270;
- water, two- and three-body Jastrow (jastrow_data_w_2b_3b_w_ecp.pkl):
  test_comparison_with_turborvb_ECP.py:362-503;
- water, two-, one- and three-body Jastrow (jastrow_data_w_2b_1b3b_w_ecp.pkl):
  test_comparison_with_turborvb_ECP.py:504-645;
- the same wavefunction through one whole Metropolis step (case j213step):
  test_comparison_with_turborvb_ECP.py:646-950;
- H2 all-electron, no Jastrow: test_comparison_with_turborvb_AE.py:64-102;
- H2 all-electron, one-, two- and three-body Jastrow
  (jastrow_data_w_1b_2b_1b3b_ae.pkl): test_comparison_with_turborvb_AE.py:163-261.
Per case c: c_old_r_up, c_old_r_dn, c_new_r_up, c_new_r_dn, the Jastrow
(c_j1_param and c_j2_param, NaN for none; c_j1_core, the core electrons per
nucleus; c_j3_matrix, empty for none, with the three-body AO basis in
c_j3_nucleus_index, c_j3_orbital_indices, c_j3_exponents, c_j3_coefficients,
c_j3_l, c_j3_m), c_wf_ratio_sq, c_kinetic, c_potential (potential with RT =
identity, Nv = 6, one nearest nucleus) and c_decimals (the decimals the
reference asserts for the three).  Case j213step adds the proposal's time step
dt and AS cutoff eps_as, TurboRVB's step scales fa and fb, T_ratio, the
geminals geminal_old and geminal_new (up electrons along rows), s_old, s_new,
f_old, f_new, r_as_old, r_as_new, reweight and final_ratio; its wf_ratio_sq
includes the AS ratio, as TurboRVB reports it.

The reference stores the Jastrows of the last three cases as pickles of its
own classes.  They are read here by a restricted unpickler that builds plain
records for the reference's classes and admits only numpy arrays and dtypes
besides, so no code of the reference runs.
Run: python tests/golden/make_trexio_golden.py
"""

import os
import pickle
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REFERENCE = "/root/reference"

from jqmc_gb300.trexio_wrapper import read_trexio_file  # noqa: E402


EXAMPLES = os.path.join(REFERENCE, "tests", "trexio_example_files")


class _Record:
    """The attributes of one pickled object of the reference, as a dict."""

    def __setstate__(self, state):
        if isinstance(state, tuple):  # (__dict__, __slots__ state) of slotted dataclasses
            merged = dict(state[0] or {})
            merged.update(state[1] or {})
            state = merged
        self.state = dict(state)


class _RestrictedUnpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if module == "jqmc" or module.startswith("jqmc."):
            return type(name, (_Record,), {})
        if module in ("numpy.core.multiarray", "numpy._core.multiarray") and name == "_reconstruct":
            return np._core.multiarray._reconstruct
        if module == "numpy" and name in ("ndarray", "dtype"):
            return getattr(np, name)
        raise pickle.UnpicklingError(f"{module}.{name} is not admitted")


def jastrow_arrays(pkl: str | None, positions: np.ndarray, natom: int) -> dict:
    """Fixture arrays of the Jastrow pickled in ``pkl`` (none for None); the
    nuclei of its one- and three-body parts must be those of the TREXIO file."""
    out = dict(j1_param=np.nan, j1_core=np.zeros(natom), j2_param=np.nan, j3_matrix=np.zeros((0, 0)),
               j3_nucleus_index=np.zeros(0, int), j3_orbital_indices=np.zeros(0, int), j3_exponents=np.zeros(0),
               j3_coefficients=np.zeros(0), j3_l=np.zeros(0, int), j3_m=np.zeros(0, int))
    if pkl is None:
        return out
    with open(os.path.join(EXAMPLES, pkl), "rb") as f:
        jd = _RestrictedUnpickler(f).load().state
    j1, j2, j3 = (jd.get(k) for k in ("jastrow_one_body_data", "jastrow_two_body_data", "jastrow_three_body_data"))
    if j1 is not None:
        a = j1.state
        assert a.get("jastrow_1b_type", "exp") == "exp"
        assert np.allclose(a["structure_data"].state["positions"], positions)
        out.update(j1_param=float(a["jastrow_1b_param"]), j1_core=np.asarray(a["core_electrons"], dtype=np.float64))
    if j2 is not None:
        a = j2.state
        assert a.get("jastrow_2b_type", "pade") == "pade"
        out.update(j2_param=float(a["jastrow_2b_param"]))
    if j3 is not None:
        a = j3.state
        o = a["orb_data"]
        assert type(o).__name__ == "AOs_sphe_data"
        o = o.state
        assert np.allclose(o["structure_data"].state["positions"], positions)
        out.update(j3_matrix=np.asarray(a["j_matrix"], dtype=np.float64),
                   j3_nucleus_index=np.asarray(o["nucleus_index"], dtype=int),
                   j3_orbital_indices=np.asarray(o["orbital_indices"], dtype=int),
                   j3_exponents=np.asarray(o["exponents"], dtype=np.float64),
                   j3_coefficients=np.asarray(o["coefficients"], dtype=np.float64),
                   j3_l=np.asarray(o["angular_momentums"], dtype=int),
                   j3_m=np.asarray(o["magnetic_quantum_numbers"], dtype=int))
        assert len(out["j3_l"]) == int(o["num_ao"]) and len(out["j3_exponents"]) == int(o["num_ao_prim"])
    return out


def dump(h5name: str, outname: str, cases: dict) -> None:
    st, aos, mu, md, gem, coul = read_trexio_file(os.path.join(EXAMPLES, h5name))
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
        c = dict(c)
        j2 = c.pop("j2_param", np.nan)
        arrays = jastrow_arrays(c.pop("jastrow_pkl", None), st.positions, len(st.atomic_numbers))
        if not np.isnan(j2):
            arrays["j2_param"] = j2
        for k, v in {**c, **arrays}.items():
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
    j23_old_up = np.array([[-1.1345038587576, -0.698914730480577, -0.006290951981744008],
                           [-2.30366220171161, 2.32528986358581, -0.20008513679678],
                           [0.390190526911041, 0.422863618938476, 1.0981171776173],
                           [-2.4014357356045, 0.623761374394509, 0.70010581636993]])
    j23_old_dn = np.array([[-1.58454340030273, -1.01943210665261, 0.37014437052153],
                           [1.90701925586575, 0.398999201990364, -0.745191606127732],
                           [-2.00590358216444, 2.3178763219103, -0.195294104680795],
                           [-0.103689059569662, -2.18500664943652, -1.56814885512335]])
    j23_new_up = j23_old_up.copy()
    j23_new_up[2] = [0.390190526911041, -0.270740090536313, 1.0981171776173]
    j213_old_up = np.array([[-2.02906771233089, -0.726280132104733, -0.006290951981744008],
                            [-0.332901524462574, 0.626165379953289, -0.60355949374895],
                            [-0.197062006804461, -0.396462287261025, 0.207245244485559],
                            [-2.13232697453793, 2.02938760506611, 0.626121128343523]])
    j213_old_dn = np.array([[-2.27723556201111, -0.226423326809174, 0.525171318204107],
                            [0.635659512640246, -0.128318768826431, -0.479396452798511],
                            [-2.00590358216444, 1.90796788491204, -0.195294104680795],
                            [-1.12726250654165, -0.739542218156325, -0.25704043697001]])
    j213_new_dn = j213_old_dn.copy()
    j213_new_dn[0] = [-2.27723556201111, 0.7469747620327, 0.525171318204107]
    s_old_up = np.array([[-1.13450385875760, -0.698914730480577, -6.290951981744008e-003],
                         [-2.25378719009775, 0.693895756460611, -4.612006323250584e-002],
                         [-0.753191857352684, 0.314330338959413, 0.456739833308641],
                         [-1.60902246286275, 0.499927465264998, 0.700105816369930]])
    s_old_dn = np.array([[-1.52590493546481, -1.13601932859996, 0.586518269898014],
                         [0.635659512640246, 0.398999201990364, -0.745191606127732],
                         [-2.00590358216444, -0.465069404417879, 0.360171216755478],
                         [-0.302866379660751, -0.890252305196045, 0.345597836490454]])
    s_new_up = s_old_up.copy()
    s_new_up[2] = [-0.753191857352684, -1.183650619518406e-002, 0.456739833308641]
    # TurboRVB prints the geminals with down electrons along rows
    s_geminal_old = np.array([
        [0.186887184114679, 7.221020612173907e-003, 2.919097229181558e-002, 5.283664938570871e-002],
        [2.711743127945612e-002, -1.872067172512451e-002, 5.968147400894821e-002, -1.363982711796792e-002],
        [0.196787090743597, 9.308561211374290e-002, 5.042625023653007e-003, 0.135256480405370],
        [0.152575006966341, -3.569426461507245e-002, 9.441528784169728e-002, 1.156481954187638e-002]]).T
    s_geminal_new = np.array([
        [0.186887184114679, 7.221020612173907e-03, 7.892154586169434e-02, 5.283664938570871e-02],
        [2.711743127945612e-02, -1.872067172512451e-02, 6.631227501216763e-02, -1.363982711796792e-02],
        [0.196787090743597, 9.308561211374290e-02, 4.145830624511430e-02, 0.135256480405370],
        [0.152575006966341, -3.569426461507245e-02, 0.140717058457383, 1.156481954187638e-02]]).T
    dump("water_ccecp_ccpvqz.h5", "water_ccecp.npz", {
        "nojas": dict(old_r_up=w_old_up, old_r_dn=w_old_dn, new_r_up=w_new_up, new_r_dn=w_old_dn, j2_param=np.nan,
                      wf_ratio_sq=0.919592366177397, kinetic=14.6961809426982,
                      potential=-17.0152290468758 + 0.328893830058865, decimals=(6, 6, 5)),
        "j2": dict(old_r_up=j_old_up, old_r_dn=j_old_dn, new_r_up=j_new_up, new_r_dn=j_old_dn, j2_param=0.676718854150191,
                   wf_ratio_sq=0.881124604511419, kinetic=11.1237599317225,
                   potential=-27.03387193107 + 0.243517439611676, decimals=(6, 6, 5)),
        "j23": dict(old_r_up=j23_old_up, old_r_dn=j23_old_dn, new_r_up=j23_new_up, new_r_dn=j23_old_dn,
                    jastrow_pkl="jastrow_data_w_2b_3b_w_ecp.pkl", wf_ratio_sq=0.858468162763939,
                    kinetic=5.82890200054949, potential=-19.1676316230828 + 0.284240877900265, decimals=(6, 6, 5)),
        "j213": dict(old_r_up=j213_old_up, old_r_dn=j213_old_dn, new_r_up=j213_old_up, new_r_dn=j213_new_dn,
                     jastrow_pkl="jastrow_data_w_2b_1b3b_w_ecp.pkl", wf_ratio_sq=0.268078593287622,
                     kinetic=9.84051921791642, potential=-27.1676371839677 + 0.02774284473669801, decimals=(6, 6, 5)),
        "j213step": dict(old_r_up=s_old_up, old_r_dn=s_old_dn, new_r_up=s_new_up, new_r_dn=s_old_dn,
                         jastrow_pkl="jastrow_data_w_2b_1b3b_w_ecp.pkl", wf_ratio_sq=0.846407844801284,
                         kinetic=13.8637480286375, potential=-30.808883190726 + 0.168465630163985, decimals=(6, 6, 5),
                         dt=2.0, eps_as=0.30, moved=(0, 2), fa=0.470249568592385, fb=0.437344721251066,
                         t_ratio=1.06518922117014, final_ratio=0.901584512996174, geminal_old=s_geminal_old,
                         geminal_new=s_geminal_new, f_old=53823.3438428566, f_new=54231.8526090902,
                         s_old=4.833741852724715e-003, s_new=5.669181330133306e-003, r_as_old=0.124245223553222,
                         r_as_new=0.116703654039403, reweight=0.151330476290540),
    })
    h_old_up = np.array([[1.24966813461677, 1.61428085239132, -0.164635126284132]])
    h_old_dn = np.array([[0.429108885274501, -0.007401675646959482, -0.528818841020972]])
    h_new_dn = h_old_dn.copy()
    h_new_dn[0] = [0.429108885274501, -0.007401675646959482, -1.65889610184907]
    j123_old_up = np.array([[-0.140725692347622, 1.794610704318, 0.541399181483924]])
    j123_old_dn = np.array([[1.18814636744078, 0.02606967395580784, -1.62047650291381]])
    j123_new_up = j123_old_up.copy()
    j123_new_up[0] = [0.985621336113153, 1.794610704318, 0.541399181483924]
    dump("H2_ae_ccpvqz.h5", "h2_ae.npz", {
        "nojas": dict(old_r_up=h_old_up, old_r_dn=h_old_dn, new_r_up=h_old_up, new_r_dn=h_new_dn, j2_param=np.nan,
                      wf_ratio_sq=1.27268619372079, kinetic=1.00473369916001, potential=-2.32849688911382,
                      decimals=(6, 6, 3)),
        "j123": dict(old_r_up=j123_old_up, old_r_dn=j123_old_dn, new_r_up=j123_new_up, new_r_dn=j123_old_dn,
                     jastrow_pkl="jastrow_data_w_1b_2b_1b3b_ae.pkl", wf_ratio_sq=0.539734425254117,
                     kinetic=0.06762960720224656, potential=-1.22497631738529, decimals=(6, 6, 2)),
    })


if __name__ == "__main__":
    main()
