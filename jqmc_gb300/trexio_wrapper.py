"""TREXIO (HDF5 back end) input, read with the package's own HDF5 reader.

``read_trexio_file`` follows jqmc/trexio_wrapper.py:63-566 and returns the same
six objects: structure, AOs, up- and down-spin MOs, the MO geminal and the
Coulomb/ECP data.  The conversions are the reference's:
- spherical AOs in TREXIO order, m = 0, +1, -1, +2, -2, ...;
- primitive coefficients c shell_factor prim_factor sqrt(4 pi)/sqrt(2l+1)
  divided by the primitive normalisation, times the AO normalisation;
- MOs with occupation >= 1e-6, lambda the identity over the paired
  orbitals (an unpaired block for N_up > N_dn);
- ECP powers shifted by 2;
- Cartesian shells (jqmc/trexio_wrapper.py:229-360) expand into their
  (l+1)(l+2)/2 components in itertools.combinations_with_replacement order
  with coefficients c shell_factor prim_factor / N_cart, N_cart the Cartesian
  primitive normalisation of the component, times the AO normalisation; they
  give AOs_cart_data (the oracle evaluates them; the walker kernels are
  spherical).
Periodic cells and complex orbitals raise NotImplementedError.
"""

from __future__ import annotations

import math

import numpy as np

from .atomic_orbital import AOs_cart_data, AOs_sphe_data, cartesian_norm, cartesian_orders
from .coulomb_potential import Coulomb_potential_data
from .determinant import Geminal_data
from .hdf5_read import File
from .molecular_orbital import MOs_data
from .structure import Structure_data

_ELEMENTS = (
    "H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
    "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb "
    "Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn"
).split()
_MO_OCC_THRESHOLD = 1.0e-6


def _atomic_number(label: str) -> int:
    sym = "".join(ch for ch in label if ch.isalpha())
    sym = sym[:1].upper() + sym[1:].lower()
    for cand in (sym, sym[:2], sym[:1]):
        if cand in _ELEMENTS:
            return _ELEMENTS.index(cand) + 1
    raise ValueError(f"unsupported atomic label {label!r}")


def _primitive_normalization(l: int, Z: float) -> float:
    """Normalisation of r^l exp(-Z r^2) over r^2 dr with the angular factor, as the
    reference divides it out (jqmc/trexio_wrapper.py:384-392)."""
    return math.sqrt(2.0 ** (2 * l + 3) * math.factorial(l + 1) * (2.0 * Z) ** (l + 1.5)
                     / (math.factorial(2 * l + 2) * math.sqrt(math.pi)))


def read_trexio_file(trexio_file: str, store_tuple: bool = False):
    """(structure_data, aos_data, mos_data_up, mos_data_dn, geminal_data,
    coulomb_potential_data) from a TREXIO HDF5 file (jqmc/trexio_wrapper.py:63)."""
    f = File(trexio_file)

    def attr(group, name, default=None):
        g = f[group]
        return g.attrs.get(name, default)

    def data(path):
        return f[path].read()

    if "pbc" in f.root and attr("pbc", "pbc_periodic", 0):
        raise NotImplementedError("periodic cells are not supported")
    n_up = int(attr("electron", "electron_up_num"))
    n_dn = int(attr("electron", "electron_dn_num"))
    labels = [str(x) for x in data("nucleus/nucleus_label")]
    coords = np.asarray(data("nucleus/nucleus_coord"), dtype=np.float64)
    seq = tuple if store_tuple else list
    structure = Structure_data(positions=coords, pbc_flag=False, atomic_numbers=seq(_atomic_number(x) for x in labels),
                               element_symbols=seq(labels), atomic_labels=seq(labels))

    cartesian = bool(int(attr("ao", "ao_cartesian", 0)))
    shell_num = int(attr("basis", "basis_shell_num"))
    shell_index = data("basis/basis_shell_index")
    shell_nucleus = data("basis/basis_nucleus_index")
    shell_l = data("basis/basis_shell_ang_mom")
    shell_factor = data("basis/basis_shell_factor")
    expo = data("basis/basis_exponent")
    coef = data("basis/basis_coefficient")
    prim_factor = data("basis/basis_prim_factor")
    ao_num = int(attr("ao", "ao_num"))
    ao_norm = data("ao/ao_normalization")
    nucleus_index, ang, mag, orb_idx, exps, coefs, powers = [], [], [], [], [], [], []
    ao = 0
    for s in range(shell_num):
        l = int(shell_l[s])
        prims = [k for k in range(len(shell_index)) if shell_index[k] == s]
        if cartesian:
            comps = cartesian_orders(l)
            pcs = [[shell_factor[s] * prim_factor[k] / cartesian_norm(l, expo[k], *pw) * coef[k] for k in prims]
                   for pw in comps]
        else:
            comps = [0] + [i * (-1) ** j for i in range(1, l + 1) for j in range(2)]
            pc = [shell_factor[s] * prim_factor[k] * math.sqrt(4.0 * math.pi) / math.sqrt(2 * l + 1)
                  / _primitive_normalization(l, expo[k]) * coef[k] for k in prims]
            pcs = [pc] * len(comps)
        for j, comp in enumerate(comps):
            nucleus_index.append(int(shell_nucleus[s]))
            ang.append(l)
            (powers if cartesian else mag).append(comp)
            for k, c in zip(prims, pcs[j]):
                orb_idx.append(ao + j)
                exps.append(float(expo[k]))
                coefs.append(float(c * ao_norm[ao + j]))
        ao += len(comps)
    if ao != ao_num:
        raise ValueError(f"ao count {ao} is inconsistent with ao_num = {ao_num}")
    if cartesian:
        pw = np.array(powers, dtype=int).reshape(-1, 3)
        aos = AOs_cart_data(structure_data=structure, nucleus_index=seq(nucleus_index), num_ao=ao, num_ao_prim=len(exps),
                            orbital_indices=seq(orb_idx), exponents=np.array(exps), coefficients=np.array(coefs),
                            angular_momentums=seq(ang), polynominal_order_x=seq(int(x) for x in pw[:, 0]),
                            polynominal_order_y=seq(int(x) for x in pw[:, 1]),
                            polynominal_order_z=seq(int(x) for x in pw[:, 2]))
    else:
        aos = AOs_sphe_data(structure_data=structure, nucleus_index=seq(nucleus_index), num_ao=ao, num_ao_prim=len(exps),
                            orbital_indices=seq(orb_idx), exponents=np.array(exps), coefficients=np.array(coefs),
                            angular_momentums=seq(ang), magnetic_quantum_numbers=seq(mag))

    if "mo_coefficient_im" in f["mo"]:
        raise NotImplementedError("complex molecular orbitals are not supported")
    mo_c = np.asarray(data("mo/mo_coefficient"), dtype=np.float64)
    mo_occ = data("mo/mo_occupation")
    mo_spin = data("mo/mo_spin") if "mo_spin" in f["mo"] else np.zeros(len(mo_occ), dtype=int)
    spin_dependent = bool(np.any(mo_spin != 0))
    if not spin_dependent:
        idx = [i for i, v in enumerate(mo_spin) if v == 0]
        c_up = c_dn = mo_c[idx]
        occ = mo_occ[idx]
        keep = [i for i, v in enumerate(occ) if v >= _MO_OCC_THRESHOLD]
        c_up, c_dn = c_up[keep], c_dn[keep]
    elif n_up != n_dn:
        iu = [i for i, v in enumerate(mo_spin) if v == 0]
        idn = [i for i, v in enumerate(mo_spin) if v == 1]
        ku = [i for i, v in enumerate(mo_occ[iu]) if v >= _MO_OCC_THRESHOLD]
        kd = [i for i, v in enumerate(mo_occ[idn]) if v >= _MO_OCC_THRESHOLD]
        if len(ku) < len(kd):
            raise ValueError("more occupied down-spin than up-spin orbitals")
        c_up, c_dn = mo_c[iu][ku], mo_c[idn][ku]
    else:
        raise NotImplementedError("spin-dependent orbitals for a closed shell")
    nmo = c_up.shape[0]
    mos_up = MOs_data(num_mo=nmo, aos_data=aos, mo_coefficients=c_up)
    mos_dn = MOs_data(num_mo=nmo, aos_data=aos, mo_coefficients=c_dn)
    diff = n_up - n_dn
    lam_p = np.pad(np.eye(n_dn), ((0, nmo - n_dn), (0, nmo - n_dn)))
    lam_u = np.pad(np.eye(diff), ((n_dn, nmo - n_dn - diff), (0, 0)))
    geminal = Geminal_data(num_electron_up=n_up, num_electron_dn=n_dn, orb_data_up_spin=mos_up, orb_data_dn_spin=mos_dn,
                           lambda_matrix=np.hstack([lam_p, lam_u]))

    if "ecp" in f.root and attr("ecp", "ecp_num") is not None:
        coul = Coulomb_potential_data(
            structure_data=structure, ecp_flag=True, z_cores=seq(int(x) for x in data("ecp/ecp_z_core")),
            max_ang_mom_plus_1=seq(int(x) for x in data("ecp/ecp_max_ang_mom_plus_1")), num_ecps=int(attr("ecp", "ecp_num")),
            ang_moms=seq(int(x) for x in data("ecp/ecp_ang_mom")),
            nucleus_index=seq(int(x) for x in data("ecp/ecp_nucleus_index")),
            exponents=seq(float(x) for x in data("ecp/ecp_exponent")),
            coefficients=seq(float(x) for x in data("ecp/ecp_coefficient")),
            powers=seq(int(x) + 2 for x in data("ecp/ecp_power")))
    else:
        coul = Coulomb_potential_data(structure_data=structure, ecp_flag=False)
    return structure, aos, mos_up, mos_dn, geminal, coul
