"""Bare Coulomb and semilocal ECP data.

Mirrors ``Coulomb_potential_data`` (jqmc/coulomb_potential.py:188-233).  Each ECP
term k belongs to nucleus ``nucleus_index[k]`` and channel ``ang_moms[k]``; the
channel l == max_ang_mom_plus_1[atom] is the local part, lower l are non-local
projector channels.  A channel's radial function is
V_l(r) = r^-2 sum_k c_k r^(n_k) exp(-alpha_k r^2) (coulomb_potential.py:601-661).
The quadrature meshes (coulomb_potential.py:96-184) are restated in
``ECP_MESHES`` below.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .structure import Structure_data


def _icosahedron():
    th = np.array([0.0, np.pi] + [np.arctan(2.0)] * 5 + [np.pi - np.arctan(2.0)] * 5)
    ph = np.array([0.0, 0.0] + [2.0 * k * np.pi / 5.0 for k in range(5)] + [(2.0 * k + 1.0) * np.pi / 5.0 for k in range(5)])
    return np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], axis=1)


def _octa18():
    p = 1.0 / np.sqrt(2.0)
    pts = [[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
           [p, p, 0], [p, -p, 0], [-p, p, 0], [-p, -p, 0], [p, 0, p], [p, 0, -p],
           [-p, 0, p], [-p, 0, -p], [0, p, p], [0, -p, p], [0, p, -p], [0, -p, -p]]
    return np.array(pts, dtype=np.float64)


_q = 1.0 / np.sqrt(3.0)
#: Nv -> (weights, unit grid points), the spherical quadratures of the reference.
ECP_MESHES = {
    4: (np.full(4, 0.25), np.array([[_q, _q, _q], [_q, -_q, -_q], [-_q, _q, -_q], [-_q, -_q, _q]])),
    6: (np.full(6, 1.0 / 6.0), np.array([[1.0, 0, 0], [-1.0, 0, 0], [0, 1.0, 0], [0, -1.0, 0], [0, 0, 1.0], [0, 0, -1.0]])),
    12: (np.full(12, 1.0 / 12.0), _icosahedron()),
    18: (np.array([1.0 / 6.0] * 6 + [1.0 / 15.0] * 12), _octa18()),
}


@dataclass(frozen=True)
class Coulomb_potential_data:
    structure_data: Structure_data = field(default_factory=Structure_data)
    ecp_flag: bool = False
    z_cores: tuple = ()
    max_ang_mom_plus_1: tuple = ()
    num_ecps: int = 0
    ang_moms: tuple = ()
    nucleus_index: tuple = ()
    exponents: tuple = ()
    coefficients: tuple = ()
    powers: tuple = ()

    def sanity_check(self) -> None:
        n = self.structure_data.natom
        if self.ecp_flag:
            if len(self.z_cores) != n or len(self.max_ang_mom_plus_1) != n:
                raise ValueError("z_cores / max_ang_mom_plus_1 must have one entry per nucleus")
            for arr in (self.ang_moms, self.nucleus_index, self.exponents, self.coefficients, self.powers):
                if len(arr) != self.num_ecps:
                    raise ValueError("ECP term arrays must have num_ecps entries")

    @property
    def effective_charges(self) -> np.ndarray:
        z = np.asarray(self.structure_data.atomic_numbers, dtype=np.float64)
        if self.ecp_flag:
            z = z - np.asarray(self.z_cores, dtype=np.float64)
        return z

    _effective_charges = effective_charges


# ---------------------------------------------------------------- evaluation (GPU: the walker initialisation's energy cache)
def compute_bare_coulomb_potential_el_ion_element_wise(coulomb_potential_data: Coulomb_potential_data, r_up_carts,
                                                       r_dn_carts):
    """(per up electron, per down electron) electron-ion Coulomb energies with the
    effective charges (jqmc/coulomb_potential.py:2285)."""
    from . import surface
    ei, _, _, _, single = surface.coulomb_terms(coulomb_potential_data, r_up_carts, r_dn_carts)
    n = np.asarray(r_up_carts).shape[-2]
    up, dn = surface.as_numpy(ei[:, :n]), surface.as_numpy(ei[:, n:])
    return (up[0], dn[0]) if single else (up, dn)


def compute_bare_coulomb_potential_el_ion(coulomb_potential_data: Coulomb_potential_data, r_up_carts, r_dn_carts):
    """Total electron-ion Coulomb energy (jqmc/coulomb_potential.py:2575)."""
    from . import surface
    ei, _, _, _, single = surface.coulomb_terms(coulomb_potential_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(ei.sum(dim=1), single)


def compute_bare_coulomb_potential_el_el(r_up_carts, r_dn_carts):
    """Electron-electron Coulomb energy (jqmc/coulomb_potential.py:2465)."""
    from . import surface
    _, _, ee, _, single = surface.coulomb_terms(None, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(ee, single)


def compute_bare_coulomb_potential_ion_ion(coulomb_potential_data: Coulomb_potential_data) -> float:
    """Ion-ion Coulomb energy with the effective charges (jqmc/coulomb_potential.py:2522)."""
    from .engine import _ion_ion
    return float(_ion_ion(np.asarray(coulomb_potential_data.structure_data.positions, dtype=np.float64),
                          np.asarray(coulomb_potential_data.effective_charges, dtype=np.float64)))


def compute_bare_coulomb_potential(coulomb_potential_data: Coulomb_potential_data, r_up_carts, r_dn_carts):
    """Ion-ion + electron-ion + electron-electron (jqmc/coulomb_potential.py:2253)."""
    from . import surface
    ei, _, ee, ion_ion, single = surface.coulomb_terms(coulomb_potential_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(ei.sum(dim=1) + ee + ion_ion, single)


def compute_ecp_local_parts_all_pairs(coulomb_potential_data: Coulomb_potential_data, r_up_carts, r_dn_carts):
    """Local ECP channel summed over all electron-nucleus pairs (jqmc/coulomb_potential.py:1145)."""
    from . import surface
    if not coulomb_potential_data.ecp_flag:
        raise ValueError("the Coulomb data carry no ECP")
    _, eloc, _, _, single = surface.coulomb_terms(coulomb_potential_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(eloc.sum(dim=1), single)


def compute_coulomb_potential(coulomb_potential_data: Coulomb_potential_data, r_up_carts, r_dn_carts, RT, NN: int = 1,
                              Nv: int = 6, wavefunction_data=None):
    """Bare Coulomb plus the local and non-local ECP, the quadrature rotated by RT
    (jqmc/coulomb_potential.py:2643): E_L - T of the walker kernels.  Without ECP
    the bare Coulomb alone; the non-local part needs wavefunction_data.  One
    nearest nucleus (NN = 1) on the walker path."""
    from . import surface
    if NN != 1:
        raise NotImplementedError("the walker path evaluates the non-local ECP at the nearest nucleus (NN = 1)")
    if not coulomb_potential_data.ecp_flag:
        return compute_bare_coulomb_potential(coulomb_potential_data, r_up_carts, r_dn_carts)
    if wavefunction_data is None:
        raise ValueError("the non-local ECP needs wavefunction_data")
    v, single = surface.potential_energy(coulomb_potential_data, wavefunction_data, r_up_carts, r_dn_carts, RT, Nv)
    return surface.scalar_or_array(v, single)


def compute_ecp_coulomb_potential(coulomb_potential_data: Coulomb_potential_data, wavefunction_data, r_up_carts,
                                  r_dn_carts, RT, NN: int = 1, Nv: int = 6):
    """Local plus non-local ECP energy (jqmc/coulomb_potential.py:2103): the total
    potential less the bare Coulomb energy."""
    from . import surface
    if not coulomb_potential_data.ecp_flag:
        raise ValueError("the Coulomb data carry no ECP")
    if NN != 1:
        raise NotImplementedError("the walker path evaluates the non-local ECP at the nearest nucleus (NN = 1)")
    v, single = surface.potential_energy(coulomb_potential_data, wavefunction_data, r_up_carts, r_dn_carts, RT, Nv)
    ei, _, ee, ion_ion, _ = surface.coulomb_terms(coulomb_potential_data, r_up_carts, r_dn_carts)
    return surface.scalar_or_array(v - (ei.sum(dim=1) + ee + ion_ion), single)
