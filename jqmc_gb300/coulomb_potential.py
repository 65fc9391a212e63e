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
