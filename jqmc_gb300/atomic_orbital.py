"""Contracted spherical Gaussian atomic orbitals (and the Cartesian data layout).

Mirrors ``jqmc/atomic_orbital.py``: the data layout of ``AOs_sphe_data``
(atomic_orbital.py:781-929) and the public calls ``compute_AOs``
(atomic_orbital.py:1886) and ``compute_AOs_value_grad_lap``
(atomic_orbital.py:3594-3640).  An AO is

    phi_mu(r) = sum_p c_p N_p exp(-Z_p |r-R|^2) * sqrt((2l+1)/4pi) * S_lm(r-R)

with N_p the primitive normalisation of atomic_orbital.py:2316-2323 and S_lm the
real regular solid harmonic scaled by sqrt(4pi/(2l+1)) (atomic_orbital.py:2353-2585).

The evaluation itself runs in the CUDA library (``ao_vgl`` in
``csrc/jqmc_gpu.cu``); this module packs the basis into the shell table the
kernels read and wraps the C-ABI call.  Unlike the reference, the batched call
takes electron positions with a leading walker axis.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from math import comb, factorial, pi, sqrt

import numpy as np

from .structure import Structure_data

L_MAX = 6


def primitive_norm(l: int, Z: float) -> float:
    """sqrt(2^(2l+3) (l+1)! (2Z)^(l+3/2) / ((2l+2)! sqrt(pi))): the radial
    normalisation of atomic_orbital.py:2316-2323, times the sqrt((2l+1)/4pi)
    angular factor that multiplies the scaled solid harmonic."""
    n2 = (2.0 ** (2 * l + 3)) * factorial(l + 1) * (2.0 * Z) ** (l + 1.5) / (factorial(2 * l + 2) * sqrt(pi))
    return sqrt(n2) * sqrt((2 * l + 1) / (4.0 * pi))


@dataclass(frozen=True)
class AOs_sphe_data:
    """Field-for-field mirror of jqmc's ``AOs_sphe_data`` (atomic_orbital.py:910-929)."""

    structure_data: Structure_data = field(default_factory=Structure_data)
    nucleus_index: tuple = ()
    num_ao: int = 0
    num_ao_prim: int = 0
    orbital_indices: tuple = ()
    exponents: np.ndarray = field(default_factory=lambda: np.zeros(0))
    coefficients: np.ndarray = field(default_factory=lambda: np.zeros(0))
    angular_momentums: tuple = ()
    magnetic_quantum_numbers: tuple = ()

    def __post_init__(self):
        object.__setattr__(self, "exponents", np.asarray(self.exponents, dtype=np.float64))
        object.__setattr__(self, "coefficients", np.asarray(self.coefficients, dtype=np.float64))

    def sanity_check(self) -> None:
        if len(self.nucleus_index) != self.num_ao:
            raise ValueError("len(nucleus_index) != num_ao")
        if len(self.angular_momentums) != self.num_ao or len(self.magnetic_quantum_numbers) != self.num_ao:
            raise ValueError("angular_momentums / magnetic_quantum_numbers must have num_ao entries")
        if len(self.orbital_indices) != self.num_ao_prim or len(self.exponents) != self.num_ao_prim:
            raise ValueError("primitive arrays must have num_ao_prim entries")
        if len(self.coefficients) != self.num_ao_prim:
            raise ValueError("len(coefficients) != num_ao_prim")
        for l, m in zip(self.angular_momentums, self.magnetic_quantum_numbers):
            if not (0 <= l <= L_MAX and -l <= m <= l):
                raise ValueError(f"(l, m)=({l}, {m}) outside the supported range l<={L_MAX}")
        if set(self.orbital_indices) != set(range(self.num_ao)):
            raise ValueError("every AO needs at least one primitive")

    @property
    def orb_num(self) -> int:
        return self.num_ao

    @property
    def _atomic_center_carts_np(self) -> np.ndarray:
        return self.structure_data.positions[np.asarray(self.nucleus_index, dtype=np.int64)]

    def primitives_of(self, ao: int):
        idx = [i for i, v in enumerate(self.orbital_indices) if v == ao]
        return self.exponents[idx], self.coefficients[idx]

    def shells(self):
        """Group AOs into shells: consecutive AOs on one nucleus with the same l and
        the same primitive list.  Returns a list of dicts with keys
        ``atom, l, exps, coefs, aos (list of AO indices), ms (list of m)``.  Every
        AO appears in exactly one shell, so evaluation per shell shares the
        exponentials across the 2l+1 AOs of a shell."""
        shells = []
        for ao in range(self.num_ao):
            e, c = self.primitives_of(ao)
            atom = int(self.nucleus_index[ao])
            l = int(self.angular_momentums[ao])
            m = int(self.magnetic_quantum_numbers[ao])
            if shells:
                s = shells[-1]
                if (s["atom"] == atom and s["l"] == l and len(s["exps"]) == len(e)
                        and np.array_equal(s["exps"], e) and np.array_equal(s["coefs"], c)
                        and m not in s["ms"] and len(s["ms"]) < 2 * l + 1):
                    s["aos"].append(ao)
                    s["ms"].append(m)
                    continue
            shells.append({"atom": atom, "l": l, "exps": e, "coefs": c, "aos": [ao], "ms": [m]})
        return shells


def cartesian_orders(l: int):
    """(nx, ny, nz) of the Cartesian components of one shell in TREXIO order,
    itertools.combinations_with_replacement("xyz", l) (trexio_wrapper.py:244-247):
    xx, xy, xz, yy, yz, zz for l = 2."""
    out = []
    for nx in range(l, -1, -1):
        for ny in range(l - nx, -1, -1):
            out.append((nx, ny, l - nx - ny))
    return out


def cartesian_norm(l: int, Z: float, nx: int, ny: int, nz: int) -> float:
    """sqrt((2Z/pi)^(3/2) (8Z)^l nx! ny! nz! / ((2nx)! (2ny)! (2nz)!)): the primitive
    normalisation of a Cartesian Gaussian (atomic_orbital.py:1984-2030, :2198-2290)."""
    ratio = factorial(nx) * factorial(ny) * factorial(nz) / (factorial(2 * nx) * factorial(2 * ny) * factorial(2 * nz))
    return sqrt((2.0 * Z / pi) ** 1.5 * (8.0 * Z) ** l * ratio)


def _poly_mul(a: dict, b: dict) -> dict:
    out = {}
    for ka, va in a.items():
        for kb, vb in b.items():
            k = (ka[0] + kb[0], ka[1] + kb[1], ka[2] + kb[2])
            out[k] = out.get(k, 0.0) + va * vb
    return out


def solid_harmonic_monomials(l: int, m: int) -> dict:
    """{(a, b, c): coefficient} of S_lm = sum coef x^a y^b z^c, the real solid
    harmonic scaled by sqrt(4pi/(2l+1)) (the convention of atomic_orbital.py:2353-2585),
    expanded from the closed form Pi_l^|m|(z, r^2) times Re/Im (x + iy)^|m|."""
    am = abs(m)
    pi = {}
    for k in range((l - am) // 2 + 1):
        ck = ((-1) ** k * 2.0 ** -l * comb(l, k) * comb(2 * l - 2 * k, l) * factorial(l - 2 * k)
              / factorial(l - 2 * k - am))
        for i in range(k + 1):
            for j in range(k - i + 1):
                q = k - i - j
                key = (2 * i, 2 * j, 2 * q + l - 2 * k - am)
                pi[key] = pi.get(key, 0.0) + ck * factorial(k) / (factorial(i) * factorial(j) * factorial(q))
    scale = sqrt(factorial(l - am) / factorial(l + am))
    if m == 0:
        return {k: v * scale for k, v in pi.items() if v != 0.0}
    part = {}
    for t in range(am + 1):   # (x + i y)^|m| = sum C(|m|, t) x^(|m|-t) (i y)^t
        if (t % 2 == 0) == (m > 0):
            sign = (-1) ** (t // 2)
            part[(am - t, t, 0)] = sign * comb(am, t)
    out = _poly_mul(pi, part)
    return {k: v * scale * sqrt(2.0) for k, v in out.items() if v != 0.0}


def spherical_to_cartesian_matrix(l: int) -> np.ndarray:
    """(2l+1, (l+1)(l+2)/2): row m + l expresses the spherical AO of m as a
    combination of the Cartesian AOs of the same shell (same exponents and
    contraction coefficients, each with its own primitive normalisation), in
    TREXIO component order.  The factor N_sph / N_cart does not depend on Z."""
    orders = cartesian_orders(l)
    T = np.zeros((2 * l + 1, len(orders)))
    for m in range(-l, l + 1):
        for key, c in solid_harmonic_monomials(l, m).items():
            T[m + l, orders.index(key)] = c * primitive_norm(l, 1.0) / cartesian_norm(l, 1.0, *key)
    return T


def aos_cart_to_sphe(aos_data):
    """(AOs_sphe_data, transform_pinv (num_ao_cart, num_ao_sph)) of a Cartesian
    basis (atomic_orbital.py:1574-1690): Cartesian AOs on one nucleus with one l
    and the same primitives form a shell, which must be complete; each shell
    gives 2l+1 spherical AOs with those primitives, m = -l..l; MO coefficients
    map by C_sph = C_cart transform_pinv, the least-squares projection (exact
    for l <= 1; higher shells drop their r^2 components)."""
    if isinstance(aos_data, AOs_sphe_data):
        return aos_data, np.eye(aos_data.num_ao)
    if not isinstance(aos_data, AOs_cart_data):
        raise ValueError("Spherical conversion is only available from Cartesian AOs.")
    shells = []
    for a in range(aos_data.num_ao):
        e, c = aos_data.primitives_of(a)
        atom, l = int(aos_data.nucleus_index[a]), int(aos_data.angular_momentums[a])
        pw = (int(aos_data.polynominal_order_x[a]), int(aos_data.polynominal_order_y[a]), int(aos_data.polynominal_order_z[a]))
        for sh in shells:
            if (sh["atom"] == atom and sh["l"] == l and len(sh["exps"]) == len(e) and np.allclose(sh["exps"], e)
                    and np.allclose(sh["coefs"], c) and pw not in sh["aos"]):
                sh["aos"][pw] = a
                break
        else:
            shells.append({"atom": atom, "l": l, "exps": e, "coefs": c, "aos": {pw: a}})
    n_sph = sum(2 * sh["l"] + 1 for sh in shells)
    T = np.zeros((n_sph, aos_data.num_ao))
    nuc, ls, ms, oi, ex, co = [], [], [], [], [], []
    row = 0
    for sh in shells:
        l = sh["l"]
        orders = cartesian_orders(l)
        if set(sh["aos"]) != set(orders):
            raise ValueError(f"Shell with l={l} at nucleus {sh['atom']} is incomplete: {len(sh['aos'])} Cartesian AOs found.")
        cols = [sh["aos"][o] for o in orders]
        T[np.ix_(range(row, row + 2 * l + 1), cols)] = spherical_to_cartesian_matrix(l)
        for m in range(-l, l + 1):
            a = len(nuc)
            nuc.append(sh["atom"])
            ls.append(l)
            ms.append(m)
            oi += [a] * len(sh["exps"])
            ex += list(sh["exps"])
            co += list(sh["coefs"])
        row += 2 * l + 1
    sph = AOs_sphe_data(structure_data=aos_data.structure_data, nucleus_index=tuple(nuc), num_ao=n_sph, num_ao_prim=len(ex),
                        orbital_indices=tuple(oi), exponents=np.array(ex), coefficients=np.array(co),
                        angular_momentums=tuple(ls), magnetic_quantum_numbers=tuple(ms))
    return sph, np.linalg.pinv(T)


@dataclass(frozen=True)
class AOs_cart_data:
    """Field-for-field mirror of jqmc's ``AOs_cart_data`` (atomic_orbital.py:88-330): an
    AO is phi(r) = sum_p c_p N_p exp(-Z_p |r-R|^2) x^nx y^ny z^nz with N_p from
    ``cartesian_norm``.  The oracle evaluates it; the walker kernels are
    spherical, so a Cartesian basis on the GPU path raises."""

    structure_data: Structure_data = field(default_factory=Structure_data)
    nucleus_index: tuple = ()
    num_ao: int = 0
    num_ao_prim: int = 0
    orbital_indices: tuple = ()
    exponents: np.ndarray = field(default_factory=lambda: np.zeros(0))
    coefficients: np.ndarray = field(default_factory=lambda: np.zeros(0))
    angular_momentums: tuple = ()
    polynominal_order_x: tuple = ()
    polynominal_order_y: tuple = ()
    polynominal_order_z: tuple = ()

    def __post_init__(self):
        object.__setattr__(self, "exponents", np.asarray(self.exponents, dtype=np.float64))
        object.__setattr__(self, "coefficients", np.asarray(self.coefficients, dtype=np.float64))

    def sanity_check(self) -> None:
        """The checks of atomic_orbital.py:260-300, and nx + ny + nz = l."""
        if len(self.nucleus_index) != self.num_ao:
            raise ValueError("dim. of self.nucleus_index is wrong")
        if len(np.unique(self.orbital_indices)) != self.num_ao:
            raise ValueError(f"num_ao={self.num_ao} and/or num_ao_prim={self.num_ao_prim} is wrong")
        if len(self.exponents) != self.num_ao_prim or len(self.coefficients) != self.num_ao_prim:
            raise ValueError("dim. of self.exponents / self.coefficients is wrong")
        for name in ("angular_momentums", "polynominal_order_x", "polynominal_order_y", "polynominal_order_z"):
            if len(getattr(self, name)) != self.num_ao:
                raise ValueError(f"dim. of self.{name} is wrong")
        for l, nx, ny, nz in zip(self.angular_momentums, self.polynominal_order_x, self.polynominal_order_y,
                                 self.polynominal_order_z):
            if min(nx, ny, nz) < 0 or nx + ny + nz != l or not 0 <= l <= L_MAX:
                raise ValueError(f"powers ({nx}, {ny}, {nz}) do not make l = {l} (l <= {L_MAX})")

    @property
    def orb_num(self) -> int:
        return self.num_ao

    @property
    def _atomic_center_carts_np(self) -> np.ndarray:
        return self.structure_data.positions[np.asarray(self.nucleus_index, dtype=np.int64)]

    def primitives_of(self, ao: int):
        idx = [i for i, v in enumerate(self.orbital_indices) if v == ao]
        return self.exponents[idx], self.coefficients[idx]


# ---------------------------------------------------------------- evaluation (GPU, jqmc_ao_vgl)
def compute_AOs(aos_data: AOs_sphe_data, r_carts) -> np.ndarray:
    """AO values (num_ao, N) at r_carts (N, 3) (jqmc/atomic_orbital.py:1886)."""
    from . import surface
    return surface.as_numpy(surface.ao_vgl(aos_data, r_carts)[0])


def compute_AOs_grad(aos_data: AOs_sphe_data, r_carts):
    """(d/dx, d/dy, d/dz) of the AOs, each (num_ao, N) (jqmc/atomic_orbital.py:3346)."""
    from . import surface
    t = surface.as_numpy(surface.ao_vgl(aos_data, r_carts))
    return t[1], t[2], t[3]


def compute_AOs_laplacian(aos_data: AOs_sphe_data, r_carts) -> np.ndarray:
    """Laplacians of the AOs (num_ao, N) (jqmc/atomic_orbital.py:2989)."""
    from . import surface
    return surface.as_numpy(surface.ao_vgl(aos_data, r_carts)[4])


def compute_AOs_value_grad_lap(aos_data: AOs_sphe_data, r_carts):
    """(val, gx, gy, gz, lap), each (num_ao, N) (jqmc/atomic_orbital.py:3594)."""
    from . import surface
    t = surface.as_numpy(surface.ao_vgl(aos_data, r_carts))
    return t[0], t[1], t[2], t[3], t[4]
