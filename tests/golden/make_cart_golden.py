"""Golden fixture for Cartesian AOs, made by running the reference's own functions.

Run from the repository root in a container that has the reference checked out
at /root/reference:

    python tests/golden/make_cart_golden.py

As in make_golden.py, the reference modules run on the NumPy stand-in for JAX in
``tests/golden/jaxshim``.  The basis is Cartesian on the water_like nuclei:
the shells of water_like's geminal basis (l <= 2) with their exponents and
contraction coefficients, every shell expanded into its (l+1)(l+2)/2 Cartesian
components in TREXIO order, plus an f and a g shell on the first nucleus.  The
reference's _compute_AOs_cart_debug, compute_AOs and compute_AOs_value_grad_lap
are evaluated at seeded points, and its Cartesian -> spherical conversion
(_aos_cart_to_sphe, MOs_data.to_spherical) is applied to the basis and to
seeded MO coefficients; inputs and outputs go to tests/golden/cart.npz.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REFERENCE = "/root/reference"
sys.path.insert(0, os.path.join(HERE, "jaxshim"))
sys.path.insert(0, REFERENCE)
sys.path.insert(0, ROOT)

import jqmc.atomic_orbital as r_ao  # noqa: E402
import jqmc.molecular_orbital as r_mo  # noqa: E402
import jqmc.structure as r_st  # noqa: E402

from jqmc_gb300 import synthetic  # noqa: E402
from jqmc_gb300.atomic_orbital import cartesian_orders  # noqa: E402


def cartesian_basis():
    """Arrays of the Cartesian basis (see the module docstring)."""
    syn = synthetic.water_like()
    st = syn.hamiltonian.structure_data
    sph = syn.hamiltonian.wavefunction_data.geminal_data.ao_basis_lambda()[0]
    shells = [(s["atom"], s["l"], s["exps"], s["coefs"]) for s in sph.shells()]
    shells += [(0, 3, np.array([1.3, 0.45]), np.array([0.6, 0.5])), (0, 4, np.array([0.9]), np.array([1.0]))]
    nuc, ls, px, py, pz, oi, ex, co = [], [], [], [], [], [], [], []
    ao = 0
    for atom, l, e, c in shells:
        for (nx, ny, nz) in cartesian_orders(l):
            nuc.append(atom)
            ls.append(l)
            px.append(nx)
            py.append(ny)
            pz.append(nz)
            oi += [ao] * len(e)
            ex += list(e)
            co += list(c)
            ao += 1
    return st, dict(nucleus_index=np.array(nuc), angular_momentums=np.array(ls), polynominal_order_x=np.array(px),
                    polynominal_order_y=np.array(py), polynominal_order_z=np.array(pz), orbital_indices=np.array(oi),
                    exponents=np.array(ex), coefficients=np.array(co))


def main():
    st, b = cartesian_basis()
    ref_st = r_st.Structure_data(positions=np.asarray(st.positions), pbc_flag=False, atomic_numbers=tuple(st.atomic_numbers),
                                 element_symbols=tuple(st.element_symbols), atomic_labels=tuple(st.atomic_labels))
    aos = r_ao.AOs_cart_data(structure_data=ref_st, nucleus_index=tuple(int(x) for x in b["nucleus_index"]),
                             num_ao=len(b["angular_momentums"]), num_ao_prim=len(b["exponents"]),
                             orbital_indices=tuple(int(x) for x in b["orbital_indices"]), exponents=b["exponents"],
                             coefficients=b["coefficients"], angular_momentums=tuple(int(x) for x in b["angular_momentums"]),
                             polynominal_order_x=tuple(int(x) for x in b["polynominal_order_x"]),
                             polynominal_order_y=tuple(int(x) for x in b["polynominal_order_y"]),
                             polynominal_order_z=tuple(int(x) for x in b["polynominal_order_z"]))
    aos.sanity_check()
    r = np.random.default_rng(31).normal(scale=1.5, size=(9, 3)) + np.asarray(st.positions)[0]
    out = dict(b, positions=np.asarray(st.positions), r=r)
    out["ao_debug"] = np.asarray(r_ao._compute_AOs_cart_debug(aos, r), dtype=np.float64)
    out["ao"] = np.asarray(r_ao.compute_AOs(aos, r), dtype=np.float64)
    for k, v in enumerate(r_ao.compute_AOs_value_grad_lap(aos, r)):
        out[f"ao_vgl.{k}"] = np.asarray(v, dtype=np.float64)
    # the reference's Cartesian -> spherical conversion (atomic_orbital.py:1574-1690,
    # molecular_orbital.py:214-236) of the same basis and of seeded MO coefficients
    sph, pinv = r_ao._aos_cart_to_sphe(aos)
    out["to_sphe_pinv"] = np.asarray(pinv, dtype=np.float64)
    out["to_sphe_l"] = np.asarray(sph.angular_momentums)
    out["to_sphe_m"] = np.asarray(sph.magnetic_quantum_numbers)
    out["to_sphe_nucleus_index"] = np.asarray(sph.nucleus_index)
    out["to_sphe_exponents"] = np.asarray(sph.exponents, dtype=np.float64)
    out["to_sphe_coefficients"] = np.asarray(sph.coefficients, dtype=np.float64)
    c_cart = np.random.default_rng(32).normal(size=(3, aos.num_ao))
    mos = r_mo.MOs_data(num_mo=3, aos_data=aos, mo_coefficients=c_cart).to_spherical()
    out["mo_cart_coefficients"] = c_cart
    out["mo_sphe_coefficients"] = np.asarray(mos.mo_coefficients, dtype=np.float64)
    path = os.path.join(HERE, "cart.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {len(out)} arrays to {path}; {aos.num_ao} AOs")


if __name__ == "__main__":
    main()
