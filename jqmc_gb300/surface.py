"""The reference's module-level evaluation functions on the GPU path.

jqmc exposes per-configuration functions beside its drivers:
- jqmc.atomic_orbital.compute_AOs*, jqmc.molecular_orbital.compute_MOs*;
- jqmc.determinant.compute_*geminal_all_elements;
- jqmc.jastrow_factor.compute_Jastrow_*;
- jqmc.wavefunction.evaluate_* and compute_kinetic_energy;
- jqmc.hamiltonians.compute_local_energy.

The modules of this package keep those names, and this file holds their
bodies.  Each call runs the walker kernels on a device copy of the data object
it receives (cached per object), with the configurations as walkers:
- r_up_carts (n_up, 3) gives a Python float, as the reference returns;
- (W, n_up, 3) gives an array over the W configurations.

AO and MO tables take points (..., 3) and return (num_orb, ...).

The kernels need a whole Hamiltonian, so partial objects are completed:
- nuclear charges of zero and no ECP where only the wavefunction matters;
- a stand-in geminal of s functions where only the Jastrow factor matters (its
  determinant outputs are not read);
- an identity pairing matrix over the AO set whose tables are asked for.

There is no CPU evaluation: without the built library or a CUDA device these
raise, like the drivers.
"""

from __future__ import annotations

from collections import OrderedDict

import numpy as np
import torch

from .atomic_orbital import AOs_sphe_data
from .coulomb_potential import Coulomb_potential_data
from .determinant import Geminal_data
from ._lib import JqmcError
from .engine import GpuSystem, WalkerSet
from .hamiltonians import Hamiltonian_data
from .jastrow_factor import Jastrow_data
from .molecular_orbital import MOs_data
from .structure import Structure_data
from .wavefunction import Wavefunction_data

_CACHE_SIZE = 8
_cache: OrderedDict = OrderedDict()   # id(data object) -> (data object, GpuSystem)


def _system(obj, build) -> GpuSystem:
    """The device copy for ``obj`` (built by ``build()`` into a Hamiltonian on first use)."""
    hit = _cache.get(id(obj))
    if hit is not None and hit[0] is obj:
        _cache.move_to_end(id(obj))
        return hit[1]
    gs = GpuSystem(build())
    _cache[id(obj)] = (obj, gs)
    while len(_cache) > _CACHE_SIZE:
        _cache.popitem(last=False)
    return gs


def _no_charges(st: Structure_data) -> Coulomb_potential_data:
    bare = Structure_data(positions=st.positions, atomic_numbers=(0,) * st.natom,
                          element_symbols=st.element_symbols, atomic_labels=st.atomic_labels)
    return Coulomb_potential_data(structure_data=bare, ecp_flag=False)


def _structure_of(orb) -> Structure_data:
    return orb.aos_data.structure_data if isinstance(orb, MOs_data) else orb.structure_data


def _ham_for_aos(aos: AOs_sphe_data) -> Hamiltonian_data:
    st = aos.structure_data
    gem = Geminal_data(num_electron_up=1, num_electron_dn=1, orb_data_up_spin=aos, orb_data_dn_spin=aos,
                       lambda_matrix=np.eye(aos.num_ao))
    return Hamiltonian_data(structure_data=st, coulomb_potential_data=_no_charges(st),
                            wavefunction_data=Wavefunction_data(jastrow_data=Jastrow_data(), geminal_data=gem))


def _ham_for_wavefunction(wf: Wavefunction_data) -> Hamiltonian_data:
    st = _structure_of(wf.geminal_data.orb_data_up_spin)
    return Hamiltonian_data(structure_data=st, coulomb_potential_data=_no_charges(st), wavefunction_data=wf)


def _stand_in_geminal(st, n_up: int, n_dn: int) -> Geminal_data:
    """A geminal for quantities that do not depend on it: n_up s functions with
    distinct exponents (0.3 to 3 bohr^-2) on nucleus 0 and a unit pairing matrix,
    so that G is non-singular for electrons at distinct distances from that
    nucleus and the walker initialisation runs through cleanly."""
    s_set = AOs_sphe_data(structure_data=st, nucleus_index=(0,) * n_up, num_ao=n_up, num_ao_prim=n_up,
                          orbital_indices=tuple(range(n_up)), exponents=np.geomspace(0.3, 3.0, n_up),
                          coefficients=np.ones(n_up), angular_momentums=(0,) * n_up, magnetic_quantum_numbers=(0,) * n_up)
    return Geminal_data(num_electron_up=n_up, num_electron_dn=n_dn, orb_data_up_spin=s_set, orb_data_dn_spin=s_set,
                        lambda_matrix=np.eye(n_up, 2 * n_up - n_dn))


def _ham_for_jastrow(jd: Jastrow_data, n_up: int, n_dn: int) -> Hamiltonian_data:
    if jd.jastrow_one_body_data is not None:
        st = jd.jastrow_one_body_data.structure_data
    elif jd.jastrow_three_body_data is not None:
        st = jd.jastrow_three_body_data.orb_data.structure_data
    else:
        st = Structure_data(positions=np.zeros((1, 3)), atomic_numbers=(0,))
    # its determinant outputs are not read, and the J outputs do not depend on it
    return Hamiltonian_data(structure_data=st, coulomb_potential_data=_no_charges(st),
                            wavefunction_data=Wavefunction_data(jastrow_data=jd, geminal_data=_stand_in_geminal(st, n_up, n_dn)))


def _ham_for_coulomb(coul, n_up: int, n_dn: int) -> Hamiltonian_data:
    """The given Coulomb/ECP data (None: no nuclear charges) with the stand-in
    geminal and no Jastrow.  The walker initialisation fills the energy cache
    (electron-ion and local ECP terms per electron, the electron-electron total),
    which is all that is read."""
    if coul is None:
        return _ham_for_jastrow(Jastrow_data(), n_up, n_dn)
    st = coul.structure_data
    return Hamiltonian_data(structure_data=st, coulomb_potential_data=coul,
                            wavefunction_data=Wavefunction_data(jastrow_data=Jastrow_data(),
                                                                geminal_data=_stand_in_geminal(st, n_up, n_dn)))


def coulomb_terms(coul, r_up_carts, r_dn_carts):
    """(electron-ion per electron (W, N), local ECP per electron (W, N), electron-
    electron (W,), ion-ion, single) from the energy cache of the walker
    initialisation; coul None: no nuclear charges (electron-electron only)."""
    r_up, r_dn, single = _configs(r_up_carts, r_dn_carts)
    n_up, n_dn = r_up.shape[1], r_dn.shape[1]
    key = ("coulomb", id(coul), n_up, n_dn)
    hit = _cache.get(key)
    if hit is not None and hit[0] is coul:
        _cache.move_to_end(key)
        gs = hit[1]
    else:
        gs = GpuSystem(_ham_for_coulomb(coul, n_up, n_dn))
        _cache[key] = (coul, gs)
        while len(_cache) > _CACHE_SIZE:
            _cache.popitem(last=False)
    ec = _walkers(gs, r_up, r_dn).ecache          # (W, N + 1, stride)
    N = n_up + n_dn
    ei, eloc, ee = ec[:, :N, 0], ec[:, :N, 1], ec[:, N, 0]
    if not (bool(torch.isfinite(ei).all()) and bool(torch.isfinite(eloc).all()) and bool(torch.isfinite(ee).all())):
        raise JqmcError("the energy cache of the Coulomb evaluation holds non-finite values")
    return ei, eloc, ee, float(gs.ion_ion), single


def _configs(r_up_carts, r_dn_carts):
    """(r_up (W, n_up, 3), r_dn (W, n_dn, 3), single configuration?)"""
    r_up = np.asarray(r_up_carts, dtype=np.float64)
    r_dn = np.asarray(r_dn_carts, dtype=np.float64)
    single = r_up.ndim == 2
    if single:
        r_up, r_dn = r_up[None], r_dn[None]
    if r_up.ndim != 3 or r_dn.ndim != 3 or r_up.shape[-1] != 3 or r_dn.shape[-1] != 3 or r_up.shape[0] != r_dn.shape[0]:
        raise ValueError(f"electron coordinates must be (n, 3) or (W, n, 3); got {r_up.shape} and {r_dn.shape}")
    return r_up, r_dn, single


def _walkers(gs: GpuSystem, r_up: np.ndarray, r_dn: np.ndarray) -> WalkerSet:
    if r_up.shape[1] != gs.n_up or r_dn.shape[1] != gs.n_dn:
        raise ValueError(f"expected {gs.n_up} up and {gs.n_dn} down electrons; got {r_up.shape[1]} and {r_dn.shape[1]}")
    return WalkerSet(gs, r_up, r_dn, precision="fp64")


def _out(t: torch.Tensor, single: bool):
    a = t.detach().cpu().numpy()
    return float(a[0]) if single else a


# ---------------------------------------------------------------- AO / MO tables
def ao_vgl(aos: AOs_sphe_data, r_carts) -> torch.Tensor:
    """(5, num_ao, ...) value, d/dx, d/dy, d/dz, Laplacian at points (..., 3), on the device."""
    gs = _system(aos, lambda: _ham_for_aos(aos))
    r = np.asarray(r_carts, dtype=np.float64)
    if r.shape[-1] != 3:
        raise ValueError(f"points must be (..., 3); got {r.shape}")
    lead = r.shape[:-1]
    out = gs.ao_vgl(torch.as_tensor(r.reshape(-1, 3)), basis=0)
    return out.reshape(5, aos.num_ao, *lead)


def mo_vgl(mos: MOs_data, r_carts) -> torch.Tensor:
    """(5, num_mo, ...) MO value, gradient and Laplacian: C times the AO tables."""
    t = ao_vgl(mos.aos_data, r_carts)
    c = torch.as_tensor(np.asarray(mos.mo_coefficients, dtype=np.float64), device=t.device)
    return torch.einsum("ma,ka...->km...", c, t)


def as_numpy(t: torch.Tensor) -> np.ndarray:
    return t.detach().cpu().numpy()


# ---------------------------------------------------------------- determinant and wavefunction
def geminal_log_det(geminal: Geminal_data, r_up_carts, r_dn_carts):
    """(ln|det G|, sign det G, G) for each configuration (walker initialisation + jqmc_log_psi)."""
    wf = Wavefunction_data(jastrow_data=Jastrow_data(), geminal_data=geminal)
    gs = _system(geminal, lambda: _ham_for_wavefunction(wf))
    r_up, r_dn, single = _configs(r_up_carts, r_dn_carts)
    ws = _walkers(gs, r_up, r_dn)
    ld, sg, _ = ws.log_psi()
    return ld, sg, ws.G, single


def as_factor(G: torch.Tensor, Ginv: torch.Tensor) -> torch.Tensor:
    """Attaccalite-Sorella factor (min(min row |G|^2, min column |G|^2) |G^-1|_F^2)^(-3/8),
    zero where that product is not positive (jqmc/determinant.py:1223-1260); G, Ginv (W, n, n)."""
    F = (Ginv * Ginv).sum(dim=(1, 2))
    S = torch.minimum((G * G).sum(dim=2).amin(dim=1), (G * G).sum(dim=1).amin(dim=1))
    SF = S * F
    return torch.where(SF > 0.0, SF.clamp_min(torch.finfo(SF.dtype).tiny) ** (-3.0 / 8.0), torch.zeros_like(SF))


def geminal_as_factor(geminal: Geminal_data, r_up_carts, r_dn_carts):
    """The AS factor of each configuration, from the walker initialisation's G and G^-1."""
    wf = Wavefunction_data(jastrow_data=Jastrow_data(), geminal_data=geminal)
    gs = _system(geminal, lambda: _ham_for_wavefunction(wf))
    r_up, r_dn, single = _configs(r_up_carts, r_dn_carts)
    ws = _walkers(gs, r_up, r_dn)
    return as_factor(ws.G, ws.Ginv), single


def wavefunction_parts(wf: Wavefunction_data, r_up_carts, r_dn_carts):
    """(ln|det G|, sign, J) for each configuration."""
    gs = _system(wf, lambda: _ham_for_wavefunction(wf))
    r_up, r_dn, single = _configs(r_up_carts, r_dn_carts)
    ld, sg, jj = _walkers(gs, r_up, r_dn).log_psi()
    return ld, sg, jj, single


def electron_tables(gs: GpuSystem, r_up_carts, r_dn_carts):
    """Per-electron derivatives of ln|psi| and kinetic elements as NumPy, (N, 9) for
    one configuration or (W, N, 9): grad ln|det| (3), lap ln|det|, grad J (3),
    lap J, T_e; and n_up (jqmc_electron_terms)."""
    r_up, r_dn, single = _configs(r_up_carts, r_dn_carts)
    a = as_numpy(_walkers(gs, r_up, r_dn).electron_terms())
    return (a[0] if single else a), gs.n_up


def discretized_kinetic(alat: float, wf: Wavefunction_data, r_up_carts, r_dn_carts, RT):
    """(r_up configurations (6N, n_up, 3), r_dn configurations (6N, n_dn, 3),
    elements (6N,)) of the six moves +-alat along the rows of RT for every
    electron, up electrons first; with a leading walker axis for (W, n, 3) inputs."""
    gs = wavefunction_system(wf)
    r_up, r_dn, single = _configs(r_up_carts, r_dn_carts)
    W, nu, nd = r_up.shape[0], r_up.shape[1], r_dn.shape[1]
    ang = angles_from_RT(RT).reshape(-1, 3)
    if ang.shape[0] == 1 and W > 1:
        ang = np.repeat(ang, W, axis=0)
    if ang.shape[0] != W:
        raise ValueError(f"{ang.shape[0]} rotations for {W} configurations")
    el = as_numpy(_walkers(gs, r_up, r_dn).kinetic_mesh(torch.as_tensor(ang), alat)).reshape(W, -1)
    rt = np.asarray(RT, dtype=np.float64).reshape(-1, 3, 3)
    if rt.shape[0] == 1:
        rt = np.repeat(rt, W, axis=0)
    shifts = alat * np.einsum("kc,wcd->wkd", np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]],
                                                      dtype=np.float64), rt)           # (W, 6, 3): rows of RT
    N = nu + nd
    cu = np.repeat(r_up[:, None], 6 * N, axis=1)
    cd = np.repeat(r_dn[:, None], 6 * N, axis=1)
    for e in range(N):
        for k in range(6):
            g = 6 * e + k
            if e < nu:
                cu[:, g, e] += shifts[:, k]
            else:
                cd[:, g, e - nu] += shifts[:, k]
    if single:
        return cu[0], cd[0], el[0]
    return cu, cd, el


def wavefunction_system(wf: Wavefunction_data) -> GpuSystem:
    return _system(wf, lambda: _ham_for_wavefunction(wf))


def geminal_system(geminal: Geminal_data) -> GpuSystem:
    wf = Wavefunction_data(jastrow_data=Jastrow_data(), geminal_data=geminal)
    return _system(geminal, lambda: _ham_for_wavefunction(wf))


def jastrow_system(jd: Jastrow_data, n_up: int, n_dn: int, key_obj=None) -> GpuSystem:
    """The stand-in system of a Jastrow factor, cached on ``key_obj`` (default ``jd``)."""
    owner = jd if key_obj is None else key_obj
    key = (id(owner), n_up, n_dn)
    hit = _cache.get(key)
    if hit is not None and hit[0] is owner:
        _cache.move_to_end(key)
        return hit[1]
    gs = GpuSystem(_ham_for_jastrow(jd, n_up, n_dn))
    _cache[key] = (owner, gs)
    while len(_cache) > _CACHE_SIZE:
        _cache.popitem(last=False)
    return gs


def jastrow_value(jd: Jastrow_data, r_up_carts, r_dn_carts, key_obj=None):
    """J (without exp) for each configuration; the device copy is cached on
    ``key_obj`` (the caller's data object; default ``jd``)."""
    r_up, r_dn, single = _configs(r_up_carts, r_dn_carts)
    gs = jastrow_system(jd, r_up.shape[1], r_dn.shape[1], key_obj)
    _, _, jj = _walkers(gs, r_up, r_dn).log_psi()
    return jj, single


def kinetic_energy(wf: Wavefunction_data, r_up_carts, r_dn_carts):
    """-1/2 sum_i lap_i psi / psi: the local energy of the wavefunction with no
    nuclear charges and no ECP, less the electron-electron repulsion."""
    gs = _system(wf, lambda: _ham_for_wavefunction(wf))
    r_up, r_dn, single = _configs(r_up_carts, r_dn_carts)
    ws = _walkers(gs, r_up, r_dn)
    angles = torch.zeros((ws.nwalk, 3), dtype=torch.float64, device=gs.device)
    eL, _ = ws.vmc_measure(angles, 0.0)
    r = ws.r
    d = torch.cdist(r, r)
    iu = torch.triu_indices(r.shape[1], r.shape[1], offset=1, device=r.device)
    vee = (1.0 / d[:, iu[0], iu[1]]).sum(dim=1)
    return eL - vee, single


# ---------------------------------------------------------------- local energy
def angles_from_RT(RT) -> np.ndarray:
    """Euler angles (alpha, beta, gamma) with RT = R(alpha, beta, gamma)^T, the
    rotation convention of the reference's drivers (jqmc_mcmc.py:724-727,
    jqmc_gfmc.py:4721-4736); RT (3, 3) or (W, 3, 3)."""
    rt = np.asarray(RT, dtype=np.float64)
    if rt.shape[-2:] != (3, 3):
        raise ValueError(f"RT must be (3, 3) or (W, 3, 3); got {rt.shape}")
    R = np.swapaxes(rt, -1, -2)
    eye = np.eye(3)
    if not np.allclose(R @ np.swapaxes(R, -1, -2), eye, atol=1e-10) or not np.allclose(np.linalg.det(R), 1.0, atol=1e-10):
        raise ValueError("RT must be a proper rotation matrix")
    beta = np.arcsin(np.clip(-R[..., 2, 0], -1.0, 1.0))
    alpha = np.arctan2(R[..., 2, 1], R[..., 2, 2])
    gamma = np.arctan2(R[..., 1, 0], R[..., 0, 0])
    return np.stack([alpha, beta, gamma], axis=-1)


def potential_energy(coul, wf: Wavefunction_data, r_up_carts, r_dn_carts, RT, Nv: int = 6):
    """(V = E_L - T for each configuration, single): bare Coulomb plus the local and
    non-local ECP with the quadrature rotated by RT, on the system of (coul, wf)
    (cached on both objects)."""
    key = ("potential", id(coul), id(wf), Nv)
    hit = _cache.get(key)
    if hit is not None and hit[0][0] is coul and hit[0][1] is wf:
        _cache.move_to_end(key)
        gs = hit[1]
    else:
        ham = Hamiltonian_data(structure_data=coul.structure_data, coulomb_potential_data=coul, wavefunction_data=wf)
        gs = GpuSystem(ham, Nv=Nv)
        _cache[key] = ((coul, wf), gs)
        while len(_cache) > _CACHE_SIZE:
            _cache.popitem(last=False)
    eL, single = local_energy(None, r_up_carts, r_dn_carts, RT, system=gs)
    t, _ = kinetic_energy(wf, r_up_carts, r_dn_carts)
    return eL - t, single


def local_energy(ham: Hamiltonian_data, r_up_carts, r_dn_carts, RT, system: GpuSystem | None = None):
    """E_L for each configuration, non-local ECP quadrature rotated by RT."""
    gs = system if system is not None else _system(ham, lambda: ham)
    r_up, r_dn, single = _configs(r_up_carts, r_dn_carts)
    ang = angles_from_RT(RT).reshape(-1, 3)
    W = r_up.shape[0]
    if ang.shape[0] == 1 and W > 1:
        ang = np.repeat(ang, W, axis=0)
    if ang.shape[0] != W:
        raise ValueError(f"{ang.shape[0]} rotations for {W} configurations")
    ws = _walkers(gs, r_up, r_dn)
    eL, _ = ws.vmc_measure(torch.as_tensor(ang, device=gs.device).contiguous(), 0.0)
    return eL, single


def scalar_or_array(t: torch.Tensor, single: bool):
    return _out(t, single)
