"""Device-side engine: packs a Hamiltonian_data into the library's tables and
drives the walker kernels on torch-owned device buffers.

PyTorch supplies device memory and the current CUDA stream; every computation
runs in libjqmc_gpu.so through the C ABI (``_lib``).  There is no CPU fallback:
constructing a ``GpuSystem`` without the built library or without a CUDA device
raises.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .atomic_orbital import cartesian_norm, cartesian_orders, primitive_norm
from .coulomb_potential import ECP_MESHES
from .hamiltonians import Hamiltonian_data

PRECISIONS = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED, "mixed_fast_energy": _lib.PREC_MIXED_FASTE}


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def pack_basis(aos):
    """(shells int32 (nshell, 8), prims float64 (nprim, 2)) for one AOs_sphe_data.

    A shell is a run of consecutive AOs on one nucleus with one l, one primitive
    list and consecutive m; each primitive row holds (Z, c N_p sqrt((2l+1)/4pi))."""
    if hasattr(aos, "polynominal_order_x"):
        return _pack_cartesian(aos)
    aos.sanity_check()
    oi = np.asarray(aos.orbital_indices, dtype=np.int64)
    ex = np.asarray(aos.exponents, dtype=np.float64)
    co = np.asarray(aos.coefficients, dtype=np.float64)
    prim_of = [np.nonzero(oi == a)[0] for a in range(aos.num_ao)]
    shells, prims = [], []
    a = 0
    while a < aos.num_ao:
        atom, l, m = int(aos.nucleus_index[a]), int(aos.angular_momentums[a]), int(aos.magnetic_quantum_numbers[a])
        z, c = ex[prim_of[a]], co[prim_of[a]]
        b = a + 1
        while (b < aos.num_ao and int(aos.nucleus_index[b]) == atom and int(aos.angular_momentums[b]) == l
               and int(aos.magnetic_quantum_numbers[b]) == m + (b - a)
               and np.array_equal(ex[prim_of[b]], z) and np.array_equal(co[prim_of[b]], c)):
            b += 1
        p0 = len(prims)
        for zz, cc in zip(z, c):
            prims.append((zz, cc * primitive_norm(l, zz)))
        shells.append((atom, l, len(z), p0, a, b - a, m, 0))
        a = b
    return np.ascontiguousarray(np.array(shells, dtype=np.int32)), np.ascontiguousarray(np.array(prims, dtype=np.float64))


def _pack_cartesian(aos):
    """Shell table of an AOs_cart_data: one shell per AO, {atom, l, nprim, prim0, ao,
    1, component, 1} with the component's index in TREXIO order and primitive
    rows (Z, c N_cart)."""
    aos.sanity_check()
    oi = np.asarray(aos.orbital_indices, dtype=np.int64)
    ex = np.asarray(aos.exponents, dtype=np.float64)
    co = np.asarray(aos.coefficients, dtype=np.float64)
    shells, prims = [], []
    for a in range(aos.num_ao):
        atom, l = int(aos.nucleus_index[a]), int(aos.angular_momentums[a])
        pw = (int(aos.polynominal_order_x[a]), int(aos.polynominal_order_y[a]), int(aos.polynominal_order_z[a]))
        idx = np.nonzero(oi == a)[0]
        p0 = len(prims)
        for zz, cc in zip(ex[idx], co[idx]):
            prims.append((zz, cc * cartesian_norm(l, zz, *pw)))
        shells.append((atom, l, len(idx), p0, a, 1, cartesian_orders(l).index(pw), 1))
    if any(shells[i][0] > shells[i + 1][0] for i in range(len(shells) - 1)):
        raise ValueError("the AOs must be grouped by nucleus")
    return np.ascontiguousarray(np.array(shells, dtype=np.int32)), np.ascontiguousarray(np.array(prims, dtype=np.float64))


def _ion_ion(pos, z):
    e = 0.0
    for i in range(len(z)):
        for j in range(i + 1, len(z)):
            e += z[i] * z[j] / np.linalg.norm(pos[i] - pos[j])
    return e


def system_desc(ham: Hamiltonian_data, Nv: int = 6, non_local_move: str = "tmove"):
    """(jqmc_system_desc, arrays it points into, sizes) for one Hamiltonian_data
    (jqmc/hamiltonians.py:83); the arrays must outlive the descriptor."""
    ham.sanity_check()
    st = ham.structure_data
    g = ham.wavefunction_data.geminal_data
    if g.num_electron_up != g.num_electron_dn:
        raise NotImplementedError("open-shell geminals (N_up != N_dn) are not supported by the walker kernels")
    n_up, n_dn = g.num_electron_up, g.num_electron_dn
    aos, lam_p, _ = g.ao_basis_lambda()
    keep = {}
    keep["pos"] = np.ascontiguousarray(st.positions, dtype=np.float64)
    coul = ham.coulomb_potential_data
    keep["zeff"] = np.ascontiguousarray(coul.effective_charges, dtype=np.float64)
    keep["dsh"], keep["dpr"] = pack_basis(aos)
    keep["lam"] = np.ascontiguousarray(lam_p, dtype=np.float64)
    A = aos.num_ao
    jd = ham.wavefunction_data.jastrow_data
    d = _lib.SystemDesc()
    d.natom, d.n_up, d.n_dn = st.natom, n_up, n_dn
    d.atom_pos = _ptr(keep["pos"], C.c_double)
    d.atom_zeff = _ptr(keep["zeff"], C.c_double)
    d.det = _lib.BasisDesc(len(keep["dsh"]), A, len(keep["dpr"]), _ptr(keep["dsh"], C.c_int32), _ptr(keep["dpr"], C.c_double))
    d.lambda_ = _ptr(keep["lam"], C.c_double)
    j1 = jd.jastrow_one_body_data
    if j1 is not None:
        keep["j1z"] = np.ascontiguousarray(j1.effective_charges, dtype=np.float64)
        d.has_j1, d.j1_type, d.j1_param = 1, {"exp": 0, "pade": 1}[j1.jastrow_1b_type], float(j1.jastrow_1b_param)
        d.j1_zeff = _ptr(keep["j1z"], C.c_double)
    j2 = jd.jastrow_two_body_data
    if j2 is not None:
        d.has_j2, d.j2_type, d.j2_param = 1, {"pade": 0, "exp": 1}[j2.jastrow_2b_type], float(j2.jastrow_2b_param)
    j3 = jd.jastrow_three_body_data
    A3 = 0
    if j3 is not None:
        keep["jsh"], keep["jpr"] = pack_basis(j3.orb_data)
        keep["j3m"] = np.ascontiguousarray(j3.j_matrix, dtype=np.float64)
        A3 = j3.orb_num
        d.has_j3 = 1
        d.j3 = _lib.BasisDesc(len(keep["jsh"]), A3, len(keep["jpr"]), _ptr(keep["jsh"], C.c_int32), _ptr(keep["jpr"], C.c_double))
        d.j3_matrix = _ptr(keep["j3m"], C.c_double)
    if coul.ecp_flag:
        M = st.natom
        chan = np.zeros((M, _lib.ECP_SLOTS, 2), dtype=np.int32)
        terms = []
        for atom in range(M):
            for slot in range(_lib.ECP_SLOTS):
                chan[atom, slot, 0] = len(terms)
                for (a, l, ex, co, pw) in zip(coul.nucleus_index, coul.ang_moms, coul.exponents, coul.coefficients, coul.powers):
                    if a == atom and l == slot and co != 0.0:
                        terms.append((co, pw, ex))
                chan[atom, slot, 1] = len(terms) - chan[atom, slot, 0]
        keep["maxl1"] = np.ascontiguousarray(coul.max_ang_mom_plus_1, dtype=np.int32)
        keep["chan"] = np.ascontiguousarray(chan)
        keep["terms"] = np.ascontiguousarray(np.array(terms, dtype=np.float64).reshape(-1, 3))
        w, pts = ECP_MESHES[Nv]
        keep["mw"] = np.ascontiguousarray(w, dtype=np.float64)
        keep["mp"] = np.ascontiguousarray(pts, dtype=np.float64)
        d.ecp_flag = 1
        d.ecp_maxl1 = _ptr(keep["maxl1"], C.c_int32)
        d.ecp_chan = _ptr(keep["chan"], C.c_int32)
        d.ecp_nterm = len(keep["terms"])
        d.ecp_terms = _ptr(keep["terms"], C.c_double)
        d.nv = Nv
        d.mesh_points = _ptr(keep["mp"], C.c_double)
        d.mesh_weights = _ptr(keep["mw"], C.c_double)
    d.ion_ion = _ion_ion(keep["pos"], keep["zeff"])
    if non_local_move not in _lib.NONLOCAL_MOVES:
        raise NotImplementedError(f"non_local_move={non_local_move!r}: 'tmove' or 'dltmove'")
    d.nonlocal_move = _lib.NONLOCAL_MOVES[non_local_move]
    return d, keep, {"n_up": n_up, "n_dn": n_dn, "A": A, "A3": A3}


class GpuSystem:
    """Device copy of one Hamiltonian_data (jqmc/hamiltonians.py:83) for the walker kernels."""

    def __init__(self, ham: Hamiltonian_data, Nv: int = 6, device: int | None = None, non_local_move: str = "tmove"):
        if not torch.cuda.is_available():
            raise _lib.JqmcError("no CUDA device: the walker path runs only on the GPU")
        self.ham = ham
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        L = _lib.lib()
        d, keep, info = system_desc(ham, Nv, non_local_move)
        self.non_local_move = non_local_move
        self.n_up, self.n_dn = info["n_up"], info["n_dn"]
        self.N = self.n_up + self.n_dn
        self.A, self.A3 = info["A"], info["A3"]
        self.ion_ion = d.ion_ion
        self.Nv = Nv
        handle = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(L.jqmc_system_create(C.byref(d), C.byref(handle)), "jqmc_system_create")
        self.handle = handle
        self._keep = keep
        self._desc = d

    def close(self):
        if getattr(self, "handle", None):
            _lib.lib().jqmc_system_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def walker_bytes(self, precision: str = "fp64") -> int:
        return int(_lib.lib().jqmc_walker_bytes(self.handle, PRECISIONS[precision]))

    def ao_vgl(self, points: torch.Tensor, basis: int = 0) -> torch.Tensor:
        """(5, nao, P) value/grad/lap of the geminal (0) or J3 (1) basis at points (P, 3)."""
        pts = points.to(self.device, torch.float64).contiguous()
        nao = self.A if basis == 0 else self.A3
        out = torch.empty((5, nao, pts.shape[0]), dtype=torch.float64, device=self.device)
        _lib.check(_lib.lib().jqmc_ao_vgl(self.handle, basis, C.c_void_p(pts.data_ptr()), pts.shape[0],
                                          C.c_void_p(out.data_ptr()), self.stream), "jqmc_ao_vgl")
        return out


class WalkerSet:
    """Per-walker state tensors (layout of jqmc_walkers in include/jqmc_gpu.h).

    precision "fp64": every table double (the plain drop-in);
    precision "mixed": G, G^-1, T tables and the J3 field in float, rebuilt in
    double from the positions by ``init`` / ``rebuild`` (an FP64 scratch of
    2 n A doubles per walker is held for that rebuild, and every build writes
    the tables' low float parts to ``tlo``); the block energy right after a
    build reads the FP64-accurate tables (T_hi + T_lo, h_hi + h_lo) with the
    electron terms and the heavy electrons' ECP elements in FP64 and the other
    mesh ratios in compensated float, and the walkers whose mesh ratios cancel
    strongly (factor above ``_lib.FAST_ENERGY_CANCEL``) are recomputed in FP64;
    precision "mixed_fast_energy": as "mixed" without that recompute."""

    def __init__(self, system: GpuSystem, r_up, r_dn, precision: str = "fp64", scratch: torch.Tensor | None = None):
        self.sys = system
        self.precision = precision
        dev = system.device
        r_up = torch.as_tensor(np.asarray(r_up), dtype=torch.float64)
        r_dn = torch.as_tensor(np.asarray(r_dn), dtype=torch.float64)
        W = r_up.shape[0]
        n, N, A, A3 = system.n_up, system.N, system.A, system.A3
        tdt = torch.float64 if precision == "fp64" else torch.float32
        self.nwalk = W
        self.r = torch.cat([r_up, r_dn], dim=1).to(dev).contiguous()
        self.G = torch.empty((W, n, n), dtype=tdt, device=dev)
        self.Ginv = torch.empty_like(self.G)
        self.Tup = torch.empty((W, n, A), dtype=tdt, device=dev)
        self.Tdn = torch.empty_like(self.Tup)
        self.h3 = torch.zeros((W, N, max(A3, 1)), dtype=tdt, device=dev)
        self.dphi = torch.empty((W, N, 4, A), dtype=tdt, device=dev)
        self.dphi3 = torch.empty((W, N, 5, max(A3, 1)), dtype=tdt, device=dev)
        self.ecache = torch.zeros((W, N + 1, _lib.ECACHE_STRIDE), dtype=torch.float64, device=dev)
        self.status = torch.zeros(W, dtype=torch.int32, device=dev)
        if precision != "fp64":
            self.scratch = scratch if scratch is not None else torch.empty((W, 2, n, A), dtype=torch.float64, device=dev)
            M = len(system._keep["pos"])
            big = N * (M + N) * 3 * 4 > 64 * 1024
            self.dcache = torch.empty((W, N * (M + N) * 3), dtype=torch.float32, device=dev) if big else None
            # low parts of the FP64-accurate T tables and J3 field, written by every
            # build and read by the block energy while no move has changed the
            # tables (fresh)
            self.tlo = torch.empty((W, 2 * n * A + N * A3), dtype=torch.float32, device=dev)
        else:
            self.scratch = None
            self.dcache = None
            self.tlo = None
        self.fresh = False
        self.init()

    @classmethod
    def empty_like(cls, other: "WalkerSet") -> "WalkerSet":
        obj = cls.__new__(cls)
        obj.sys = other.sys
        obj.nwalk = other.nwalk
        obj.precision = other.precision
        for name in ("r", "G", "Ginv", "Tup", "Tdn", "h3", "dphi", "dphi3", "ecache", "status"):
            setattr(obj, name, torch.empty_like(getattr(other, name)))
        obj.scratch = other.scratch   # the rebuild scratch is shared: it holds no state between calls
        obj.dcache = other.dcache     # so are the displacement caches (rebuilt every projection step)
        obj.tlo = other.tlo           # and the low table parts (valid only from a build to the next move)
        obj.fresh = False
        return obj

    def desc(self, tlo: bool = False) -> _lib.Walkers:
        """The C descriptor; ``tlo`` passes the low table parts (builds write them,
        the block energy reads them while the tables are fresh)."""
        d = _lib.Walkers()
        d.nwalk = self.nwalk
        d.precision = PRECISIONS[self.precision]
        for name in ("r", "G", "Ginv", "Tup", "Tdn", "h3", "dphi", "dphi3", "ecache", "status"):
            setattr(d, name, C.c_void_p(getattr(self, name).data_ptr()))
        d.scratch = C.c_void_p(self.scratch.data_ptr()) if self.scratch is not None else None
        d.dcache = C.c_void_p(self.dcache.data_ptr()) if self.dcache is not None else None
        d.tlo = C.c_void_p(self.tlo.data_ptr()) if (tlo and self.tlo is not None) else None
        return d

    @property
    def r_up(self):
        return self.r[:, : self.sys.n_up]

    @property
    def r_dn(self):
        return self.r[:, self.sys.n_up:]

    def init(self):
        d = self.desc(tlo=True)
        _lib.check(_lib.lib().jqmc_walker_init(self.sys.handle, C.byref(d), self.sys.stream), "jqmc_walker_init")
        self.fresh = True

    def rebuild(self):
        """FP64 rebuild of G, G^-1 (+ one refinement step), T and the J3 field from
        the positions; the exact per-electron caches are kept."""
        d = self.desc(tlo=True)
        _lib.check(_lib.lib().jqmc_lu_rebuild_refine(self.sys.handle, C.byref(d), self.sys.stream), "jqmc_lu_rebuild_refine")
        self.fresh = True

    def dlnpsi_dparam(self, lam: bool = True):
        """Raw per-walker derivative blocks of ln|psi| (FP64 walkers): (d_j1 (W,),
        d_j2 (W,), d_j3 (W, A3, A3+1) or None, d_lambda_AO (W, A, A) or None)."""
        dev = self.sys.device
        W, n, A, A3 = self.nwalk, self.sys.n_up, self.sys.A, self.sys.A3
        j1 = torch.empty(W, dtype=torch.float64, device=dev)
        j2 = torch.empty_like(j1)
        j3 = torch.empty((W, A3, A3 + 1), dtype=torch.float64, device=dev) if A3 else None
        dl = torch.empty((W, A, A), dtype=torch.float64, device=dev) if lam else None
        work = torch.empty((W, 2, n, A), dtype=torch.float64, device=dev) if lam else None
        ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        d = self.desc()
        _lib.check(_lib.lib().jqmc_dlnpsi_dparam(self.sys.handle, C.byref(d), ptr(j1), ptr(j2), ptr(j3), ptr(dl), ptr(work),
                                                 self.sys.stream), "jqmc_dlnpsi_dparam")
        return j1, j2, j3, dl

    def log_psi(self):
        dev = self.sys.device
        ld = torch.empty(self.nwalk, dtype=torch.float64, device=dev)
        sg = torch.empty_like(ld)
        jj = torch.empty_like(ld)
        d = self.desc()
        _lib.check(_lib.lib().jqmc_log_psi(self.sys.handle, C.byref(d), C.c_void_p(ld.data_ptr()), C.c_void_p(sg.data_ptr()),
                                           C.c_void_p(jj.data_ptr()), self.sys.stream), "jqmc_log_psi")
        return ld, sg, jj

    def electron_terms(self) -> torch.Tensor:
        """(W, N, 9) per electron: grad ln|det| (3), lap ln|det|, grad J (3), lap J,
        kinetic element T_e (FP64 walkers; jqmc_electron_terms)."""
        out = torch.empty((self.nwalk, self.sys.N, 9), dtype=torch.float64, device=self.sys.device)
        d = self.desc()
        _lib.check(_lib.lib().jqmc_electron_terms(self.sys.handle, C.byref(d), C.c_void_p(out.data_ptr()), self.sys.stream),
                   "jqmc_electron_terms")
        return out

    def kinetic_mesh(self, angles: torch.Tensor, alat: float) -> torch.Tensor:
        """(W, N, 6) discretised kinetic elements of the six rotated lattice moves of
        every electron (FP64 walkers; jqmc_kinetic_mesh)."""
        out = torch.empty((self.nwalk, self.sys.N, 6), dtype=torch.float64, device=self.sys.device)
        ang = angles.to(self.sys.device, torch.float64).contiguous()
        d = self.desc()
        _lib.check(_lib.lib().jqmc_kinetic_mesh(self.sys.handle, C.byref(d), C.c_void_p(ang.data_ptr()), float(alat),
                                                C.c_void_p(out.data_ptr()), self.sys.stream), "jqmc_kinetic_mesh")
        return out

    def vmc_sweep(self, idraw: torch.Tensor, fdraw: torch.Tensor, Dt: float, eps_AS: float, accept: torch.Tensor):
        K = idraw.shape[1]
        self.fresh = False
        d = self.desc()
        _lib.check(_lib.lib().jqmc_vmc_sweep(self.sys.handle, C.byref(d), K, C.c_void_p(idraw.data_ptr()),
                                             C.c_void_p(fdraw.data_ptr()), float(Dt), float(eps_AS),
                                             C.c_void_p(accept.data_ptr()), self.sys.stream), "jqmc_vmc_sweep")

    def vmc_measure(self, angles: torch.Tensor, eps_AS: float):
        eL = torch.empty(self.nwalk, dtype=torch.float64, device=self.sys.device)
        wL = torch.empty_like(eL)
        d = self.desc()
        _lib.check(_lib.lib().jqmc_vmc_measure(self.sys.handle, C.byref(d), C.c_void_p(angles.data_ptr()), float(eps_AS),
                                               C.c_void_p(eL.data_ptr()), C.c_void_p(wL.data_ptr()), self.sys.stream),
                   "jqmc_vmc_measure")
        return eL, wL

    def lrdmc_project(self, draws: torch.Tensor, alat: float, E_scf: float, w: torch.Tensor):
        K = draws.shape[1]
        self.fresh = False
        d = self.desc()
        _lib.check(_lib.lib().jqmc_lrdmc_project(self.sys.handle, C.byref(d), K, C.c_void_p(draws.data_ptr()), float(alat),
                                                 float(E_scf), C.c_void_p(w.data_ptr()), self.sys.stream), "jqmc_lrdmc_project")

    def lrdmc_project_t(self, draws: torch.Tensor, alat: float, w: torch.Tensor, tau_left: torch.Tensor,
                        nsteps: torch.Tensor, eL: torch.Tensor):
        """GFMC_t projections until tau_left is spent or the K draws (W, K, 5) are used."""
        self.fresh = False
        K = draws.shape[1]
        d = self.desc()
        _lib.check(_lib.lib().jqmc_lrdmc_project_t(self.sys.handle, C.byref(d), K, C.c_void_p(draws.data_ptr()), float(alat),
                                                   C.c_void_p(w.data_ptr()), C.c_void_p(tau_left.data_ptr()),
                                                   C.c_void_p(nsteps.data_ptr()), C.c_void_p(eL.data_ptr()),
                                                   self.sys.stream), "jqmc_lrdmc_project_t")

    def lrdmc_energy(self, last_draw: torch.Tensor, alat: float):
        """(e_L, V_diag) with one rotation per walker: last_draw holds 4 doubles per
        walker (three Euler angles and the unused move uniform of a GFMC_n draw)."""
        last_draw = last_draw.contiguous()
        if last_draw.dtype != torch.float64 or last_draw.numel() != 4 * self.nwalk:
            raise ValueError(f"lrdmc_energy needs 4 float64 draws per walker; got {tuple(last_draw.shape)} {last_draw.dtype}")
        eL = torch.empty(self.nwalk, dtype=torch.float64, device=self.sys.device)
        vd = torch.empty_like(eL)
        d = self.desc(tlo=self.fresh)
        _lib.check(_lib.lib().jqmc_lrdmc_energy(self.sys.handle, C.byref(d), C.c_void_p(last_draw.data_ptr()), float(alat),
                                                C.c_void_p(eL.data_ptr()), C.c_void_p(vd.data_ptr()), self.sys.stream),
                   "jqmc_lrdmc_energy")
        return eL, vd

    def energy_cancellation(self) -> torch.Tensor:
        """Per-walker cancellation factors of the compensated block energy's mesh
        ratios, as left by the last ``lrdmc_energy`` in precision "mixed" (the
        first double of each walker's rebuild scratch; overwritten by the next
        rebuild).  Walkers above ``_lib.FAST_ENERGY_CANCEL`` were recomputed in FP64."""
        if self.precision != "mixed":
            raise ValueError("cancellation factors are kept in precision 'mixed' only")
        return self.scratch.view(self.nwalk, -1)[:, 0].clone()

    def gather_from(self, src: "WalkerSet", chosen: torch.Tensor):
        self.fresh = False
        ds, dd = src.desc(), self.desc()
        _lib.check(_lib.lib().jqmc_walker_gather(self.sys.handle, C.byref(ds), C.byref(dd), C.c_void_p(chosen.data_ptr()),
                                                 self.sys.stream), "jqmc_walker_gather")


def branch_comb(w: torch.Tensor, zeta: float, chosen: torch.Tensor | None = None, scratch: torch.Tensor | None = None):
    """Comb reconfiguration indices on the device (jqmc_gfmc.py:2010-2090)."""
    W = w.shape[0]
    if chosen is None:
        chosen = torch.empty(W, dtype=torch.int32, device=w.device)
    if scratch is None:
        scratch = torch.empty(W, dtype=torch.float64, device=w.device)
    stream = C.c_void_p(torch.cuda.current_stream(w.device).cuda_stream)
    _lib.check(_lib.lib().jqmc_branch_comb(W, C.c_void_p(w.data_ptr()), float(zeta), C.c_void_p(chosen.data_ptr()),
                                           C.c_void_p(scratch.data_ptr()), stream), "jqmc_branch_comb")
    return chosen
