"""ctypes binding of libjqmc_gpu.so (the C ABI declared in include/jqmc_gpu.h).

The library is built in-tree by ``jqmc_gb300.build.build()`` (nvcc, sm_103a).
Loading fails loudly when the shared object is missing: there is no CPU path.
"""

from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libjqmc_gpu.so")

JQMC_OK = 0
ERRORS = {-1: "bad argument", -2: "size above a compiled maximum", -3: "CUDA runtime error", -4: "shared-memory footprint too large"}
ECP_SLOTS = 8
ECACHE_STRIDE = 24
MAX_NUP = 128

ST_SINGULAR, ST_ZERO_RATIO, ST_NAN = 1, 2, 4

i32, i64, f64 = C.c_int32, C.c_int64, C.c_double
pi32, pf64, vp = C.POINTER(C.c_int32), C.POINTER(C.c_double), C.c_void_p


class BasisDesc(C.Structure):
    _fields_ = [("nshell", i32), ("nao", i32), ("nprim", i32), ("shells", pi32), ("prims", pf64)]


class SystemDesc(C.Structure):
    _fields_ = [
        ("natom", i32), ("n_up", i32), ("n_dn", i32),
        ("atom_pos", pf64), ("atom_zeff", pf64),
        ("det", BasisDesc), ("lambda_", pf64),
        ("has_j1", i32), ("j1_type", i32), ("j1_param", f64), ("j1_zeff", pf64),
        ("has_j2", i32), ("j2_type", i32), ("j2_param", f64),
        ("has_j3", i32), ("j3", BasisDesc), ("j3_matrix", pf64),
        ("ecp_flag", i32), ("ecp_maxl1", pi32), ("ecp_chan", pi32), ("ecp_nterm", i32), ("ecp_terms", pf64),
        ("nv", i32), ("mesh_points", pf64), ("mesh_weights", pf64),
        ("ion_ion", f64), ("nonlocal_move", i32),
    ]


class Walkers(C.Structure):
    _fields_ = [("nwalk", i32), ("precision", i32), ("r", vp), ("G", vp), ("Ginv", vp), ("Tup", vp), ("Tdn", vp), ("h3", vp),
                ("dphi", vp), ("dphi3", vp), ("ecache", vp), ("scratch", vp), ("dcache", vp), ("status", vp),
                ("tlo", vp)]


PREC_FP64, PREC_MIXED, PREC_MIXED_FASTE = 0, 1, 2
NONLOCAL_MOVES = {"tmove": 0, "dltmove": 1}   # JQMC_NONLOCAL_TMOVE, JQMC_NONLOCAL_DLTMOVE
FAST_ENERGY_CANCEL = 10.0   # JQMC_FAST_ENERGY_CANCEL: cancellation factor above which a block energy is recomputed in FP64


class JqmcError(RuntimeError):
    pass


_lib = None


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise JqmcError(f"{LIB_PATH} is missing: run jqmc_gb300.build.build() (nvcc, sm_103a) first; "
                            "the walker path has no CPU fallback")
        L = C.CDLL(LIB_PATH)
        L.jqmc_system_create.argtypes = [C.POINTER(SystemDesc), C.POINTER(vp)]
        L.jqmc_system_destroy.argtypes = [vp]
        L.jqmc_walker_bytes.argtypes = [vp, i32]
        L.jqmc_walker_bytes.restype = i64
        L.jqmc_ao_vgl.argtypes = [vp, i32, vp, i64, vp, vp]
        L.jqmc_walker_init.argtypes = [vp, C.POINTER(Walkers), vp]
        L.jqmc_lu_rebuild_refine.argtypes = [vp, C.POINTER(Walkers), vp]
        L.jqmc_dlnpsi_dparam.argtypes = [vp, C.POINTER(Walkers), vp, vp, vp, vp, vp, vp]
        L.jqmc_lrdmc_project_t.argtypes = [vp, C.POINTER(Walkers), i32, vp, f64, vp, vp, vp, vp, vp]
        L.jqmc_batch_create.argtypes = [i32, C.POINTER(vp), C.POINTER(Walkers), C.POINTER(vp)]
        L.jqmc_batch_destroy.argtypes = [vp]
        L.jqmc_batch_walkers.argtypes = [vp]
        L.jqmc_vmc_sweep_batch.argtypes = [vp, i32, vp, vp, f64, f64, vp, i32, i32, vp]
        L.jqmc_batch_rebuild.argtypes = [vp, i32, vp]
        L.jqmc_dlnpsi_dR.argtypes = [vp, C.POINTER(Walkers), vp, vp]
        L.jqmc_electron_terms.argtypes = [vp, C.POINTER(Walkers), vp, vp]
        L.jqmc_kinetic_mesh.argtypes = [vp, C.POINTER(Walkers), vp, f64, vp, vp]
        L.jqmc_log_psi.argtypes = [vp, C.POINTER(Walkers), vp, vp, vp, vp]
        L.jqmc_vmc_sweep.argtypes = [vp, C.POINTER(Walkers), i32, vp, vp, f64, f64, vp, vp]
        L.jqmc_vmc_measure.argtypes = [vp, C.POINTER(Walkers), vp, f64, vp, vp, vp]
        L.jqmc_lrdmc_project.argtypes = [vp, C.POINTER(Walkers), i32, vp, f64, f64, vp, vp]
        L.jqmc_lrdmc_energy.argtypes = [vp, C.POINTER(Walkers), vp, f64, vp, vp, vp]
        L.jqmc_branch_comb.argtypes = [i32, vp, f64, vp, vp, vp]
        L.jqmc_walker_gather.argtypes = [vp, C.POINTER(Walkers), C.POINTER(Walkers), vp, vp]
        L.jqmc_probe_fp64.argtypes = [i64, i32, vp, pf64, vp]
        L.jqmc_branch_comb_noalloc.argtypes = [i32, vp, f64, vp, vp]
        L.jqmc_probe_fp32.argtypes = [i64, i32, vp, pf64, vp]
        L.jqmc_tensor_core_rebuild.argtypes = [vp]
        for name in ("jqmc_probe_fp64", "jqmc_system_create", "jqmc_system_destroy", "jqmc_ao_vgl", "jqmc_walker_init", "jqmc_log_psi",
                     "jqmc_vmc_sweep", "jqmc_vmc_measure", "jqmc_lrdmc_project", "jqmc_lrdmc_energy",
                     "jqmc_branch_comb", "jqmc_walker_gather", "jqmc_branch_comb_noalloc", "jqmc_probe_fp32",
                     "jqmc_lu_rebuild_refine", "jqmc_dlnpsi_dparam", "jqmc_lrdmc_project_t", "jqmc_batch_create",
                     "jqmc_batch_destroy", "jqmc_batch_walkers", "jqmc_vmc_sweep_batch", "jqmc_batch_rebuild",
                     "jqmc_dlnpsi_dR", "jqmc_electron_terms", "jqmc_kinetic_mesh", "jqmc_tensor_core_rebuild"):
            getattr(L, name).restype = C.c_int
        _lib = L
    return _lib


def check(rc: int, what: str) -> None:
    if rc != JQMC_OK:
        raise JqmcError(f"{what} failed: {ERRORS.get(rc, rc)} (code {rc})")


EXPORTED = ("jqmc_system_create", "jqmc_system_destroy", "jqmc_walker_bytes", "jqmc_ao_vgl", "jqmc_walker_init",
            "jqmc_log_psi", "jqmc_vmc_sweep", "jqmc_vmc_measure", "jqmc_lrdmc_project", "jqmc_lrdmc_energy",
            "jqmc_branch_comb", "jqmc_walker_gather", "jqmc_probe_fp64", "jqmc_branch_comb_noalloc", "jqmc_probe_fp32",
            "jqmc_lu_rebuild_refine", "jqmc_dlnpsi_dparam", "jqmc_lrdmc_project_t", "jqmc_batch_create",
            "jqmc_batch_destroy", "jqmc_batch_walkers", "jqmc_vmc_sweep_batch", "jqmc_batch_rebuild",
            "jqmc_dlnpsi_dR", "jqmc_electron_terms", "jqmc_kinetic_mesh", "jqmc_tensor_core_rebuild")
