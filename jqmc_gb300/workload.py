"""Algorithmic work model of the walker kernels (for roofline accounting).

Operation counts per unit of work, counted from the algorithm the kernels
implement (not from profiler counters):  FMA = 2, add / sub / mul / div /
sqrt / compare = 1.  An exponential counts as the instructions that evaluate
it: EXP_FLOPS = 20 in FP64 (a software range reduction and polynomial), and
EXP_F32 = 2 in the float kernels (one multiply by log2 e and one SFU ex2: the
float mesh uses the fast intrinsic).  The convention is stated with every
number that uses it.

Bytes per unit are the walker-state bytes a step must read and write in HBM.
"""

from __future__ import annotations

import numpy as np

EXP_FLOPS = 20.0
EXP_F32 = 2.0


def _sh_flops(l: int) -> float:
    return 0.0 if l < 2 else 4.0 * (2 * l + 1)


def ao_point_flops(shells: np.ndarray, exp_flops: float = EXP_FLOPS) -> float:
    """Value of every AO of a packed basis at one point, dotted with a vector."""
    f = 0.0
    for sh in shells:
        l, np_, nm = int(sh[1]), int(sh[2]), int(sh[5])
        f += 8 + np_ * (3 + exp_flops) + _sh_flops(l) + nm * 3
    return f


def ao_vgl_flops(shells: np.ndarray) -> float:
    f = 0.0
    for sh in shells:
        l, np_, nm = int(sh[1]), int(sh[2]), int(sh[5])
        f += 10 + np_ * (8 + EXP_FLOPS) + 4 * _sh_flops(l) + nm * 20
    return f


def _step_parts(gs, ecp_fraction: float, exp_mesh: float = EXP_FLOPS):
    """Operation counts of one GFMC_n projection of one walker, by phase, as the
    walker kernels execute it (streaming caches: the AO derivative tables and the
    per-electron energy cache are read every step and recomputed only for the
    moved electron)."""
    keep = gs._keep
    N, n, A, M = gs.N, gs.n_up, gs.A, len(keep["pos"])
    A3 = gs.A3
    det_p = ao_point_flops(keep["dsh"], exp_mesh)
    j3_p = ao_point_flops(keep["jsh"], exp_mesh) if A3 else 0.0
    det_v = ao_vgl_flops(keep["dsh"])
    j3_v = ao_vgl_flops(keep["jsh"]) if A3 else 0.0
    # psi(r')/psi(r) at one mesh point: AO values dotted with the T row / J3 field,
    # J1 over nuclei, J2 over electrons, the exponential of the Jastrow difference
    ratio = det_p + j3_p + M * (12 + 2 * exp_mesh) + N * 16 + exp_mesh + 3
    mesh = 6 * N * (ratio + 8) + gs.Nv * N * ecp_fraction * (ratio + 40)
    # electron terms: cached derivative tables dotted with T rows and J3 fields
    elec_dots = N * (2 * (4 * A + 5 * A3) + 40)
    # rank-1 move: AO values at the old and new position, lam^T dphi, T/G/G^-1
    # updates, J3 field update
    move = 2 * (det_p + j3_p) + 2 * A * A + 10 * A * n + 8 * n * n + 2 * A3 * A3 + 2 * N * A3
    # FP64 in both forms: derivative tables of the moved electron, its energy-cache
    # row and the pair updates, the (diag, nondiag) sums and the move choice
    fp64 = det_v + j3_v + M * (30 + EXP_FLOPS) + N * 27 + 6 * N * 6 + gs.Nv * N * 2 + 12 * N * 3
    return mesh, elec_dots, move, fp64


def lrdmc_step_split(gs, ecp_fraction: float):
    """(float part, FP64 part) of one projection of one walker in the mixed form:
    the mesh ratios, the electron-term dots and the rank-1 table updates run in
    float; the moved electron's derivative tables, the energy cache, the sums and
    the move choice stay in double."""
    mesh, elec_dots, move, fp64 = _step_parts(gs, ecp_fraction, EXP_F32)
    return mesh + elec_dots + move, fp64


def lrdmc_step_flops(gs, ecp_fraction: float) -> float:
    """Operations of one GFMC_n projection of one walker (all FP64 in the plain form)."""
    return sum(_step_parts(gs, ecp_fraction))


def lrdmc_step_bytes(gs, table_bytes: int = 8) -> float:
    """HBM bytes of one projection of one walker with tables of `table_bytes`:
    - read: the AO derivative tables of every electron (N 4 A + N 5 A3), the T
      rows (2 n A) and J3 field (N A3) of the electron terms and the mesh, the
      energy cache (8-byte rows of the stride);
    - the rank-1 updates read and write T_up, T_dn (2 n A each way) and the J3
      field (N A3 each way);
    - written: the moved electron's derivative tables (4 A + 5 A3) and cache row.
    G and G^-1 stay in shared memory for the whole block (read and written once
    per block, amortised away)."""
    n, N, A, A3 = gs.n_up, gs.N, gs.A, max(gs.A3, 0)
    tables = (N * 4 * A + N * 5 * A3) + (2 * n * A + N * A3) + 2 * (2 * n * A + N * A3) + (4 * A + 5 * A3)
    return float(table_bytes) * tables + 8.0 * (N + 2) * 24


def rebuild_gemm_flops(gs) -> float:
    """Operations of the rebuild's lambda-GEMM per walker: M_up = Phi_up lambda and
    M_dn = Phi_dn lambda^T, 2 x 2 n A^2 (one product; the split form issues 21
    bf16 slice products per product on the tensor cores)."""
    return 2.0 * 2.0 * gs.n_up * gs.A * gs.A


def dlnpsi_flops(gs, lam: bool = True) -> float:
    """FP64 operations of jqmc_dlnpsi_dparam for one walker: J1 / J2 parameter
    sums, J3 AO values and the A3 x (A3+1) block, and (lam) the AO values of
    every electron, X = G^-T Psi_dn (n^2 A) and the A x A block (n A^2)."""
    keep = gs._keep
    N, n, A, M, A3 = gs.N, gs.n_up, gs.A, len(keep["pos"]), gs.A3
    f = N * M * (12 + EXP_FLOPS) + N * (N - 1) / 2 * 14
    if A3:
        f += N * ao_point_flops(keep["jsh"]) + 2 * N * A3 * A3 + 2 * N * A3
    if lam:
        f += N * ao_point_flops(keep["dsh"]) + 2 * n * n * A + 2 * n * A * A
    return f


def dlnpsi_bytes(gs, lam: bool = True) -> float:
    """HBM bytes of jqmc_dlnpsi_dparam per walker: positions and G^-1 in, the
    blocks out, the Phi / X work rows written and read back."""
    n, A, N, A3 = gs.n_up, gs.A, gs.N, gs.A3
    b = 8.0 * (3 * N + n * n + 2 + A3 * (A3 + 1))
    if lam:
        b += 8.0 * (A * A + 3 * 2 * n * A)
    return b
