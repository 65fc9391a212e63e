"""Algorithmic work model of the walker kernels (for roofline accounting).

FP64 operation counts per unit of work, counted from the algorithm the kernels
implement (not from profiler counters):  FMA = 2, add / sub / mul / div /
sqrt / compare = 1, and one FP64 exponential = EXP_FLOPS (a range reduction
plus a degree-10 polynomial in FP64 is about 20 operations; this is the
convention, stated with every number that uses it).

Bytes per unit are the walker-state bytes a step must read and write in HBM.
"""

from __future__ import annotations

import numpy as np

EXP_FLOPS = 20.0


def _sh_flops(l: int) -> float:
    return 0.0 if l < 2 else 4.0 * (2 * l + 1)


def ao_point_flops(shells: np.ndarray) -> float:
    """Value of every AO of a packed basis at one point, dotted with a vector."""
    f = 0.0
    for sh in shells:
        l, np_, nm = int(sh[1]), int(sh[2]), int(sh[5])
        f += 8 + np_ * (3 + EXP_FLOPS) + _sh_flops(l) + nm * 3
    return f


def ao_vgl_flops(shells: np.ndarray) -> float:
    f = 0.0
    for sh in shells:
        l, np_, nm = int(sh[1]), int(sh[2]), int(sh[5])
        f += 10 + np_ * (8 + EXP_FLOPS) + 4 * _sh_flops(l) + nm * 20
    return f


def lrdmc_step_split(gs, ecp_fraction: float):
    """(mesh + move ops, electron-term ops) of one projection of one walker: the
    first part runs in float in the mixed form, the second stays in double."""
    keep = gs._keep
    N, n, A, M = gs.N, gs.n_up, gs.A, len(keep["pos"])
    A3 = gs.A3
    det_p = ao_point_flops(keep["dsh"])
    j3_p = ao_point_flops(keep["jsh"]) if A3 else 0.0
    ratio = det_p + j3_p + M * (8 + EXP_FLOPS + 6) + N * 12 + EXP_FLOPS + 3
    mesh = 6 * N * (ratio + 8) + gs.Nv * N * ecp_fraction * (ratio + 40 + 2 * EXP_FLOPS)
    move = 2 * (det_p + j3_p) + 4 * A * n + 4 * n * n + 2 * A * A + 6 * A * n + 4 * n * n + 4 * A3 * A3 + N * A3
    elec = N * (ao_vgl_flops(keep["dsh"]) + (ao_vgl_flops(keep["jsh"]) if A3 else 0.0) + M * (30 + EXP_FLOPS) + N * 27)
    sums = 6 * N * 6 + N * N * 5 + N * M * (12 + EXP_FLOPS) + 12 * N * 3
    return mesh + move, elec + sums


def lrdmc_step_flops(gs, ecp_fraction: float) -> float:
    """FP64 operations of one GFMC_n projection of one walker (jqmc_gb300 kernels)."""
    keep = gs._keep
    N, n, A, M = gs.N, gs.n_up, gs.A, len(keep["pos"])
    A3 = gs.A3
    det_p = ao_point_flops(keep["dsh"])
    j3_p = ao_point_flops(keep["jsh"]) if A3 else 0.0
    ratio = det_p + j3_p + M * (8 + EXP_FLOPS + 6) + N * 12 + EXP_FLOPS + 3
    kin_mesh = 6 * N * (ratio + 8)
    ecp_mesh = gs.Nv * N * ecp_fraction * (ratio + 40 + 2 * EXP_FLOPS)
    elec = N * (ao_vgl_flops(keep["dsh"]) + (ao_vgl_flops(keep["jsh"]) if A3 else 0.0) + M * (30 + EXP_FLOPS) + N * 27)
    sums = 6 * N * 6 + N * N * 5 + N * M * (12 + EXP_FLOPS)
    move = 2 * (det_p + j3_p) + 4 * A * n + 4 * n * n + 2 * A * A + 6 * A * n + 4 * n * n + 4 * A3 * A3 + N * A3
    cdf = 12 * N * 3
    return kin_mesh + ecp_mesh + elec + sums + move + cdf


def lrdmc_step_bytes(gs) -> float:
    """HBM bytes of one projection of one walker: the rank-1 updates read and write
    T_up, T_dn (2 n A doubles each way), the J3 field (N A3), and G, G^-1 once per
    block (amortised, ignored)."""
    return 8.0 * (2 * 2 * gs.n_up * gs.A + 2 * gs.N * max(gs.A3, 0))
